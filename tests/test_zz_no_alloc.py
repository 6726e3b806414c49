"""cg_generate_for_box_noalloc: the span mesher for callers that cannot
allocate device memory (graph capture, a foreign allocator owning the GPU, a
per-frame LOD loop).  It runs on a fixed workspace inside the library, so it
must give exactly what the allocating entry point gives -- on two calls in a
row, because the second call reuses the first one's workspace contents.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from cantucci_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def noalloc_mesh(cg, span, shape, res, vcap, icap):
    """One call through the C ABI; returns host copies of the outputs."""
    import torch
    from cantucci_gb300 import _ffi
    verts = torch.zeros((vcap, 7), dtype=torch.float32, device="cuda")
    idx = torch.zeros(icap, dtype=torch.int32, device="cuda")
    counts = torch.full((3,), 0xFFFF, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    _ffi.check(_ffi.load().cg_generate_for_box_noalloc(
        C.byref(span.to_c()), C.byref(shape._cshape()), res, C.c_void_p(verts.data_ptr()), vcap,
        C.c_void_p(idx.data_ptr()), icap, C.c_void_p(counts.data_ptr()),
        C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    nv, nq, status = counts.cpu().numpy().astype(np.int64).tolist()
    return (verts[:nv].cpu().numpy(), idx[:6 * nq].cpu().numpy().view(np.uint32), nv, 6 * nq,
            status)


def allocating_mesh(cg, span, shape, res):
    m = cg.Mesher(0)
    try:
        v, i, nv, ni, _ = m.generate(span, shape, res, strict=False)
        return v[:nv].view(np.float32).reshape(-1, 7), i[:ni], m.last_status
    finally:
        m.close()


def test_noalloc_matches_allocating_entry_point_twice(cg):
    shape = cg.Mandelbulb.classic(15, 2.5)
    spans = [(cg.Span(*W.SPAN_C1), 64)]
    s, _, _, _ = W.batched_spans(32, seed=5)
    spans.append((cg.Span(s[3][:3], s[3][3:]), 32))
    # Two calls in a row, the second on a different span and resolution, so
    # stale workspace contents from the first would show up in the second.
    for span, res in spans:
        v, i, nv, ni, status = noalloc_mesh(cg, span, shape, res, res ** 3, 18 * res ** 3)
        rv, ri, rstatus = allocating_mesh(cg, span, shape, res)
        assert (nv, ni) == (len(rv), len(ri))
        assert status == (1 if rstatus == 3 else 0)
        # Same kernels, same inputs: bit-identical (the tests' tolerance for
        # the mesh index list and for Mandelbulb vertices on one GPU).
        assert np.array_equal(i, ri)
        assert np.array_equal(v.view(np.uint32), rv.view(np.uint32))


def test_noalloc_rejects_large_resolution(cg):
    from cantucci_gb300 import _ffi
    with pytest.raises(_ffi.CantucciError) as e:
        noalloc_mesh(cg, cg.Span(*W.SPAN_C1), cg.Mandelbulb.classic(15, 2.5), 128, 16, 96)
    assert e.value.status == _ffi.CG_EINVAL
    assert "64" in str(e.value)
