"""cg_generate_for_box_noalloc: the span mesher for callers that cannot
allocate device memory (a foreign allocator owning the GPU, a per-frame LOD
loop that cannot take cudaMalloc's synchronisation).  It runs on a fixed
workspace inside the library, so it must give exactly what the allocating
entry point gives -- on two calls in a row, because the second call reuses
the first one's workspace contents.

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


@pytest.mark.parametrize("kind", ["p8", "sphere", "polar"])
def test_noalloc_matches_allocating_entry_point_twice(cg, kind):
    shape = {"p8": lambda: cg.Mandelbulb.classic(15, 2.5),
             "sphere": lambda: cg.Sphere((0.1, -0.05, 0.02), 0.9),
             "polar": lambda: cg.MandelbulbPolar(8.3, 15, 2.5, (0.2, 0.1, 0.0))}[kind]()
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


def test_noalloc_outputs_cut_at_capacity(cg):
    """Outputs smaller than the mesh: the call still returns CG_OK and
    reports the full counts; it writes the first vertex_cap vertices and
    index_cap indices of the full mesh and nothing past them.  The buffers
    are larger than the capacities passed, filled with a sentinel, so a
    write past a capacity would show."""
    import torch
    from cantucci_gb300 import _ffi
    shape = cg.Mandelbulb.classic(15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    res = 32
    fv, fi, nv, ni, _ = noalloc_mesh(cg, span, shape, res, res ** 3, 18 * res ** 3)
    vcap, icap = nv // 3, (ni // 2) - 5
    pad = 4096
    verts = torch.full((vcap + pad, 7), -7.0, dtype=torch.float32, device="cuda")
    idx = torch.full((icap + pad,), -7, dtype=torch.int32, device="cuda")
    counts = torch.zeros(3, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    st = _ffi.load().cg_generate_for_box_noalloc(
        C.byref(span.to_c()), C.byref(shape._cshape()), res, C.c_void_p(verts.data_ptr()), vcap,
        C.c_void_p(idx.data_ptr()), icap, C.c_void_p(counts.data_ptr()),
        C.c_void_p(stream.cuda_stream))
    stream.synchronize()
    assert st == _ffi.CG_OK
    c = counts.cpu().numpy().astype(np.int64)
    assert (int(c[0]), 6 * int(c[1])) == (nv, ni)
    v = verts.cpu().numpy()
    i = idx.cpu().numpy().view(np.uint32)
    assert np.array_equal(v[:vcap].view(np.uint32), fv[:vcap].view(np.uint32))
    assert np.all(v[vcap:] == -7.0)
    # whole quads only: the last partial quad is not written
    done = (icap // 6) * 6
    assert np.array_equal(i[:done], fi[:done])
    assert np.all(idx.cpu().numpy()[done:] == -7)
