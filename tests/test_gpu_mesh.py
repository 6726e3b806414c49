"""GPU span mesher (MeshBuffer::generate_for_box) against goldens and oracle.

Bar: the cell -> vertex-id table and the triangle index list are bit-exact
(P=8 and Sphere); vertex positions/normals/distances, which depend on the
final ln of the corner distances, are compared with the tolerances stated;
the Sphere mesh (no libm at all) is bit-exact everywhere.
"""
import hashlib

import numpy as np
import pytest

from cantucci_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# Central-difference normals subtract two distances that each carry the final
# logf's last-bit difference (CUDA vs glibc); 0.1 degree is the angular bar.
NORMAL_DEG = 0.1


def sha(a) -> bytes:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()


def as7(v):
    return np.ascontiguousarray(v).view(np.float32).reshape(-1, 7)


def angle_deg(a, b):
    a = a / np.linalg.norm(a, axis=1, keepdims=True)
    b = b / np.linalg.norm(b, axis=1, keepdims=True)
    return np.degrees(np.arccos(np.clip(np.sum(a * b, axis=1), -1, 1)))


@pytest.fixture(scope="module")
def mesher(cg):
    m = cg.Mesher(0)
    yield m
    m.close()


def test_c1_topology_matches_golden(cg, golden, mesher):
    s = cg.Mandelbulb.classic(15, 2.5)
    buf, t = cg.MeshBuffer.generate_for_box(cg.Span(*W.SPAN_C1), s, 64, mesher=mesher)
    assert [len(buf.vertices), len(buf.indices)] == golden["c1_counts"].tolist()
    assert (t.vertices, t.faces * 6) == tuple(golden["c1_counts"].tolist())
    assert sha(buf.indices) == golden["c1_indices_sha"].tobytes()
    pts = mesher.last_points().cpu().numpy().astype(np.uint32)
    assert sha(pts) == golden["c1_points_sha"].tobytes()
    assert np.array_equal(buf.indices[:6000], golden["c1_index_head"])
    v = as7(buf.vertices)[::37]
    g = golden["c1_vertex_sample"]
    np.testing.assert_allclose(v[:, :3], g[:, :3], rtol=0, atol=1e-6)
    assert angle_deg(v[:, 3:6], g[:, 3:6]).max() < NORMAL_DEG
    np.testing.assert_allclose(v[:, 6], g[:, 6], rtol=1e-4, atol=1e-7)


def ulp_diff(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def placement_vs_oracle(orc, mesher, a, indices, res, status):
    """The oracle's steps 2-3 (buffer.rs:85-372) fed the GPU's own corner
    distances: the surface cells, the vertex positions (the 12-edge lerps
    and their centroid, buffer.rs:187-250) and the quads follow from the
    distances alone, so they must match bit for bit.  Only the estimator
    calls at the vertex differ, through CUDA's logf against glibc's: the two
    ln r are within 1.82 ulp (CUDA's logf is within 1 ulp, glibc's within
    0.82), and the product by r and the quotient by dr round once more on
    each side (half an ulp each), so the distances at the vertex differ by
    less than (1.82 + 1 + 1) 2^-23 relative, which is under 8 ulp: at most
    7; 99% must be within 2 ulp.  The six-sample normal within 0.1 degree
    for 99.9%."""
    d = mesher.last_dists().cpu().numpy()
    ref = orc.mesh_from_dists(orc.mandelbulb(8, 15, 2.5), np.array(W.SPAN_C1).ravel(), res, d,
                              vcap=len(a) + 1, icap=len(indices) + 1)
    assert ref["rc"] == status
    assert ref["nv"] == len(a) and np.array_equal(indices, ref["indices"])
    b = as7(ref["vertices"])
    assert np.array_equal(a[:, :3].view(np.uint32), b[:, :3].view(np.uint32))
    fin = np.isfinite(b[:, 6])
    assert np.array_equal(np.isfinite(a[:, 6]), fin)
    du = ulp_diff(a[fin, 6], b[fin, 6])
    assert du.max() <= 7 and np.mean(du <= 2) >= 0.99, (du.max(), np.mean(du <= 2))
    ok = np.all(np.isfinite(b[:, 3:6]), axis=1)
    ang = angle_deg(a[ok, 3:6], b[ok, 3:6])
    assert np.mean(ang < NORMAL_DEG) >= 0.999, (np.mean(ang < NORMAL_DEG), ang.max())


def test_c1_vertices_vs_oracle(cg, orc, mesher):
    s = cg.Mandelbulb.classic(15, 2.5)
    buf, _ = cg.MeshBuffer.generate_for_box(cg.Span(*W.SPAN_C1), s, 64, mesher=mesher)
    ref = orc.generate_for_box(orc.mandelbulb(8, 15, 2.5), np.array(W.SPAN_C1).ravel(), 64)
    assert np.array_equal(buf.indices, ref["indices"])
    placement_vs_oracle(orc, mesher, as7(buf.vertices), buf.indices, 64, orc.ORC_OK)


@pytest.mark.parametrize("n", range(6))
def test_small_spans_match_golden(cg, golden, mesher, n):
    P, it, rr = golden["small%d_meta" % n].tolist()
    sp = golden["small%d_span" % n]
    buf, _ = cg.MeshBuffer.generate_for_box(cg.Span(sp[:3], sp[3:]), cg.Mandelbulb(P, it, 2.5), rr,
                                            mesher=mesher)
    pts = mesher.last_points().cpu().numpy().astype(np.uint32)
    d = mesher.last_dists().cpu().numpy()
    gd = golden["small%d_dists" % n]
    if P == 8:
        assert np.array_equal(pts, golden["small%d_points" % n])
        assert np.array_equal(buf.indices, golden["small%d_indices" % n])
    else:
        # Trig path: a sign may flip only where the reference's own distance
        # is tiny compared with the cell size.
        flip = np.signbit(d) != np.signbit(gd)
        cell = float(np.max(sp[3:] - sp[:3])) / rr
        assert np.all(np.abs(gd[flip]) < 1e-3 * cell), np.abs(gd[flip]).max()
        if not flip.any():
            assert np.array_equal(buf.indices, golden["small%d_indices" % n])
        close = np.abs(d - gd) <= 1e-6 + 1e-3 * np.abs(gd)
        assert close.mean() >= 0.99, close.mean()
        return
    np.testing.assert_allclose(d, gd, rtol=1e-3, atol=1e-6)


@pytest.mark.parametrize("n", range(2))
def test_sphere_mesh_bit_exact(cg, golden, mesher, n):
    meta = golden["sphere%d_meta" % n]
    sp = golden["sphere%d_span" % n]
    buf, _ = cg.MeshBuffer.generate_for_box(cg.Span(sp[:3], sp[3:]), cg.Sphere(meta[:3], meta[3]),
                                            int(meta[4]), mesher=mesher)
    assert np.array_equal(as7(buf.vertices).view(np.uint32),
                          golden["sphere%d_vertices" % n].view(np.uint32))
    assert np.array_equal(buf.indices, golden["sphere%d_indices" % n])


@pytest.mark.parametrize("span,res", [(((0, 0, 0), (-1, 1, 1)), 8), (((0, 0, 0), (1, 1, 1)), 6),
                                      (((0, 0, 0), (1, 1, 1)), 0), (((0, 0, 0), (1, 1, 1)), 1),
                                      (((0, 0, 0), (1, 1, 1)), 2048)])
def test_invalid_arguments(cg, mesher, span, res):
    with pytest.raises(cg.CantucciError) as e:
        cg.MeshBuffer.generate_for_box(cg.Span(*span), cg.Mandelbulb(8, 15, 2.5), res,
                                       mesher=mesher)
    assert e.value.status == 1


def test_capacity_reported(cg, mesher):
    s = cg.Mandelbulb(8, 15, 2.5)
    verts = np.zeros(10, cg.VERTEX_DTYPE)
    idx = np.zeros(12, np.uint32)
    with pytest.raises(cg.CantucciError) as e:
        mesher.generate(cg.Span(*W.SPAN_C1), s, 16, vertices=verts, indices=idx)
    assert e.value.status == 2
    full, _ = cg.MeshBuffer.generate_for_box(cg.Span(*W.SPAN_C1), s, 16, mesher=mesher)
    # what fits was written, nothing beyond
    assert np.array_equal(idx, full.indices[:12])
    assert np.array_equal(verts.view(np.uint8), full.vertices[:10].view(np.uint8))


def test_c2_panics_like_the_reference(cg, mesher):
    """generate_for_box raises CG_ELERP where the reference's lerp asserts."""
    with pytest.raises(cg.CantucciError) as e:
        cg.MeshBuffer.generate_for_box(cg.Span(*W.SPAN_C1), cg.Mandelbulb.classic(15, 2.5), 512,
                                       mesher=mesher)
    assert e.value.status == 3


def test_device_output_matches_host(cg, mesher):
    import torch
    s = cg.Mandelbulb(8, 15, 2.5)
    host, _ = cg.MeshBuffer.generate_for_box(cg.Span(*W.SPAN_C1), s, 32, mesher=mesher)
    v = torch.empty((32 ** 3, 7), dtype=torch.float32, device="cuda")
    i = torch.empty(18 * 32 ** 3, dtype=torch.int32, device="cuda")
    nv, ni, _ = mesher.generate_device(cg.Span(*W.SPAN_C1), s, 32, v, i)
    assert (nv, ni) == (len(host.vertices), len(host.indices))
    assert np.array_equal(v[:nv].cpu().numpy().view(np.uint32), as7(host.vertices).view(np.uint32))
    assert np.array_equal(i[:ni].cpu().numpy().view(np.uint32), host.indices)


def test_two_meshers_in_threads(cg):
    """The reference meshes spans from a thread pool; each worker owns a mesher."""
    import threading
    spans = [cg.Span(*W.SPAN_C1)] + [cg.Span(s[:3], s[3:]) for s in W.batched_spans(6, 2)[0]]
    results = {}

    def work(k):
        m = cg.Mesher(0)
        out = []
        for sp in spans:
            b, _ = cg.MeshBuffer.generate_for_box(sp, cg.Mandelbulb(8, 15, 2.5), 32, mesher=m)
            out.append(sha(b.indices) + sha(b.vertices))
        m.close()
        results[k] = out

    th = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert results[0] == results[1]


@pytest.mark.slow
def test_c2_full_size_vs_oracle(cg, orc, mesher):
    """513^3 corners: cell table and index list bit-exact against the oracle.

    At this resolution the reference panics (src/math.rs:19): four corners in
    the y=0 plane evaluate to NaN next to outside corners.  Both sides report
    that (CG_ELERP / ORC_ELERP) and complete the mesh identically."""
    s = cg.Mandelbulb.classic(15, 2.5)
    n = 512 ** 3
    verts = np.empty(6_000_000, cg.VERTEX_DTYPE)
    idx = np.empty(40_000_000, np.uint32)
    v, i, nv, ni, tm = mesher.generate(cg.Span(*W.SPAN_C1), s, 512, vertices=verts, indices=idx,
                                       strict=False)
    assert mesher.last_status == 3  # CG_ELERP
    gpu_points = mesher.last_points().cpu().numpy().astype(np.uint32)
    ref = orc.generate_for_box(orc.mandelbulb(8, 15, 2.5), np.array(W.SPAN_C1).ravel(), 512,
                               want_grids=True, vcap=6_000_000, icap=40_000_000)
    assert ref["rc"] == orc.ORC_ELERP
    assert (nv, ni) == (ref["nv"], ref["ni"])
    assert np.array_equal(gpu_points, ref["points"])
    assert np.array_equal(idx[:ni], ref["indices"])
    a, b = as7(verts[:nv]), as7(ref["vertices"])
    np.testing.assert_allclose(a[:, :3], b[:, :3], rtol=0, atol=1e-6)
    assert n == gpu_points.size
    placement_vs_oracle(orc, mesher, a, idx[:ni], 512, orc.ORC_ELERP)


@pytest.mark.parametrize("kind", ["polar", "p8", "p6", "sphere"])
def test_analytic_normals(cg, orc, kind):
    """Analytic (forward-mode) normals: the same mesh except the normals,
    which match the FP64 gradient at the vertex (for Mandelbulb<8> the
    gradient of the reference's polynomial itself)."""
    rot = (0.2, 0.1, 0.0)
    shape, oshape = {
        "polar": (cg.MandelbulbPolar(8.3, 15, 2.5, rot), orc.mandelbulb_polar(8.3, 15, 2.5, rot)),
        "p8": (cg.Mandelbulb(8, 15, 2.5), orc.mandelbulb(8, 15, 2.5)),
        "p6": (cg.Mandelbulb(6, 12, 2.5), orc.mandelbulb(6, 12, 2.5)),
        "sphere": (cg.Sphere((0.1, -0.05, 0.02), 0.9), orc.sphere((0.1, -0.05, 0.02), 0.9)),
    }[kind]
    span = cg.Span(*W.SPAN_C1)
    m = cg.Mesher(0)
    try:
        v0, i0, nv0, ni0, _ = m.generate(span, shape, 64)
        m.set_normals("analytic")
        v1, i1, nv1, ni1, _ = m.generate(span, shape, 64)
    finally:
        m.close()
    assert (nv0, ni0) == (nv1, ni1) and nv0 > 1000
    a, b = as7(v0[:nv0]), as7(v1[:nv1])
    assert np.array_equal(i0[:ni0], i1[:ni1])
    assert np.array_equal(a[:, [0, 1, 2, 6]].view(np.uint32), b[:, [0, 1, 2, 6]].view(np.uint32))
    g = orc.de_grad_f64(oshape, b[:, :3])
    ok = np.all(np.isfinite(g[:, 1:4]), axis=1) & np.all(np.isfinite(b[:, 3:6]), axis=1)
    assert ok.mean() > 0.99
    ang = angle_deg(b[ok, 3:6].astype(np.float64), g[ok, 1:4])
    if kind == "sphere":
        assert ang.max() < 1e-3, ang.max()
    else:
        assert np.median(ang) < 0.01 and np.mean(ang < 0.1) >= 0.9, np.quantile(ang, [0.5, 0.9])
        # the six-sample normal is much further from the gradient
        ang_fd = angle_deg(a[ok, 3:6], g[ok, 1:4])
        assert np.median(ang_fd) > np.median(ang)


@pytest.mark.parametrize("res", [64, 128, 256])
def test_pinned_host_outputs_match_device(cg, mesher, res):
    """Pinned host outputs: up to res 128 through device staging and a
    replayed graph, above it the overlapped path (vertices stored by the GPU
    straight into host memory, the index copy overlapping placement); same
    bits as the device-output mesh either way."""
    import torch
    s = cg.Mandelbulb(8, 15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    vcap, icap = res ** 3 // 8, 18 * res ** 3 // 8
    v = torch.empty((vcap, 7), dtype=torch.float32, device="cuda")
    i = torch.empty(icap, dtype=torch.int32, device="cuda")
    nv, ni, _ = mesher.generate_device(span, s, res, v, i)
    vh = torch.zeros((vcap, 7), dtype=torch.float32, pin_memory=True)
    ih = torch.zeros(icap, dtype=torch.int32, pin_memory=True)
    vnp = vh.numpy().view(cg.VERTEX_DTYPE).reshape(-1)
    inp = ih.numpy().view(np.uint32)
    _, _, nv2, ni2, tm = mesher.generate(span, s, res, vertices=vnp, indices=inp)
    assert (nv2, ni2) == (nv, ni)
    assert np.array_equal(vh[:nv].numpy().view(np.uint32), v[:nv].cpu().numpy().view(np.uint32))
    assert np.array_equal(ih[:ni].numpy(), i[:ni].cpu().numpy())
    assert tm.first_ms > 0 and tm.second_ms > 0 and tm.third_ms > 0


@pytest.mark.parametrize("offset", [1, 2, 4])
def test_pinned_host_outputs_offset_buffers(cg, mesher, offset):
    """The overlapped path copies the indices with a kernel in 16-byte units
    when both buffers are 16-byte aligned (offset 4 words), else with a
    copy-engine transfer (offsets 1 and 2); index counts 6q leave a 2-word
    tail when q is odd.  Same words either way, nothing written past them."""
    import torch
    s = cg.Mandelbulb(8, 15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    res = 256
    vcap, icap = res ** 3 // 8, 18 * res ** 3 // 8
    v = torch.empty((vcap, 7), dtype=torch.float32, device="cuda")
    i = torch.empty(icap, dtype=torch.int32, device="cuda")
    nv, ni, _ = mesher.generate_device(span, s, res, v, i)
    vh = torch.zeros((vcap, 7), dtype=torch.float32, pin_memory=True)
    ih = torch.full((icap + offset + 8,), -7, dtype=torch.int32, pin_memory=True)
    inp = ih.numpy().view(np.uint32)[offset:offset + icap]
    _, _, nv2, ni2, _ = mesher.generate(span, s, res,
                                        vertices=vh.numpy().view(cg.VERTEX_DTYPE).reshape(-1),
                                        indices=inp)
    assert (nv2, ni2) == (nv, ni)
    got = ih.numpy()
    assert np.array_equal(got[offset:offset + ni], i[:ni].cpu().numpy())
    assert np.all(got[:offset] == -7) and np.all(got[offset + ni:] == -7)
    assert np.array_equal(vh[:nv].numpy().view(np.uint32), v[:nv].cpu().numpy().view(np.uint32))


def test_pinned_host_outputs_capacity(cg, mesher):
    """Too-small pinned outputs: CG_ECAPACITY with the full counts, and the
    prefix that fits is the mesh's."""
    import torch
    s = cg.Mandelbulb(8, 15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    full_v, full_i, nv, ni, _ = mesher.generate(span, s, 64)
    vh = torch.zeros((1000, 7), dtype=torch.float32, pin_memory=True)
    ih = torch.zeros(3000, dtype=torch.int32, pin_memory=True)
    with pytest.raises(cg.CantucciError):
        mesher.generate(span, s, 64, vertices=vh.numpy().view(cg.VERTEX_DTYPE).reshape(-1),
                        indices=ih.numpy().view(np.uint32))
    got = vh.numpy().view(np.uint32)
    want = full_v[:1000].view(np.float32).reshape(-1, 7).view(np.uint32)
    assert np.array_equal(got, want)
    assert np.array_equal(ih.numpy().view(np.uint32), full_i[:3000])


def test_pinned_host_outputs_capacity_overlapped(cg, mesher):
    """The overlapped path (res 256) into too-small, 16-byte aligned pinned
    outputs: the index copy takes its length from the device counters, cut
    at the capacity; CG_ECAPACITY with the full counts, the prefix that fits
    is the mesh's, and nothing is written past either capacity."""
    import torch
    s = cg.Mandelbulb(8, 15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    res = 256
    full_v, full_i, nv, ni, _ = mesher.generate(span, s, res)
    vcap, icap, guard = 1000, 3000, 64
    vh = torch.full((vcap + guard, 7), -7.0, dtype=torch.float32, pin_memory=True)
    ih = torch.full((icap + guard,), -7, dtype=torch.int32, pin_memory=True)
    vnp = vh.numpy().view(cg.VERTEX_DTYPE).reshape(-1)[:vcap]
    inp = ih.numpy().view(np.uint32)[:icap]
    with pytest.raises(cg.CantucciError):
        mesher.generate(span, s, res, vertices=vnp, indices=inp)
    got_v = vh.numpy()
    want_v = full_v[:vcap].view(np.float32).reshape(-1, 7)
    assert np.array_equal(got_v[:vcap].view(np.uint32), want_v.view(np.uint32))
    assert np.all(got_v[vcap:] == -7.0)
    got_i = ih.numpy()
    assert np.array_equal(got_i[:icap].view(np.uint32), full_i[:icap])
    assert np.all(got_i[icap:] == -7)


@pytest.mark.parametrize("span,res", [
    (([1.5, 1.5, 1.5], [2.0, 2.0, 2.0]), 16),      # all outside: no surface
    (([-0.05, -0.05, -0.05], [0.05, 0.05, 0.05]), 8),  # all inside (the origin is NaN, "inside")
    (([-1.2, -1.2, -1.2], [1.2, 1.2, 1.2]), 2),     # the smallest resolution
    (([-0.9, 0.1, -0.3], [-0.5, 0.5, 0.1]), 4),
])
def test_edge_spans_match_oracle(cg, orc, mesher, span, res):
    """Includes res 2 over the whole box, whose widened grid has the origin
    (NaN) next to outside corners: the reference panics there, and both
    sides report CG_ELERP with the same completed mesh."""
    s = cg.Mandelbulb(8, 15, 2.5)
    v, i, nv, ni, _ = mesher.generate(cg.Span(*span), s, res, strict=False)
    ref = orc.generate_for_box(orc.mandelbulb(8, 15, 2.5),
                               np.array(span, np.float32).ravel(), res)
    assert mesher.last_status == ref["rc"]
    assert np.array_equal(i[:ni], ref["indices"])
    assert nv == len(ref["vertices"])
    if nv:
        np.testing.assert_allclose(as7(v[:nv])[:, :3], as7(ref["vertices"])[:, :3],
                                   rtol=0, atol=1e-6)


def test_empty_mesh_batch_and_device(cg, mesher):
    """A span with no surface gives zero counts on every path."""
    import torch
    from cantucci_gb300.batch import BatchMesher
    s = cg.Mandelbulb(8, 15, 2.5)
    sp = cg.Span([1.5, 1.5, 1.5], [2.0, 2.0, 2.0])
    v = torch.empty((16, 7), dtype=torch.float32, device="cuda")
    i = torch.empty(16, dtype=torch.int32, device="cuda")
    assert mesher.generate_device(sp, s, 32, v, i)[:2] == (0, 0)
    b = BatchMesher(np.array([[1.5, 1.5, 1.5, 2.0, 2.0, 2.0]], np.float32), [32])
    out = b.run(s, graph=True)
    vv, ii = out.mesh(0)
    assert len(vv) == 0 and len(ii) == 0 and out.status == 0
    b.close()


@pytest.mark.parametrize("shape_kind", ["p8", "polar"])
def test_root_crossings(cg, shape_kind):
    """Root-found crossings: same cells and indices as the reference's lerp,
    every vertex stays in its cell, and the vertices sit much closer to the
    surface (|DE at the vertex| drops)."""
    s = cg.Mandelbulb(8, 15, 2.5) if shape_kind == "p8" else cg.MandelbulbPolar(8.3, 15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    res = 64
    m = cg.Mesher(0)
    try:
        v0, i0, nv0, ni0, _ = m.generate(span, s, res, strict=False)
        pts0 = m.last_points().cpu().numpy()
        m.set_crossings("root", 6)
        v1, i1, nv1, ni1, _ = m.generate(span, s, res, strict=False)
        with pytest.raises(cg.CantucciError):
            m.set_crossings("root", 0)
    finally:
        m.close()
    assert (nv0, ni0) == (nv1, ni1)
    assert np.array_equal(i0[:ni0], i1[:ni1])
    a, b = as7(v0[:nv0]), as7(v1[:nv1])
    # each vertex inside its (widened-span) cell
    lo = np.asarray(span.start, np.float64) - (np.asarray(span.end) - np.asarray(span.start)) / res
    step = (np.asarray(span.end, np.float64) - np.asarray(span.start)) * (res + 2) / res / res
    cells = np.argwhere(pts0 != 0xFFFFFFFF)  # (x, y, z) in vertex-id order
    order = pts0[cells[:, 0], cells[:, 1], cells[:, 2]].astype(np.int64)
    cmin = lo + cells * step
    ok = np.all((b[order, :3] >= cmin - 1e-5) & (b[order, :3] <= cmin + step + 1e-5), axis=1)
    assert ok.mean() > 0.999
    da, db = np.abs(a[:, 6]), np.abs(b[:, 6])
    fin = np.isfinite(da) & np.isfinite(db)
    assert np.median(db[fin]) < 0.5 * np.median(da[fin]), (np.median(db[fin]), np.median(da[fin]))


@pytest.mark.slow
def test_max_resolution_span(cg, orc):
    """Resolution 1024 (the largest the ABI takes: 1025^3 corners, a 4.3 GB
    distance grid): the mesh completes, every index refers to a vertex,
    sampled corners of the grid equal the point estimator at the same
    coordinates bit for bit, and the oracle's steps 2-3 on the GPU's own
    distances give the same index list and vertex positions bit for bit."""
    import torch
    s = cg.Mandelbulb(8, 15, 2.5)
    span = cg.Span([-1.2] * 3, [1.2] * 3)
    res = 1024
    m = cg.Mesher(0)
    try:
        vcap, icap = 24 << 20, 160 << 20
        v = torch.empty((vcap, 7), dtype=torch.float32, device="cuda")
        i = torch.empty(icap, dtype=torch.int32, device="cuda")
        nv, ni, tm = m.generate_device(span, s, res, v, i, strict=False)
        assert m.last_status in (0, 3)  # OK or the reference's lerp panic (completed)
        assert 0 < nv <= vcap and 0 < ni <= icap and ni % 6 == 0
        idx = i[:ni].to(torch.int64) & 0xFFFFFFFF
        assert int(idx.max()) < nv
        d = m.last_dists()
        n = res + 1
        rng = np.random.default_rng(11)
        cells = rng.integers(0, n, size=(10000, 3))
        rf = np.float32(res)
        st = (span.start + -((span.end - span.start) / rf)).astype(np.float32)
        en = (span.end + (span.end - span.start) / rf).astype(np.float32)
        pts = (st + (en - st) * (cells.astype(np.float32) * (np.float32(1) / rf))).astype(np.float32)
        want = s.batch_min_distance_from(pts)
        got = d[cells[:, 0], cells[:, 1], cells[:, 2]].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        del d
        a = v[:nv].cpu().numpy()
        ih = i[:ni].cpu().numpy().view(np.uint32)
        placement_vs_oracle(orc, m, a, ih, res, m.last_status)
    finally:
        m.close()


@pytest.mark.parametrize("kind", ["p8", "p6", "polar"])
def test_fast_numerics_mesh(cg, kind):
    """CG_NUMERICS_FAST for a whole mesh: the corner signs agree with the
    exact grid almost everywhere (>= 99.9%), the vertex and quad counts stay
    within 1% of the reference's, every index names a vertex, every vertex
    lies in its cell; fast numerics together with another placement option
    is refused."""
    from oracle import qef
    s = {"p8": cg.Mandelbulb(8, 15, 2.5), "p6": cg.Mandelbulb(6, 12, 2.5),
         "polar": cg.MandelbulbPolar(8.3, 15, 2.5, (0.2, 0.1, 0.0))}[kind]
    span = cg.Span(*W.SPAN_C1)
    res = 128
    m = cg.Mesher(0)
    try:
        v0, i0, nv0, ni0, _ = m.generate(span, s, res, strict=False)
        d0 = m.last_dists().cpu().numpy()
        m.set_numerics("fast")
        v1, i1, nv1, ni1, _ = m.generate(span, s, res, strict=False)
        d1 = m.last_dists().cpu().numpy()
        pts = m.last_points().cpu().numpy()
        m.set_placement("qef")
        with pytest.raises(cg.CantucciError):
            m.generate(span, s, 16)
    finally:
        m.close()
    assert np.mean(np.signbit(d0) == np.signbit(d1)) >= 0.999
    assert abs(nv1 - nv0) <= 0.01 * nv0 and abs(ni1 - ni0) <= 0.01 * ni0
    assert ni1 > 0 and int(i1[:ni1].max()) < nv1
    b = as7(v1[:nv1])
    cells = np.argwhere(pts != 0xFFFFFFFF)
    order = pts[cells[:, 0], cells[:, 1], cells[:, 2]].astype(np.int64)
    start, step = qef.span_setup(np.array(W.SPAN_C1), res)
    lo = (start + cells.astype(np.float32) * step).astype(np.float32)
    ok = np.all((b[order, :3] >= lo - 1e-6) & (b[order, :3] <= lo + step + 1e-6), axis=1)
    assert ok.all()


def test_launch_knobs_change_no_bit(cg):
    """The placement grid and the side stream's priority are launch shapes
    only: meshes under other settings equal the default mesh bit for bit."""
    s = cg.Mandelbulb(8, 15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    lib = cg.load()
    meshes = []
    try:
        for bps, prio in ((128, 1), (1, 0), (16, 1), (1024, 0)):
            assert lib.cg_set_option(b"place_blocks_per_sm", bps) == 0
            assert lib.cg_set_option(b"side_stream_priority", prio) == 0
            m = cg.Mesher(0)
            try:
                v, i, nv, ni, _ = m.generate(span, s, 128)
            finally:
                m.close()
            meshes.append((as7(v[:nv]).view(np.uint32).copy(), i[:ni].copy()))
        assert lib.cg_set_option(b"place_blocks_per_sm", 0) != 0
        assert lib.cg_set_option(b"side_stream_priority", 2) != 0
    finally:
        lib.cg_set_option(b"place_blocks_per_sm", 128)
        lib.cg_set_option(b"side_stream_priority", 1)
    for v, i in meshes[1:]:
        assert np.array_equal(v, meshes[0][0]) and np.array_equal(i, meshes[0][1])


def test_graph_replay_matches_direct_launches(cg):
    """A mesher replays one captured graph for every span of the same
    resolution and shape (the span goes in through a parameter block) and
    captures again when the resolution changes (res 256 is launched
    directly): each mesh equals the one direct launches give, bit for bit,
    timings included."""
    lib = cg.load()
    s = cg.Mandelbulb(8, 15, 2.5)
    jobs = [((-1.2, -1.2, -1.2), (0.0, 0.0, 0.0), 32), ((0.0, -1.2, 0.0), (1.2, 0.0, 1.2), 32),
            ((-0.6, 0.0, -0.6), (0.0, 0.6, 0.0), 32), ((-1.2, -1.2, -1.2), (1.2, 1.2, 1.2), 64),
            ((0.3, 0.3, -0.9), (0.9, 0.9, -0.3), 32), ((-1.2, -1.2, -1.2), (1.2, 1.2, 1.2), 256),
            ((-1.2, -1.2, -1.2), (0.0, 0.0, 0.0), 128)]
    out = {}
    try:
        for graphs in (1, 0):
            assert lib.cg_set_option(b"mesh_graphs", graphs) == 0
            m = cg.Mesher(0)
            try:
                res_list = []
                for a, b, r in jobs:
                    v, i, nv, ni, tm = m.generate(cg.Span(a, b), s, r)
                    assert tm.first_ms > 0 and tm.second_ms > 0
                    res_list.append((as7(v[:nv]).view(np.uint32).copy(), i[:ni].copy()))
            finally:
                m.close()
            out[graphs] = res_list
    finally:
        lib.cg_set_option(b"mesh_graphs", 1)
    for (va, ia), (vb, ib) in zip(out[1], out[0]):
        assert len(va) > 0 and np.array_equal(va, vb) and np.array_equal(ia, ib)
