"""Dual-contouring placement (CG_PLACEMENT_QEF) and the spatial gradient it
is built on (cg_de_spatial_grad), against the oracle's FP64 forward-mode
gradients and the FP64 placement model in oracle/qef.py.

The cell table and the index list stay the reference's bit for bit; only
the vertex inside each surface cell moves.  Tolerances: near the surface
the f32 gradient follows the chaotic estimator (test_gpu_adjoint explains
the bars), and the pseudo-inverse drops eigenvalues below a threshold, so a
cell whose middle eigenvalue sits at the threshold may take the other
solution.  The bars are in test_qef_matches_fp64_model; every vertex
stays inside its cell, and the DE stored with each vertex is the
estimator's at its position, bit for bit.
"""
import numpy as np
import pytest

from cantucci_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def angle_deg(a, b):
    a = a / np.linalg.norm(a, axis=1, keepdims=True)
    b = b / np.linalg.norm(b, axis=1, keepdims=True)
    return np.degrees(np.arccos(np.clip(np.sum(a * b, axis=1), -1, 1)))


def as7(v):
    return np.ascontiguousarray(v).view(np.float32).reshape(-1, 7)


def shapes(cg, orc, kind):
    if kind == "p8":
        return cg.Mandelbulb(8, 15, 2.5), orc.mandelbulb(8, 15, 2.5)
    if kind == "p8_it5":
        return cg.Mandelbulb(8, 5, 2.5), orc.mandelbulb(8, 5, 2.5)
    if kind == "p6":
        return cg.Mandelbulb(6, 12, 2.5), orc.mandelbulb(6, 12, 2.5)
    if kind in ("polar", "polar_it5"):
        rot, it = (0.2, 0.1, 0.0), (5 if kind == "polar_it5" else 15)
        return cg.MandelbulbPolar(8.3, it, 2.5, rot), orc.mandelbulb_polar(8.3, it, 2.5, rot)
    return cg.Sphere((0.1, -0.05, 0.02), 0.9), orc.sphere((0.1, -0.05, 0.02), 0.9)


def near_surface(shape, n, seed):
    """Uniform points in the box marched 8 steps along random directions by
    the shape's own estimator."""
    import torch
    rng = np.random.default_rng(seed)
    p = torch.as_tensor(rng.uniform(-1.2, 1.2, size=(n, 3)).astype(np.float32)).cuda()
    d = torch.as_tensor(rng.normal(size=(n, 3)).astype(np.float32)).cuda()
    d = d / d.norm(dim=1, keepdim=True)
    for _ in range(8):
        p = p + d * shape.batch_min_distance_from(p)[:, None]
    return p


@pytest.mark.parametrize("kind", ["p8", "p6", "polar", "sphere"])
def test_spatial_grad_matches_fp64(cg, orc, kind):
    """dDE/dp in one forward-mode pass: >= 99% within 0.1 degree of the FP64
    gradient away from the surface; in the band |DE| < 1e-3, median below
    0.01 degree and >= 90% within 0.1 degree.  Column 0 is the estimator's
    value, bit for bit."""
    import torch
    from cantucci_gb300.autograd import spatial_grad
    s, o = shapes(cg, orc, kind)
    rng = np.random.default_rng(11)
    far = torch.as_tensor(rng.uniform(-1.2, 1.2, size=(20000, 3)).astype(np.float32)).cuda()
    de = s.batch_min_distance_from(far)
    far = far[(de > 0.02) & (de < 0.3)][:4000]
    band = near_surface(s, 40000, 12)
    db = s.batch_min_distance_from(band)
    band = band[torch.isfinite(db) & (db.abs() < 1e-3)][:4000]
    assert len(far) > 500 and len(band) > 500
    for pts, bar in ((far, "far"), (band, "band")):
        g = spatial_grad(pts, s).cpu().numpy()
        ref = orc.de_grad_f64(o, pts.cpu().numpy())
        ok = np.all(np.isfinite(ref[:, 1:4]), axis=1) & (np.linalg.norm(ref[:, 1:4], axis=1) > 0)
        assert ok.mean() > 0.99
        ang = angle_deg(g[ok, 1:4].astype(np.float64), ref[ok, 1:4])
        if bar == "far":
            assert np.mean(ang < 0.1) >= 0.99, np.quantile(ang, [0.5, 0.99, 1.0])
        else:
            assert np.median(ang) < 0.01 and np.mean(ang < 0.1) >= 0.9, np.quantile(ang, [0.5, 0.9])
        est = s.batch_min_distance_from(pts).cpu().numpy()
        assert np.array_equal(g[:, 0].view(np.uint32), est.view(np.uint32))


def _qef_case(cg, orc, kind, res, crossings=None):
    from oracle import qef
    s, o = shapes(cg, orc, kind)
    span = cg.Span(*W.SPAN_C1)
    m = cg.Mesher(0)
    try:
        v0, i0, nv0, ni0, _ = m.generate(span, s, res, strict=False)
        if crossings:
            m.set_crossings(crossings, 6)
        m.set_placement("qef")
        v1, i1, nv1, ni1, _ = m.generate(span, s, res, strict=False)
        pts = m.last_points().cpu().numpy()
        dists = m.last_dists().cpu().numpy()
    finally:
        m.close()
    assert (nv0, ni0) == (nv1, ni1) and nv0 > 100
    assert np.array_equal(i0[:ni0], i1[:ni1])
    cells = np.argwhere(pts != 0xFFFFFFFF)
    order = pts[cells[:, 0], cells[:, 1], cells[:, 2]].astype(np.int64)
    cells_by_id = np.empty_like(cells)
    cells_by_id[order] = cells
    start, step = qef.span_setup(np.array(W.SPAN_C1), res)
    return s, o, as7(v0[:nv0]), as7(v1[:nv1]), cells_by_id, start, step, dists


@pytest.mark.parametrize("kind", ["p8_it5", "polar_it5", "p8", "polar", "sphere"])
def test_qef_matches_fp64_model(cg, orc, kind):
    """Same mesh topology; vertices near the FP64 model's on the GPU's own
    corner distances, inside their cells, and the stored DE is the
    estimator's at the new position.  With 5 iterations (f32 and FP64
    trajectories still track) and on the sphere, >= 99% within 1e-3 of a
    cell; with 15, where the band's f32 gradients scatter, >= 70% within
    1e-3 and >= 95% within 0.05 of a cell."""
    from oracle import qef
    res = 64 if kind != "sphere" else 32
    s, o, a, b, cells, start, step, dists = _qef_case(cg, orc, kind, res)
    ref = qef.qef_vertices(o, dists, cells, start, step)
    err = np.max(np.abs(b[:, :3] - ref) / step, axis=1)
    q = np.quantile(err, [0.5, 0.8, 0.97, 0.99, 1.0])
    if kind in ("p8_it5", "polar_it5", "sphere"):
        assert np.mean(err < 1e-3) >= 0.99, q
    else:
        assert np.mean(err < 1e-3) >= 0.7 and np.mean(err < 0.05) >= 0.95, q
    lo = (start + cells.astype(np.float32) * step).astype(np.float32)
    hi = (lo + step).astype(np.float32)
    assert np.all((b[:, :3] >= lo) & (b[:, :3] <= hi))
    est = s.batch_min_distance_from(b[:, :3])
    assert np.array_equal(np.asarray(est).view(np.uint32), b[:, 6].view(np.uint32))


def test_qef_on_the_sphere(cg, orc):
    """Dual contouring puts the sphere's vertices on it: radial error below
    0.05 of a cell, against about a fifth of a cell for the reference's
    centroids."""
    s, o, a, b, cells, start, step, dists = _qef_case(cg, orc, "sphere", 32)
    c = np.array([0.1, -0.05, 0.02])
    rq = np.abs(np.linalg.norm(b[:, :3] - c, axis=1) - 0.9) / step[0]
    rc = np.abs(np.linalg.norm(a[:, :3] - c, axis=1) - 0.9) / step[0]
    assert rq.max() < 0.05 and np.median(rc) > 5 * np.median(rq), (rq.max(), np.median(rc))


@pytest.mark.parametrize("crossings", [None, "root"])
def test_qef_mandelbulb_nearer_surface(cg, orc, crossings):
    """On the P=8 Mandelbulb the QEF vertices sit nearer the surface than the
    reference's centroids (median |DE| at least 2x lower), also with
    root-found crossings."""
    s, o, a, b, cells, start, step, dists = _qef_case(cg, orc, "p8", 64, crossings)
    da, db = np.abs(a[:, 6]), np.abs(b[:, 6])
    fin = np.isfinite(da) & np.isfinite(db)
    assert np.median(db[fin]) < 0.5 * np.median(da[fin]), (np.median(db[fin]), np.median(da[fin]))
    lo = (start + cells.astype(np.float32) * step).astype(np.float32)
    assert np.all((b[:, :3] >= lo) & (b[:, :3] <= (lo + step).astype(np.float32)))


def test_qef_host_and_device_outputs_agree(cg):
    """The pinned-host pipeline and the device-output mesh give the same bits
    with dual contouring on."""
    import torch
    s = cg.MandelbulbPolar(8.3, 15, 2.5, (0.2, 0.1, 0.0))
    span = cg.Span(*W.SPAN_C1)
    res = 64
    m = cg.Mesher(0)
    try:
        m.set_placement("qef")
        m.set_normals("analytic")
        hv = torch.empty((res ** 3, 7), dtype=torch.float32).pin_memory()
        hi = torch.empty(18 * res ** 3, dtype=torch.int32).pin_memory()
        _, _, nv, ni, _ = m.generate(span, s, res, vertices=hv, indices=hi)
        dv = torch.empty((res ** 3, 7), dtype=torch.float32, device="cuda")
        di = torch.empty(18 * res ** 3, dtype=torch.int32, device="cuda")
        nv2, ni2, _ = m.generate_device(span, s, res, dv, di)
    finally:
        m.close()
    assert (nv, ni) == (nv2, ni2)
    assert torch.equal(hv[:nv].view(torch.int32), dv[:nv].cpu().view(torch.int32))
    assert torch.equal(hi[:ni], di[:ni].cpu())


def test_placement_rejects_unknown_mode(cg):
    lib = cg.load()
    m = cg.Mesher(0)
    try:
        assert lib.cg_mesher_set_placement(m.handle, 2) != 0
        assert lib.cg_mesher_set_placement(m.handle, 1) == 0
    finally:
        m.close()


@pytest.mark.parametrize("res", [2, 4, 8])
def test_qef_small_resolutions(cg, res):
    """The smallest spans (res 2 is the least the reference accepts): the
    same topology as the centroid mesh and every vertex inside its cell."""
    from oracle import qef
    s = cg.Sphere((0.1, -0.05, 0.02), 0.9)
    span = cg.Span(*W.SPAN_C1)
    m = cg.Mesher(0)
    try:
        v0, i0, nv0, ni0, _ = m.generate(span, s, res)
        m.set_placement("qef")
        v1, i1, nv1, ni1, _ = m.generate(span, s, res)
        pts = m.last_points().cpu().numpy()
    finally:
        m.close()
    assert (nv0, ni0) == (nv1, ni1) and nv0 > 0
    assert np.array_equal(i0[:ni0], i1[:ni1])
    b = as7(v1[:nv1])
    cells = np.argwhere(pts != 0xFFFFFFFF)
    order = pts[cells[:, 0], cells[:, 1], cells[:, 2]].astype(np.int64)
    start, step = qef.span_setup(np.array(W.SPAN_C1), res)
    lo = (start + cells.astype(np.float32) * step).astype(np.float32)
    assert np.all((b[order, :3] >= lo) & (b[order, :3] <= (lo + step).astype(np.float32)))


def test_qef_empty_span(cg):
    """A span the surface does not cross: no vertices, no quads, no edges,
    through both the device and the pinned-host pipelines."""
    import torch
    s = cg.Mandelbulb(8, 15, 2.5)
    span = cg.Span((1.5, 1.5, 1.5), (1.9, 1.9, 1.9))
    m = cg.Mesher(0)
    try:
        m.set_placement("qef")
        _, _, nv, ni, _ = m.generate(span, s, 32)
        hv = torch.empty((1024, 7), dtype=torch.float32).pin_memory()
        hi = torch.empty(4096, dtype=torch.int32).pin_memory()
        _, _, nv2, ni2, _ = m.generate(span, s, 32, vertices=hv, indices=hi)
    finally:
        m.close()
    assert (nv, ni) == (0, 0) and (nv2, ni2) == (0, 0)
