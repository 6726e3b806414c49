"""Adjoint kernel against the FP64 forward-mode oracle and FP64 central
differences, and the autograd.Function against the adjoint itself.

Tolerances: the estimator iterates a chaotic map (angles are multiplied by
the power every step), so in the surface band |DE| < 1e-3 a few percent of
points follow an f32 trajectory that has left the FP64 one (their f32
distance is ~1% off FP64).  No f32 method can match FP64 there.  So the bars
are: away from the surface (0.02 < DE < 0.3), and in the band with 5
iterations, where the trajectories still track, >= 99% of normals within
0.1 degree of FP64 and the power / rotation derivatives within 1e-3 (1e-2 in
the band); over the whole 15-iteration band, median error below 0.01 degree
and >= 90% within 0.1 degree.
"""
import numpy as np
import pytest

from cantucci_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def angle_deg(a, b):
    a = a / np.linalg.norm(a, axis=1, keepdims=True)
    b = b / np.linalg.norm(b, axis=1, keepdims=True)
    return np.degrees(np.arccos(np.clip(np.sum(a * b, axis=1), -1, 1)))


def band_points(cg, n, power=8.0, rot=(0.0, 0.0, 0.0), seed=0):
    """Points near the surface: uniform in the box, marched 8 steps along
    random directions, then kept where |DE| < 1e-3."""
    import torch
    shape = cg.MandelbulbPolar(power, 15, 2.5, rot)
    rng = np.random.default_rng(seed)
    p = torch.as_tensor(rng.uniform(-1.2, 1.2, size=(8 * n, 3)).astype(np.float32)).cuda()
    d = torch.as_tensor(rng.normal(size=(8 * n, 3)).astype(np.float32)).cuda()
    d = d / d.norm(dim=1, keepdim=True)
    for _ in range(8):
        p = p + d * shape.batch_min_distance_from(p)[:, None]
    de = shape.batch_min_distance_from(p)
    keep = torch.isfinite(de) & (de.abs() < 1e-3)
    return p[keep][:n].contiguous()


def test_adjoint_matches_fp64_forward_mode(cg, orc):
    import torch
    from cantucci_gb300.autograd import de_grad
    rot = (0.2, 0.1, 0.0)
    pts = band_points(cg, 4000, 8.3, rot)
    assert pts.shape[0] >= 1000
    g = de_grad(pts, 8.3, rot).cpu().numpy().astype(np.float64)
    ref = orc.de_grad_f64(orc.mandelbulb_polar(8.3, 15, 2.5, rot), pts.cpu().numpy())
    fin = np.all(np.isfinite(ref), axis=1) & np.all(np.isfinite(g), axis=1)
    assert fin.mean() > 0.99
    ang = angle_deg(g[fin, 1:4], ref[fin, 1:4])
    assert np.median(ang) < 0.01 and np.mean(ang < 0.1) >= 0.9, np.quantile(ang, [0.5, 0.9])


def test_adjoint_band_few_iterations(cg, orc):
    """The same band points with max_iters 5: the f32 trajectory still tracks
    FP64, so every output of the adjoint must."""
    from cantucci_gb300.autograd import de_grad
    rot = (0.2, 0.1, 0.0)
    pts = band_points(cg, 4000, 8.3, rot, seed=4)
    g = de_grad(pts, 8.3, rot, max_iters=5).cpu().numpy().astype(np.float64)
    ref = orc.de_grad_f64(orc.mandelbulb_polar(8.3, 5, 2.5, rot), pts.cpu().numpy())
    fin = np.all(np.isfinite(ref), axis=1) & np.all(np.isfinite(g), axis=1)
    ang = angle_deg(g[fin, 1:4], ref[fin, 1:4])
    assert np.mean(ang < 0.1) >= 0.99, np.quantile(ang, [0.5, 0.99])
    rel = np.abs(g[fin, 4] - ref[fin, 4]) / np.maximum(np.abs(ref[fin, 4]), 1e-6)
    assert np.mean(rel < 1e-2) >= 0.99, np.quantile(rel, [0.5, 0.99])
    rot_err = np.abs(g[fin, 5:8] - ref[fin, 5:8]) / np.maximum(
        np.linalg.norm(ref[fin, 5:8], axis=1, keepdims=True), 1e-6)
    assert np.mean(np.all(rot_err < 1e-2, axis=1)) >= 0.99, np.quantile(rot_err.max(1), [0.5, 0.99])
    # the DE itself is the forward estimator's value, bit for bit
    d = cg.MandelbulbPolar(8.3, 5, 2.5, rot).batch_min_distance_from(pts).cpu().numpy()
    np.testing.assert_array_equal(d.view(np.uint32), g[:, 0].astype(np.float32).view(np.uint32))


def test_adjoint_away_from_surface(cg, orc):
    """Points 0.02..0.3 from the surface: no chaos, tight agreement."""
    import torch
    from cantucci_gb300.autograd import de_grad
    rot = (0.2, 0.1, 0.0)
    shape = cg.MandelbulbPolar(8.3, 15, 2.5, rot)
    p = torch.as_tensor(W.uniform_points(200_000, seed=21)).cuda()
    d = shape.batch_min_distance_from(p)
    p = p[(d > 0.02) & (d < 0.3)][:3000].contiguous()
    g = de_grad(p, 8.3, rot).cpu().numpy().astype(np.float64)
    ref = orc.de_grad_f64(orc.mandelbulb_polar(8.3, 15, 2.5, rot), p.cpu().numpy())
    ang = angle_deg(g[:, 1:4], ref[:, 1:4])
    assert np.mean(ang < 0.01) >= 0.99, np.quantile(ang, [0.5, 0.99])
    rel = np.abs(g[:, 4:8] - ref[:, 4:8]) / np.maximum(np.abs(ref[:, 4:8]), 1e-4)
    assert np.mean(np.all(rel < 1e-3, axis=1)) >= 0.99, np.quantile(rel, 0.99, axis=0)


def test_adjoint_matches_fp64_central_differences(cg, orc):
    """Against FP64 central differences with h = 1e-4 (the benchmark's check),
    where the DE is smooth at that scale."""
    from cantucci_gb300.autograd import de_grad
    pts = band_points(cg, 2000, 8.0, seed=1)
    p64 = pts.cpu().numpy().astype(np.float64)
    g = de_grad(pts, 8.0).cpu().numpy().astype(np.float64)
    s = orc.mandelbulb_polar(8.0, 15, 2.5)
    h = 1e-4
    fd = np.zeros((len(p64), 3))
    for a in range(3):
        e = np.zeros(3)
        e[a] = h
        plus = np.array([orc.lib().orc_de_f64(s, *(p + e)) for p in p64])
        minus = np.array([orc.lib().orc_de_f64(s, *(p - e)) for p in p64])
        fd[:, a] = (plus - minus) / (2 * h)
    ref = orc.de_grad_f64(s, pts.cpu().numpy())[:, 1:4]
    smooth = angle_deg(fd, ref) < 0.1  # where h = 1e-4 resolves the gradient
    assert smooth.mean() > 0.25
    ang = angle_deg(g[smooth, 1:4], fd[smooth])
    assert np.mean(ang < 0.1) >= 0.9


def test_autograd_function(cg):
    import torch
    from cantucci_gb300.autograd import de_grad, mandelbulb_de
    pts = band_points(cg, 512, 8.3, (0.2, 0.1, 0.0), seed=2).requires_grad_(True)
    power = torch.tensor(8.3, requires_grad=True)
    rot = torch.tensor([0.2, 0.1, 0.0], requires_grad=True)
    w = torch.linspace(-1, 1, pts.shape[0], device=pts.device)
    loss = (mandelbulb_de(pts, power, rot) * w).sum()
    loss.backward()
    full = de_grad(pts.detach(), 8.3, (0.2, 0.1, 0.0))
    np.testing.assert_allclose(pts.grad.cpu().numpy(), (full[:, 1:4] * w[:, None]).cpu().numpy(),
                               rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(float(power.grad), float((full[:, 4] * w).sum()), rtol=1e-3,
                               atol=1e-4)
    np.testing.assert_allclose(rot.grad.numpy(), (full[:, 5:8] * w[:, None]).sum(0).cpu().numpy(),
                               rtol=1e-3, atol=1e-4)


def test_backward_partials_reuse_and_capture(cg):
    """The parameter gradients' per-warp partials live in a buffer of the
    calling thread that later calls reuse: calls alternating between two
    streams, a larger call that grows the buffer, and a call captured in a
    CUDA graph (which allocates its own) all give the first call's bits."""
    import ctypes as C
    import torch
    from cantucci_gb300 import _ffi
    lib = cg.load()
    shape = cg.MandelbulbPolar(8.3, 15, 2.5, (0.2, 0.1, 0.0))._cshape()

    def backward(pts, g, params, stream):
        _ffi.check(lib.cg_de_backward(C.byref(shape), C.c_void_p(pts.data_ptr()),
                                      C.c_void_p(g.data_ptr()), pts.shape[0], None,
                                      C.c_void_p(params.data_ptr()),
                                      C.c_void_p(stream.cuda_stream)))

    small = band_points(cg, 4096, 8.3, (0.2, 0.1, 0.0), seed=5)
    large = band_points(cg, 1 << 19, 8.3, (0.2, 0.1, 0.0), seed=6)
    gs = torch.linspace(-1, 1, small.shape[0], device="cuda")
    gl = torch.linspace(-1, 1, large.shape[0], device="cuda")
    s0, s1 = torch.cuda.Stream(), torch.cuda.Stream()
    want_s, want_l = torch.empty(4, device="cuda"), torch.empty(4, device="cuda")
    backward(small, gs, want_s, s0)
    s0.synchronize()
    backward(large, gl, want_l, s0)
    s0.synchronize()
    outs = [torch.empty(4, device="cuda") for _ in range(6)]
    for k, o in enumerate(outs):
        st = s0 if k % 2 == 0 else s1
        backward(large if k == 3 else small, gl if k == 3 else gs, o, st)
    torch.cuda.synchronize()
    for k, o in enumerate(outs):
        want = want_l if k == 3 else want_s
        assert torch.equal(o.view(torch.int32), want.view(torch.int32)), k
    # captured: the graph replays the same sums
    gout = torch.empty(4, device="cuda")
    cap = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=cap):
        backward(small, gs, gout, cap)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(gout.view(torch.int32), want_s.view(torch.int32))


def test_fd_grad_matches_adjoint_on_smooth_points(cg):
    """GPU six-evaluation central differences agree with the adjoint where
    the field is smooth at the step."""
    from cantucci_gb300.autograd import de_grad, fd_grad
    pts = band_points(cg, 4000, 8.0, seed=3)
    shape = cg.MandelbulbPolar(8.0, 15, 2.5)
    a = de_grad(pts, 8.0).cpu().numpy()[:, 1:4]
    f1 = fd_grad(pts, shape, 1e-3).cpu().numpy()
    f2 = fd_grad(pts, shape, 5e-4).cpu().numpy()
    smooth = angle_deg(f1, f2) < 0.05
    assert np.median(angle_deg(a[smooth], f2[smooth])) < 0.5


def test_adjoint_rejects_other_shapes(cg):
    import torch
    from cantucci_gb300.autograd import de_grad, _shape
    import ctypes as C
    from cantucci_gb300 import _ffi
    s = cg.Mandelbulb(8, 15, 2.5)._cshape()
    pts = torch.zeros((4, 3), device="cuda")
    out = torch.empty((4, 8), device="cuda")
    assert _ffi.load().cg_de_grad(C.byref(s), C.c_void_p(pts.data_ptr()), 4,
                                  C.c_void_p(out.data_ptr()), None) == _ffi.CG_EINVAL


def test_tangent_mode_matches_adjoint(cg, orc):
    """Forward mode linearises the same f32 trajectory as the adjoint: the
    two agree far more tightly than either agrees with FP64."""
    from cantucci_gb300.autograd import de_grad
    rot = (0.2, 0.1, 0.0)
    pts = band_points(cg, 4000, 8.3, rot, seed=8)
    a = de_grad(pts, 8.3, rot).cpu().numpy().astype(np.float64)
    t = de_grad(pts, 8.3, rot, mode="tangent").cpu().numpy().astype(np.float64)
    # the DE column is the forward estimator's, bit for bit
    d = cg.MandelbulbPolar(8.3, 15, 2.5, rot).batch_min_distance_from(pts).cpu().numpy()
    np.testing.assert_array_equal(d.view(np.uint32), t[:, 0].astype(np.float32).view(np.uint32))
    fin = np.all(np.isfinite(a), axis=1) & np.all(np.isfinite(t), axis=1)
    assert fin.mean() > 0.99
    ang = angle_deg(t[fin, 1:4], a[fin, 1:4])
    assert np.mean(ang < 0.01) >= 0.99, np.quantile(ang, [0.5, 0.99])
    rel = np.abs(t[fin, 4:8] - a[fin, 4:8]) / np.maximum(
        np.linalg.norm(a[fin, 4:8], axis=1, keepdims=True), 1e-6)
    assert np.mean(np.all(rel < 1e-3, axis=1)) >= 0.99, np.quantile(rel.max(1), [0.5, 0.99])
    # against FP64 forward mode, the same bar as the adjoint
    ref = orc.de_grad_f64(orc.mandelbulb_polar(8.3, 15, 2.5, rot), pts.cpu().numpy())
    ok = fin & np.all(np.isfinite(ref), axis=1)
    ang64 = angle_deg(t[ok, 1:4], ref[ok, 1:4])
    assert np.median(ang64) < 0.01 and np.mean(ang64 < 0.1) >= 0.9


def test_tangent_mode_away_from_surface(cg, orc):
    import torch
    from cantucci_gb300.autograd import de_grad
    rot = (0.2, 0.1, 0.0)
    shape = cg.MandelbulbPolar(8.3, 15, 2.5, rot)
    p = torch.as_tensor(W.uniform_points(200_000, seed=22)).cuda()
    d = shape.batch_min_distance_from(p)
    p = p[(d > 0.02) & (d < 0.3)][:3000].contiguous()
    g = de_grad(p, 8.3, rot, mode="tangent").cpu().numpy().astype(np.float64)
    ref = orc.de_grad_f64(orc.mandelbulb_polar(8.3, 15, 2.5, rot), p.cpu().numpy())
    ang = angle_deg(g[:, 1:4], ref[:, 1:4])
    assert np.mean(ang < 0.01) >= 0.99, np.quantile(ang, [0.5, 0.99])
    rel = np.abs(g[:, 4:8] - ref[:, 4:8]) / np.maximum(np.abs(ref[:, 4:8]), 1e-4)
    assert np.mean(np.all(rel < 1e-3, axis=1)) >= 0.99, np.quantile(rel, 0.99, axis=0)


def test_tangent_mode_without_power(cg):
    from cantucci_gb300.autograd import de_grad
    rot = (0.2, 0.1, 0.0)
    pts = band_points(cg, 2000, 8.3, rot, seed=9)
    full = de_grad(pts, 8.3, rot, mode="tangent").cpu().numpy()
    pt = de_grad(pts, 8.3, rot, mode="tangent", with_power=False).cpu().numpy()
    assert np.all(pt[:, 4] == 0)
    np.testing.assert_array_equal(pt[:, 0].view(np.uint32), full[:, 0].view(np.uint32))
    cols = [1, 2, 3, 5, 6, 7]
    scale = np.maximum(np.linalg.norm(full[:, 1:4], axis=1, keepdims=True), 1e-6)
    err = np.abs(pt[:, cols] - full[:, cols]) / scale
    assert np.nanmax(err) < 1e-5


def test_tangent_mode_any_max_iters(cg, orc):
    """Forward mode has no checkpoint table, so max_iters above the
    adjoint's 64 works."""
    import torch
    from cantucci_gb300.autograd import de_grad
    p = torch.as_tensor(W.uniform_points(2000, seed=23)).cuda()
    g = de_grad(p, 8.0, max_iters=80, mode="tangent").cpu().numpy().astype(np.float64)
    d = cg.MandelbulbPolar(8.0, 80, 2.5).batch_min_distance_from(p).cpu().numpy()
    np.testing.assert_array_equal(d.view(np.uint32), g[:, 0].astype(np.float32).view(np.uint32))


def test_tangent_fast_numerics(cg, orc):
    """Forward mode with the fast polar arithmetic: normals close to the
    exact forward mode away from the surface, and in the band most of them
    still within 0.1 degree of FP64."""
    import torch
    from cantucci_gb300.autograd import de_grad
    shape = cg.MandelbulbPolar(8.0, 15, 2.5)
    p = torch.as_tensor(W.uniform_points(200_000, seed=24)).cuda()
    d = shape.batch_min_distance_from(p)
    far = p[(d > 0.02) & (d < 0.3)][:3000].contiguous()
    a = de_grad(far, 8.0, mode="tangent", with_power=False).cpu().numpy()
    b = de_grad(far, 8.0, mode="tangent", with_power=False, fast=True).cpu().numpy()
    ang = angle_deg(b[:, 1:4].astype(np.float64), a[:, 1:4].astype(np.float64))
    assert np.mean(ang < 0.01) >= 0.99, np.quantile(ang, [0.5, 0.99])
    band = band_points(cg, 2000, 8.0, seed=25)
    g = de_grad(band, 8.0, mode="tangent", with_power=False, fast=True).cpu().numpy()
    ref = orc.de_grad_f64(orc.mandelbulb_polar(8.0, 15, 2.5), band.cpu().numpy())
    ok = np.all(np.isfinite(ref[:, 1:4]), axis=1) & np.all(np.isfinite(g[:, 1:4]), axis=1)
    ang64 = angle_deg(g[ok, 1:4].astype(np.float64), ref[ok, 1:4])
    assert np.mean(ang64 < 0.1) >= 0.8, np.mean(ang64 < 0.1)
    with pytest.raises(ValueError):
        de_grad(band, 8.0, fast=True)


@pytest.mark.parametrize("ck", [4, 5, 8])
def test_adjoint_fast_recompute(cg, orc, ck):
    """cg_set_option("adjoint_recompute", 1): every segment but the last is
    recomputed from its exact checkpoint in the fast polar arithmetic.  The
    DE column stays the forward estimator's, bit for bit; the gradient keeps
    the exact recompute's bar against FP64 (median below 0.01 degree, >= 90%
    within 0.1 degree) at every checkpoint interval.  Against the exact
    recompute it drifts with the length of the replayed segment (up to
    interval - 1 fast steps, each amplified by the orbit): within 0.1 degree
    for 98% of the band points at intervals 4 and 5 (measured 98.95% at 5)
    and 97% at 8 (measured 97.65%); the exact adjoint itself is within
    0.1 degree of FP64 for ~93%."""
    from cantucci_gb300 import _ffi
    from cantucci_gb300.autograd import de_grad
    lib = _ffi.load()
    rot = (0.2, 0.1, 0.0)
    pts = band_points(cg, 4000, 8.3, rot, seed=3)
    _ffi.check(lib.cg_set_option(b"adjoint_ck", ck))
    try:
        exact = de_grad(pts, 8.3, rot).cpu().numpy().astype(np.float64)
        _ffi.check(lib.cg_set_option(b"adjoint_recompute", 1))
        fast = de_grad(pts, 8.3, rot).cpu().numpy().astype(np.float64)
    finally:
        lib.cg_set_option(b"adjoint_recompute", 0)
        lib.cg_set_option(b"adjoint_ck", 5)
    d = cg.MandelbulbPolar(8.3, 15, 2.5, rot).batch_min_distance_from(pts).cpu().numpy()
    np.testing.assert_array_equal(d.view(np.uint32), fast[:, 0].astype(np.float32).view(np.uint32))
    ref = orc.de_grad_f64(orc.mandelbulb_polar(8.3, 15, 2.5, rot), pts.cpu().numpy())
    fin = np.all(np.isfinite(ref), axis=1) & np.all(np.isfinite(fast), axis=1)
    assert fin.mean() > 0.99
    ang = angle_deg(fast[fin, 1:4], ref[fin, 1:4])
    assert np.median(ang) < 0.01 and np.mean(ang < 0.1) >= 0.9, np.quantile(ang, [0.5, 0.9])
    ang_e = angle_deg(fast[fin, 1:4], exact[fin, 1:4])
    assert np.mean(ang_e < 0.1) >= (0.98 if ck <= 5 else 0.97), np.quantile(ang_e, [0.5, 0.98])
