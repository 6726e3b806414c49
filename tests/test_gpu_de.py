"""GPU distance estimator against the golden fixtures and the oracle.

Bar: the loop state (r, dr, steps, escaped) of the exact P=8 path is
bit-identical to the reference's; the DE differs only through the final ln
(CUDA logf vs glibc logf), so it is compared to 2 ulp; NaN outputs carry the
x86 bit pattern 0xFFC00000.  Trigonometric paths (P != 8, the polar form)
are compared with the tolerances stated in each test.
"""
import numpy as np
import pytest

from cantucci_gb300 import workloads as W

pytestmark = pytest.mark.gpu

P8_SHAPES = {"p8_i8_b5": (8, 8, 5.0), "p8_i15_b2.5": (8, 15, 2.5)}
TRIG_SHAPES = {"p6_i10_b2.5": (6, 10, 2.5), "p10_i20_b2.5": (10, 20, 2.5), "p3_i6_b2": (3, 6, 2.0)}
DE_ULPS = 2  # CUDA logf vs glibc logf in the final ln(r)


def ulp_diff(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def gpu_state(cg, shape, pts):
    import ctypes as C
    import torch
    from cantucci_gb300 import _ffi
    p = torch.as_tensor(np.ascontiguousarray(pts, np.float32)).cuda()
    out = torch.empty((p.shape[0], 4), dtype=torch.float32, device="cuda")
    _ffi.check(_ffi.load().cg_mandelbulb_state(C.byref(shape._cshape()), C.c_void_p(p.data_ptr()),
                                               p.shape[0], C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def same_bits(a, b):
    """Bit equality, except that any two NaNs match (CUDA's canonical NaN and
    x86's default NaN differ in sign and payload inside the loop state)."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    nan = np.isnan(a) & np.isnan(b)
    return bool(np.all(nan | (a.view(np.uint32) == b.view(np.uint32))))


def test_bench_points_state_bit_exact(cg, golden):
    pts = golden["points"]
    for name, (P, it, b) in P8_SHAPES.items():
        st = gpu_state(cg, cg.Mandelbulb(P, it, b), pts)
        assert same_bits(st[:, 0], golden["r_" + name]), name
        assert same_bits(st[:, 1], golden["dr_" + name]), name
        assert np.array_equal(st[:, 2].view(np.uint32), golden["steps_" + name]), name
        assert np.array_equal(st[:, 3].view(np.uint32), golden["esc_" + name]), name


def test_bench_points_de(cg, golden):
    pts = golden["points"]
    for name, (P, it, b) in P8_SHAPES.items():
        d = cg.Mandelbulb(P, it, b).batch_min_distance_from(pts)
        g = golden["de_" + name]
        nan = np.isnan(g)
        assert np.array_equal(np.isnan(d), nan)
        assert np.all(d[nan].view(np.uint32) == 0xFFC00000), "NaN must carry the x86 sign"
        assert ulp_diff(d[~nan], g[~nan]).max() <= DE_ULPS, name


def test_trig_powers_close(cg, golden):
    """P != 8 runs acosf/atan2f/sinf/cosf; CUDA's and glibc's differ in the
    last bit, which the iteration amplifies near the surface."""
    pts = golden["points"]
    for name, (P, it, b) in TRIG_SHAPES.items():
        st = gpu_state(cg, cg.Mandelbulb(P, it, b), pts)
        steps = st[:, 2].view(np.uint32)
        assert np.mean(steps == golden["steps_" + name]) >= 0.9, name
        d = cg.Mandelbulb(P, it, b).batch_min_distance_from(pts)
        g = golden["de_" + name]
        ok = np.isfinite(g) & (steps == golden["steps_" + name])
        np.testing.assert_allclose(d[ok], g[ok], rtol=1e-3, atol=1e-5)


def test_random_points_state_bit_exact_vs_oracle(cg, orc):
    pts = W.uniform_points(200_000, seed=11, lo=-1.3, hi=1.3)
    s = cg.Mandelbulb(8, 15, 2.5)
    st = gpu_state(cg, s, pts)
    ref = orc.batch_state(orc.mandelbulb(8, 15, 2.5), pts)
    assert same_bits(st, ref)


def test_span_grid_signs_match_golden(cg, golden):
    import torch
    s = cg.Mandelbulb.classic(15, 2.5)
    d = s.span_grid(cg.Span(*W.SPAN_C1), 64)
    torch.cuda.synchronize()
    d = d.cpu().numpy()
    assert np.array_equal(np.packbits(np.signbit(d).ravel()), golden["c1_signbits"])
    sample = d.ravel()[::97]
    g = golden["c1_dist_sample"]
    nan = np.isnan(g)
    assert np.array_equal(np.isnan(sample), nan)
    assert ulp_diff(sample[~nan], g[~nan]).max() <= DE_ULPS


def set_grid_kernel(v):
    import ctypes as C
    from cantucci_gb300 import _ffi
    _ffi.check(_ffi.load().cg_set_option(b"de_grid_kernel", v))


@pytest.mark.parametrize("res", [16, 64, 128])
def test_grid_kernel_variants_bit_identical(cg, golden, res):
    """Linear, 2x4x4-brick and packed 4x4x4-brick step-1 kernels agree bit
    for bit, on the distances and (through the mesher) on the sign words."""
    import torch
    s = cg.Mandelbulb.classic(15, 2.5)
    span = cg.Span(*W.SPAN_C1)
    outs, meshes = [], []
    try:
        for v in (1, 2, 3):
            set_grid_kernel(v)
            d = s.span_grid(span, res)
            torch.cuda.synchronize()
            outs.append(d.cpu().numpy().view(np.uint32))
            buf, _ = cg.MeshBuffer.generate_for_box(span, s, res)
            meshes.append(buf.indices)
    finally:
        set_grid_kernel(0)
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    for m in meshes[1:]:
        assert np.array_equal(m, meshes[0])
    if res == 64:
        assert np.array_equal(np.packbits(np.signbit(outs[0].view(np.float32)).ravel()),
                              golden["c1_signbits"])


def test_span_grid_vs_fp64(cg, orc):
    """Distances of the 65^3 grid against the FP64 oracle.  The GPU loop is
    bit-identical to the reference's f32 loop, so these statistics are the
    reference's own f32 error: signs agree everywhere, >= 99.9% of points are
    within 1e-6 absolute, >= 97% within 1e-5 relative."""
    import torch
    s = cg.Mandelbulb.classic(15, 2.5)
    d32 = s.span_grid(cg.Span(*W.SPAN_C1), 64)
    torch.cuda.synchronize()
    d32 = d32.cpu().numpy().ravel().astype(np.float64)
    n = 65
    rf = np.float32(64)
    st = np.float32(-1.2) + -(np.float32(2.4) / rf)
    en = np.float32(1.2) + np.float32(2.4) / rf
    c = (st + np.float32(en - st) * (np.arange(n, dtype=np.float32) / rf)).astype(np.float32)
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    d64 = orc.de_f64(orc.mandelbulb(8, 15, 2.5), pts)
    fin = np.isfinite(d64) & np.isfinite(d32)
    assert np.array_equal(np.signbit(d32[fin]), np.signbit(d64[fin]))
    err = np.abs(d32[fin] - d64[fin])
    assert np.mean(err <= 1e-6) >= 0.999
    assert np.mean(err <= 1e-5 * np.abs(d64[fin])) >= 0.97


def test_contains(cg, orc):
    pts = W.uniform_points(50_000, seed=3)
    s = cg.Mandelbulb(8, 15, 2.5)
    c = s.batch_contains(pts)
    d = orc.min_distance_from(orc.mandelbulb(8, 15, 2.5), pts)
    assert np.array_equal(c, d < 0.0)
    sp = cg.Sphere((0.1, 0.2, 0.3), 0.7)
    c2 = sp.batch_contains(pts)
    ref = np.array([orc.contains(orc.sphere((0.1, 0.2, 0.3), 0.7), *p) for p in pts[:2000]], bool)
    assert np.array_equal(c2[:2000], ref)


def test_fast_numerics_close(cg):
    """CG_NUMERICS_FAST (FMA, approximate div/sqrt/log) against exact."""
    pts = W.uniform_points(200_000, seed=5)
    s = cg.Mandelbulb(8, 15, 2.5)
    a = s.batch_min_distance_from(pts)
    b = s.fast().batch_min_distance_from(pts)
    fin = np.isfinite(a) & np.isfinite(b)
    assert np.mean(np.signbit(a[fin]) == np.signbit(b[fin])) >= 0.999
    assert np.mean(np.abs(a[fin] - b[fin]) <= 1e-5 + 1e-3 * np.abs(a[fin])) >= 0.99


def test_polar_vs_oracle(cg, orc):
    pts = W.uniform_points(100_000, seed=7)
    s = cg.MandelbulbPolar(8.3, 15, 2.5, (0.2, 0.1, 0.0))
    d = s.batch_min_distance_from(pts)
    ref = orc.min_distance_from(orc.mandelbulb_polar(8.3, 15, 2.5, (0.2, 0.1, 0.0)), pts)
    fin = np.isfinite(ref) & np.isfinite(d)
    assert np.mean(np.signbit(d[fin]) == np.signbit(ref[fin])) >= 0.999
    assert np.mean(np.abs(d[fin] - ref[fin]) <= 1e-5 + 1e-4 * np.abs(ref[fin])) >= 0.99


def test_sphere_bit_exact(cg, orc):
    pts = W.uniform_points(100_000, seed=9)
    d = cg.Sphere((0.1, -0.2, 0.05), 0.9).batch_min_distance_from(pts)
    ref = orc.min_distance_from(orc.sphere((0.1, -0.2, 0.05), 0.9), pts)
    assert np.array_equal(d.view(np.uint32), ref.view(np.uint32))


def test_reference_shaders_fixture(cg):
    """The GPU's sphere and polar estimators against cantucci's own shaders
    (src/shape/shape.frag, src/shape/mandelbulb.frag) compiled as C++ with
    their placeholders filled as the shapes fill them, at 5371 points
    including signed zeros, infinities and NaN coordinates
    (tests/golden/shader_de.npz, made by tests/golden/make_shader_golden.py).
    Sphere: the same bits (IEEE operations only).  Polar form at P = 3, 6,
    8, 10: CUDA's acosf/atan2f/powf/sincosf/logf against glibc's, so the
    bar of test_polar_vs_oracle (>= 99.9% same sign, >= 99% within
    1e-5 + 1e-4 |d|), and NaN where the shader gives NaN."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "shader_de.npz"))
    pts = g["points"]
    for name, kind, par in zip(g["names"], g["kinds"], g["params"]):
        ref = g["de_" + str(name)]
        nan = np.isnan(ref)
        if str(kind) == "sphere":
            d = cg.Sphere(tuple(float(v) for v in par[:3]), float(par[3])).batch_min_distance_from(pts)
            assert np.array_equal(np.isnan(d), nan), name
            assert np.array_equal(d[~nan].view(np.uint32), ref[~nan].view(np.uint32)), name
            continue
        d = cg.MandelbulbPolar(float(par[0]), int(par[1]), float(par[2])).batch_min_distance_from(pts)
        assert np.mean(np.isnan(d) == nan) >= 0.999, name
        fin = np.isfinite(ref) & np.isfinite(d)
        assert np.mean(np.signbit(d[fin]) == np.signbit(ref[fin])) >= 0.999, name
        assert np.mean(np.abs(d[fin] - ref[fin]) <= 1e-5 + 1e-4 * np.abs(ref[fin])) >= 0.99, name


def test_march_matches_golden(cg, golden):
    hits, hit = cg.march(cg.Mandelbulb(8, 15, 2.5), golden["march_origins"], golden["march_dirs"],
                         100, 1e-6)
    assert np.array_equal(hit, golden["march_hit"])
    np.testing.assert_allclose(hits, golden["march_hits"], rtol=0, atol=1e-5)


def test_invalid_shape_raises(cg):
    with pytest.raises(cg.CantucciError):
        m = cg.Mandelbulb(8, 15, 2.5)
        m.max_iters = 0
        m.batch_min_distance_from(np.zeros((4, 3), np.float32))


@pytest.mark.parametrize("P", [3, 6, 10])
def test_int_power_trig_free_path(cg, orc, P):
    """Fast numerics for integer P != 8: the complex-power form is as close
    to the FP64 trig formula as the (libm) trig path is."""
    import torch
    pts = W.uniform_points(200_000, seed=30 + P)
    p = torch.as_tensor(pts).cuda()
    exact = cg.Mandelbulb(P, 15, 2.5)
    d_exact = exact.batch_min_distance_from(p).cpu().numpy().astype(np.float64)
    d_fast = exact.fast().batch_min_distance_from(p).cpu().numpy().astype(np.float64)
    ref = orc.de_f64(orc.mandelbulb(P, 15, 2.5), pts)
    ok = np.isfinite(ref)
    scale = np.maximum(np.abs(ref[ok]), 1e-6)
    close_fast = np.mean(np.abs(d_fast[ok] - ref[ok]) / scale < 1e-3)
    close_exact = np.mean(np.abs(d_exact[ok] - ref[ok]) / scale < 1e-3)
    assert close_fast >= 0.99 and close_fast >= close_exact - 0.005, (close_fast, close_exact)
    assert np.mean(np.sign(d_fast[ok]) == np.sign(ref[ok])) >= 0.999
