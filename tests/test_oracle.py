"""The CPU oracle against the golden fixtures and against itself (no GPU).

On x86-64 (where the fixtures were made) every value must match bit for
bit.  On other hosts libm's logf/acosf/... may round differently, so values
that pass through libm are compared to a few ulp and everything computed
with IEEE add/mul/div/sqrt only is still compared bit for bit.
"""
import hashlib
import os
import platform

import numpy as np
import pytest

from cantucci_gb300 import workloads as W

X86 = platform.machine() == "x86_64"
SHAPES = {"p8_i8_b5": (8, 8, 5.0), "p8_i15_b2.5": (8, 15, 2.5), "p6_i10_b2.5": (6, 10, 2.5),
          "p10_i20_b2.5": (10, 20, 2.5), "p3_i6_b2": (3, 6, 2.0)}


def ulp_diff(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def same_bits_or_close(a, b, ulps):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    if X86:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all(both_nan | (ulp_diff(a, b) <= ulps)))


def test_bench_points_match_golden(orc, golden):
    pts = golden["points"]
    assert np.array_equal(pts[:20], W.bench_points())
    for name, (P, it, b) in SHAPES.items():
        s = orc.mandelbulb(P, it, b)
        de = orc.min_distance_from(s, pts)
        assert same_bits_or_close(de, golden["de_" + name], 2), name
        st = np.array([orc.state(s, p) for p in pts])
        assert np.array_equal(st[:, 2].astype(np.uint32), golden["steps_" + name])
        assert np.array_equal(st[:, 3].astype(np.uint32), golden["esc_" + name])
        if P == 8:  # trig-free path: the loop state is libm-independent
            r = st[:, 0].astype(np.float32)
            assert np.array_equal(r.view(np.uint32)[:20], golden["r_" + name].view(np.uint32)[:20])


def test_origin_is_negative_nan(orc):
    """0/0 at the origin gives x86's default NaN (sign set): inside."""
    s = orc.mandelbulb(8, 15, 2.5)
    d = orc.min_distance_from(s, np.zeros((1, 3), np.float32))
    assert d.view(np.uint32)[0] == 0xFFC00000


def test_de_f32_close_to_f64(orc, golden):
    """f32 oracle vs FP64 on the fixture points (all near the surface, where
    f32 rounding is amplified by the iteration): same sign, and 1e-4 absolute
    where the escape step agrees."""
    pts = golden["points"]
    for name, (P, it, b) in SHAPES.items():
        s = orc.mandelbulb(P, it, b)
        d32 = orc.min_distance_from(s, pts).astype(np.float64)
        d64, k64 = orc.de_f64(s, pts, with_steps=True)
        k32 = golden["steps_" + name]
        ok = np.isfinite(d64) & np.isfinite(d32) & (k64 == k32)
        err = np.abs(d32[ok] - d64[ok])
        assert np.all(err <= 1e-4 + 1e-5 * np.abs(d64[ok])), (name, err.max(), np.argmax(err))
        assert np.array_equal(np.signbit(d32[ok]), np.signbit(d64[ok])), name


def test_grad_f64_against_central_differences(orc):
    pts = W.bench_points()[:6].astype(np.float64)
    for s in (orc.mandelbulb(8, 15, 2.5), orc.mandelbulb(6, 10, 2.5),
              orc.mandelbulb_polar(8.3, 15, 2.5, (0.2, 0.1, 0.0))):
        g = orc.de_grad_f64(s, pts.astype(np.float32))
        checked = 0

        def fd(p, h):
            out = []
            for k in range(3):
                e = np.zeros(3)
                e[k] = h
                out.append((orc.lib().orc_de_f64(s, *(p + e)) - orc.lib().orc_de_f64(s, *(p - e))) / (2 * h))
            return np.array(out)

        for i, p in enumerate(pts.astype(np.float32).astype(np.float64)):
            a, b = fd(p, 1e-9), fd(p, 1e-8)
            # The DE is only piecewise smooth (the escape step jumps); test
            # where the two step sizes agree.
            if np.linalg.norm(a - b) > 1e-2 * np.linalg.norm(a):
                continue
            checked += 1
            np.testing.assert_allclose(g[i, 1:4], a, rtol=0, atol=1e-4 * np.linalg.norm(a))
        assert checked >= 3


def test_c1_mesh_matches_golden(orc, golden):
    s = orc.mandelbulb(8, 15, 2.5)
    m = orc.generate_for_box(s, np.array(W.SPAN_C1).ravel(), 64, want_grids=True)
    assert m["rc"] == 0
    assert [m["nv"], m["ni"]] == golden["c1_counts"].tolist()
    assert np.array_equal(np.packbits(np.signbit(m["dists"]).ravel()), golden["c1_signbits"])
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()
    assert sha(m["points"]) == golden["c1_points_sha"].tobytes()
    assert sha(m["indices"]) == golden["c1_indices_sha"].tobytes()
    if X86:
        assert sha(m["dists"]) == golden["c1_dists_sha"].tobytes()
        assert sha(m["vertices"]) == golden["c1_vertices_sha"].tobytes()


def test_mesh_is_deterministic_across_threads(orc):
    s = orc.mandelbulb(8, 15, 2.5)
    a = orc.generate_for_box(s, np.array(W.SPAN_C1).ravel(), 32, nthreads=1)
    b = orc.generate_for_box(s, np.array(W.SPAN_C1).ravel(), 32, nthreads=7)
    assert np.array_equal(a["indices"], b["indices"])
    assert np.array_equal(a["vertices"].view(np.uint8), b["vertices"].view(np.uint8))


def test_small_and_sphere_meshes_match_golden(orc, golden):
    for n in range(6):
        P, it, rr = golden["small%d_meta" % n].tolist()
        m = orc.generate_for_box(orc.mandelbulb(P, it, 2.5), golden["small%d_span" % n], rr,
                                 want_grids=True)
        assert m["rc"] == 0
        assert np.array_equal(m["points"], golden["small%d_points" % n])
        assert np.array_equal(m["indices"], golden["small%d_indices" % n])
    for n in range(2):
        meta = golden["sphere%d_meta" % n]
        m = orc.generate_for_box(orc.sphere(meta[:3], meta[3]), golden["sphere%d_span" % n],
                                 int(meta[4]), want_grids=True)
        assert np.array_equal(m["vertices"].view(np.float32).reshape(-1, 7).view(np.uint32),
                              golden["sphere%d_vertices" % n].view(np.uint32))
        assert np.array_equal(m["indices"], golden["sphere%d_indices" % n])


def test_mesh_topology_invariants(orc):
    """Every quad references surface cells; every surface cell is used."""
    s = orc.mandelbulb(8, 15, 2.5)
    m = orc.generate_for_box(s, np.array(W.SPAN_C1).ravel(), 32, want_grids=True)
    idx = m["indices"]
    assert len(idx) % 6 == 0
    assert idx.max() < m["nv"]
    assert len(np.unique(idx)) == m["nv"]
    pts = m["points"].ravel()
    surf = pts != 0xFFFFFFFF
    assert np.array_equal(pts[surf], np.arange(m["nv"], dtype=np.uint32))


@pytest.mark.parametrize("shape,res", [("p8", 32), ("p8", 64), ("sphere", 16)])
def test_mesh_from_dists_reproduces_the_mesher(orc, shape, res):
    """Steps 2-3 on given corner distances (the entry the GPU parity tests
    feed with the GPU's own grid) reproduce generate_for_box bit for bit when
    given its own step-1 grid; a changed distance changes the mesh there."""
    s = orc.mandelbulb(8, 15, 2.5) if shape == "p8" else orc.sphere((0.1, -0.05, 0.02), 0.9)
    span = np.array(W.SPAN_C1, np.float32).ravel()
    full = orc.generate_for_box(s, span, res, want_grids=True)
    again = orc.mesh_from_dists(s, span, res, full["dists"])
    assert again["rc"] == full["rc"] and (again["nv"], again["ni"]) == (full["nv"], full["ni"])
    assert np.array_equal(again["indices"], full["indices"])
    assert np.array_equal(again["points"], full["points"])
    assert np.array_equal(again["vertices"].view(np.uint8), full["vertices"].view(np.uint8))
    # flip the sign of one inside corner next to the surface: the cell table moves
    d = full["dists"].copy().reshape(-1)
    k = int(np.flatnonzero((d < 0) & (d > -0.05))[0])
    d[k] = -d[k]
    moved = orc.mesh_from_dists(s, span, res, d)
    assert not np.array_equal(moved["points"], full["points"])


def test_mesh_from_dists_rejects_a_null_grid(orc):
    import ctypes as C
    lib = orc.lib()
    nv, ni = C.c_uint64(), C.c_uint64()
    span = np.array(W.SPAN_C1, np.float32).ravel()
    rc = lib.orc_mesh_from_dists(C.byref(orc.mandelbulb(8, 15, 2.5)), span.ctypes.data, 8, 1,
                                 None, None, None, 0, None, 0, C.byref(nv), C.byref(ni))
    assert rc == orc.ORC_EINVAL


def test_sphere_vertices_near_surface(orc):
    c, r = np.array([0.1, -0.2, 0.05], np.float32), 0.9
    m = orc.generate_for_box(orc.sphere(c, r), np.array([-1, -1, -1, 1, 1, 1], np.float32), 32)
    p = m["vertices"]["position"]
    dist = np.linalg.norm(p - c, axis=1) - r
    assert np.abs(dist).max() < 2.0 / 32
    n = m["vertices"]["normal"]
    radial = (p - c) / np.linalg.norm(p - c, axis=1, keepdims=True)
    assert np.min(np.sum(n * radial, axis=1)) > 0.99


@pytest.mark.parametrize("span,res", [((0, 0, 0, -1, 1, 1), 8), ((0, 0, 0, 1, 1, 1), 6),
                                      ((0, 0, 0, 1, 1, 1), 0), ((0, 0, 0, 1, 1, 1), 1)])
def test_invalid_span_or_resolution(orc, span, res):
    m = orc.generate_for_box(orc.mandelbulb(8, 15, 2.5), np.array(span, np.float32), res, vcap=0,
                             icap=0)
    assert m["rc"] == orc.ORC_EINVAL


def test_capacity_reporting(orc):
    s = orc.mandelbulb(8, 15, 2.5)
    m = orc.generate_for_box(s, np.array(W.SPAN_C1).ravel(), 16, vcap=10, icap=10)
    assert m["rc"] == orc.ORC_ECAPACITY
    full = orc.generate_for_box(s, np.array(W.SPAN_C1).ravel(), 16)
    assert (m["nv"], m["ni"]) == (full["nv"], full["ni"])


def test_march_matches_golden(orc, golden):
    hits, hit = orc.march(orc.mandelbulb(8, 15, 2.5), golden["march_origins"], golden["march_dirs"],
                          100, 1e-6)
    assert np.array_equal(hit, golden["march_hit"])
    assert same_bits_or_close(hits, golden["march_hits"], 64)


def test_create_spans_order(orc):
    parent = np.array([-1.2, -1.2, -1.2, 1.2, 1.2, 1.2], np.float32)
    ch = orc.create_spans(parent)
    # child 3 = x lower, y upper, z upper (src/octree/mod.rs:322)
    assert np.allclose(ch[3], [-1.2, 0, 0, 0, 1.2, 1.2])
    vol = np.prod(ch[:, 3:] - ch[:, :3], axis=1)
    assert np.allclose(vol.sum(), 2.4 ** 3, rtol=1e-6)


def test_qef_model(orc):
    """The FP64 dual-contouring model: on a sphere its vertices lie within a
    tenth of a cell of the surface (the reference's centroids: about a fifth
    of a cell off, the worst most of a cell) and inside their cells; on the
    P=8 Mandelbulb the median |DE| at the vertices is well below the
    centroids'."""
    from oracle import qef
    sh = orc.sphere((0.1, -0.05, 0.02), 0.9)
    m, cells, start, step = qef.mesh_cells(sh, np.array(W.SPAN_C1), 16)
    v = qef.qef_vertices(sh, m["dists"], cells, start, step)
    c = np.array([0.1, -0.05, 0.02])
    rq = np.abs(np.linalg.norm(v - c, axis=1) - 0.9) / step[0]
    rc = np.abs(np.linalg.norm(m["vertices"]["position"] - c, axis=1) - 0.9) / step[0]
    assert rq.max() < 0.1 and np.median(rc) > 4 * np.median(rq)
    lo = (start + cells.astype(np.float32) * step).astype(np.float64)
    assert np.all((v >= lo) & (v <= lo + step.astype(np.float64)))
    mb = orc.mandelbulb(8, 15, 2.5)
    m, cells, start, step = qef.mesh_cells(mb, np.array(W.SPAN_C1), 32)
    v = qef.qef_vertices(mb, m["dists"], cells, start, step)
    dq = np.abs(orc.de_f64(mb, v.astype(np.float32)))
    dc = np.abs(orc.de_f64(mb, m["vertices"]["position"]))
    assert np.median(dq) < 0.5 * np.median(dc)


# ---- the reference's own estimator shaders (oracle/ref_build.py) --------

SHADER_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "shader_de.npz")


def shader_shape(orc, kind, par):
    """The oracle shape a filled shader describes: mandelbulb.frag with
    power P is the polar form at power P without rotation."""
    if kind == "mandelbulb":
        return orc.mandelbulb_polar(float(par[0]), int(par[1]), float(par[2]), (0.0, 0.0, 0.0))
    return orc.sphere(tuple(float(v) for v in par[:3]), float(par[3]))


def shader_agrees(ours, ref):
    """Same bits wherever the shader's value is a number (on x86-64; 2 ulps
    elsewhere, where libm differs), NaN on both sides where it is NaN (the
    oracle returns x86's default NaN for every NaN; the compiled shader keeps
    the sign glibc gives)."""
    ours = np.asarray(ours, np.float32)
    ref = np.asarray(ref, np.float32)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(ours), nan)
    return same_bits_or_close(ours[~nan], ref[~nan], 2)


def test_oracle_matches_reference_shader_fixture(orc):
    """The oracle's polar and sphere estimators against cantucci's own
    shaders (src/shape/mandelbulb.frag, src/shape/shape.frag) compiled as
    C++ with their placeholders filled as src/shape/mandelbulb.rs:82-85 and
    src/shape/sphere.rs:42-46 fill them (tests/golden/make_shader_golden.py):
    five Mandelbulb powers and two spheres at 5371 points, including signed
    zeros, infinities and NaN coordinates."""
    g = np.load(SHADER_GOLDEN)
    pts = g["points"]
    assert np.array_equal(pts[:20], W.bench_points())
    for name, kind, par in zip(g["names"], g["kinds"], g["params"]):
        ours = orc.min_distance_from(shader_shape(orc, str(kind), par), pts)
        assert shader_agrees(ours, g["de_" + str(name)]), name


def test_oracle_matches_reference_shader_live(orc):
    """The same against the shader library built from the reference tree
    here, at 200,000 further seeded points (skipped where the reference tree
    and an earlier build are both absent)."""
    if orc.ref_shader() is None:
        pytest.skip("reference shaders not built")
    from oracle import ref_build
    g = np.load(SHADER_GOLDEN)
    rng = np.random.default_rng(77)
    pts = rng.uniform(-1.6, 1.6, (200_000, 3)).astype(np.float32)
    for i, (name, kind, par) in enumerate(ref_build.CONFIGS):
        ref = orc.ref_shader_de(i, pts)
        assert shader_agrees(orc.min_distance_from(shader_shape(orc, kind, par), pts), ref), name
        # the fixture is what this build computes
        fx = orc.ref_shader_de(i, g["points"])
        assert np.array_equal(np.isnan(fx), np.isnan(g["de_" + name]))
        ok = ~np.isnan(fx)
        assert np.array_equal(fx[ok].view(np.uint32), g["de_" + name][ok].view(np.uint32)), name


def test_shader_placeholder_formatting():
    """The recipe fills the shaders' placeholders with Rust's Display of an
    f32 (shortest round-trip digits, no exponent, no trailing ".0"), as
    src/shape/mandelbulb.rs:83 and src/shape/sphere.rs:43-46 do."""
    from oracle.ref_build import rust_f32
    cases = {2.5: "2.5", 5.0: "5", -0.05: "-0.05", 1e-7: "0.0000001", 1e10: "10000000000",
             0.1: "0.1", -0.0: "-0", 8.3: "8.3", 1.0 / 3.0: "0.33333334"}
    for v, want in cases.items():
        assert rust_f32(v) == want, (v, rust_f32(v))
