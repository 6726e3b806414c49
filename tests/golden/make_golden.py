"""Generates the golden fixtures in this directory from the CPU oracle.

The reference ships no expected values (its benches assert nothing), so the
fixtures are the oracle's restatement of the reference, computed on x86-64
with glibc libm -- the only platform the reference builds on.  Run from the
repository root:  python tests/golden/make_golden.py
"""
import hashlib
import os
import platform
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from cantucci_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def special_points() -> np.ndarray:
    """Edge cases: origin, the z axis (rotate_on_z_axis path), tiny x/y,
    cube corners, points far outside (escape at the first test)."""
    pts = [[0, 0, 0], [0, 0, 0.5], [0, 0, -0.5], [0, 0, 1.1], [0, 0, -1.1], [-0.0, 0.0, 0.3],
           [0.0, -0.0, -0.3], [0, 0, 1.2375], [1e-20, 0, 0.5], [0, 1e-20, -0.5], [1e-30, 1e-30, 0.7],
           [1.2, 1.2, 1.2], [-1.2375, -1.2375, -1.2375], [3.0, 0, 0], [0, 3.0, 0], [0.9, 0.9, 0.9],
           [0.3, 0.0, 0.0], [0.0, 0.3, 0.0], [-0.3, 0.0, 0.0], [1e-3, 1e-3, 1e-3]]
    return np.array(pts, np.float32)


def state_arrays(shape, pts):
    st = np.array([O.state(shape, p) for p in pts], dtype=np.float64)
    r = st[:, 0].astype(np.float32)
    dr = st[:, 1].astype(np.float32)
    return r, dr, st[:, 2].astype(np.uint32), st[:, 3].astype(np.uint32)


def main():
    if platform.machine() != "x86_64":
        raise SystemExit("golden fixtures are generated on x86-64 (the reference's platform)")
    g = {}
    pts = np.concatenate([W.bench_points(), special_points()])
    g["points"] = pts
    shapes = {"p8_i8_b5": O.mandelbulb(8, 8, 5.0), "p8_i15_b2.5": O.mandelbulb(8, 15, 2.5),
              "p6_i10_b2.5": O.mandelbulb(6, 10, 2.5), "p10_i20_b2.5": O.mandelbulb(10, 20, 2.5),
              "p3_i6_b2": O.mandelbulb(3, 6, 2.0)}
    for name, s in shapes.items():
        g["de_" + name] = O.min_distance_from(s, pts)
        r, dr, k, e = state_arrays(s, pts)
        g["r_" + name], g["dr_" + name], g["steps_" + name], g["esc_" + name] = r, dr, k, e
        g["de64_" + name] = O.de_f64(s, pts)
    polar = O.mandelbulb_polar(8.3, 15, 2.5, (0.2, 0.1, 0.0))
    g["de_polar"] = O.min_distance_from(polar, pts)
    g["de64_polar"] = O.de_f64(polar, pts)
    g["grad64_polar"] = O.de_grad_f64(polar, pts)
    g["grad64_p8"] = O.de_grad_f64(shapes["p8_i15_b2.5"], pts)

    # Single span, res 64 (65^3 corners): full mesh digests plus samples.
    s = shapes["p8_i15_b2.5"]
    m = O.generate_for_box(s, np.array(W.SPAN_C1).ravel(), 64, want_grids=True)
    assert m["rc"] == 0
    d = m["dists"]
    g["c1_counts"] = np.array([m["nv"], m["ni"]], np.uint64)
    g["c1_signbits"] = np.packbits(np.signbit(d).ravel())
    g["c1_dists_sha"] = np.frombuffer(bytes.fromhex(sha(d)), np.uint8)
    g["c1_points_sha"] = np.frombuffer(bytes.fromhex(sha(m["points"])), np.uint8)
    g["c1_indices_sha"] = np.frombuffer(bytes.fromhex(sha(m["indices"])), np.uint8)
    g["c1_vertices_sha"] = np.frombuffer(bytes.fromhex(sha(m["vertices"])), np.uint8)
    g["c1_dist_sample"] = d.ravel()[::97].copy()
    g["c1_vertex_sample"] = m["vertices"].view(np.float32).reshape(-1, 7)[::37].copy()
    g["c1_index_head"] = m["indices"][:6000].copy()

    # Small spans of the batched workload generator, full meshes.
    spans, res, _, _ = W.batched_spans(256, seed=0)
    small, used = [], set()
    for P, it in ((6, 10), (8, 15), (10, 20)):
        for rr in (8, 16):
            for i in range(len(spans)):  # first unused span that meets the surface
                if i in used:
                    continue
                t = O.generate_for_box(O.mandelbulb(P, it, 2.5), spans[i], rr)
                if t["rc"] == 0 and t["nv"] > 20:
                    used.add(i)
                    small.append((P, it, spans[i], rr))
                    break
    for n, (P, it, sp, rr) in enumerate(small):
        mm = O.generate_for_box(O.mandelbulb(P, it, 2.5), sp, rr, want_grids=True)
        assert mm["rc"] == 0, mm["rc"]
        g["small%d_meta" % n] = np.array([P, it, rr], np.int64)
        g["small%d_span" % n] = sp
        g["small%d_dists" % n] = mm["dists"]
        g["small%d_points" % n] = mm["points"]
        g["small%d_vertices" % n] = mm["vertices"].view(np.float32).reshape(-1, 7)
        g["small%d_indices" % n] = mm["indices"]

    # Sphere: every value is IEEE add/mul/div/sqrt, so the whole mesh is bit-exact.
    for n, (c, rad, sp, rr) in enumerate((((0.1, -0.2, 0.05), 0.9, (-1, -1, -1, 1, 1, 1), 16),
                                           ((0.0, 0.0, 0.0), 0.5, (0, 0, 0, 0.6, 0.6, 0.6), 8))):
        mm = O.generate_for_box(O.sphere(c, rad), np.array(sp, np.float32), rr, want_grids=True)
        assert mm["rc"] == 0
        g["sphere%d_meta" % n] = np.array([*c, rad, rr], np.float32)
        g["sphere%d_span" % n] = np.array(sp, np.float32)
        g["sphere%d_dists" % n] = mm["dists"]
        g["sphere%d_points" % n] = mm["points"]
        g["sphere%d_vertices" % n] = mm["vertices"].view(np.float32).reshape(-1, 7)
        g["sphere%d_indices" % n] = mm["indices"]

    # March loop of get_focii on a fan of rays from a camera at distance 2.5.
    o = np.tile(np.array([[0.0, 0.0, 2.5]], np.float32), (25, 1))
    u, v = np.meshgrid(np.linspace(-0.3, 0.3, 5), np.linspace(-0.3, 0.3, 5))
    dirs = np.stack([u.ravel(), v.ravel(), -np.ones(25)], 1)
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    hits, hit = O.march(s, o, dirs, 100, 1e-6)
    g["march_origins"], g["march_dirs"], g["march_hits"], g["march_hit"] = o, dirs, hits, hit

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes;", "c1 counts", g["c1_counts"])


if __name__ == "__main__":
    main()
