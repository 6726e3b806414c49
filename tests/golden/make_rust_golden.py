"""Generates tests/golden/rust_ref.npz from cantucci's own Rust source: the
estimator (src/shape/mandelbulb.rs, src/shape/sphere.rs) and the mesher
(src/mesh/buffer.rs with src/math.rs, src/util/grid.rs, src/util/iter.rs),
translated into C++ and compiled by oracle/rust_build.py.  Needs the
reference tree and x86-64 (the reference is x86-only).  Run from the
repository root:

    CANTUCCI_REFERENCE=<cantucci source tree> python tests/golden/make_rust_golden.py

The fixture pins, wherever the tests run (the GPU machine has no reference tree):
  - the oracle, bit for bit: the estimator at the reference's BENCH_POINTS,
    edge points and 200,000 seeded points (by digest), whole meshes
    (distance grid, cell table, vertices, indices; by digest), and the
    513^3-corner span, where the reference panics in lerp (its distance grid
    by digest, the panic, the NaN corners);
  - the GPU, within what its logf allows: distance signs and index lists
    bit for bit, distances within 7 ulp (99% within 2).
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

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rust_ref.npz")

# (name, power, max_iters, bailout).  p8_i8_b5 is the reference's own bench
# shape, Mandelbulb::classic(8, 5.0) (src/shape/bench.rs:15).
DE_CONFIGS = [("p8_i15_b2.5", 8, 15, 2.5), ("p8_i8_b5", 8, 8, 5.0), ("p6_i10_b2.5", 6, 10, 2.5),
              ("p10_i20_b2.5", 10, 20, 2.5), ("p3_i6_b2", 3, 6, 2.0)]
RAND_SEED, RAND_N, RAND_KEEP = 20261204, 200_000, 8192
# (name, shape args, span, res): config 1 (res 64), smaller spans, a sphere,
# the other integer powers of the batched workload.
MESHES = [("c1", ("mandelbulb", 8, 15, 2.5), W.SPAN_C1, 64),
          ("p8_r16", ("mandelbulb", 8, 15, 2.5), W.SPAN_C1, 16),
          ("p8_r8_leaf", ("mandelbulb", 8, 15, 2.5), ((0.3, -0.6, -0.3), (0.6, -0.3, 0.0)), 8),
          ("p6_r32", ("mandelbulb", 6, 10, 2.5), W.SPAN_C1, 32),
          ("p10_r32", ("mandelbulb", 10, 20, 2.5), W.SPAN_C1, 32),
          ("sphere_r16", ("sphere", (0.1, -0.05, 0.02), 0.9), W.SPAN_C1, 16)]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def edge_points() -> np.ndarray:
    """The origin and the z axis (rotate_on_z_axis) with every sign of zero,
    tiny and subnormal x/y, points far outside the bailout, and infinite and
    NaN coordinates."""
    z = [0.0, -0.0]
    pts = [[a, b, c] for a in z for b in z for c in (0.0, -0.0, 0.3, -0.7, 1.1, 2.0)]
    pts += [[1e-40, 0.0, 0.5], [0.0, -1e-42, -0.3], [1e-45, 1e-45, 0.1], [1e-20, 1e-20, 0.6],
            [1e-3, 1e-3, 1e-3], [3.0, 0.0, 0.0], [1e30, 0.0, 0.0], [0.9, 0.9, 0.9],
            [np.inf, 0.0, 0.0], [0.0, 0.0, np.inf], [np.nan, 0.0, 0.0], [-np.inf, 0.5, 0.5],
            [0.0, 0.0, 1.2375], [-1.2375, -1.2375, -1.2375]]
    return np.array(pts, np.float32)


def rand_points() -> np.ndarray:
    rng = np.random.default_rng(RAND_SEED)
    return rng.uniform(-1.5, 1.5, (RAND_N, 3)).astype(np.float32)


def make_shape(args):
    if args[0] == "sphere":
        return O.sphere(args[1], args[2])
    return O.mandelbulb(*args[1:])


def main():
    if platform.machine() != "x86_64":
        raise SystemExit("the reference's Rust source is x86-64 only")
    if O.rust_ref() is None:
        raise SystemExit("set CANTUCCI_REFERENCE to the cantucci source tree")
    g = {"bench_points": W.bench_points(), "edge_points": edge_points(),
         "rand_seed": np.int64(RAND_SEED), "rand_n": np.int64(RAND_N),
         "de_configs": np.array([[p, i, b] for _, p, i, b in DE_CONFIGS], np.float64),
         "de_names": np.array([c[0] for c in DE_CONFIGS])}
    rnd = rand_points()
    g["rand_head"] = rnd[:RAND_KEEP]
    for name, p, it, b in DE_CONFIGS:
        s = O.mandelbulb(p, it, b)
        g["de_bench_" + name] = O.rust_ref_de(s, W.bench_points())
        g["de_edge_" + name] = O.rust_ref_de(s, edge_points())
        g["contains_edge_" + name] = O.rust_ref_contains(s, edge_points())
        d = O.rust_ref_de(s, rnd)
        g["de_rand_head_" + name] = d[:RAND_KEEP]
        g["de_rand_sha_" + name] = np.array(sha(d))
    sph = O.sphere((0.1, -0.05, 0.02), 0.9)
    g["de_edge_sphere"] = O.rust_ref_de(sph, edge_points())
    g["contains_edge_sphere"] = O.rust_ref_contains(sph, edge_points())
    g["de_rand_sha_sphere"] = np.array(sha(O.rust_ref_de(sph, rnd)))
    for name, args, span, res in MESHES:
        m = O.rust_ref_generate_for_box(make_shape(args), np.array(span, np.float32).ravel(), res)
        if m["rc"] != O.RR_OK:
            raise SystemExit("mesh %s: rc %d" % (name, m["rc"]))
        g["mesh_%s_span" % name] = np.array(span, np.float32).ravel()
        g["mesh_%s_res" % name] = np.int64(res)
        g["mesh_%s_counts" % name] = np.array([m["nv"], m["ni"]], np.int64)
        for part in ("dists", "points", "vertices", "indices"):
            g["mesh_%s_sha_%s" % (name, part)] = np.array(sha(m[part]))
        g["mesh_%s_signbits_sha" % name] = np.array(sha(np.packbits(np.signbit(m["dists"]))))
        if res <= 16:  # small meshes travel whole
            g["mesh_%s_vertices" % name] = m["vertices"].view(np.float32).reshape(-1, 7)
            g["mesh_%s_indices" % name] = m["indices"]
    # config 2, the 513^3-corner span: the reference panics in lerp (a NaN
    # corner next to an outside one); its distance grid is complete by then
    m = O.rust_ref_generate_for_box(O.mandelbulb(8, 15, 2.5),
                                    np.array(W.SPAN_C1, np.float32).ravel(), 512, vcap=1, icap=1)
    g["c2_rc"] = np.int64(m["rc"])
    g["c2_sha_dists"] = np.array(sha(m["dists"]))
    g["c2_nan_corners"] = np.argwhere(np.isnan(m["dists"])).astype(np.int64)
    np.savez_compressed(OUT, **g)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
