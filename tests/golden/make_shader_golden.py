"""Generates tests/golden/shader_de.npz: cantucci's own estimator shaders
(src/shape/mandelbulb.frag, src/shape/shape.frag), compiled as C++ by
oracle/ref_build.py with their placeholders filled as the shapes fill them,
evaluated at fixed points.  Needs the reference tree (to build the shader
library) and x86-64 with glibc, where the reference runs.  Run from the
repository root:  python tests/golden/make_shader_golden.py

The fixture then pins, wherever the tests run:
  - the oracle's polar and sphere estimators, bit for bit;
  - the GPU's, within the tolerance its trigonometric functions need.
"""
import os
import platform
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import oracle as O  # noqa: E402
from oracle import ref_build as RB  # noqa: E402
from cantucci_gb300 import workloads as W  # noqa: E402
from make_golden import special_points  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "shader_de.npz")


def points() -> np.ndarray:
    """The reference's BENCH_POINTS, the mesh fixtures' special points, every
    combination of a few awkward coordinates (signed zeros, tiny, infinite,
    NaN, outside the bailout) and 4000 seeded uniform points in [-1.5, 1.5]^3."""
    vals = np.array([0.0, -0.0, 1e-30, -1e-30, 0.5, -0.5, 1.1, np.inf, -np.inf, np.nan, 3.0],
                    np.float32)
    grid = np.stack(np.meshgrid(vals, vals, vals, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(20240601)
    uni = rng.uniform(-1.5, 1.5, (4000, 3)).astype(np.float32)
    return np.concatenate([W.bench_points(), special_points(), grid, uni]).astype(np.float32)


def main():
    if platform.machine() != "x86_64":
        raise SystemExit("shader fixtures are generated on x86-64 (the reference's platform)")
    if O.ref_shader() is None:
        raise SystemExit("the reference tree is needed to build oracle/_ref/libref_shader.so")
    pts = points()
    g = {"points": pts,
         "names": np.array([c[0] for c in RB.CONFIGS]),
         "kinds": np.array([c[1] for c in RB.CONFIGS]),
         "params": np.array([list(c[2]) + [0.0] * (4 - len(c[2])) for c in RB.CONFIGS],
                            np.float64)}
    for i, (name, _, _) in enumerate(RB.CONFIGS):
        g["de_" + name] = O.ref_shader_de(i, pts)
    np.savez_compressed(OUT, **g)
    print(OUT, {k: v.shape for k, v in g.items()})


if __name__ == "__main__":
    main()
