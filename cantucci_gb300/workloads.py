"""The benchmark workloads, as synthetic inputs with the stated shapes.

single_span(res):  Mandelbulb P=8, max_iters 15, bailout 2.5, span
                   [-1.2, 1.2]^3, `res` cells per axis (64: 65^3 corners,
                   512: 513^3 corners).
batched_spans():   4096 octree spans, centres on the shell of radius
                   0.8..1.15, edge 2^-k with k in {3..7}, res in
                   {8, 16, 32, 64}; one power from {6, 8, 10} and one
                   max_iters from {10, 15, 20} per batch; seeded.
"""
import numpy as np

SPAN_C1 = ((-1.2, -1.2, -1.2), (1.2, 1.2, 1.2))


def bench_points() -> np.ndarray:
    """BENCH_POINTS of src/shape/mod.rs:111-133: 20 points near the P=8 surface."""
    return np.array([
        [-0.73772496, -0.002343091, -0.7382717],
        [-0.7484558, -0.8255949, -0.0026540023],
        [-1.0951594, -0.0014639703, -0.0027306266],
        [-0.60622436, -0.16786861, 0.7227598],
        [-0.6000897, -0.5997089, 0.028461732],
        [-0.6077231, -0.8336551, -0.004541016],
        [-0.05153041, -0.5906257, -0.7647207],
        [-0.73772484, -0.0030531297, -0.7382715],
        [-1.09658, -0.032518614, 0.026089936],
        [-0.74845594, -0.8255949, -0.0033077204],
        [-0.0031473506, 0.59545904, 0.7711717],
        [0.59178185, -0.009300065, 0.70574695],
        [0.5934337, -0.0065053166, -0.8548532],
        [0.5906368, 0.5906708, 0.0002929632],
        [0.5909915, 0.6001409, -0.4285654],
        [-0.004541016, 0.5956404, 0.36293367],
        [-0.00073693885, 0.5916996, -0.8447121],
        [0.59545904, -0.004541016, 0.35817686],
        [0.59545904, -0.004541016, -0.3581769],
        [0.60028464, -0.36826742, 0.6579103],
    ], dtype=np.float32)


def batched_spans(n: int = 4096, seed: int = 0):
    """Returns (spans (n, 6) float32 [start, end], res (n,) uint32, power, max_iters)."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    radius = rng.uniform(0.8, 1.15, size=(n, 1))
    centre = (d * radius).astype(np.float32)
    k = rng.integers(3, 8, size=n)
    edge = np.ldexp(np.float32(1.0), -k).astype(np.float32)[:, None]
    half = (edge / np.float32(2.0)).astype(np.float32)
    spans = np.concatenate([centre - half, centre + half], axis=1).astype(np.float32)
    res = rng.choice(np.array([8, 16, 32, 64], np.uint32), size=n)
    power = int(rng.choice([6, 8, 10]))
    max_iters = int(rng.choice([10, 15, 20]))
    return spans, res.astype(np.uint32), power, max_iters


def uniform_points(n: int, seed: int = 1, lo: float = -1.2, hi: float = 1.2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
