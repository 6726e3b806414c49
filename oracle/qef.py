"""FP64 model of the dual-contouring vertex placement (CG_PLACEMENT_QEF).

Test infrastructure only: the tests compare the GPU mesher's QEF vertices
with this model.  Nothing in the product imports it.

The reference has no dual contouring; src/mesh/buffer.rs:53-54 names it as
the successor of its naive surface nets (issue #2).  The model follows the
published method (Ju, Losasso, Schaefer and Warren, "Dual Contouring of
Hermite Data", SIGGRAPH 2002) with the choices the GPU path makes:

  * crossings: the zero of the linear interpolant of the corner distances
    on each sign-changing edge (not the reference's lerp point, which sits
    mirrored about the edge midpoint: see crossings());
  * normals: the FP64 forward-mode gradient of the shape's estimator at each
    crossing (oracle de_grad_f64), normalised; zero or non-finite gradients
    add no plane;
  * the vertex x minimises sum_i (n_i . (x - p_i))^2 as c + pinv(A) (b - A c)
    in coordinates relative to the cell's first corner, c the crossings'
    mass point, the pseudo-inverse dropping eigenvalues of A = sum n n^T at
    or below TRUNCATE times the largest; then each coordinate is clamped to
    the cell.
"""
import numpy as np

from . import de_grad_f64, generate_for_box

f32 = np.float32
TRUNCATE = 0.01

# EDGES (buffer.rs:155-176): x edges, y edges, z edges, corner k = 4x + 2y + z.
EDGE_FROM = np.array([0, 1, 2, 3, 0, 1, 4, 5, 0, 2, 4, 6])
EDGE_TO = np.array([4, 5, 6, 7, 2, 3, 6, 7, 1, 3, 5, 7])
CORNER = np.array([[(k >> 2) & 1, (k >> 1) & 1, k & 1] for k in range(8)])


def span_setup(span, res):
    """Span widening and step of buffer.rs:64-67,101 in f32: start - overflow,
    end + overflow with overflow = (end - start) / res, step = (end - start) / res."""
    sp = np.asarray(span, f32).reshape(2, 3)
    rf = f32(res)
    ov = (sp[1] - sp[0]) / rf
    start = sp[0] + (-ov)
    end = sp[1] + ov
    step = (end - start) / rf
    return start.astype(f32), step.astype(f32)


def crossings(dists, cells, start, step):
    """Crossing points (V, 12, 3) f32 and their mask (V, 12) of the cells
    (V, 3) integer (x, y, z): on each sign-changing edge a + t (b - a) with
    t = d_a / (d_a - d_b), the zero of the linear interpolant of the corner
    distances (0.5 where that is not in [0, 1]).  The reference's lerp
    (buffer.rs:203-240) puts the point at 1 - t instead -- its weight
    d_to / (d_to - d_from) multiplies the `to` corner -- which suits a
    centroid but not a tangent plane."""
    cells = np.asarray(cells, np.int64)
    corner = cells[:, None, :] + CORNER[None, :, :]                    # (V, 8, 3)
    dd = dists[corner[..., 0], corner[..., 1], corner[..., 2]].astype(f32)  # (V, 8)
    p0 = (start[None, :] + cells.astype(f32) * step[None, :]).astype(f32)  # (V, 3)
    f0, f1 = dd[:, EDGE_FROM], dd[:, EDGE_TO]
    mask = np.signbit(f0) != np.signbit(f1)
    with np.errstate(invalid="ignore", divide="ignore"):
        t = (f0 / (f0 - f1)).astype(f32)
    t = np.where((t >= 0) & (t <= 1), t, f32(0.5)).astype(f32)
    # The edge's lower corner from its own grid coordinate, start + c * step
    # in f32, and the crossing a + t e with one rounding per coordinate (an
    # FMA: t e is exact in FP64).
    corner_lo = (cells[:, None, :] + CORNER[EDGE_FROM][None]).astype(f32)
    a = (start + (corner_lo * step).astype(f32)).astype(f32)
    e = (np.where(CORNER[EDGE_TO][None] == 1, step, f32(0))
         - np.where(CORNER[EDGE_FROM][None] == 1, step, f32(0))).astype(f32)
    pts = (a.astype(np.float64) + t[..., None].astype(np.float64) * e.astype(np.float64)).astype(f32)
    return pts, mask, p0


def qef_vertices(shape, dists, cells, start, step, nthreads=None):
    """Dual-contouring vertex (V, 3) float64 of every cell."""
    pts, mask, p0 = crossings(dists, cells, start, step)
    V = len(cells)
    flat = pts[mask]                                                   # (K, 3)
    g = de_grad_f64(shape, flat, nthreads=nthreads)[:, 1:4] if len(flat) else np.zeros((0, 3))
    grad = np.zeros((V, 12, 3))
    grad[mask] = g
    rel = np.where(mask[..., None], pts.astype(np.float64) - p0[:, None, :].astype(np.float64), 0.0)
    n_pts = mask.sum(1)
    c = rel.sum(1) / n_pts[:, None]
    l2 = (grad ** 2).sum(-1)
    ok = mask & np.isfinite(l2) & (l2 > 0)
    with np.errstate(invalid="ignore", divide="ignore"):
        n = np.where(ok[..., None], grad / np.sqrt(np.where(ok, l2, 1.0))[..., None], 0.0)
    A = np.einsum("vki,vkj->vij", n, n)
    bvec = np.einsum("vki,vk->vi", n, (n * rel).sum(-1))
    rhs = bvec - np.einsum("vij,vj->vi", A, c)
    lam, vec = np.linalg.eigh(A)
    lmax = lam.max(1, keepdims=True)
    keep = lam > TRUNCATE * lmax
    with np.errstate(invalid="ignore", divide="ignore"):
        coef = np.where(keep, np.einsum("vij,vi->vj", vec, rhs) / np.where(keep, lam, 1.0), 0.0)
    dx = np.einsum("vij,vj->vi", vec, coef)
    fin = np.isfinite(dx).all(1) & ok.any(1)
    x = c + np.where(fin[:, None], dx, 0.0)
    x = np.clip(x, 0.0, step.astype(np.float64)[None, :])
    return p0.astype(np.float64) + x


def mesh_cells(shape, span, res, nthreads=None):
    """The oracle's mesh with its grids, the surface cells (V, 3) in vertex
    order, and the span's f32 start and step."""
    m = generate_for_box(shape, span, res, nthreads=nthreads, want_grids=True)
    pts = m["points"]
    idx = np.nonzero(pts.reshape(-1) != 0xFFFFFFFF)[0]
    order = np.argsort(pts.reshape(-1)[idx], kind="stable")
    flat = idx[order]
    cells = np.stack([flat // (res * res), (flat // res) % res, flat % res], 1)
    start, step = span_setup(span, res)
    return m, cells, start, step
