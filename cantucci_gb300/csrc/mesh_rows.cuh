// mesh_rows.cuh -- the per-row and per-vertex bodies of naive surface nets
// (MeshBuffer::naive_surface_nets, src/mesh/buffer.rs:85-372), shared by the
// single-span kernels (mesh.cu) and the batched multi-span kernels
// (mesh_batch.cu).  All pointers are already offset to one span's arrays.
//
// Layout per span (res cells per axis, n = res + 1 corners per axis):
//   dists    f32 [n][n][n]     x-major, z fastest (GridTable, src/util/grid.rs:45-48)
//   sgn      u32 [n][n][W]     W = ceil(n/32); bit b of word w = is_sign_positive(dists[x][y][32w+b])
//   cellbits u32 [res][res][Wc] Wc = ceil(res/32); bit = cell (x, y, 32w+b) crosses the surface
//   wordoff  u32 [res][res][Wc] surface cells of the row before word w
//   rowoff   u32 [res*res]     vertices before cell row (x, y) (exclusive scan)
// A vertex id is rowoff[x,y] + wordoff[x,y,w] + popc(cellbits[x,y,w] & below(b)):
// the running count of surface cells in cube() order that the reference
// assigns with vertices.len() - 1 (buffer.rs:274).
#pragma once

#include <cstdint>

#include "adjoint.cuh"
#include "de.cuh"
#include "kernels.cuh"
#include "qef.cuh"

namespace cg {

__device__ __forceinline__ uint32_t valid_mask(uint32_t res, uint32_t w) {
    const uint32_t lo = w * 32;
    return (lo + 32 <= res) ? 0xFFFFFFFFu : ((1u << (res - lo)) - 1u);
}

// Sign word of corner row `row` shifted by one corner: bit b = corner 32w+b+1.
__device__ __forceinline__ uint32_t sign_hi(const uint32_t* __restrict__ sgn, const MeshDims& d,
                                            uint32_t row, uint32_t w) {
    const uint32_t lo = CG_AT(sgn, row * d.W + w, (uint64_t)d.n * d.n * d.W);
    const uint32_t nx = (w + 1 < d.W) ? CG_AT(sgn, row * d.W + w + 1, (uint64_t)d.n * d.n * d.W) : 0u;
    return (lo >> 1) | (nx << 31);
}

// Surface cells of word w of cell row r = (x, y) (buffer.rs:116-147): a
// cell crosses iff the sign bits of its 8 corners are not all equal.
__device__ __forceinline__ uint32_t cells_word(const uint32_t* __restrict__ sgn, const MeshDims& d,
                                               uint32_t r, uint32_t w) {
    const uint32_t x = r / d.res, y = r % d.res;
    const uint32_t r00 = x * d.n + y, r01 = r00 + 1, r10 = r00 + d.n, r11 = r10 + 1;
    [[maybe_unused]] const uint64_t ns = (uint64_t)d.n * d.n * d.W;
    const uint32_t a0 = CG_AT(sgn, r00 * d.W + w, ns), a1 = CG_AT(sgn, r01 * d.W + w, ns);
    const uint32_t a2 = CG_AT(sgn, r10 * d.W + w, ns), a3 = CG_AT(sgn, r11 * d.W + w, ns);
    const uint32_t b0 = sign_hi(sgn, d, r00, w), b1 = sign_hi(sgn, d, r01, w);
    const uint32_t b2 = sign_hi(sgn, d, r10, w), b3 = sign_hi(sgn, d, r11, w);
    const uint32_t all1 = a0 & a1 & a2 & a3 & b0 & b1 & b2 & b3;
    const uint32_t any1 = a0 | a1 | a2 | a3 | b0 | b1 | b2 | b3;
    return any1 & ~all1 & valid_mask(d.res, w);
}

// The surface cells of cell row r, word by word, with each word's running
// count before it; returns the row's count.
__device__ __forceinline__ uint32_t cells_row(const uint32_t* __restrict__ sgn, const MeshDims& d,
                                              uint32_t r, uint32_t* __restrict__ cellbits,
                                              uint32_t* __restrict__ wordoff) {
    uint32_t run = 0;
    for (uint32_t w = 0; w < d.Wc; ++w) {
        const uint32_t surf = cells_word(sgn, d, r, w);
        CG_AT(cellbits, r * d.Wc + w, (uint64_t)d.res * d.res * d.Wc) = surf;
        CG_AT(wordoff, r * d.Wc + w, (uint64_t)d.res * d.res * d.Wc) = run;
        run += __popc(surf);
    }
    return run;
}

// Inclusive scan of v over aligned groups of L lanes (L a power of two <=
// 32; sub = lane % L); every lane of the warp calls it.
__device__ __forceinline__ uint32_t group_inclusive_scan(uint32_t v, uint32_t sub, uint32_t L) {
    for (uint32_t o = 1; o < L; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o, L);
        if (sub >= o) v += t;
    }
    return v;
}

// Cell index (within its span) of every vertex of cell row r, written at the
// row's vertex ids starting from `base` (only ids below `cap`); `tag` (if
// any) receives `tag_value` at the same ids.
__device__ __forceinline__ void vertex_list_row(const MeshDims& d, uint32_t r,
                                                const uint32_t* __restrict__ cellbits,
                                                const uint32_t* __restrict__ wordoff, uint32_t base,
                                                uint64_t cap, uint32_t* __restrict__ cellidx,
                                                uint32_t* __restrict__ tag, uint32_t tag_value) {
    for (uint32_t w = 0; w < d.Wc; ++w) {
        uint32_t bits = CG_AT(cellbits, r * d.Wc + w, (uint64_t)d.res * d.res * d.Wc);
        uint32_t v = base + CG_AT(wordoff, r * d.Wc + w, (uint64_t)d.res * d.res * d.Wc);
        while (bits) {
            const uint32_t b = __ffs(bits) - 1;
            bits &= bits - 1;
            if (v < cap) {
                CG_AT(cellidx, v, cap) = r * d.res + w * 32 + b;
                if (tag) CG_AT(tag, v, cap) = tag_value;
            }
            ++v;
        }
    }
}

struct PlaceParams {
    float start[3], step[3], delta[3];
};

PlaceParams place_params(const SpanSetup& su);

// Corner k of a cell's eight distances without a dynamic register index.
__device__ __forceinline__ float pick8(const float (&dd)[8], uint32_t k) {
    float v = dd[0];
#pragma unroll
    for (uint32_t j = 1; j < 8; ++j) v = k == j ? dd[j] : v;
    return v;
}

// EDGES (buffer.rs:155-176) packed 4 bits per edge: from / to corner of edge k.
constexpr uint64_t kEdgeFrom = 0x642054103210ull;  // 0,1,2,3, 0,1,4,5, 0,2,4,6
constexpr uint64_t kEdgeTo = 0x753176327654ull;    // 4,5,6,7, 2,3,6,7, 1,3,5,7

// Dual contouring's edge table.  Edge (a, x, y, z) joins corner (x, y, z)
// to its +a neighbour; row r = a n^2 + x n + y holds the edges of corner
// row (x, y) along axis a, 32 corners per word.  An edge's id is
// eoff[r] + ewoff[r W + w] + popc(bits below z), so the edges of all cells
// are numbered once, and table entry `id` holds (t, dDE/dp) of the edge's
// crossing a + t (b - a).
struct EdgeTable {
    const uint32_t* sgn;
    const uint32_t* eoff;   // edges before row r (3 n^2)
    const uint32_t* ewoff;  // edges before word w within row r (3 n^2 W)
    const float4* data;     // per edge: t, gradient
    uint32_t edges;         // entries of data
};

// Sign-change bits of the axis-a edges of corner row (x, y), word w.
__device__ __forceinline__ uint32_t edge_bits(const uint32_t* __restrict__ sgn, const MeshDims& d,
                                              uint32_t a, uint32_t x, uint32_t y, uint32_t w) {
    const uint32_t row = x * d.n + y;
    [[maybe_unused]] const uint64_t ns = (uint64_t)d.n * d.n * d.W;
    const uint32_t base = CG_AT(sgn, row * d.W + w, ns);
    if (a == 0) return x + 1 < d.n ? base ^ CG_AT(sgn, (row + d.n) * d.W + w, ns) : 0u;
    if (a == 1) return y + 1 < d.n ? base ^ CG_AT(sgn, (row + 1) * d.W + w, ns) : 0u;
    return (base ^ sign_hi(sgn, d, row, w)) & valid_mask(d.res, w);
}

// The reference's crossing on edge (from, to) of a cell with first corner
// p0 (buffer.rs:187-250): the factor w = (d_from + delta) / delta, delta =
// d_to - d_from, after the distances are oriented so that d_from < 0 (0.5
// for equal distances), then Point3::lerp a (1 - w) + b w (src/math.rs:
// 45-49).  A factor outside [0, 1] (math.rs:19 panics there) sets `bad`
// and uses 0.
__device__ __forceinline__ void lerp_crossing(const PlaceParams& pp, float p0x, float p0y,
                                              float p0z, int from, int to, float df0, float dt0,
                                              bool& bad, float& cx, float& cy, float& cz) {
    float df, dt;
    if (df0 < 0.0f) {
        df = df0;
        dt = dt0;
    } else {
        df = -df0;
        dt = -dt0;
    }
    float wgt;
    if (dt == df) {
        wgt = 0.5f;
    } else {
        const float delta = __fsub_rn(dt, df);
        wgt = __fdiv_rn(__fadd_rn(df, delta), delta);
    }
    if (!(wgt >= 0.0f && wgt <= 1.0f)) {
        bad = true;
        wgt = 0.0f;
    }
    const float ax = __fadd_rn(p0x, ((from >> 2) & 1) ? pp.step[0] : 0.0f);
    const float ay = __fadd_rn(p0y, ((from >> 1) & 1) ? pp.step[1] : 0.0f);
    const float az = __fadd_rn(p0z, (from & 1) ? pp.step[2] : 0.0f);
    const float bx = __fadd_rn(p0x, ((to >> 2) & 1) ? pp.step[0] : 0.0f);
    const float by = __fadd_rn(p0y, ((to >> 1) & 1) ? pp.step[1] : 0.0f);
    const float bz = __fadd_rn(p0z, (to & 1) ? pp.step[2] : 0.0f);
    const float omt = __fsub_rn(1.0f, wgt);
    cx = __fadd_rn(__fmul_rn(ax, omt), __fmul_rn(bx, wgt));
    cy = __fadd_rn(__fmul_rn(ay, omt), __fmul_rn(by, wgt));
    cz = __fadd_rn(__fmul_rn(az, omt), __fmul_rn(bz, wgt));
}

// The DE's root on the edge a + t e, t in [0, 1], by `iters` Illinois
// (modified regula falsi) steps from the corner distances f0 (t = 0) and f1
// (t = 1), whose sign bits differ; NaN counts as inside, as the sign bit
// says.  A step that leaves the bracket (NaN or degenerate) bisects.
template <int M>
__device__ __forceinline__ float root_on_edge(const ShapeDev& s, float ax, float ay, float az,
                                              float ex, float ey, float ez, float f0, float f1,
                                              uint32_t iters) {
    const uint32_t in0 = __float_as_uint(f0) >> 31;
    float t0 = 0.0f, t1 = 1.0f, t = 0.5f;
    int side = 0;
    for (uint32_t it = 0; it < iters; ++it) {
        float tc = (t0 * f1 - t1 * f0) / (f1 - f0);
        if (!(tc > t0 && tc < t1)) tc = 0.5f * (t0 + t1);
        const float fc = eval<M>(s, ax + tc * ex, ay + tc * ey, az + tc * ez);
        if ((__float_as_uint(fc) >> 31) == in0) {
            t0 = tc;
            f0 = fc;
            if (side == -1) f1 *= 0.5f;
            side = -1;
        } else {
            t1 = tc;
            f1 = fc;
            if (side == 1) f0 *= 0.5f;
            side = 1;
        }
        t = tc;
    }
    return t;
}

// The zero of the linear interpolant of an edge's corner distances, t in
// [0, 1] (0.5 where that is undefined).  The reference's lerp sits at 1 - t:
// its weight d_to / (d_to - d_from) multiplies the `to` corner.
__device__ __forceinline__ float linear_root(float f0, float f1) {
    const float t = f0 / (f0 - f1);
    return (t >= 0.0f && t <= 1.0f) ? t : 0.5f;
}

// Vertex of one surface cell (buffer.rs:149-274): centroid of the lerped edge
// crossings, DE at the vertex and the six-sample central-difference normal.
// With AN the normal is instead the normalised analytic gradient from one
// forward-mode pass (shape_gradient: for P = 8 the reference's polynomial
// in dual numbers), which also gives the DE at the vertex (the same bits as
// the estimator's; for other integer powers one more estimator call).  With ROOT each crossing is not the
// reference's distance-weighted lerp but the root of the DE along the edge,
// found by root_iters Illinois (regula falsi) steps from the edge's corner
// distances -- the refinement buffer.rs:178-186 leaves for
// later (issue #1).  With QEF the vertex is not the crossings' centroid but
// the dual-contouring minimiser of their tangent planes (qef.cuh; issue #2),
// from the edge table `et` (crossing and gradient per edge, built by
// k_edge_data: roots or zeros of the linear interpolant of the corner
// distances, not the reference's lerp points, which sit mirrored about the
// edge midpoint); ROOT is then unused.
// Neither changes the cell table or the index list.
// Returns false if a lerp factor left [0, 1] (src/math.rs:19 panics there).
// Cell c's corner distances, its corner p0, and its sign-changing edges'
// lerp crossings summed in EDGES order (buffer.rs:187-250); `bad` when a
// lerp factor left [0, 1].
struct CellCrossings {
    uint32_t x, y, z;
    float dd[8];
    float p0x, p0y, p0z;
    float sx, sy, sz;
    uint32_t count, xmask;
    bool bad;
};

__device__ __forceinline__ void cell_crossings(const PlaceParams& pp, const MeshDims& d,
                                               const float* __restrict__ dists, uint32_t c,
                                               CellCrossings& q) {
    q.z = c % d.res;
    const uint32_t xy = c / d.res;
    q.y = xy % d.res;
    q.x = xy / d.res;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t cx = q.x + ((k >> 2) & 1), cy = q.y + ((k >> 1) & 1), cz = q.z + (k & 1);
        q.dd[k] = CG_AT(dists, ((size_t)cx * d.n + cy) * d.n + cz, (uint64_t)d.n * d.n * d.n);
    }
    q.p0x = __fadd_rn(pp.start[0], __fmul_rn((float)q.x, pp.step[0]));
    q.p0y = __fadd_rn(pp.start[1], __fmul_rn((float)q.y, pp.step[1]));
    q.p0z = __fadd_rn(pp.start[2], __fmul_rn((float)q.z, pp.step[2]));
    // EDGES (buffer.rs:155-176): x edges, y edges, z edges.
    const uint8_t EF[12] = {0, 1, 2, 3, 0, 1, 4, 5, 0, 2, 4, 6};
    const uint8_t ET[12] = {4, 5, 6, 7, 2, 3, 6, 7, 1, 3, 5, 7};
    q.sx = q.sy = q.sz = 0.0f;
    q.count = q.xmask = 0;
    q.bad = false;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
        const int from = EF[k], to = ET[k];
        const float df0 = q.dd[from], dt0 = q.dd[to];
        if ((__float_as_uint(df0) >> 31) == (__float_as_uint(dt0) >> 31)) continue;
        q.xmask |= 1u << k;
        float cx, cy, cz;
        lerp_crossing(pp, q.p0x, q.p0y, q.p0z, from, to, df0, dt0, q.bad, cx, cy, cz);
        q.sx = __fadd_rn(q.sx, cx);
        q.sy = __fadd_rn(q.sy, cy);
        q.sz = __fadd_rn(q.sz, cz);
        ++q.count;
    }
}

// Sample k of a vertex (buffer.rs:254-266): 0 is the vertex itself; 1..6
// are p + unit * (+-delta) along x, y, z, i.e. p + (delta, +0, +0) and
// p + (-delta, -0, -0) etc.
__device__ __forceinline__ void sample_point(const PlaceParams& pp, int k, float vx, float vy,
                                             float vz, float& qx, float& qy, float& qz) {
    qx = vx;
    qy = vy;
    qz = vz;
    if (k > 0) {
        const int axis = (k - 1) >> 1;
        const bool neg = ((k - 1) & 1) != 0;
        const float zero = neg ? -0.0f : 0.0f;
        const float dd0 = axis == 0 ? pp.delta[0] : (axis == 1 ? pp.delta[1] : pp.delta[2]);
        const float off = neg ? -dd0 : dd0;
        qx = __fadd_rn(vx, axis == 0 ? off : zero);
        qy = __fadd_rn(vy, axis == 1 ? off : zero);
        qz = __fadd_rn(vz, axis == 2 ? off : zero);
    }
}

// The vertex record from its position and its seven samples' distances:
// the normal is cgmath's normalize of the central differences,
// v * (1 / |v|) with |v| = sqrt((x*x + y*y) + z*z).
__device__ __forceinline__ void vertex_record(const float (&de)[7], float vx, float vy, float vz,
                                              float* __restrict__ o) {
    const float nx = __fsub_rn(de[1], de[2]);
    const float ny = __fsub_rn(de[3], de[4]);
    const float nz = __fsub_rn(de[5], de[6]);
    const float inv = __fdiv_rn(1.0f, magnitude<Exact>(nx, ny, nz));
    o[0] = vx;
    o[1] = vy;
    o[2] = vz;
    o[3] = __fmul_rn(nx, inv);
    o[4] = __fmul_rn(ny, inv);
    o[5] = __fmul_rn(nz, inv);
    o[6] = de[0];
}

template <int M, bool AN = false, bool ROOT = false, bool QEF = false>
__device__ __forceinline__ bool place_vertex(const ShapeDev& s, const PlaceParams& pp,
                                             const MeshDims& d, const float* __restrict__ dists,
                                             uint32_t c, float* __restrict__ o,
                                             uint32_t root_iters = 0,
                                             const EdgeTable* et = nullptr) {
    CellCrossings cc;
    cell_crossings(pp, d, dists, c, cc);
    const uint32_t x = cc.x, y = cc.y, z = cc.z;
    const float(&dd)[8] = cc.dd;
    const float p0x = cc.p0x, p0y = cc.p0y, p0z = cc.p0z;
    float sx = cc.sx, sy = cc.sy, sz = cc.sz;
    const uint32_t count = cc.count, xmask = cc.xmask;
    const bool bad = cc.bad;
    if constexpr (ROOT && !QEF) {
        sx = sy = sz = 0.0f;
#pragma unroll 1
        for (uint32_t m = xmask; m; m &= m - 1) {
            const uint32_t k = __ffs(m) - 1;
            const uint32_t from = (uint32_t)(kEdgeFrom >> (4 * k)) & 7u;
            const uint32_t to = (uint32_t)(kEdgeTo >> (4 * k)) & 7u;
            const float ax = p0x + (((from >> 2) & 1) ? pp.step[0] : 0.0f);
            const float ay = p0y + (((from >> 1) & 1) ? pp.step[1] : 0.0f);
            const float az = p0z + ((from & 1) ? pp.step[2] : 0.0f);
            const float ex = (((to >> 2) & 1) ? pp.step[0] : 0.0f) - (((from >> 2) & 1) ? pp.step[0] : 0.0f);
            const float ey = (((to >> 1) & 1) ? pp.step[1] : 0.0f) - (((from >> 1) & 1) ? pp.step[1] : 0.0f);
            const float ez = ((to & 1) ? pp.step[2] : 0.0f) - ((from & 1) ? pp.step[2] : 0.0f);
            const float t = root_on_edge<M>(s, ax, ay, az, ex, ey, ez, pick8(dd, from),
                                            pick8(dd, to), root_iters);
            sx += ax + t * ex;
            sy += ay + t * ey;
            sz += az + t * ez;
        }
    }
    Qef q = {};
    if constexpr (QEF) {
        // Each crossing edge's (t, gradient) from the edge table; `from` is
        // the edge's lower corner, so the crossing is at t along +axis from
        // it, in coordinates relative to p0.
#pragma unroll 1
        for (uint32_t m = xmask; m; m &= m - 1) {
            const uint32_t k = __ffs(m) - 1;
            const uint32_t from = (uint32_t)(kEdgeFrom >> (4 * k)) & 7u;
            const uint32_t a = k >> 2;  // EDGES: x edges, then y, then z
            const uint32_t cx = x + ((from >> 2) & 1), cy = y + ((from >> 1) & 1),
                           cz = z + (from & 1);
            const uint32_t w = cz >> 5, b = cz & 31;
            const uint32_t r = a * d.n * d.n + cx * d.n + cy;
            const uint32_t bits = edge_bits(et->sgn, d, a, cx, cy, w);
            [[maybe_unused]] const uint64_t nr = 3ull * d.n * d.n;
            const uint32_t id = CG_AT(et->eoff, r, nr) + CG_AT(et->ewoff, r * d.W + w, nr * d.W) +
                                __popc(bits & ((1u << b) - 1u));
            const float4 e = CG_AT(et->data, id, et->edges);
            float rx = ((from >> 2) & 1) ? pp.step[0] : 0.0f;
            float ry = ((from >> 1) & 1) ? pp.step[1] : 0.0f;
            float rz = (from & 1) ? pp.step[2] : 0.0f;
            if (a == 0) rx += e.x * pp.step[0];
            else if (a == 1) ry += e.x * pp.step[1];
            else rz += e.x * pp.step[2];
            qef_add(q, rx, ry, rz, e.y, e.z, e.w);
        }
    }
    const float cf = (float)count;
    float vx = __fadd_rn(0.0f, __fdiv_rn(sx, cf));
    float vy = __fadd_rn(0.0f, __fdiv_rn(sy, cf));
    float vz = __fadd_rn(0.0f, __fdiv_rn(sz, cf));
    if constexpr (QEF) {
        float rx, ry, rz;
        qef_solve(q, pp.step[0], pp.step[1], pp.step[2], rx, ry, rz);
        vx = p0x + rx;
        vy = p0y + ry;
        vz = p0z + rz;
    }
    // The seven samples (sample_point) one after another; the loop is kept
    // rolled so that one copy of the estimator is in the code.
    if constexpr (AN) {
        float g[4];
        shape_gradient<M>(s, vx, vy, vz, g);
        if constexpr (M == MODE_INT) g[0] = eval<M>(s, vx, vy, vz);  // the estimator's bits
        const float inv = __fdiv_rn(1.0f, magnitude<Exact>(g[1], g[2], g[3]));
        if (o) {
            o[0] = vx;
            o[1] = vy;
            o[2] = vz;
            o[3] = __fmul_rn(g[1], inv);
            o[4] = __fmul_rn(g[2], inv);
            o[5] = __fmul_rn(g[3], inv);
            o[6] = g[0];
        }
        return !bad;
    } else {
        float de[7];
#pragma unroll 1
        for (int k = 0; k < 7; ++k) {
            float qx, qy, qz;
            sample_point(pp, k, vx, vy, vz, qx, qy, qz);
            const float val = eval<M>(s, qx, qy, qz);
#pragma unroll
            for (int j = 0; j < 7; ++j) de[j] = (j == k) ? val : de[j];
        }
        if (o) vertex_record(de, vx, vy, vz, o);
        return !bad;
    }
}

// Edge crossings of the corners of one corner row, 32 corners per word
// (buffer.rs:299-371): bit b of ex/ey/ez = the +x/+y/+z edge of corner
// (x, y, 32w+b) emits a quad.
struct EdgeWords {
    uint32_t ex, ey, ez;
};

__device__ __forceinline__ EdgeWords edge_words(const uint32_t* __restrict__ sgn, const MeshDims& d,
                                                uint32_t x, uint32_t y, uint32_t w) {
    const uint32_t r = x * d.n + y;
    [[maybe_unused]] const uint64_t ns = (uint64_t)d.n * d.n * d.W;
    const uint32_t base = CG_AT(sgn, r * d.W + w, ns);
    const uint32_t valid = valid_mask(d.res, w);
    const uint32_t zpos = valid & (w == 0 ? ~1u : ~0u);
    EdgeWords e;
    e.ex = (y > 0) ? ((base ^ CG_AT(sgn, (r + d.n) * d.W + w, ns)) & zpos) : 0u;
    e.ey = (x > 0) ? ((base ^ CG_AT(sgn, (r + 1) * d.W + w, ns)) & zpos) : 0u;
    e.ez = (x > 0 && y > 0) ? ((base ^ sign_hi(sgn, d, r, w)) & valid) : 0u;
    return e;
}

__device__ __forceinline__ uint32_t quad_count_row(const uint32_t* __restrict__ sgn,
                                                   const MeshDims& d, uint32_t r) {
    const uint32_t x = r / d.res, y = r % d.res;
    uint32_t c = 0;
    for (uint32_t w = 0; w < d.Wc; ++w) {
        const EdgeWords e = edge_words(sgn, d, x, y, w);
        c += __popc(e.ex) + __popc(e.ey) + __popc(e.ez);
    }
    return c;
}

__device__ __forceinline__ uint32_t vertex_id(const MeshDims& d, const uint32_t* __restrict__ cellbits,
                                              const uint32_t* __restrict__ wordoff,
                                              const uint32_t* __restrict__ rowoff, uint32_t x,
                                              uint32_t y, uint32_t z) {
    const uint32_t r = x * d.res + y, w = z >> 5, b = z & 31;
    [[maybe_unused]] const uint64_t nc = (uint64_t)d.res * d.res * d.Wc;
    return CG_AT(rowoff, r, (uint64_t)d.res * d.res) + CG_AT(wordoff, r * d.Wc + w, nc) +
           __popc(CG_AT(cellbits, r * d.Wc + w, nc) & ((1u << b) - 1u));
}

// Quad indices of corner row (x, y), sign word w (buffer.rs:288-372), from
// quad q on: corner order, then +x, +y, +z; winding by dists[(x, y, z)] <
// 0.0.  Vertex ids are rowoff-based minus `vbase`; quad q is written from
// index 6 * q (capacity icap).  Returns the next quad.
__device__ __forceinline__ uint64_t quad_emit_word(const EdgeWords& e, const MeshDims& d,
                                                   const float* __restrict__ dists,
                                                   const uint32_t* __restrict__ cellbits,
                                                   const uint32_t* __restrict__ wordoff,
                                                   const uint32_t* __restrict__ rowoff,
                                                   uint32_t vbase, uint64_t q,
                                                   uint32_t* __restrict__ idx, uint64_t icap,
                                                   uint32_t x, uint32_t y, uint32_t w) {
    uint32_t any = e.ex | e.ey | e.ez;
    while (any) {
        const uint32_t b = __ffs(any) - 1;
        any &= any - 1;
        const uint32_t z = w * 32 + b;
        const bool neg = CG_AT(dists, ((size_t)x * d.n + y) * d.n + z, (uint64_t)d.n * d.n * d.n) < 0.0f;
        const uint32_t bit = 1u << b;
        uint32_t t[6];
        if (e.ex & bit) {
            const uint32_t v0 = vertex_id(d, cellbits, wordoff, rowoff, x, y - 1, z - 1) - vbase;
            const uint32_t v1 = vertex_id(d, cellbits, wordoff, rowoff, x, y - 1, z) - vbase;
            const uint32_t v2 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z - 1) - vbase;
            const uint32_t v3 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z) - vbase;
            if (neg) { t[0] = v0; t[1] = v2; t[2] = v1; t[3] = v1; t[4] = v2; t[5] = v3; }
            else     { t[0] = v0; t[1] = v1; t[2] = v2; t[3] = v1; t[4] = v3; t[5] = v2; }
            if (6 * q + 6 <= icap)
                for (int k = 0; k < 6; ++k) CG_AT(idx, 6 * q + k, icap) = t[k];
            ++q;
        }
        if (e.ey & bit) {
            const uint32_t v0 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y, z - 1) - vbase;
            const uint32_t v1 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y, z) - vbase;
            const uint32_t v2 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z - 1) - vbase;
            const uint32_t v3 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z) - vbase;
            if (neg) { t[0] = v0; t[1] = v1; t[2] = v2; t[3] = v1; t[4] = v3; t[5] = v2; }
            else     { t[0] = v0; t[1] = v2; t[2] = v1; t[3] = v1; t[4] = v2; t[5] = v3; }
            if (6 * q + 6 <= icap)
                for (int k = 0; k < 6; ++k) CG_AT(idx, 6 * q + k, icap) = t[k];
            ++q;
        }
        if (e.ez & bit) {
            const uint32_t v0 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y - 1, z) - vbase;
            const uint32_t v1 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y, z) - vbase;
            const uint32_t v2 = vertex_id(d, cellbits, wordoff, rowoff, x, y - 1, z) - vbase;
            const uint32_t v3 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z) - vbase;
            if (neg) { t[0] = v0; t[1] = v2; t[2] = v1; t[3] = v1; t[4] = v2; t[5] = v3; }
            else     { t[0] = v0; t[1] = v1; t[2] = v2; t[3] = v1; t[4] = v3; t[5] = v2; }
            if (6 * q + 6 <= icap)
                for (int k = 0; k < 6; ++k) CG_AT(idx, 6 * q + k, icap) = t[k];
            ++q;
        }
    }
    return q;
}

// The quads of corner row r, one word after another from quad q.
__device__ __forceinline__ void quad_emit_row(const uint32_t* __restrict__ sgn, const MeshDims& d,
                                              const float* __restrict__ dists,
                                              const uint32_t* __restrict__ cellbits,
                                              const uint32_t* __restrict__ wordoff,
                                              const uint32_t* __restrict__ rowoff, uint32_t vbase,
                                              uint64_t q, uint32_t* __restrict__ idx, uint64_t icap,
                                              uint32_t r) {
    const uint32_t x = r / d.res, y = r % d.res;
    for (uint32_t w = 0; w < d.Wc; ++w)
        q = quad_emit_word(edge_words(sgn, d, x, y, w), d, dists, cellbits, wordoff, rowoff, vbase,
                           q, idx, icap, x, y, w);
}

}  // namespace cg
