// mesh.cu -- steps 2 and 3 of naive surface nets
// (MeshBuffer::naive_surface_nets, src/mesh/buffer.rs:85-372) on the GPU.
//
// Data layout in HBM (res = cells per axis, n = res + 1 corners per axis):
//   dists    f32 [n][n][n]               x-major, z fastest (GridTable, src/util/grid.rs:45-48)
//   sgn      u32 [n][n][W], W = ceil(n/32)  bit b of word w = is_sign_positive(dists[x][y][32w+b])
//   cellbits u32 [res][res][Wc], Wc = ceil(res/32)  bit = cell (x,y,32w+b) crosses the surface
//   wordoff  u32 [res][res][Wc]          surface cells of the row before word w
//   rowoff   u32 [res*res]               vertices before cell row (x,y): exclusive scan
// A vertex id is rowoff[x,y] + wordoff[x,y,w] + popc(cellbits[x,y,w] & below(b)),
// which is the running count of surface cells in cube() order that the
// reference assigns with vertices.len() - 1 (buffer.rs:274).
#include "common.cuh"
#include "kernels.cuh"

namespace cg {

MeshDims mesh_dims(uint32_t res) {
    MeshDims d;
    d.res = res;
    d.n = res + 1;
    d.W = (d.n + 31) / 32;
    d.Wc = (res + 31) / 32;
    return d;
}

static size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

size_t mesh_workspace_layout(uint32_t res, char* base, MeshWork* w) {
    const MeshDims d = mesh_dims(res);
    const size_t n3 = (size_t)d.n * d.n * d.n;
    const size_t rows_c = (size_t)d.n * d.n;
    const size_t rows = (size_t)res * res;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += align_up(bytes);
        return p;
    };
    MeshWork t;
    t.dists = (float*)take(n3 * 4);
    t.sgn = (uint32_t*)take(rows_c * d.W * 4);
    t.cellbits = (uint32_t*)take(rows * d.Wc * 4);
    t.wordoff = (uint32_t*)take(rows * d.Wc * 4);
    t.rowcnt = (uint32_t*)take(rows * 4);
    t.rowoff = (uint32_t*)take(rows * 4);
    t.quadcnt = (uint32_t*)take(rows * 4);
    t.quadoff = (uint32_t*)take(rows * 4);
    t.cellidx = (uint32_t*)take((size_t)res * res * res * 4);
    t.scratch = (uint32_t*)take(scan_scratch_words((uint32_t)rows) * 4);
    t.counters = (MeshCounters*)take(sizeof(MeshCounters));
    if (w) *w = t;
    return off;
}

__device__ __forceinline__ uint32_t valid_mask(uint32_t res, uint32_t w) {
    const uint32_t lo = w * 32;
    return (lo + 32 <= res) ? 0xFFFFFFFFu : ((1u << (res - lo)) - 1u);
}

// Sign word of corner row `row` shifted by one corner: bit b = corner 32w+b+1.
__device__ __forceinline__ uint32_t sign_hi(const uint32_t* __restrict__ sgn, uint32_t row,
                                            uint32_t W, uint32_t w) {
    const uint32_t lo = sgn[row * W + w];
    const uint32_t nx = (w + 1 < W) ? sgn[row * W + w + 1] : 0u;
    return (lo >> 1) | (nx << 31);
}

// f32::is_sign_positive of every corner, packed 32 corners of a z row per
// word with a warp ballot.
__global__ void __launch_bounds__(256) k_sign_words(const float* __restrict__ dists, uint32_t n,
                                                    uint32_t W, uint32_t* __restrict__ sgn) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t total = n * n * W;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t wi = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < total; wi += nwarps) {
        const uint32_t row = wi / W, w = wi % W;
        const uint32_t z = w * 32 + lane;
        bool pos = false;
        if (z < n) pos = (__float_as_uint(dists[(size_t)row * n + z]) >> 31) == 0u;
        const uint32_t bits = __ballot_sync(0xFFFFFFFFu, pos);
        if (lane == 0) sgn[wi] = bits;
    }
}

// Surface cells of every cell row (buffer.rs:116-147): a cell crosses iff the
// sign bits of its 8 corners are not all equal.  One thread per row (x, y).
__global__ void __launch_bounds__(256) k_cells(const uint32_t* __restrict__ sgn, MeshDims d,
                                               uint32_t* __restrict__ cellbits,
                                               uint32_t* __restrict__ wordoff,
                                               uint32_t* __restrict__ rowcnt) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const uint32_t x = r / d.res, y = r % d.res;
        const uint32_t r00 = x * d.n + y, r01 = r00 + 1, r10 = r00 + d.n, r11 = r10 + 1;
        uint32_t run = 0;
        for (uint32_t w = 0; w < d.Wc; ++w) {
            const uint32_t a0 = sgn[r00 * d.W + w], a1 = sgn[r01 * d.W + w];
            const uint32_t a2 = sgn[r10 * d.W + w], a3 = sgn[r11 * d.W + w];
            const uint32_t b0 = sign_hi(sgn, r00, d.W, w), b1 = sign_hi(sgn, r01, d.W, w);
            const uint32_t b2 = sign_hi(sgn, r10, d.W, w), b3 = sign_hi(sgn, r11, d.W, w);
            const uint32_t all1 = a0 & a1 & a2 & a3 & b0 & b1 & b2 & b3;
            const uint32_t any1 = a0 | a1 | a2 | a3 | b0 | b1 | b2 | b3;
            const uint32_t surf = any1 & ~all1 & valid_mask(d.res, w);
            cellbits[r * d.Wc + w] = surf;
            wordoff[r * d.Wc + w] = run;
            run += __popc(surf);
        }
        rowcnt[r] = run;
    }
}

// Cell index of every vertex, in vertex-id order.
__global__ void __launch_bounds__(256) k_vertex_list(MeshDims d, const uint32_t* __restrict__ cellbits,
                                                     const uint32_t* __restrict__ wordoff,
                                                     const uint32_t* __restrict__ rowoff,
                                                     uint32_t* __restrict__ cellidx) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const uint32_t base = rowoff[r];
        for (uint32_t w = 0; w < d.Wc; ++w) {
            uint32_t bits = cellbits[r * d.Wc + w];
            uint32_t v = base + wordoff[r * d.Wc + w];
            while (bits) {
                const uint32_t b = __ffs(bits) - 1;
                bits &= bits - 1;
                cellidx[v++] = r * d.res + w * 32 + b;
            }
        }
    }
}

struct PlaceParams {
    float start[3], step[3], delta[3];
};

// Vertex of one surface cell (buffer.rs:149-274): centroid of the lerped edge
// crossings, DE at the vertex and the six-sample central-difference normal.
__global__ void __launch_bounds__(128) k_place(ShapeDev s, PlaceParams pp, MeshDims d,
                                               const float* __restrict__ dists,
                                               const uint32_t* __restrict__ cellidx,
                                               MeshCounters* __restrict__ cnt,
                                               cg_vertex* __restrict__ verts, uint64_t vcap) {
    const uint32_t V = cnt->vertices;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const uint32_t c = cellidx[v];
        const uint32_t z = c % d.res, xy = c / d.res, y = xy % d.res, x = xy / d.res;
        float dd[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t cx = x + ((k >> 2) & 1), cy = y + ((k >> 1) & 1), cz = z + (k & 1);
            dd[k] = dists[((size_t)cx * d.n + cy) * d.n + cz];
        }
        const float p0x = __fadd_rn(pp.start[0], __fmul_rn((float)x, pp.step[0]));
        const float p0y = __fadd_rn(pp.start[1], __fmul_rn((float)y, pp.step[1]));
        const float p0z = __fadd_rn(pp.start[2], __fmul_rn((float)z, pp.step[2]));
        // EDGES (buffer.rs:155-176): x edges, y edges, z edges.
        const uint8_t EF[12] = {0, 1, 2, 3, 0, 1, 4, 5, 0, 2, 4, 6};
        const uint8_t ET[12] = {4, 5, 6, 7, 2, 3, 6, 7, 1, 3, 5, 7};
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        uint32_t count = 0;
        bool bad = false;
#pragma unroll
        for (int k = 0; k < 12; ++k) {
            const int from = EF[k], to = ET[k];
            const float df0 = dd[from], dt0 = dd[to];
            if ((__float_as_uint(df0) >> 31) == (__float_as_uint(dt0) >> 31)) continue;
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
            // math::lerp asserts 0 <= t <= 1 (src/math.rs:19).
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
            // Point3::lerp: self * (1 - t) + other * t (src/math.rs:45-49).
            const float omt = __fsub_rn(1.0f, wgt);
            sx = __fadd_rn(sx, __fadd_rn(__fmul_rn(ax, omt), __fmul_rn(bx, wgt)));
            sy = __fadd_rn(sy, __fadd_rn(__fmul_rn(ay, omt), __fmul_rn(by, wgt)));
            sz = __fadd_rn(sz, __fadd_rn(__fmul_rn(az, omt), __fmul_rn(bz, wgt)));
            ++count;
        }
        if (bad) atomicOr(&cnt->status, MESH_LERP_FAIL);
        const float cf = (float)count;
        const float vx = __fadd_rn(0.0f, __fdiv_rn(sx, cf));
        const float vy = __fadd_rn(0.0f, __fdiv_rn(sy, cf));
        const float vz = __fadd_rn(0.0f, __fdiv_rn(sz, cf));
        const float dist_p = shape_de(s, vx, vy, vz);
        const float dx = pp.delta[0], dy = pp.delta[1], dz = pp.delta[2];
        // p + unit * delta = p + (delta, +0, +0); p + unit * -delta = p + (-delta, -0, -0)
        const float nx = __fsub_rn(
            shape_de(s, __fadd_rn(vx, dx), __fadd_rn(vy, 0.0f), __fadd_rn(vz, 0.0f)),
            shape_de(s, __fadd_rn(vx, -dx), __fadd_rn(vy, -0.0f), __fadd_rn(vz, -0.0f)));
        const float ny = __fsub_rn(
            shape_de(s, __fadd_rn(vx, 0.0f), __fadd_rn(vy, dy), __fadd_rn(vz, 0.0f)),
            shape_de(s, __fadd_rn(vx, -0.0f), __fadd_rn(vy, -dy), __fadd_rn(vz, -0.0f)));
        const float nz = __fsub_rn(
            shape_de(s, __fadd_rn(vx, 0.0f), __fadd_rn(vy, 0.0f), __fadd_rn(vz, dz)),
            shape_de(s, __fadd_rn(vx, -0.0f), __fadd_rn(vy, -0.0f), __fadd_rn(vz, -dz)));
        // cgmath normalize: v * (1 / |v|), |v| = sqrt((x*x + y*y) + z*z).
        const float inv = __fdiv_rn(1.0f, magnitude<Exact>(nx, ny, nz));
        if (v < vcap) {
            float* o = reinterpret_cast<float*>(verts + v);
            o[0] = vx;
            o[1] = vy;
            o[2] = vz;
            o[3] = __fmul_rn(nx, inv);
            o[4] = __fmul_rn(ny, inv);
            o[5] = __fmul_rn(nz, inv);
            o[6] = dist_p;
        }
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
    const uint32_t base = sgn[r * d.W + w];
    const uint32_t valid = valid_mask(d.res, w);
    const uint32_t zpos = valid & (w == 0 ? ~1u : ~0u);
    EdgeWords e;
    e.ex = (y > 0) ? ((base ^ sgn[(r + d.n) * d.W + w]) & zpos) : 0u;
    e.ey = (x > 0) ? ((base ^ sgn[(r + 1) * d.W + w]) & zpos) : 0u;
    e.ez = (x > 0 && y > 0) ? ((base ^ sign_hi(sgn, r, d.W, w)) & valid) : 0u;
    return e;
}

__global__ void __launch_bounds__(256) k_quad_count(const uint32_t* __restrict__ sgn, MeshDims d,
                                                    uint32_t* __restrict__ quadcnt) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const uint32_t x = r / d.res, y = r % d.res;
        uint32_t c = 0;
        for (uint32_t w = 0; w < d.Wc; ++w) {
            const EdgeWords e = edge_words(sgn, d, x, y, w);
            c += __popc(e.ex) + __popc(e.ey) + __popc(e.ez);
        }
        quadcnt[r] = c;
    }
}

__device__ __forceinline__ uint32_t vertex_id(const MeshDims& d, const uint32_t* __restrict__ cellbits,
                                              const uint32_t* __restrict__ wordoff,
                                              const uint32_t* __restrict__ rowoff, uint32_t x,
                                              uint32_t y, uint32_t z) {
    const uint32_t r = x * d.res + y, w = z >> 5, b = z & 31;
    return rowoff[r] + wordoff[r * d.Wc + w] + __popc(cellbits[r * d.Wc + w] & ((1u << b) - 1u));
}

// Quad indices (buffer.rs:288-372): corner order, then +x, +y, +z; winding
// by dists[(x, y, z)] < 0.0.
__global__ void __launch_bounds__(256) k_quad_emit(const uint32_t* __restrict__ sgn, MeshDims d,
                                                   const float* __restrict__ dists,
                                                   const uint32_t* __restrict__ cellbits,
                                                   const uint32_t* __restrict__ wordoff,
                                                   const uint32_t* __restrict__ rowoff,
                                                   const uint32_t* __restrict__ quadoff,
                                                   uint32_t* __restrict__ idx, uint64_t icap) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const uint32_t x = r / d.res, y = r % d.res;
        uint64_t q = quadoff[r];
        for (uint32_t w = 0; w < d.Wc; ++w) {
            const EdgeWords e = edge_words(sgn, d, x, y, w);
            uint32_t any = e.ex | e.ey | e.ez;
            while (any) {
                const uint32_t b = __ffs(any) - 1;
                any &= any - 1;
                const uint32_t z = w * 32 + b;
                const bool neg = dists[((size_t)x * d.n + y) * d.n + z] < 0.0f;
                const uint32_t bit = 1u << b;
                uint32_t t[6];
                if (e.ex & bit) {
                    const uint32_t v0 = vertex_id(d, cellbits, wordoff, rowoff, x, y - 1, z - 1);
                    const uint32_t v1 = vertex_id(d, cellbits, wordoff, rowoff, x, y - 1, z);
                    const uint32_t v2 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z - 1);
                    const uint32_t v3 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z);
                    if (neg) { t[0] = v0; t[1] = v2; t[2] = v1; t[3] = v1; t[4] = v2; t[5] = v3; }
                    else     { t[0] = v0; t[1] = v1; t[2] = v2; t[3] = v1; t[4] = v3; t[5] = v2; }
                    if (6 * q + 6 <= icap)
                        for (int k = 0; k < 6; ++k) idx[6 * q + k] = t[k];
                    ++q;
                }
                if (e.ey & bit) {
                    const uint32_t v0 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y, z - 1);
                    const uint32_t v1 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y, z);
                    const uint32_t v2 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z - 1);
                    const uint32_t v3 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z);
                    if (neg) { t[0] = v0; t[1] = v1; t[2] = v2; t[3] = v1; t[4] = v3; t[5] = v2; }
                    else     { t[0] = v0; t[1] = v2; t[2] = v1; t[3] = v1; t[4] = v2; t[5] = v3; }
                    if (6 * q + 6 <= icap)
                        for (int k = 0; k < 6; ++k) idx[6 * q + k] = t[k];
                    ++q;
                }
                if (e.ez & bit) {
                    const uint32_t v0 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y - 1, z);
                    const uint32_t v1 = vertex_id(d, cellbits, wordoff, rowoff, x - 1, y, z);
                    const uint32_t v2 = vertex_id(d, cellbits, wordoff, rowoff, x, y - 1, z);
                    const uint32_t v3 = vertex_id(d, cellbits, wordoff, rowoff, x, y, z);
                    if (neg) { t[0] = v0; t[1] = v2; t[2] = v1; t[3] = v1; t[4] = v2; t[5] = v3; }
                    else     { t[0] = v0; t[1] = v1; t[2] = v2; t[3] = v1; t[4] = v3; t[5] = v2; }
                    if (6 * q + 6 <= icap)
                        for (int k = 0; k < 6; ++k) idx[6 * q + k] = t[k];
                    ++q;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_points_table(MeshDims d,
                                                     const uint32_t* __restrict__ cellbits,
                                                     const uint32_t* __restrict__ wordoff,
                                                     const uint32_t* __restrict__ rowoff,
                                                     uint32_t* __restrict__ points) {
    const uint32_t total = d.res * d.res * d.res;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < total;
         c += gridDim.x * blockDim.x) {
        const uint32_t z = c % d.res, r = c / d.res;
        const uint32_t word = cellbits[r * d.Wc + (z >> 5)];
        points[c] = ((word >> (z & 31)) & 1u)
                        ? vertex_id(d, cellbits, wordoff, rowoff, r / d.res, r % d.res, z)
                        : 0xFFFFFFFFu;
    }
}

cg_status launch_points_table(const MeshDims& d, const MeshWork& w, uint32_t* points,
                              cudaStream_t st) {
    const uint64_t total = (uint64_t)d.res * d.res * d.res;
    const unsigned B = 256, G = grid_for(total, B, 8);
    k_points_table<<<G, B, 0, st>>>(d, w.cellbits, w.wordoff, w.rowoff, points);
    CG_CHECK_LAUNCH("k_points_table");
    return CG_OK;
}

cg_status launch_mesh_from_dists(const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                                 const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                                 uint32_t* idx, uint64_t icap, cudaStream_t st,
                                 cudaEvent_t ev_after_vertices, bool signs_ready) {
    const uint32_t rows = d.res * d.res;
    CG_CUDA(cudaMemsetAsync(w.counters, 0, sizeof(MeshCounters), st));
    if (!signs_ready) {
        const uint64_t warps = (uint64_t)d.n * d.n * d.W;
        const unsigned B = 256, G = grid_for(warps * 32, B, 8);
        k_sign_words<<<G, B, 0, st>>>(w.dists, d.n, d.W, w.sgn);
        CG_CHECK_LAUNCH("k_sign_words");
    }
    {
        const unsigned B = 256, G = grid_for(rows, B, 8);
        k_cells<<<G, B, 0, st>>>(w.sgn, d, w.cellbits, w.wordoff, w.rowcnt);
        CG_CHECK_LAUNCH("k_cells");
    }
    CG_TRY(launch_exclusive_scan(w.rowcnt, w.rowoff, rows, w.scratch, &w.counters->vertices, st));
    {
        const unsigned B = 256, G = grid_for(rows, B, 8);
        k_vertex_list<<<G, B, 0, st>>>(d, w.cellbits, w.wordoff, w.rowoff, w.cellidx);
        CG_CHECK_LAUNCH("k_vertex_list");
    }
    {
        PlaceParams pp;
        for (int k = 0; k < 3; ++k) {
            pp.start[k] = su.start[k];
            pp.step[k] = su.step[k];
            pp.delta[k] = su.delta[k];
        }
        const unsigned B = 128;
        const unsigned G = (unsigned)sm_count() * 16;
        k_place<<<G, B, 0, st>>>(s, pp, d, w.dists, w.cellidx, w.counters, verts, vcap);
        CG_CHECK_LAUNCH("k_place");
    }
    if (ev_after_vertices) CG_CUDA(cudaEventRecord(ev_after_vertices, st));
    {
        const unsigned B = 256, G = grid_for(rows, B, 8);
        k_quad_count<<<G, B, 0, st>>>(w.sgn, d, w.quadcnt);
        CG_CHECK_LAUNCH("k_quad_count");
    }
    CG_TRY(launch_exclusive_scan(w.quadcnt, w.quadoff, rows, w.scratch, &w.counters->quads, st));
    {
        const unsigned B = 256, G = grid_for(rows, B, 8);
        k_quad_emit<<<G, B, 0, st>>>(w.sgn, d, w.dists, w.cellbits, w.wordoff, w.rowoff,
                                     w.quadoff, idx, icap);
        CG_CHECK_LAUNCH("k_quad_emit");
    }
    return CG_OK;
}

}  // namespace cg
