// mesh.cu -- steps 2 and 3 of naive surface nets
// (MeshBuffer::naive_surface_nets, src/mesh/buffer.rs:85-372) on one span.
// The per-row and per-vertex bodies (and the data layout) are in
// mesh_rows.cuh; the batched multi-span version is mesh_batch.cu.
#include <atomic>
#include <cstring>

#include "common.cuh"
#include "kernels.cuh"
#include "mesh_rows.cuh"

namespace cg {

CG_OOB_READER(mesh)

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
        if (z < n) pos = (__float_as_uint(CG_AT(dists, (size_t)row * n + z, (uint64_t)n * n * n)) >> 31) == 0u;
        const uint32_t bits = __ballot_sync(0xFFFFFFFFu, pos);
        if (lane == 0) CG_AT(sgn, wi, total) = bits;
    }
}

// The row kernels below give a cell row's Wc words (res <= 1024, so Wc is a
// power of two <= 32) to Wc lanes, 32 / Wc rows per warp: each lane streams
// its word, and a scan over the row's lanes gives what a walk along the row
// would (running counts, row totals).  The loop bound is warp-uniform, so
// every lane reaches every shuffle.
struct RowLanes {
    uint32_t L, per_warp, sub, lane_row, warp, nwarps;
    __device__ RowLanes(const MeshDims& d) {
        const uint32_t lane = threadIdx.x & 31;
        L = d.Wc;
        per_warp = 32 / L;
        sub = lane % L;
        lane_row = lane / L;
        warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        nwarps = (gridDim.x * blockDim.x) >> 5;
    }
};

static uint64_t row_lanes(const MeshDims& d) { return (uint64_t)d.res * d.res * d.Wc; }

// Surface cells of every cell row (x, y), with each word's running count
// and the row's total.  Also clears the counters the later kernels
// accumulate into (the totals come from the scans), in place of a memset.
__global__ void __launch_bounds__(256) k_cells(const uint32_t* __restrict__ sgn, MeshDims d,
                                               uint32_t* __restrict__ cellbits,
                                               uint32_t* __restrict__ wordoff,
                                               uint32_t* __restrict__ rowcnt,
                                               MeshCounters* __restrict__ cnt) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        cnt->status = 0;
        cnt->edges = 0;
    }
    const uint32_t rows = d.res * d.res;
    [[maybe_unused]] const uint64_t nc = (uint64_t)rows * d.Wc;
    const RowLanes g(d);
    for (uint32_t r0 = g.warp * g.per_warp; r0 < rows; r0 += g.nwarps * g.per_warp) {
        const uint32_t r = r0 + g.lane_row;
        const bool ok = r < rows;
        const uint32_t surf = ok ? cells_word(sgn, d, r, g.sub) : 0u;
        const uint32_t here = __popc(surf);
        const uint32_t inc = group_inclusive_scan(here, g.sub, g.L);
        if (ok) {
            CG_AT(cellbits, r * d.Wc + g.sub, nc) = surf;
            CG_AT(wordoff, r * d.Wc + g.sub, nc) = inc - here;
            if (g.sub == g.L - 1) CG_AT(rowcnt, r, rows) = inc;
        }
    }
}

// Cell index of every vertex, in vertex-id order.
__global__ void __launch_bounds__(256) k_vertex_list(MeshDims d, const uint32_t* __restrict__ cellbits,
                                                     const uint32_t* __restrict__ wordoff,
                                                     const uint32_t* __restrict__ rowoff,
                                                     uint32_t* __restrict__ cellidx) {
    const uint32_t rows = d.res * d.res;
    [[maybe_unused]] const uint64_t nc = (uint64_t)rows * d.Wc;
#ifdef CG_CHECKED
    const uint64_t cap = (uint64_t)rows * d.res;
#endif
    const RowLanes g(d);
    for (uint32_t r0 = g.warp * g.per_warp; r0 < rows; r0 += g.nwarps * g.per_warp) {
        const uint32_t r = r0 + g.lane_row;
        if (r >= rows) continue;
        uint32_t bits = CG_AT(cellbits, r * d.Wc + g.sub, nc);
        uint32_t v = CG_AT(rowoff, r, rows) + CG_AT(wordoff, r * d.Wc + g.sub, nc);
        while (bits) {
            const uint32_t b = __ffs(bits) - 1;
            bits &= bits - 1;
            CG_AT(cellidx, v, cap) = r * d.res + g.sub * 32 + b;
            ++v;
        }
    }
}

// One vertex per thread (buffer.rs:149-274).  A warp places 32 consecutive
// vertices and stores them through shared memory as 16-byte chunks (32
// vertices = 896 bytes = 56 float4), so the stores are coalesced whether
// `verts` is device memory or pinned host memory written over the C2C link.
template <int M, bool AN, bool ROOT, bool QEF>
__global__ void __launch_bounds__(128) k_place(ShapeDev s, PlaceParams pp, MeshDims d,
                                               const float* __restrict__ dists,
                                               const uint32_t* __restrict__ cellidx,
                                               MeshCounters* __restrict__ cnt,
                                               cg_vertex* __restrict__ verts, uint64_t vcap,
                                               uint32_t root_iters, EdgeTable et,
                                               const PlaceParams* __restrict__ ppp) {
    if (ppp) pp = *ppp;
    __shared__ __align__(16) float stage[4][32 * 7];
    const uint32_t V = cnt->vertices;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool vec_ok = ((uintptr_t)verts & 15u) == 0u;
    float* st = stage[wid];
    bool bad = false;
    // warp-uniform loop over groups of 32 consecutive vertex ids
    for (uint32_t base = blockIdx.x * blockDim.x + wid * 32; base < V;
         base += gridDim.x * blockDim.x) {
        const uint32_t v = base + lane;
        float o[7] = {0, 0, 0, 0, 0, 0, 0};
        if (v < V)
            bad |= !place_vertex<M, AN, ROOT, QEF>(s, pp, d, dists,
                                                   CG_AT(cellidx, v, (uint64_t)d.res * d.res * d.res),
                                                   o, root_iters, &et);
#pragma unroll
        for (int k = 0; k < 7; ++k) st[lane * 7 + k] = o[k];
        __syncwarp();
        const uint64_t room = base < vcap ? vcap - base : 0;
        uint32_t nw = V - base < 32u ? V - base : 32u;
        if ((uint64_t)nw > room) nw = (uint32_t)room;
        if (nw == 32 && vec_ok) {
            // 32 vertices from base (a multiple of 32) = 56 float4 units
            const float4* src4 = reinterpret_cast<const float4*>(st);
#ifdef CG_CHECKED
            float4* v4 = reinterpret_cast<float4*>(verts);
            const uint64_t b4 = (uint64_t)base * 7 / 4, n4 = vcap * 7 / 4;
            CG_AT(v4, b4 + lane, n4) = src4[lane];
            if (lane < 24) CG_AT(v4, b4 + 32 + lane, n4) = src4[32 + lane];
#else
            float4* dst4 = reinterpret_cast<float4*>(verts + base);
            dst4[lane] = src4[lane];
            if (lane < 24) dst4[32 + lane] = src4[32 + lane];
#endif
        } else {
            float* vf = reinterpret_cast<float*>(verts);
            for (uint32_t i = lane; i < nw * 7; i += 32) CG_AT(vf, (uint64_t)base * 7 + i, vcap * 7) = st[i];
        }
        __syncwarp();
    }
    if (bad) atomicOr(&cnt->status, MESH_LERP_FAIL);
}

// Small spans: the seven samples of a vertex on seven lanes of a group of
// eight (four vertices per warp), so a vertex waits for one estimator call
// instead of seven in a row; lane 0 of the group forms the record.  The
// same operations as k_place<M, false, false, false>, so the same bits.
// The loop bound is warp-uniform, so every lane reaches the shuffles.
template <int M>
__global__ void __launch_bounds__(128) k_place_spread(ShapeDev s, PlaceParams pp, MeshDims d,
                                                      const float* __restrict__ dists,
                                                      const uint32_t* __restrict__ cellidx,
                                                      MeshCounters* __restrict__ cnt,
                                                      cg_vertex* __restrict__ verts,
                                                      uint64_t vcap,
                                                      const PlaceParams* __restrict__ ppp) {
    if (ppp) pp = *ppp;
    const uint32_t V = cnt->vertices;
    const uint32_t lane = threadIdx.x & 31, k = lane & 7, g0 = lane & ~7u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    float* vf = reinterpret_cast<float*>(verts);
    bool bad = false;
    for (uint32_t base = warp * 4; base < V; base += nwarps * 4) {
        const uint32_t v = base + (lane >> 3);
        const bool live = v < V;
        float vx = 0.0f, vy = 0.0f, vz = 0.0f, val = 0.0f;
        if (live) {
            CellCrossings cc;
            cell_crossings(pp, d, dists, CG_AT(cellidx, v, (uint64_t)d.res * d.res * d.res), cc);
            const float cf = (float)cc.count;
            vx = __fadd_rn(0.0f, __fdiv_rn(cc.sx, cf));
            vy = __fadd_rn(0.0f, __fdiv_rn(cc.sy, cf));
            vz = __fadd_rn(0.0f, __fdiv_rn(cc.sz, cf));
            if (k == 0) bad |= cc.bad;
            if (k < 7) {
                float qx, qy, qz;
                sample_point(pp, (int)k, vx, vy, vz, qx, qy, qz);
                val = eval<M>(s, qx, qy, qz);
            }
        }
        float de[7];
#pragma unroll
        for (int j = 0; j < 7; ++j) de[j] = __shfl_sync(0xFFFFFFFFu, val, g0 + j);
        if (live && k == 0 && v < vcap) {
            float o[7];
            vertex_record(de, vx, vy, vz, o);
#pragma unroll
            for (int j = 0; j < 7; ++j) CG_AT(vf, (uint64_t)v * 7 + j, vcap * 7) = o[j];
        }
    }
    if (bad) atomicOr(&cnt->status, MESH_LERP_FAIL);
}

// Spans up to this resolution place with k_place_spread and emit quads with
// k_quad_emit_fine: their few thousand vertices leave most of the GPU
// idle, so the seven estimator calls in a row and a row's quads in a row
// are the time.  (At res 128 the pair measured slower: 0.180 against
// 0.169 ms per mesh.)
constexpr uint32_t kSpreadMaxRes = 64;

// One resident wave of k_place_spread blocks, and no more than the span's
// cells can fill (four vertices per warp).
template <int M>
static unsigned spread_grid(const MeshDims& d) {
    static int per_sm = 0;
    if (!per_sm) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_place_spread<M>, 128, 0) !=
                cudaSuccess || b < 1)
            b = 1;
        per_sm = b;
    }
    const uint64_t cap = (uint64_t)sm_count() * per_sm;
    const uint64_t need = ((uint64_t)d.res * d.res * d.res + 15) / 16;  // 16 vertices a block
    return (unsigned)(need < cap ? need : cap);
}

template <int M>
static void launch_place_spread(const ShapeDev& s, const PlaceParams& pp, const MeshDims& d,
                                const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                                cudaStream_t st, const PlaceParams* pp_dev) {
    k_place_spread<M><<<spread_grid<M>(d), 128, 0, st>>>(s, pp, d, w.dists, w.cellidx,
                                                         w.counters, verts, vcap, pp_dev);
}

// Edge table, pass 1: per row r = a n^2 + x n + y (axis a, corner row
// (x, y)), the sign-changing edges before each word and in the row.
__global__ void __launch_bounds__(256) k_edge_rows(const uint32_t* __restrict__ sgn, MeshDims d,
                                                   uint32_t* __restrict__ ewoff,
                                                   uint32_t* __restrict__ ecount) {
    const uint32_t n2 = d.n * d.n, rows = 3 * n2;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const uint32_t a = r / n2, row = r % n2, x = row / d.n, y = row % d.n;
        uint32_t run = 0;
        for (uint32_t w = 0; w < d.W; ++w) {
            CG_AT(ewoff, r * d.W + w, (uint64_t)rows * d.W) = run;
            run += __popc(edge_bits(sgn, d, a, x, y, w));
        }
        CG_AT(ecount, r, rows) = run;
    }
}

// Pass 2: the edges in id order, each as the code r n + z.
__global__ void __launch_bounds__(256) k_edge_list(const uint32_t* __restrict__ sgn, MeshDims d,
                                                   const uint32_t* __restrict__ eoff,
                                                   const uint32_t* __restrict__ ewoff,
                                                   uint32_t* __restrict__ list, uint32_t E) {
    const uint32_t n2 = d.n * d.n, rows = 3 * n2;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const uint32_t a = r / n2, row = r % n2, x = row / d.n, y = row % d.n;
        for (uint32_t w = 0; w < d.W; ++w) {
            uint32_t bits = edge_bits(sgn, d, a, x, y, w);
            uint32_t v = CG_AT(eoff, r, rows) + CG_AT(ewoff, r * d.W + w, (uint64_t)rows * d.W);
            while (bits) {
                const uint32_t b = __ffs(bits) - 1;
                bits &= bits - 1;
                CG_AT(list, v++, E) = r * d.n + w * 32 + b;
            }
        }
    }
}

// Pass 3, one edge per thread: its crossing t (the root with ROOT, else the
// zero of the linear interpolant of its corner distances) and the DE's
// gradient there.
template <int M, bool ROOT>
__global__ void __launch_bounds__(128) k_edge_data(ShapeDev s, PlaceParams pp, MeshDims d,
                                                   const float* __restrict__ dists,
                                                   const uint32_t* __restrict__ list,
                                                   const MeshCounters* __restrict__ cnt,
                                                   float4* __restrict__ data, uint32_t root_iters) {
    const uint32_t E = cnt->edges, n2 = d.n * d.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < E; i += gridDim.x * blockDim.x) {
        const uint32_t code = CG_AT(list, i, E);
        const uint32_t z = code % d.n, r = code / d.n;
        const uint32_t a = r / n2, row = r % n2, x = row / d.n, y = row % d.n;
        const uint32_t x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
        const float f0 = CG_AT(dists, ((size_t)x * d.n + y) * d.n + z, (uint64_t)d.n * d.n * d.n);
        const float f1 = CG_AT(dists, ((size_t)x1 * d.n + y1) * d.n + z1, (uint64_t)d.n * d.n * d.n);
        const float ax = __fadd_rn(pp.start[0], __fmul_rn((float)x, pp.step[0]));
        const float ay = __fadd_rn(pp.start[1], __fmul_rn((float)y, pp.step[1]));
        const float az = __fadd_rn(pp.start[2], __fmul_rn((float)z, pp.step[2]));
        const float ex = a == 0 ? pp.step[0] : 0.0f;
        const float ey = a == 1 ? pp.step[1] : 0.0f;
        const float ez = a == 2 ? pp.step[2] : 0.0f;
        float t;
        if constexpr (ROOT)
            t = root_on_edge<M>(s, ax, ay, az, ex, ey, ez, f0, f1, root_iters);
        else
            t = linear_root(f0, f1);
        // The crossing a + t e, one rounding per coordinate (e is 0 off the
        // edge's axis).
        float g[4];
        shape_gradient<M>(s, __fmaf_rn(t, ex, ax), __fmaf_rn(t, ey, ay), __fmaf_rn(t, ez, az), g);
        CG_AT(data, i, E) = make_float4(t, g[1], g[2], g[3]);
    }
}

// Quads of every corner row, one thread per row: the per-lane version of
// the kernels above measured slower here (22 against 17 us at res 512).
__global__ void __launch_bounds__(256) k_quad_count(const uint32_t* __restrict__ sgn, MeshDims d,
                                                    uint32_t* __restrict__ quadcnt) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x)
        CG_AT(quadcnt, r, rows) = quad_count_row(sgn, d, r);
}

__global__ void __launch_bounds__(256) k_quad_emit(const uint32_t* __restrict__ sgn, MeshDims d,
                                                   const float* __restrict__ dists,
                                                   const uint32_t* __restrict__ cellbits,
                                                   const uint32_t* __restrict__ wordoff,
                                                   const uint32_t* __restrict__ rowoff,
                                                   const uint32_t* __restrict__ quadoff,
                                                   uint32_t* __restrict__ idx, uint64_t icap) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x)
        quad_emit_row(sgn, d, dists, cellbits, wordoff, rowoff, 0u, CG_AT(quadoff, r, rows), idx,
                      icap, r);
}

// Small spans: one warp per (corner row, sign word), one lane per corner.
// A lane's first quad is the row's offset, plus the quads of the row's
// earlier words, plus those of the word's corners below it; the lane then
// emits its corner's (at most three) quads.  The same list as k_quad_emit
// with a corner's quads, not a row's, in a row.
__global__ void __launch_bounds__(256) k_quad_emit_fine(const uint32_t* __restrict__ sgn,
                                                        MeshDims d, const float* __restrict__ dists,
                                                        const uint32_t* __restrict__ cellbits,
                                                        const uint32_t* __restrict__ wordoff,
                                                        const uint32_t* __restrict__ rowoff,
                                                        const uint32_t* __restrict__ quadoff,
                                                        uint32_t* __restrict__ idx, uint64_t icap) {
    const uint32_t rows = d.res * d.res, units = rows * d.Wc;
    const uint32_t lane = threadIdx.x & 31, bit = 1u << lane;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < units; u += nwarps) {
        const uint32_t r = u / d.Wc, w = u % d.Wc, x = r / d.res, y = r % d.res;
        uint64_t q = CG_AT(quadoff, r, rows);
        for (uint32_t w2 = 0; w2 < w; ++w2) {
            const EdgeWords e2 = edge_words(sgn, d, x, y, w2);
            q += __popc(e2.ex) + __popc(e2.ey) + __popc(e2.ez);
        }
        const EdgeWords e = edge_words(sgn, d, x, y, w);
        const uint32_t below = bit - 1u;
        q += __popc(e.ex & below) + __popc(e.ey & below) + __popc(e.ez & below);
        const EdgeWords mine = {e.ex & bit, e.ey & bit, e.ez & bit};
        quad_emit_word(mine, d, dists, cellbits, wordoff, rowoff, 0u, q, idx, icap, x, y, w);
    }
}

// Copy of the first n words of src (n <= src_cap) to dst (n <= dst_cap),
// both 16-byte aligned, as 16-byte units: the quad indices into mapped host
// memory.  With `cnt`, n is read on the device instead: the mesh's
// 6 * quads, cut at dst_cap, so the copy needs no count on the host.  A few
// blocks keep the link busy; beside the placement they cost less than a
// copy-engine transfer, whose traffic competes with the placement's own
// stores into host memory.
static constexpr unsigned kCopyBlocks = 16;

__global__ void __launch_bounds__(256) k_copy_words(const uint32_t* __restrict__ src,
                                                    uint64_t src_cap, uint32_t* __restrict__ dst,
                                                    uint64_t dst_cap, uint64_t n,
                                                    const MeshCounters* __restrict__ cnt) {
    if (cnt) {
        const uint64_t q = 6ull * cnt->quads;
        n = q < dst_cap ? q : dst_cap;
        if (n > src_cap) n = src_cap;
    }
    const uint64_t n4 = n / 4, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (uint64_t i = t; i < n4; i += stride) CG_AT(d4, i, dst_cap / 4) = CG_AT(s4, i, src_cap / 4);
    for (uint64_t i = n4 * 4 + t; i < n; i += stride) CG_AT(dst, i, dst_cap) = CG_AT(src, i, src_cap);
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
        const uint32_t word = CG_AT(cellbits, r * d.Wc + (z >> 5), (uint64_t)d.res * d.res * d.Wc);
        CG_AT(points, c, total) = ((word >> (z & 31)) & 1u)
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

PlaceParams place_params(const SpanSetup& su) {
    PlaceParams pp;
    for (int k = 0; k < 3; ++k) {
        pp.start[k] = su.start[k];
        pp.step[k] = su.step[k];
        pp.delta[k] = su.delta[k];
    }
    return pp;
}

// Blocks of k_place per SM (cg_set_option "place_blocks_per_sm").  Many
// short blocks (128 per SM, about 14 waves) rather than one resident wave:
// blocks then finish throughout the launch, so the quad kernels on the
// higher-priority side stream get SMs early and end under the placement
// (measured on the 513^3 span: 3.39 ms per mesh against 3.45 with 16 per
// SM and equal priorities).
static std::atomic<uint32_t> g_place_blocks_per_sm{128};

uint32_t place_blocks_per_sm() { return g_place_blocks_per_sm.load(); }

// The placement grid: place_blocks_per_sm per SM, but no more blocks than
// the span's res^3 cells (the most vertices it can have) fill.  Blocks past
// the vertex count exit at once, yet each still has to be scheduled: on a
// res-64 span the full grid is 19,456 blocks for some 150 with work.
static unsigned place_grid(const MeshDims& d, unsigned block) {
    const uint64_t cap = (uint64_t)sm_count() * g_place_blocks_per_sm.load();
    const uint64_t need = ((uint64_t)d.res * d.res * d.res + block - 1) / block;
    return (unsigned)(need < cap ? need : cap);
}

int set_place_option(const char* name, int64_t v) {
    if (strcmp(name, "place_blocks_per_sm") || v < 1 || v > 1024) return 0;
    g_place_blocks_per_sm.store((uint32_t)v);
    return 1;
}

template <int M, bool AN>
static void launch_place_mode(const ShapeDev& s, const PlaceParams& pp, const MeshDims& d,
                              const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                              cudaStream_t st, const PlaceOptions& opt, const EdgeTable& et) {
    const unsigned B = 128;
    const unsigned G = place_grid(d, B);
    if (opt.qef)
        k_place<M, AN, false, true><<<G, B, 0, st>>>(s, pp, d, w.dists, w.cellidx, w.counters,
                                                     verts, vcap, 0, et, opt.pp_dev);
    else if (opt.root_iters)
        k_place<M, AN, true, false><<<G, B, 0, st>>>(s, pp, d, w.dists, w.cellidx, w.counters,
                                                     verts, vcap, opt.root_iters, et, opt.pp_dev);
    else if (!AN && d.res <= kSpreadMaxRes)
        launch_place_spread<M>(s, pp, d, w, verts, vcap, st, opt.pp_dev);
    else
        k_place<M, AN, false, false><<<G, B, 0, st>>>(s, pp, d, w.dists, w.cellidx, w.counters,
                                                      verts, vcap, 0, et, opt.pp_dev);
}

// The per-row part of the edge table for `res`: ecount, eoff (3 n^2 each),
// ewoff (3 n^2 W) and the scan's block sums, in edge_rows.
struct EdgeRows {
    uint32_t *ecount, *eoff, *ewoff, *scratch;
};

static size_t edge_rows_layout(const MeshDims& d, char* base, EdgeRows* e) {
    const size_t rows = 3ull * d.n * d.n;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return (uint32_t*)p;
    };
    EdgeRows t;
    t.ecount = take(rows * 4);
    t.eoff = take(rows * 4);
    t.ewoff = take(rows * d.W * 4);
    t.scratch = take(scan_scratch_words((uint32_t)rows) * 4);
    if (e) *e = t;
    return off;
}

cg_status grow_scratch(DeviceScratch* b, size_t bytes) {
    if (b->ptr && b->bytes >= bytes) return CG_OK;
    if (b->ptr) CG_CUDA(cudaFree(b->ptr));
    b->ptr = nullptr;
    b->bytes = 0;
    CG_CUDA(cudaMalloc(&b->ptr, bytes ? bytes : 1));
    b->bytes = bytes;
    return CG_OK;
}

// Edge table, first half: row counts and their scan; the edge total lands
// in w.counters->edges.
static cg_status launch_edge_rows(const MeshDims& d, const MeshWork& w, const PlaceOptions& opt,
                                  cudaStream_t st) {
    if (!opt.edge_rows || !opt.edge_data) {
        set_error("dual contouring needs edge scratch buffers");
        return CG_EINVAL;
    }
    CG_TRY(grow_scratch(opt.edge_rows, edge_rows_layout(d, nullptr, nullptr)));
    EdgeRows e;
    edge_rows_layout(d, (char*)opt.edge_rows->ptr, &e);
    const uint32_t rows = 3 * d.n * d.n;
    const unsigned B = 256, G = grid_for(rows, B, 8);
    k_edge_rows<<<G, B, 0, st>>>(w.sgn, d, e.ewoff, e.ecount);
    CG_CHECK_LAUNCH("k_edge_rows");
    return launch_exclusive_scan(e.ecount, e.eoff, rows, e.scratch, &w.counters->edges, st);
}

// Second half, once the host knows the edge total E: the list and the
// per-edge crossing and gradient.
static cg_status launch_edge_data(const ShapeDev& s, const PlaceParams& pp, const MeshDims& d,
                                  const MeshWork& w, const PlaceOptions& opt, uint32_t E,
                                  cudaStream_t st, EdgeTable* et) {
    CG_TRY(grow_scratch(opt.edge_data, (size_t)E * 20 + 16));
    EdgeRows e;
    edge_rows_layout(d, (char*)opt.edge_rows->ptr, &e);
    float4* data = (float4*)opt.edge_data->ptr;
    uint32_t* list = (uint32_t*)(data + E);
    {
        const uint32_t rows = 3 * d.n * d.n;
        const unsigned B = 256, G = grid_for(rows, B, 8);
        k_edge_list<<<G, B, 0, st>>>(w.sgn, d, e.eoff, e.ewoff, list, E);
        CG_CHECK_LAUNCH("k_edge_list");
    }
    const unsigned B = 128, G = (unsigned)sm_count() * 16;
    switch (mode_of(s, CG_NUMERICS_EXACT)) {
#define CG_EDGE_DATA(MODE)                                                                    \
    if (opt.root_iters)                                                                       \
        k_edge_data<MODE, true><<<G, B, 0, st>>>(s, pp, d, w.dists, list, w.counters, data,   \
                                                 opt.root_iters);                             \
    else                                                                                      \
        k_edge_data<MODE, false><<<G, B, 0, st>>>(s, pp, d, w.dists, list, w.counters, data, 0);
    case MODE_P8: CG_EDGE_DATA(MODE_P8) break;
    case MODE_INT: CG_EDGE_DATA(MODE_INT) break;
    case MODE_POLAR: CG_EDGE_DATA(MODE_POLAR) break;
    default: CG_EDGE_DATA(MODE_SPHERE) break;
#undef CG_EDGE_DATA
    }
    CG_CHECK_LAUNCH("k_edge_data");
    et->sgn = w.sgn;
    et->eoff = e.eoff;
    et->ewoff = e.ewoff;
    et->data = data;
    et->edges = E;
    return CG_OK;
}

// The fast estimators (CG_NUMERICS_FAST) with the reference's placement.
template <int M>
static void launch_place_plain(const ShapeDev& s, const PlaceParams& pp, const MeshDims& d,
                               const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                               cudaStream_t st, const PlaceParams* pp_dev) {
    if (d.res <= kSpreadMaxRes) {
        launch_place_spread<M>(s, pp, d, w, verts, vcap, st, pp_dev);
        return;
    }
    const unsigned B = 128;
    const unsigned G = place_grid(d, B);
    k_place<M, false, false, false><<<G, B, 0, st>>>(s, pp, d, w.dists, w.cellidx, w.counters,
                                                     verts, vcap, 0, EdgeTable{}, pp_dev);
}

static cg_status launch_place(const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                              const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                              cudaStream_t st, const PlaceOptions& opt,
                              const EdgeTable& et = EdgeTable{}) {
    const PlaceParams pp = place_params(su);
    if (opt.numerics == CG_NUMERICS_FAST &&
        (opt.analytic_normals || opt.root_iters || opt.qef)) {
        set_error("fast numerics mesh with the default placement only");
        return CG_EINVAL;
    }
    switch (mode_of(s, opt.numerics)) {
    case MODE_P8_FAST: launch_place_plain<MODE_P8_FAST>(s, pp, d, w, verts, vcap, st, opt.pp_dev); break;
    case MODE_INT_POLY: launch_place_plain<MODE_INT_POLY>(s, pp, d, w, verts, vcap, st, opt.pp_dev); break;
    case MODE_POLAR_FAST: launch_place_plain<MODE_POLAR_FAST>(s, pp, d, w, verts, vcap, st, opt.pp_dev); break;
#define CG_PLACE_MODE(MODE)                                                        \
    if (opt.analytic_normals)                                                      \
        launch_place_mode<MODE, true>(s, pp, d, w, verts, vcap, st, opt, et);      \
    else                                                                           \
        launch_place_mode<MODE, false>(s, pp, d, w, verts, vcap, st, opt, et);
    // (P = 8 takes the rolled loop: with seven estimator calls per vertex the
    // unrolled one measured slower here)
    case MODE_P8: CG_PLACE_MODE(MODE_P8) break;
    case MODE_INT: CG_PLACE_MODE(MODE_INT) break;
    case MODE_POLAR: CG_PLACE_MODE(MODE_POLAR) break;
    default: CG_PLACE_MODE(MODE_SPHERE) break;
#undef CG_PLACE_MODE
    }
    CG_CHECK_LAUNCH("k_place");
    return CG_OK;
}

// Surface cells, their scan and the vertex list (step 2 up to placement).
static cg_status launch_cells(const MeshDims& d, const MeshWork& w, cudaStream_t st,
                              bool signs_ready) {
    const uint32_t rows = d.res * d.res;
    if (!signs_ready) {
        const uint64_t warps = (uint64_t)d.n * d.n * d.W;
        const unsigned B = 256, G = grid_for(warps * 32, B, 8);
        k_sign_words<<<G, B, 0, st>>>(w.dists, d.n, d.W, w.sgn);
        CG_CHECK_LAUNCH("k_sign_words");
    }
    {
        const unsigned B = 256, G = grid_for(row_lanes(d), B, 8);
        k_cells<<<G, B, 0, st>>>(w.sgn, d, w.cellbits, w.wordoff, w.rowcnt, w.counters);
        CG_CHECK_LAUNCH("k_cells");
    }
    CG_TRY(launch_exclusive_scan(w.rowcnt, w.rowoff, rows, w.scratch, &w.counters->vertices, st));
    {
        const unsigned B = 256, G = grid_for(row_lanes(d), B, 8);
        k_vertex_list<<<G, B, 0, st>>>(d, w.cellbits, w.wordoff, w.rowoff, w.cellidx);
        CG_CHECK_LAUNCH("k_vertex_list");
    }
    return CG_OK;
}

static cg_status launch_quad_count(const MeshDims& d, const MeshWork& w, cudaStream_t st) {
    const uint32_t rows = d.res * d.res;
    const unsigned B = 256, G = grid_for(rows, B, 8);
    k_quad_count<<<G, B, 0, st>>>(w.sgn, d, w.quadcnt);
    CG_CHECK_LAUNCH("k_quad_count");
    CG_TRY(launch_exclusive_scan(w.quadcnt, w.quadoff, rows, w.scratch, &w.counters->quads, st));
    return CG_OK;
}

static cg_status launch_quad_emit(const MeshDims& d, const MeshWork& w, uint32_t* idx,
                                  uint64_t icap, cudaStream_t st) {
    if (d.res <= kSpreadMaxRes) {
        const uint64_t lanes = (uint64_t)d.res * d.res * d.Wc * 32;
        const unsigned B = 256, G = grid_for(lanes, B, 8);
        k_quad_emit_fine<<<G, B, 0, st>>>(w.sgn, d, w.dists, w.cellbits, w.wordoff, w.rowoff,
                                          w.quadoff, idx, icap);
        CG_CHECK_LAUNCH("k_quad_emit_fine");
        return CG_OK;
    }
    const uint32_t rows = d.res * d.res;
    const unsigned B = 256, G = grid_for(rows, B, 8);
    k_quad_emit<<<G, B, 0, st>>>(w.sgn, d, w.dists, w.cellbits, w.wordoff, w.rowoff, w.quadoff,
                                 idx, icap);
    CG_CHECK_LAUNCH("k_quad_emit");
    return CG_OK;
}

cg_status launch_mesh_from_dists(const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                                 const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                                 uint32_t* idx, uint64_t icap, cudaStream_t st,
                                 cudaEvent_t ev_after_vertices, bool signs_ready,
                                 const PlaceOptions& opt, const SideStream* side) {
    CG_TRY(launch_cells(d, w, st, signs_ready));
    // Dual contouring: the edge table (its size is read back once).
    auto edge_table = [&](EdgeTable* et) -> cg_status {
        CG_TRY(launch_edge_rows(d, w, opt, st));
        uint32_t E = 0;
        CG_CUDA(cudaMemcpyAsync(&E, &w.counters->edges, sizeof E, cudaMemcpyDeviceToHost, st));
        CG_CUDA(cudaStreamSynchronize(st));
        return launch_edge_data(s, place_params(su), d, w, opt, E, st, et);
    };
    EdgeTable et{};
    if (side) {
        // The quads need only the cell table and the signs: they run on the
        // side stream while the (compute-bound) vertex placement runs here.
        CG_CUDA(cudaEventRecord(side->fork, st));
        CG_CUDA(cudaStreamWaitEvent(side->stream, side->fork, 0));
        CG_TRY(launch_quad_count(d, w, side->stream));
        CG_TRY(launch_quad_emit(d, w, idx, icap, side->stream));
        CG_CUDA(cudaEventRecord(side->join, side->stream));
        if (opt.qef) CG_TRY(edge_table(&et));
        CG_TRY(launch_place(s, su, d, w, verts, vcap, st, opt, et));
        if (ev_after_vertices) CG_CUDA(record_event(ev_after_vertices, st));
        CG_CUDA(cudaStreamWaitEvent(st, side->join, 0));
        return CG_OK;
    }
    if (opt.qef) CG_TRY(edge_table(&et));
    CG_TRY(launch_place(s, su, d, w, verts, vcap, st, opt, et));
    if (ev_after_vertices) CG_CUDA(record_event(ev_after_vertices, st));
    CG_TRY(launch_quad_count(d, w, st));
    CG_TRY(launch_quad_emit(d, w, idx, icap, st));
    return CG_OK;
}

cg_status launch_mesh_to_host(const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                              const MeshWork& w, cg_vertex* host_verts, uint64_t vcap,
                              uint32_t* dev_idx, uint32_t* host_idx, uint64_t icap,
                              cudaStream_t st, cudaStream_t copy_st, cudaEvent_t ev_counts,
                              cudaEvent_t ev_quads, MeshCounters* hcnt,
                              const PlaceOptions& opt) {
    CG_TRY(launch_cells(d, w, st, /*signs_ready=*/true));
    CG_TRY(launch_quad_count(d, w, st));
    const bool aligned = (((uintptr_t)host_idx | (uintptr_t)dev_idx) & 15u) == 0u;
    if (!opt.qef && aligned) {
        // Nothing below needs a count on the host: the quads and their copy
        // (which reads its length on the device) go to copy_st, beside the
        // placement on st, with no synchronisation in between.
        CG_CUDA(cudaEventRecord(ev_counts, st));
        CG_CUDA(cudaStreamWaitEvent(copy_st, ev_counts, 0));
        CG_TRY(launch_quad_emit(d, w, dev_idx, icap, copy_st));
        CG_CUDA(cudaEventRecord(ev_quads, copy_st));
        if (icap) {
            k_copy_words<<<kCopyBlocks, 256, 0, copy_st>>>(dev_idx, icap, host_idx, icap, 0,
                                                           w.counters);
            CG_CHECK_LAUNCH("k_copy_words");
        }
        return launch_place(s, su, d, w, host_verts, vcap, st, opt);
    }
    // Unaligned buffers take a copy-engine transfer and dual contouring
    // sizes its edge table: both need the counts on the host first.
    if (opt.qef) CG_TRY(launch_edge_rows(d, w, opt, st));
    CG_CUDA(cudaMemcpyAsync(hcnt, w.counters, sizeof(MeshCounters), cudaMemcpyDeviceToHost, st));
    CG_CUDA(cudaEventRecord(ev_counts, st));
    CG_CUDA(cudaEventSynchronize(ev_counts));
    const uint64_t ni = 6ull * hcnt->quads;
    const uint64_t ci = ni < icap ? ni : icap;
    // The quads and their copy on copy_st, beside the placement on st.
    CG_CUDA(cudaStreamWaitEvent(copy_st, ev_counts, 0));
    CG_TRY(launch_quad_emit(d, w, dev_idx, icap, copy_st));
    CG_CUDA(cudaEventRecord(ev_quads, copy_st));
    if (ci && aligned) {
        k_copy_words<<<kCopyBlocks, 256, 0, copy_st>>>(dev_idx, icap, host_idx, icap, ci,
                                                       nullptr);
        CG_CHECK_LAUNCH("k_copy_words");
    } else if (ci) {
        CG_CUDA(cudaMemcpyAsync(host_idx, dev_idx, ci * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                copy_st));
    }
    EdgeTable et{};
    if (opt.qef) CG_TRY(launch_edge_data(s, place_params(su), d, w, opt, hcnt->edges, st, &et));
    CG_TRY(launch_place(s, su, d, w, host_verts, vcap, st, opt, et));
    return CG_OK;
}

}  // namespace cg
