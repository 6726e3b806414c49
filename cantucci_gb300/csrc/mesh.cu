// mesh.cu -- steps 2 and 3 of naive surface nets
// (MeshBuffer::naive_surface_nets, src/mesh/buffer.rs:85-372) on one span.
// The per-row and per-vertex bodies (and the data layout) are in
// mesh_rows.cuh; the batched multi-span version is mesh_batch.cu.
#include "common.cuh"
#include "kernels.cuh"
#include "mesh_rows.cuh"

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

// Surface cells of every cell row; one thread per row (x, y).
__global__ void __launch_bounds__(256) k_cells(const uint32_t* __restrict__ sgn, MeshDims d,
                                               uint32_t* __restrict__ cellbits,
                                               uint32_t* __restrict__ wordoff,
                                               uint32_t* __restrict__ rowcnt) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x)
        rowcnt[r] = cells_row(sgn, d, r, cellbits, wordoff);
}

// Cell index of every vertex, in vertex-id order.
__global__ void __launch_bounds__(256) k_vertex_list(MeshDims d, const uint32_t* __restrict__ cellbits,
                                                     const uint32_t* __restrict__ wordoff,
                                                     const uint32_t* __restrict__ rowoff,
                                                     uint32_t* __restrict__ cellidx) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x)
        vertex_list_row(d, r, cellbits, wordoff, rowoff[r], ~0ull, cellidx, nullptr, 0);
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
                                               uint32_t root_iters) {
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
        if (v < V) bad |= !place_vertex<M, AN, ROOT, QEF>(s, pp, d, dists, cellidx[v], o, root_iters);
#pragma unroll
        for (int k = 0; k < 7; ++k) st[lane * 7 + k] = o[k];
        __syncwarp();
        const uint64_t room = base < vcap ? vcap - base : 0;
        uint32_t nw = V - base < 32u ? V - base : 32u;
        if ((uint64_t)nw > room) nw = (uint32_t)room;
        float* dst = reinterpret_cast<float*>(verts + base);
        if (nw == 32 && vec_ok) {
            const float4* src4 = reinterpret_cast<const float4*>(st);
            float4* dst4 = reinterpret_cast<float4*>(dst);
            dst4[lane] = src4[lane];
            if (lane < 24) dst4[32 + lane] = src4[32 + lane];
        } else {
            for (uint32_t i = lane; i < nw * 7; i += 32) dst[i] = st[i];
        }
        __syncwarp();
    }
    if (bad) atomicOr(&cnt->status, MESH_LERP_FAIL);
}

__global__ void __launch_bounds__(256) k_quad_count(const uint32_t* __restrict__ sgn, MeshDims d,
                                                    uint32_t* __restrict__ quadcnt) {
    const uint32_t rows = d.res * d.res;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x)
        quadcnt[r] = quad_count_row(sgn, d, r);
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
        quad_emit_row(sgn, d, dists, cellbits, wordoff, rowoff, 0u, quadoff[r], idx, icap, r);
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

PlaceParams place_params(const SpanSetup& su) {
    PlaceParams pp;
    for (int k = 0; k < 3; ++k) {
        pp.start[k] = su.start[k];
        pp.step[k] = su.step[k];
        pp.delta[k] = su.delta[k];
    }
    return pp;
}

template <int M, bool AN, bool QEF>
static void launch_place_qef(const ShapeDev& s, const PlaceParams& pp, const MeshDims& d,
                             const MeshWork& w, cg_vertex* verts, uint64_t vcap, cudaStream_t st,
                             uint32_t root_iters) {
    const unsigned B = 128;
    const unsigned G = (unsigned)sm_count() * 16;
    if (root_iters)
        k_place<M, AN, true, QEF><<<G, B, 0, st>>>(s, pp, d, w.dists, w.cellidx, w.counters,
                                                   verts, vcap, root_iters);
    else
        k_place<M, AN, false, QEF><<<G, B, 0, st>>>(s, pp, d, w.dists, w.cellidx, w.counters,
                                                    verts, vcap, 0);
}

template <int M, bool AN>
static void launch_place_mode(const ShapeDev& s, const PlaceParams& pp, const MeshDims& d,
                              const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                              cudaStream_t st, const PlaceOptions& opt) {
    if (opt.qef)
        launch_place_qef<M, AN, true>(s, pp, d, w, verts, vcap, st, opt.root_iters);
    else
        launch_place_qef<M, AN, false>(s, pp, d, w, verts, vcap, st, opt.root_iters);
}

static cg_status launch_place(const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                              const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                              cudaStream_t st, const PlaceOptions& opt) {
    const PlaceParams pp = place_params(su);
    switch (mode_of(s, CG_NUMERICS_EXACT)) {
    case MODE_P8:
        launch_place_mode<MODE_P8, false>(s, pp, d, w, verts, vcap, st, opt);
        break;
    case MODE_INT:
        launch_place_mode<MODE_INT, false>(s, pp, d, w, verts, vcap, st, opt);
        break;
    case MODE_POLAR:
        if (opt.analytic_normals)
            launch_place_mode<MODE_POLAR, true>(s, pp, d, w, verts, vcap, st, opt);
        else
            launch_place_mode<MODE_POLAR, false>(s, pp, d, w, verts, vcap, st, opt);
        break;
    default:
        launch_place_mode<MODE_SPHERE, false>(s, pp, d, w, verts, vcap, st, opt);
        break;
    }
    CG_CHECK_LAUNCH("k_place");
    return CG_OK;
}

// Surface cells, their scan and the vertex list (step 2 up to placement).
static cg_status launch_cells(const MeshDims& d, const MeshWork& w, cudaStream_t st,
                              bool signs_ready) {
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
    if (side) {
        // The quads need only the cell table and the signs: they run on the
        // side stream while the (compute-bound) vertex placement runs here.
        CG_CUDA(cudaEventRecord(side->fork, st));
        CG_CUDA(cudaStreamWaitEvent(side->stream, side->fork, 0));
        CG_TRY(launch_quad_count(d, w, side->stream));
        CG_TRY(launch_quad_emit(d, w, idx, icap, side->stream));
        CG_CUDA(cudaEventRecord(side->join, side->stream));
        CG_TRY(launch_place(s, su, d, w, verts, vcap, st, opt));
        if (ev_after_vertices) CG_CUDA(cudaEventRecord(ev_after_vertices, st));
        CG_CUDA(cudaStreamWaitEvent(st, side->join, 0));
        return CG_OK;
    }
    CG_TRY(launch_place(s, su, d, w, verts, vcap, st, opt));
    if (ev_after_vertices) CG_CUDA(cudaEventRecord(ev_after_vertices, st));
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
    CG_CUDA(cudaMemcpyAsync(hcnt, w.counters, sizeof(MeshCounters), cudaMemcpyDeviceToHost, st));
    CG_CUDA(cudaEventRecord(ev_counts, st));
    CG_CUDA(cudaEventSynchronize(ev_counts));
    const uint64_t ni = 6ull * hcnt->quads;
    const uint64_t ci = ni < icap ? ni : icap;
    // The quads and their copy on copy_st, beside the placement on st.
    CG_CUDA(cudaStreamWaitEvent(copy_st, ev_counts, 0));
    CG_TRY(launch_quad_emit(d, w, dev_idx, icap, copy_st));
    CG_CUDA(cudaEventRecord(ev_quads, copy_st));
    if (ci)
        CG_CUDA(cudaMemcpyAsync(host_idx, dev_idx, ci * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                copy_st));
    CG_TRY(launch_place(s, su, d, w, host_verts, vcap, st, opt));
    return CG_OK;
}

}  // namespace cg
