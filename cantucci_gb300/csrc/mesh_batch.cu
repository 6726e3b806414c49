// mesh_batch.cu -- many octree spans meshed together: the GPU form of
// ShapeMesh::update's thread pool, which runs one generate_for_box job per
// empty leaf (src/mesh/mod.rs:129-161).
//
// Every span of a batch keeps its own arrays (same layout as one span,
// mesh_rows.cuh) at offsets given by a span table, so each span's mesh is
// exactly what generate_for_box gives for it alone.
//
//   step 1   one persistent kernel; warps take chunks of work items from an
//            atomic queue.  An item is a 2x4x4 brick of corners (spans with
//            res >= the batch's brick_min_res) or 32 consecutive corners in
//            GridTable order (smaller spans, where bricks would leave lanes
//            idle).
//   step 2/3 grid-stride kernels over the cell rows of all spans; one
//            exclusive scan over all rows gives every span's vertex range
//            (and, for quads, its index range) in span order.  The quads run
//            on a side stream beside the vertex placement.
// No launch depends on a host-side count, so a batch is captured into one
// CUDA graph and replayed.
//
// Launch shapes are per batch (cg_batch_tuning: step-1 block size and queue
// chunk, the resolution from which spans use bricks, the placement block
// size).  cg_batch_autotune picks them by timing the batch itself:
// coordinate descent over a small candidate list, one knob at a time.  No
// knob changes any output bit.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "mesh_rows.cuh"

namespace cg {

CG_OOB_READER(mesh_batch)

struct BatchJob {
    float start[3], across[3];  // widened span (buffer.rs:64-67,77)
    float inv_res;
    PlaceParams pp;             // start, step, FD delta
    MeshDims d;
    uint64_t dist_off;          // floats into dists
    uint64_t sgn_off;           // words into sgn
    uint64_t cw_off;            // words into cellbits / wordoff
    uint32_t row_begin;         // first global cell row
    uint32_t item_begin;        // first global step-1 work item
    uint32_t items;
    uint32_t brick;             // 1: runs of 8 2x4x4 bricks along z, 0: 32 consecutive corners
};

struct BatchTotals {
    uint32_t vertices, quads, status, queue;
};

// Defaults of new batches (cg_set_option "batch_chunk", "batch_block",
// "batch_brick_min_res", "batch_place_block").
static cg_batch_tuning g_batch_default = {256, 4, 8, 128};

static bool valid_block(int64_t v, int64_t hi) {
    return v >= 64 && v <= hi && (v & (v - 1)) == 0;
}

static bool valid_tuning(const cg_batch_tuning& t) {
    return valid_block(t.de_block, 512) && t.de_chunk >= 1 && t.de_chunk <= 4096 &&
           t.brick_min_res >= 2 && t.brick_min_res <= (1u << 20) && valid_block(t.place_block, 256);
}

int set_batch_option(const char* name, int64_t v) {
    cg_batch_tuning t = g_batch_default;
    if (!strcmp(name, "batch_chunk")) t.de_chunk = (uint32_t)v;
    else if (!strcmp(name, "batch_block")) t.de_block = (uint32_t)v;
    else if (!strcmp(name, "batch_brick_min_res")) t.brick_min_res = (uint32_t)v;
    else if (!strcmp(name, "batch_place_block")) t.place_block = (uint32_t)v;
    else return 0;
    if (v < 1 || v > (1 << 20) || !valid_tuning(t)) return 0;
    g_batch_default = t;
    return 1;
}

// Index of the last entry of a non-decreasing table with key <= v.
__device__ __forceinline__ uint32_t find_job(const BatchJob* __restrict__ jobs, uint32_t njobs,
                                             uint32_t v, bool by_item) {
    uint32_t lo = 0, hi = njobs;  // answer in [lo, hi)
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t key = by_item ? jobs[mid].item_begin : jobs[mid].row_begin;
        if (key <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ float job_coord(const BatchJob& j, int k, uint32_t v) {
    return __fadd_rn(j.start[k], __fmul_rn(j.across[k], __fmul_rn((float)v, j.inv_res)));
}

// Step 1 over all spans: persistent warps pull chunks of items from `queue`.
template <int M>
__global__ void k_batch_de(ShapeDev s, const BatchJob* __restrict__ jobs, uint32_t njobs,
                           uint32_t total_items, uint32_t chunk, BatchTotals* __restrict__ tot,
                           float* __restrict__ dists, uint32_t* __restrict__ sgn) {
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&tot->queue, chunk);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= total_items) break;
        const uint32_t end = min(base + chunk, total_items);
        uint32_t j = find_job(jobs, njobs, base, true);
        for (uint32_t item = base; item < end; ++item) {
            while (j + 1 < njobs && jobs[j + 1].item_begin <= item) ++j;
            const BatchJob& J = jobs[j];
            const uint32_t n = J.d.n, W = J.d.W;
            float* out = dists + J.dist_off;
            uint32_t* sg = sgn + J.sgn_off;
            const uint32_t local = item - J.item_begin;
            if (J.brick) {
                // Unit (bx, by, gz): the 8 bricks along z of sign word gz, as
                // k_de_grid_brick walks them; the word is stored whole.
                const uint32_t BY = (n + 3) >> 2, BZ = (n + 3) >> 2;
                const uint32_t gz = local % W, t = local / W, by = t % BY, bx = t / BY;
                const uint32_t dx = lane >> 4, dy = (lane >> 2) & 3, dz = lane & 3;
                const uint32_t x = 2 * bx + dx, y = 4 * by + dy;
                const bool row_ok = x < n && y < n;
                const float px = job_coord(J, 0, x), py = job_coord(J, 1, y);
                const uint32_t bz_end = min(8 * gz + 8, BZ);
                uint32_t word = 0;
                for (uint32_t bz = 8 * gz; bz < bz_end; ++bz) {
                    const uint32_t z = 4 * bz + dz;
                    bool pos = false;
                    if (row_ok && z < n) {
                        const float d = eval<M>(s, px, py, job_coord(J, 2, z));
                        out[((size_t)x * n + y) * n + z] = d;
                        pos = (__float_as_uint(d) >> 31) == 0u;
                    }
                    const uint32_t b = __ballot_sync(0xFFFFFFFFu, pos);
                    word |= ((b >> (lane & ~3u)) & 0xFu) << ((4 * bz) & 31);
                }
                if (dz == 0 && row_ok) sg[(x * n + y) * W + gz] = word;
            } else {
                const uint32_t i = local * 32 + lane;
                if (i < n * n * n) {
                    const uint32_t z = i % n, row = i / n, y = row % n, x = row / n;
                    const float d = eval<M>(s, job_coord(J, 0, x), job_coord(J, 1, y),
                                            job_coord(J, 2, z));
                    out[i] = d;
                    if (!(__float_as_uint(d) >> 31)) atomicOr(&sg[row * W + (z >> 5)], 1u << (z & 31));
                }
            }
        }
    }
}

__global__ void k_batch_cells(const BatchJob* __restrict__ jobs, uint32_t njobs, uint32_t rows,
                              const uint32_t* __restrict__ sgn, uint32_t* __restrict__ cellbits,
                              uint32_t* __restrict__ wordoff, uint32_t* __restrict__ rowcnt) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const BatchJob& J = jobs[find_job(jobs, njobs, r, false)];
        rowcnt[r] = cells_row(sgn + J.sgn_off, J.d, r - J.row_begin, cellbits + J.cw_off,
                              wordoff + J.cw_off);
    }
}

__global__ void k_batch_vertex_list(const BatchJob* __restrict__ jobs, uint32_t njobs,
                                    uint32_t rows, const uint32_t* __restrict__ cellbits,
                                    const uint32_t* __restrict__ wordoff,
                                    const uint32_t* __restrict__ rowoff, uint64_t vcap,
                                    uint32_t* __restrict__ cellidx,
                                    uint32_t* __restrict__ celljob) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const uint32_t j = find_job(jobs, njobs, r, false);
        const BatchJob& J = jobs[j];
        // Vertex ids at or past the capacity are not listed (and not placed);
        // the totals still report the full count.
        vertex_list_row(J.d, r - J.row_begin, cellbits + J.cw_off, wordoff + J.cw_off, rowoff[r],
                        vcap, cellidx, celljob, j);
    }
}

template <int M, bool AN>
__global__ void __launch_bounds__(256) k_batch_place(ShapeDev s, const BatchJob* __restrict__ jobs,
                                                     const float* __restrict__ dists,
                                                     const uint32_t* __restrict__ cellidx,
                                                     const uint32_t* __restrict__ celljob,
                                                     BatchTotals* __restrict__ tot,
                                                     cg_vertex* __restrict__ verts, uint64_t vcap) {
    const uint32_t V = (uint32_t)min((uint64_t)tot->vertices, vcap);
    bool bad = false;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const BatchJob& J = jobs[celljob[v]];
        bad |= !place_vertex<M, AN>(s, J.pp, J.d, dists + J.dist_off, cellidx[v],
                                reinterpret_cast<float*>(verts + v));
    }
    if (bad) atomicOr(&tot->status, MESH_LERP_FAIL);
}

__global__ void k_batch_quad_count(const BatchJob* __restrict__ jobs, uint32_t njobs,
                                   uint32_t rows, const uint32_t* __restrict__ sgn,
                                   uint32_t* __restrict__ quadcnt) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const BatchJob& J = jobs[find_job(jobs, njobs, r, false)];
        quadcnt[r] = quad_count_row(sgn + J.sgn_off, J.d, r - J.row_begin);
    }
}

__global__ void k_batch_quad_emit(const BatchJob* __restrict__ jobs, uint32_t njobs,
                                  uint32_t rows, const uint32_t* __restrict__ sgn,
                                  const float* __restrict__ dists,
                                  const uint32_t* __restrict__ cellbits,
                                  const uint32_t* __restrict__ wordoff,
                                  const uint32_t* __restrict__ rowoff,
                                  const uint32_t* __restrict__ quadoff, uint32_t* __restrict__ idx,
                                  uint64_t icap) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows;
         r += gridDim.x * blockDim.x) {
        const BatchJob& J = jobs[find_job(jobs, njobs, r, false)];
        const uint32_t* ro = rowoff + J.row_begin;
        quad_emit_row(sgn + J.sgn_off, J.d, dists + J.dist_off, cellbits + J.cw_off,
                      wordoff + J.cw_off, ro, ro[0], quadoff[r], idx, icap, r - J.row_begin);
    }
}

// Per-span vertex and index ranges.
__global__ void k_batch_results(const BatchJob* __restrict__ jobs, uint32_t njobs,
                                const uint32_t* __restrict__ rowoff,
                                const uint32_t* __restrict__ quadoff,
                                const BatchTotals* __restrict__ tot,
                                cg_job_mesh* __restrict__ out) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < njobs;
         j += gridDim.x * blockDim.x) {
        const uint32_t r0 = jobs[j].row_begin;
        const bool last = j + 1 == njobs;
        const uint32_t v0 = rowoff[r0], q0 = quadoff[r0];
        const uint32_t v1 = last ? tot->vertices : rowoff[jobs[j + 1].row_begin];
        const uint32_t q1 = last ? tot->quads : quadoff[jobs[j + 1].row_begin];
        cg_job_mesh m;
        m.vertex_offset = v0;
        m.index_offset = 6ull * q0;
        m.vertices = v1 - v0;
        m.indices = 6u * (q1 - q0);
        out[j] = m;
    }
}

}  // namespace cg

using namespace cg;

struct cg_batch {
    int device = 0;
    uint32_t njobs = 0;
    uint32_t total_items = 0;
    uint32_t rows = 0;
    uint64_t vertex_cap = 0;
    char* work = nullptr;
    BatchJob* jobs = nullptr;  // device
    float* dists = nullptr;
    uint32_t *sgn = nullptr, *cellbits = nullptr, *wordoff = nullptr;
    uint32_t *rowcnt = nullptr, *rowoff = nullptr, *quadcnt = nullptr, *quadoff = nullptr;
    uint32_t *cellidx = nullptr, *celljob = nullptr, *scratch = nullptr;
    BatchTotals* tot = nullptr;
    size_t sgn_words = 0;
    std::vector<uint32_t> res;    // per job, host copy
    std::vector<BatchJob> hjobs;  // host copy of the span table
    // workspace capacities (from creation): a new job list must fit them
    uint32_t cap_jobs = 0;
    uint64_t cap_dist = 0, cap_sgnw = 0, cap_cw = 0, cap_rows = 0;
    uint32_t plan_gen = 0;  // bumped by cg_batch_set_jobs (graphs recapture)
    uint32_t normals = CG_NORMALS_FD;       // cg_batch_set_normals
    uint32_t numerics = CG_NUMERICS_EXACT;  // cg_batch_set_numerics
    // quads are built on `side` beside the vertex placement
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cg_batch_tuning tune = {256, 64, 32, 128};
    uint32_t planned_brick_min_res = 0;  // the threshold the device table holds
    // graph cache
    cudaGraphExec_t exec = nullptr;
    unsigned char graph_key[160] = {0};
    std::mutex mu;
};

namespace {

struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

size_t al(size_t v) { return (v + 255) & ~(size_t)255; }

// Step-1 work items of every job for a brick threshold: 2x4x4 bricks for
// res >= brick_min_res, runs of 32 corners in GridTable order below it.
cg_status plan_items(std::vector<BatchJob>& jobs, uint32_t brick_min_res, uint32_t* total) {
    uint64_t items = 0;
    for (BatchJob& J : jobs) {
        const uint64_t n = J.d.n;
        J.brick = J.d.res >= brick_min_res ? 1u : 0u;
        J.items = J.brick ? (uint32_t)(((n + 1) >> 1) * ((n + 3) >> 2) * J.d.W)
                          : (uint32_t)((n * n * n + 31) / 32);
        J.item_begin = (uint32_t)items;
        items += J.items;
        if (items > 0x7FFFFFFFull) {
            set_error("batch too large: %llu step-1 work items", (unsigned long long)items);
            return CG_EINVAL;
        }
    }
    *total = (uint32_t)items;
    return CG_OK;
}

struct PlanTotals {
    uint64_t dist = 0, sgnw = 0, cw = 0, rows = 0;
};

// The span table of a job list (everything but the step-1 items) and its
// workspace totals; validates each job as generate_for_box does.
cg_status build_jobs(const cg_span_job* host_jobs, uint32_t n_jobs, std::vector<BatchJob>& jobs,
                     PlanTotals* t) {
    jobs.assign(n_jobs, BatchJob{});
    PlanTotals acc;
    for (uint32_t i = 0; i < n_jobs; ++i) {
        const cg_span_job& hj = host_jobs[i];
        const uint32_t res = hj.resolution;
        for (int k = 0; k < 3; ++k) {
            if (!(hj.span.start[k] < hj.span.end[k])) {
                set_error("job %u: span.start[%d] < span.end[%d] does not hold", i, k, k);
                return CG_EINVAL;
            }
        }
        if (res < 2 || (res & (res - 1)) || res > 1024) {
            set_error("job %u: resolution %u must be a power of two in [2, 1024]", i, res);
            return CG_EINVAL;
        }
        const SpanSetup su = setup_span(hj.span, res);
        BatchJob& J = jobs[i];
        memset(&J, 0, sizeof J);
        for (int k = 0; k < 3; ++k) {
            J.start[k] = su.start[k];
            J.across[k] = su.across[k];
        }
        J.inv_res = 1.0f / (float)res;
        J.pp = place_params(su);
        J.d = mesh_dims(res);
        const uint64_t n = J.d.n;
        J.dist_off = acc.dist;
        J.sgn_off = acc.sgnw;
        J.cw_off = acc.cw;
        J.row_begin = (uint32_t)acc.rows;
        acc.dist += n * n * n;
        acc.sgnw += n * n * J.d.W;
        acc.cw += (uint64_t)res * res * J.d.Wc;
        acc.rows += (uint64_t)res * res;
        if (acc.rows > (16u << 20) || acc.dist > 0xFFFFFFFFull * 4) {
            set_error("batch too large: %llu cell rows", (unsigned long long)acc.rows);
            return CG_EINVAL;
        }
    }
    *t = acc;
    return CG_OK;
}

// Brings the device span table in line with the batch's brick threshold
// (synchronous; never called while a capture is running).
cg_status sync_plan(cg_batch* b) {
    if (b->planned_brick_min_res == b->tune.brick_min_res) return CG_OK;
    uint32_t total = 0;
    CG_TRY(plan_items(b->hjobs, b->tune.brick_min_res, &total));
    CG_CUDA(cudaMemcpy(b->jobs, b->hjobs.data(), sizeof(BatchJob) * b->njobs,
                       cudaMemcpyHostToDevice));
    b->total_items = total;
    b->planned_brick_min_res = b->tune.brick_min_res;
    return CG_OK;
}

// Resident blocks per SM of a kernel at a block size (cached per device).
template <class K>
unsigned resident_grid(K kernel, unsigned block) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)block, 0) !=
            cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    return (unsigned)(sm_count() * per_sm);
}

template <int M>
cg_status launch_batch_de(cg_batch* b, const ShapeDev& s, cudaStream_t st) {
    const unsigned B = b->tune.de_block;
    const unsigned G = resident_grid(k_batch_de<M>, B);
    k_batch_de<M><<<G, B, 0, st>>>(s, b->jobs, b->njobs, b->total_items, b->tune.de_chunk, b->tot,
                                   b->dists, b->sgn);
    CG_CHECK_LAUNCH("k_batch_de");
    return CG_OK;
}

template <int M, bool AN = false>
cg_status launch_batch_place(cg_batch* b, const ShapeDev& s, cg_vertex* vertices,
                             uint64_t vertex_cap, cudaStream_t st) {
    const unsigned B = b->tune.place_block;
    // Eight waves of blocks rather than one resident wave, so that blocks
    // finish throughout the launch (as k_place: measured 10.19 -> 10.02 ms
    // on the 4096-span batch together with the side stream's priority).
    // No more blocks than the spans' cells (the most vertices they can have)
    // fill: a small batch would otherwise schedule thousands of empty blocks.
    uint64_t cells = 0;
    for (uint32_t r : b->res) cells += (uint64_t)r * r * r;
    const uint64_t need = (cells + B - 1) / B;
    const uint64_t full = (uint64_t)resident_grid(k_batch_place<M, AN>, B) * 8;
    const unsigned G = (unsigned)(need < full ? (need ? need : 1) : full);
    k_batch_place<M, AN><<<G, B, 0, st>>>(s, b->jobs, b->dists, b->cellidx, b->celljob, b->tot,
                                      vertices, vertex_cap);
    CG_CHECK_LAUNCH("k_batch_place");
    return CG_OK;
}

}  // namespace

extern "C" {

cg_status cg_batch_create(int device, const cg_span_job* host_jobs, uint32_t n_jobs,
                          uint64_t vertex_cap, cg_batch** out) {
    if (!out || (!host_jobs && n_jobs) || n_jobs == 0) {
        set_error("bad arguments to cg_batch_create");
        return CG_EINVAL;
    }
    *out = nullptr;
    std::vector<BatchJob> jobs;
    PlanTotals t;
    CG_TRY(build_jobs(host_jobs, n_jobs, jobs, &t));
    const uint64_t dist = t.dist, sgnw = t.sgnw, cw = t.cw, rows = t.rows;
    const cg_batch_tuning tune = g_batch_default;
    uint32_t items = 0;
    CG_TRY(plan_items(jobs, tune.brick_min_res, &items));
    cg_batch* b = new (std::nothrow) cg_batch();
    if (!b) return CG_ENOMEM;
    b->device = device;
    b->njobs = n_jobs;
    b->total_items = items;
    b->rows = (uint32_t)rows;
    b->vertex_cap = vertex_cap;
    b->sgn_words = sgnw;
    b->tune = tune;
    b->planned_brick_min_res = tune.brick_min_res;
    b->res.resize(n_jobs);
    for (uint32_t i = 0; i < n_jobs; ++i) b->res[i] = host_jobs[i].resolution;
    b->cap_jobs = n_jobs;
    b->cap_dist = dist;
    b->cap_sgnw = sgnw;
    b->cap_cw = cw;
    b->cap_rows = rows;
    size_t off = 0;
    std::vector<std::pair<void**, size_t>> parts = {
        {(void**)&b->jobs, sizeof(BatchJob) * n_jobs},
        {(void**)&b->dists, dist * 4},
        {(void**)&b->sgn, sgnw * 4},
        {(void**)&b->cellbits, cw * 4},
        {(void**)&b->wordoff, cw * 4},
        {(void**)&b->rowcnt, rows * 4},
        {(void**)&b->rowoff, rows * 4},
        {(void**)&b->quadcnt, rows * 4},
        {(void**)&b->quadoff, rows * 4},
        {(void**)&b->cellidx, (vertex_cap ? vertex_cap : 1) * 4},
        {(void**)&b->celljob, (vertex_cap ? vertex_cap : 1) * 4},
        {(void**)&b->scratch, scan_scratch_words((uint32_t)rows) * 4},
        {(void**)&b->tot, sizeof(BatchTotals)},
    };
    for (auto& p : parts) off += al(p.second);
    DeviceScope g(device);
    cg_status st = cuda_status(cudaMalloc(&b->work, off), "cudaMalloc", __FILE__, __LINE__);
    if (st != CG_OK) {
        delete b;
        return st;
    }
    off = 0;
    for (auto& p : parts) {
        *p.first = b->work + off;
        off += al(p.second);
    }
    st = cuda_status(cudaMemcpy(b->jobs, jobs.data(), sizeof(BatchJob) * n_jobs,
                                cudaMemcpyHostToDevice),
                     "cudaMemcpy", __FILE__, __LINE__);
    if (st != CG_OK) {
        cudaFree(b->work);
        delete b;
        return st;
    }
    b->hjobs = std::move(jobs);
    // The quads' side stream at the highest priority: its short kernels take
    // SMs ahead of the placement's waiting blocks and end under it.
    int prio_lo = 0, prio_hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess) prio_hi = 0;
    if (cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        cg_batch_destroy(b);
        set_error("cudaStreamCreate / cudaEventCreate failed");
        return CG_ECUDA;
    }
    *out = b;
    return CG_OK;
}

void cg_batch_destroy(cg_batch* b) {
    if (!b) return;
    DeviceScope g(b->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->work) cudaFree(b->work);
    delete b;
}

cg_status cg_batch_set_jobs(cg_batch* b, const cg_span_job* host_jobs, uint32_t n_jobs) {
    if (!b || !host_jobs || n_jobs == 0) {
        set_error("bad arguments to cg_batch_set_jobs");
        return CG_EINVAL;
    }
    std::vector<BatchJob> jobs;
    PlanTotals t;
    CG_TRY(build_jobs(host_jobs, n_jobs, jobs, &t));
    if (n_jobs > b->cap_jobs || t.dist > b->cap_dist || t.sgnw > b->cap_sgnw ||
        t.cw > b->cap_cw || t.rows > b->cap_rows) {
        set_error("job list does not fit the batch's workspace (create a larger batch)");
        return CG_ECAPACITY;
    }
    uint32_t items = 0;
    CG_TRY(plan_items(jobs, b->tune.brick_min_res, &items));
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceScope g(b->device);
    CG_CUDA(cudaMemcpy(b->jobs, jobs.data(), sizeof(BatchJob) * n_jobs, cudaMemcpyHostToDevice));
    b->hjobs = std::move(jobs);
    b->njobs = n_jobs;
    b->total_items = items;
    b->rows = (uint32_t)t.rows;
    b->sgn_words = t.sgnw;
    b->planned_brick_min_res = b->tune.brick_min_res;
    b->res.assign(n_jobs, 0);
    for (uint32_t i = 0; i < n_jobs; ++i) b->res[i] = host_jobs[i].resolution;
    ++b->plan_gen;
    return CG_OK;
}

cg_status cg_batch_set_normals(cg_batch* b, uint32_t normals) {
    if (!b || normals > CG_NORMALS_ADJOINT) {
        set_error("bad batch or normals mode");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(b->mu);
    b->normals = normals;
    return CG_OK;
}

cg_status cg_batch_set_numerics(cg_batch* b, uint32_t numerics) {
    if (!b || numerics > CG_NUMERICS_FAST) {
        set_error("numerics: CG_NUMERICS_EXACT or CG_NUMERICS_FAST");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(b->mu);
    b->numerics = numerics;
    return CG_OK;
}

cg_status cg_batch_get_tuning(const cg_batch* b, cg_batch_tuning* t) {
    if (!b || !t) {
        set_error("bad arguments to cg_batch_get_tuning");
        return CG_EINVAL;
    }
    *t = b->tune;
    return CG_OK;
}

cg_status cg_batch_set_tuning(cg_batch* b, const cg_batch_tuning* t) {
    if (!b || !t || !valid_tuning(*t)) {
        set_error("bad batch tuning: de_block and place_block are powers of two in [64, 512] "
                  "and [64, 256], de_chunk in [1, 4096], brick_min_res in [2, 2^20]");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceScope g(b->device);
    b->tune = *t;
    return sync_plan(b);
}

cg_status cg_batch_mesh(cg_batch* b, const cg_shape* shape, cg_vertex* vertices,
                        uint64_t vertex_cap, uint32_t* indices, uint64_t index_cap,
                        cg_job_mesh* results, uint32_t* totals, void* stream) {
    if (!b || !shape || !results || !totals || (vertex_cap && !vertices) ||
        (index_cap && !indices)) {
        set_error("bad arguments to cg_batch_mesh");
        return CG_EINVAL;
    }
    if (b->planned_brick_min_res != b->tune.brick_min_res) {
        set_error("batch span table out of date (cg_batch_set_tuning did not finish)");
        return CG_EINVAL;
    }
    if (vertex_cap > b->vertex_cap) vertex_cap = b->vertex_cap;
    if (shape->kind == CG_SHAPE_MANDELBULB && (shape->power < 0 || shape->power > 255 ||
                                                shape->max_iters < 1)) {
        set_error("bad Mandelbulb parameters");
        return CG_EINVAL;
    }
    const ShapeDev s = make_shape_dev(*shape);
    cudaStream_t st = (cudaStream_t)stream;
    CG_CUDA(cudaMemsetAsync(b->tot, 0, sizeof(BatchTotals), st));
    CG_CUDA(cudaMemsetAsync(b->sgn, 0, b->sgn_words * 4, st));
    const bool an = b->normals == CG_NORMALS_ADJOINT;
    if (an && b->numerics == CG_NUMERICS_FAST) {
        set_error("fast numerics with the six-sample normals only");
        return CG_EINVAL;
    }
    switch (mode_of(s, b->numerics)) {
    case MODE_P8:
        if (p8_unrolled(s)) CG_TRY(launch_batch_de<MODE_P8_IT15>(b, s, st));
        else CG_TRY(launch_batch_de<MODE_P8>(b, s, st));
        break;
    case MODE_INT: CG_TRY(launch_batch_de<MODE_INT>(b, s, st)); break;
    case MODE_POLAR: CG_TRY(launch_batch_de<MODE_POLAR>(b, s, st)); break;
    case MODE_P8_FAST:
        if (p8_unrolled(s)) CG_TRY(launch_batch_de<MODE_P8_FAST_IT15>(b, s, st));
        else CG_TRY(launch_batch_de<MODE_P8_FAST>(b, s, st));
        break;
    case MODE_INT_POLY: CG_TRY(launch_batch_de<MODE_INT_POLY>(b, s, st)); break;
    case MODE_POLAR_FAST: CG_TRY(launch_batch_de<MODE_POLAR_FAST>(b, s, st)); break;
    default: CG_TRY(launch_batch_de<MODE_SPHERE>(b, s, st)); break;
    }
    const unsigned G = grid_for(b->rows, 256, 8);
    k_batch_cells<<<G, 256, 0, st>>>(b->jobs, b->njobs, b->rows, b->sgn, b->cellbits, b->wordoff,
                                     b->rowcnt);
    CG_CHECK_LAUNCH("k_batch_cells");
    CG_TRY(launch_exclusive_scan(b->rowcnt, b->rowoff, b->rows, b->scratch, &b->tot->vertices, st));
    k_batch_vertex_list<<<G, 256, 0, st>>>(b->jobs, b->njobs, b->rows, b->cellbits, b->wordoff,
                                           b->rowoff, vertex_cap, b->cellidx, b->celljob);
    CG_CHECK_LAUNCH("k_batch_vertex_list");
    // Quads (cell table and signs only) on the side stream, beside the
    // compute-bound placement.
    cudaStream_t qs = st;
    if (b->side) {
        CG_CUDA(cudaEventRecord(b->fork, st));
        CG_CUDA(cudaStreamWaitEvent(b->side, b->fork, 0));
        qs = b->side;
    }
    k_batch_quad_count<<<G, 256, 0, qs>>>(b->jobs, b->njobs, b->rows, b->sgn, b->quadcnt);
    CG_CHECK_LAUNCH("k_batch_quad_count");
    CG_TRY(launch_exclusive_scan(b->quadcnt, b->quadoff, b->rows, b->scratch, &b->tot->quads, qs));
    k_batch_quad_emit<<<G, 256, 0, qs>>>(b->jobs, b->njobs, b->rows, b->sgn, b->dists, b->cellbits,
                                         b->wordoff, b->rowoff, b->quadoff, indices, index_cap);
    CG_CHECK_LAUNCH("k_batch_quad_emit");
    if (b->side) CG_CUDA(cudaEventRecord(b->join, b->side));
#define CG_BATCH_PLACE(MODE)                                                      \
    if (an) CG_TRY((launch_batch_place<MODE, true>(b, s, vertices, vertex_cap, st))); \
    else CG_TRY((launch_batch_place<MODE, false>(b, s, vertices, vertex_cap, st)));
    switch (mode_of(s, b->numerics)) {
    case MODE_P8: CG_BATCH_PLACE(MODE_P8) break;  // rolled, as k_place
    case MODE_INT: CG_BATCH_PLACE(MODE_INT) break;
    case MODE_POLAR: CG_BATCH_PLACE(MODE_POLAR) break;
    case MODE_P8_FAST:
        CG_TRY((launch_batch_place<MODE_P8_FAST, false>(b, s, vertices, vertex_cap, st)));
        break;
    case MODE_INT_POLY:
        CG_TRY((launch_batch_place<MODE_INT_POLY, false>(b, s, vertices, vertex_cap, st)));
        break;
    case MODE_POLAR_FAST:
        CG_TRY((launch_batch_place<MODE_POLAR_FAST, false>(b, s, vertices, vertex_cap, st)));
        break;
    default: CG_BATCH_PLACE(MODE_SPHERE) break;
    }
#undef CG_BATCH_PLACE
    if (b->side) CG_CUDA(cudaStreamWaitEvent(st, b->join, 0));
    k_batch_results<<<grid_for(b->njobs, 256, 4), 256, 0, st>>>(b->jobs, b->njobs, b->rowoff,
                                                                 b->quadoff, b->tot, results);
    CG_CHECK_LAUNCH("k_batch_results");
    CG_CUDA(cudaMemcpyAsync(totals, b->tot, 3 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    return CG_OK;
}

cg_status cg_batch_mesh_graph(cg_batch* b, const cg_shape* shape, cg_vertex* vertices,
                              uint64_t vertex_cap, uint32_t* indices, uint64_t index_cap,
                              cg_job_mesh* results, uint32_t* totals, void* stream) {
    if (!b || !shape) {
        set_error("bad arguments to cg_batch_mesh_graph");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceScope g(b->device);
    // The graph bakes in every argument and the launch shapes: recapture
    // when any of them changes.
    unsigned char key[160];
    memset(key, 0, sizeof key);
    size_t o = 0;
    auto put = [&](const void* p, size_t n) {
        memcpy(key + o, p, n);
        o += n;
    };
    put(shape, sizeof(cg_shape));
    put(&vertices, sizeof vertices);
    put(&vertex_cap, 8);
    put(&indices, sizeof indices);
    put(&index_cap, 8);
    put(&results, sizeof results);
    put(&totals, sizeof totals);
    put(&b->tune, sizeof b->tune);
    put(&b->plan_gen, sizeof b->plan_gen);
    put(&b->normals, sizeof b->normals);
    put(&b->numerics, sizeof b->numerics);
    cudaStream_t st = (cudaStream_t)stream;
    if (!b->exec || memcmp(key, b->graph_key, sizeof key) != 0) {
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        cudaStream_t cap = nullptr;
        CG_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cg_status rs = cuda_status(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal),
                                   "cudaStreamBeginCapture", __FILE__, __LINE__);
        if (rs == CG_OK) {
            rs = cg_batch_mesh(b, shape, vertices, vertex_cap, indices, index_cap, results, totals,
                               cap);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(cap, &graph);
            if (rs == CG_OK) rs = cuda_status(e, "cudaStreamEndCapture", __FILE__, __LINE__);
            if (rs == CG_OK)
                rs = cuda_status(cudaGraphInstantiate(&b->exec, graph, 0), "cudaGraphInstantiate",
                                 __FILE__, __LINE__);
            if (graph) cudaGraphDestroy(graph);
        }
        cudaStreamDestroy(cap);
        if (rs != CG_OK) {
            b->exec = nullptr;
            return rs;
        }
        memcpy(b->graph_key, key, sizeof key);
    }
    CG_CUDA(cudaGraphLaunch(b->exec, st));
    return CG_OK;
}

cg_status cg_batch_autotune(cg_batch* b, const cg_shape* shape, cg_vertex* vertices,
                            uint64_t vertex_cap, uint32_t* indices, uint64_t index_cap,
                            cg_job_mesh* results, uint32_t* totals, void* stream, uint32_t reps,
                            cg_batch_tuning* best, float* best_ms) {
    if (!b || !shape || reps < 1 || reps > 100) {
        set_error("bad arguments to cg_batch_autotune");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(b->mu);
    DeviceScope g(b->device);
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CG_CUDA(cudaEventCreate(&e0));
    cg_status rs = cuda_status(cudaEventCreate(&e1), "cudaEventCreate", __FILE__, __LINE__);
    // Best of `reps` timed runs after one untimed run.
    auto time_it = [&](const cg_batch_tuning& t, float* ms) -> cg_status {
        b->tune = t;
        CG_TRY(sync_plan(b));
        CG_TRY(cg_batch_mesh(b, shape, vertices, vertex_cap, indices, index_cap, results, totals,
                             st));
        float lo = 3.4e38f;
        for (uint32_t r = 0; r < reps; ++r) {
            CG_CUDA(cudaEventRecord(e0, st));
            CG_TRY(cg_batch_mesh(b, shape, vertices, vertex_cap, indices, index_cap, results,
                                 totals, st));
            CG_CUDA(cudaEventRecord(e1, st));
            CG_CUDA(cudaEventSynchronize(e1));
            float v = 0.0f;
            CG_CUDA(cudaEventElapsedTime(&v, e0, e1));
            lo = std::min(lo, v);
        }
        *ms = lo;
        return CG_OK;
    };
    static const uint32_t kBrick[] = {8, 16, 32, 64, 1u << 20};
    static const uint32_t kDeBlock[] = {128, 256, 512};
    static const uint32_t kChunk[] = {4, 16, 64, 256};
    static const uint32_t kPlace[] = {64, 128, 256};
    cg_batch_tuning cur = b->tune;
    float cur_ms = 0.0f;
    if (rs == CG_OK) rs = time_it(cur, &cur_ms);
    // Coordinate descent: each knob over its candidates with the others
    // fixed, until a full pass changes nothing (at most three passes).
    for (int pass = 0; pass < 3 && rs == CG_OK; ++pass) {
        bool moved = false;
        for (int knob = 0; knob < 4 && rs == CG_OK; ++knob) {
            const uint32_t* vals = knob == 0 ? kBrick : knob == 1 ? kDeBlock : knob == 2 ? kChunk
                                                                                      : kPlace;
            const int nv = knob == 0 ? 5 : knob == 2 ? 4 : 3;
            for (int i = 0; i < nv && rs == CG_OK; ++i) {
                cg_batch_tuning t = cur;
                uint32_t* field = knob == 0 ? &t.brick_min_res : knob == 1 ? &t.de_block
                                                 : knob == 2 ? &t.de_chunk : &t.place_block;
                if (*field == vals[i]) continue;
                *field = vals[i];
                float ms = 0.0f;
                rs = time_it(t, &ms);
                if (rs == CG_OK && ms < 0.97f * cur_ms) {  // 3% to beat timing noise
                    cur = t;
                    cur_ms = ms;
                    moved = true;
                }
            }
        }
        if (!moved) break;
    }
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    b->tune = cur;
    const cg_status ps = sync_plan(b);
    if (rs != CG_OK) return rs;
    if (ps != CG_OK) return ps;
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return CG_OK;
}

cg_status cg_batch_dists(cg_batch* b, uint32_t job, const float** dists) {
    if (!b || job >= b->njobs || !dists) {
        set_error("bad arguments to cg_batch_dists");
        return CG_EINVAL;
    }
    uint64_t off = 0;
    for (uint32_t i = 0; i < job; ++i) {
        const uint64_t n = b->res[i] + 1;
        off += n * n * n;
    }
    *dists = b->dists + off;
    return CG_OK;
}

}  // extern "C"
