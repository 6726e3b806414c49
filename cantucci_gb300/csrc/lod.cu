// lod.cu -- ShapeMesh: the level-of-detail driver around the mesher
// (src/mesh/mod.rs:24-243), GPU-first.
//
// The reference keeps an octree of leaves, each empty, "requested" (a
// generate_for_box job on its thread pool) or "ready" (a mesh).  Every frame
// it marches 5 x 5 focus rays from the camera, splits each ready leaf around
// a focus point closer than twice the leaf's width, collects the meshes the
// pool has finished, and starts a job for every empty leaf.
//
// Here the octree and the update rules stay on the host (they are tiny and
// branchy) and the two data-parallel parts go to the GPU: the focus rays are
// one k_march launch, and all of an update's jobs are one batched mesher run
// (mesh_batch.cu) on the driver's stream, left in flight until a later
// update finds its event complete.  Like the reference's thread pool, which
// takes new jobs while older ones run, an update starts a run for the
// leaves that became empty even while earlier runs are in flight (up to
// kMaxRuns queued on the stream; they finish and are collected in launch
// order).  A run writes one vertex and one index buffer (a "generation");
// ready leaves point into it, and a generation is freed when no leaf points
// into it any more.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace cg {
namespace {

constexpr uint32_t kFocusPoints = 5;        // FOCUS_POINTS (mod.rs:88)
constexpr uint32_t kFocusSteps = 100;       // MAX_ITERS of get_focii (mod.rs:207)
constexpr float kFocusEpsilon = 0.000001f;  // EPSILON of get_focii (mod.rs:206)
constexpr uint32_t kMaxRuns = 4;            // batched runs queued at once

struct V3 {
    float x, y, z;
};
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 scale(V3 a, float k) { return {a.x * k, a.y * k, a.z * k}; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// cgmath normalize: v * (1 / |v|).
V3 normalize(V3 a) { return scale(a, 1.0f / std::sqrt(dot(a, a))); }

// Octree::leaf_around_mut's containment test (src/octree/mod.rs:25-31).
bool span_contains(const cg_span& s, V3 p) {
    return s.start[0] <= p.x && s.start[1] <= p.y && s.start[2] <= p.z && p.x < s.end[0] &&
           p.y < s.end[1] && p.z < s.end[2];
}

// create_spans (src/octree/mod.rs:300-328): children 0..7 = (-x,-y,-z),
// (-x,-y,+z), (-x,+y,-z), ..., (+x,+y,+z).
void child_spans(const cg_span& p, cg_span out[8]) {
    float c[3];
    for (int k = 0; k < 3; ++k) c[k] = p.start[k] + (p.end[k] - p.start[k]) / 2.0f;
    for (int i = 0; i < 8; ++i) {
        const int bit[3] = {(i >> 2) & 1, (i >> 1) & 1, i & 1};
        for (int k = 0; k < 3; ++k) {
            out[i].start[k] = bit[k] ? c[k] : p.start[k];
            out[i].end[k] = bit[k] ? p.end[k] : c[k];
        }
    }
}

struct Node {
    cg_span span;
    int32_t child = -1;  // first of 8 consecutive children; -1 for a leaf
    uint32_t depth = 0;
    uint32_t status = 0;  // 0 empty, 1 requested, 2 ready
    int32_t gen = -1;     // generation holding the mesh (ready)
    uint64_t voff = 0, ioff = 0;
    uint32_t nv = 0, ni = 0;
};

struct Generation {
    cg_vertex* verts = nullptr;
    uint32_t* idx = nullptr;
    uint32_t refs = 0;
};

// One batched mesher run and what it needs until it is collected.
struct Run {
    cg_batch* batch = nullptr;
    cudaEvent_t done = nullptr;
    bool inflight = false;
    int32_t gen = -1;
    uint64_t vcap = 0, icap = 0;
    std::vector<cg_span_job> jobs;
    cg_job_mesh* d_results = nullptr;  // device, batch capacity
    cg_job_mesh* h_results = nullptr;  // pinned
    uint32_t results_cap = 0;
    uint32_t* d_totals = nullptr;      // device, 4 words
    uint32_t* h_totals = nullptr;      // pinned
};

}  // namespace
}  // namespace cg

using namespace cg;

struct cg_shape_mesh {
    int device = 0;
    cg_shape shape{};
    ShapeDev sdev{};
    uint32_t res = 64;
    cudaStream_t stream = nullptr;  // mesh jobs
    cudaStream_t fstream = nullptr; // focus rays (not queued behind the jobs)
    std::vector<Node> nodes;
    std::vector<Generation> gens;
    uint32_t normals = CG_NORMALS_FD, numerics = CG_NUMERICS_EXACT;
    // run slots; `queue` holds the ones in flight, oldest first
    Run runs[kMaxRuns];
    std::vector<uint32_t> queue;
    // focus rays
    float* d_rays = nullptr;  // org | dir | hits, 3 x 3 x F^2 floats
    uint8_t* d_hit = nullptr;
    float* h_rays = nullptr;  // pinned mirror
    uint8_t* h_hit = nullptr;
    std::vector<float> focii;
    std::mutex mu;
};

namespace {

struct DevScope {
    int prev = -1;
    explicit DevScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DevScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

int32_t leaf_around(const cg_shape_mesh* sm, V3 p) {
    if (!span_contains(sm->nodes[0].span, p)) return -1;
    int32_t i = 0;
    while (sm->nodes[i].child >= 0) {
        int32_t next = -1;
        for (int c = 0; c < 8 && next < 0; ++c)
            if (span_contains(sm->nodes[sm->nodes[i].child + c].span, p)) next = sm->nodes[i].child + c;
        if (next < 0) return -1;  // p on a gap between children (cannot happen for create_spans)
        i = next;
    }
    return i;
}

void release(cg_shape_mesh* sm, Node& n) {
    if (n.gen >= 0) {
        Generation& g = sm->gens[n.gen];
        if (g.refs && --g.refs == 0) {
            cudaFreeAsync(g.verts, sm->stream);
            cudaFreeAsync(g.idx, sm->stream);
            g.verts = nullptr;
            g.idx = nullptr;
        }
    }
    n.gen = -1;
    n.nv = n.ni = 0;
}

void split(cg_shape_mesh* sm, int32_t i) {
    release(sm, sm->nodes[i]);
    sm->nodes[i].status = 0;
    cg_span ch[8];
    child_spans(sm->nodes[i].span, ch);
    const int32_t first = (int32_t)sm->nodes.size();
    const uint32_t depth = sm->nodes[i].depth + 1;
    for (int c = 0; c < 8; ++c) {
        Node n;
        n.span = ch[c];
        n.depth = depth;
        sm->nodes.push_back(n);
    }
    sm->nodes[i].child = first;
}

// Leaves in Octree::iter order: pop a node, push its children 0..7.
std::vector<int32_t> leaves_in_order(const cg_shape_mesh* sm) {
    std::vector<int32_t> out, stack{0};
    while (!stack.empty()) {
        const int32_t i = stack.back();
        stack.pop_back();
        if (sm->nodes[i].child < 0) {
            out.push_back(i);
        } else {
            for (int c = 0; c < 8; ++c) stack.push_back(sm->nodes[i].child + c);
        }
    }
    return out;
}

cg_status focus_rays(const cg_view& v, uint32_t F, float* org, float* dir) {
    if (F == 0 || !(v.fov_y > 0.0f) || !(v.aspect > 0.0f) || !(v.near_plane > 0.0f)) {
        set_error("bad view: fov_y, aspect and near_plane must be > 0");
        return CG_EINVAL;
    }
    const V3 pos = {v.position[0], v.position[1], v.position[2]};
    V3 d = {v.direction[0], v.direction[1], v.direction[2]};
    if (dot(d, d) == 0.0f) {
        set_error("bad view: zero direction (Camera::new asserts)");
        return CG_EINVAL;
    }
    d = normalize(d);
    // Projection::near_plane_dimension and Camera::near_plane_bb (camera.rs:117-134,184-189).
    const float height = 2.0f * v.near_plane * std::tan(v.fov_y * 0.5f);
    const float width = height * v.aspect;
    const V3 tl = {-width / 2.0f, -height / 2.0f, -v.near_plane};
    const V3 br = {width / 2.0f, height / 2.0f, -v.near_plane};
    const float sh = width / (float)F, sv = height / (float)F;
    const float den = 2.0f * (float)F;  // Vector3 / f32 divides each component
    const V3 cdiff = {(br.x - tl.x) / den, (br.y - tl.y) / den, (br.z - tl.z) / den};
    // Matrix4::look_at_rh(pos, pos + d, +z) maps world to view space with
    // rows s, u, -f; its inverse (a rigid motion) maps a view-space point c
    // to pos + c.x s + c.y u - c.z f.
    const V3 f = normalize(sub(add(pos, d), pos));
    const V3 s = normalize(cross(f, V3{0.0f, 0.0f, 1.0f}));
    const V3 u = cross(s, f);
    uint32_t k = 0;
    for (uint32_t x = 0; x < F; ++x) {
        for (uint32_t y = 0; y < F; ++y, ++k) {
            const V3 c = add(add(tl, V3{(float)x * sh, (float)y * sv, 0.0f}), cdiff);
            const V3 p = add(add(add(pos, scale(s, c.x)), scale(u, c.y)), scale(f, -c.z));
            const V3 r = normalize(sub(p, pos));
            org[3 * k] = pos.x;
            org[3 * k + 1] = pos.y;
            org[3 * k + 2] = pos.z;
            dir[3 * k] = r.x;
            dir[3 * k + 1] = r.y;
            dir[3 * k + 2] = r.z;
        }
    }
    return CG_OK;
}

// Grows the run's batch to hold `jobs` (a new batch when the job list does
// not fit).
cg_status fit_batch(cg_shape_mesh* sm, Run& run, const std::vector<cg_span_job>& jobs) {
    const uint32_t n = (uint32_t)jobs.size();
    if (run.batch) {
        const cg_status st = cg_batch_set_jobs(run.batch, jobs.data(), n);
        if (st == CG_OK) return CG_OK;
        if (st != CG_ECAPACITY) return st;
        cg_batch_destroy(run.batch);
        run.batch = nullptr;
    }
    // Room for twice as many jobs, so the next updates rarely reallocate.
    std::vector<cg_span_job> padded(jobs);
    while (padded.size() < 2 * jobs.size()) padded.push_back(jobs.back());
    const uint64_t r3 = (uint64_t)sm->res * sm->res * sm->res;
    CG_TRY(cg_batch_create(sm->device, padded.data(), (uint32_t)padded.size(),
                           r3 * padded.size(), &run.batch));
    CG_TRY(cg_batch_set_jobs(run.batch, jobs.data(), n));
    if (run.results_cap < padded.size()) {
        if (run.d_results) cudaFree(run.d_results);
        if (run.h_results) cudaFreeHost(run.h_results);
        run.d_results = nullptr;
        run.h_results = nullptr;
        run.results_cap = 0;
        CG_CUDA(cudaMalloc(&run.d_results, sizeof(cg_job_mesh) * padded.size()));
        CG_CUDA(cudaMallocHost(&run.h_results, sizeof(cg_job_mesh) * padded.size()));
        run.results_cap = (uint32_t)padded.size();
    }
    if (!run.d_totals) {
        CG_CUDA(cudaMalloc(&run.d_totals, 4 * sizeof(uint32_t)));
        CG_CUDA(cudaMallocHost(&run.h_totals, 4 * sizeof(uint32_t)));
    }
    if (!run.done) CG_CUDA(cudaEventCreateWithFlags(&run.done, cudaEventDisableTiming));
    return CG_OK;
}

// Launches the run's batch into its generation with its current capacities.
cg_status launch_run(cg_shape_mesh* sm, Run& run) {
    Generation& g = sm->gens[run.gen];
    CG_TRY(cg_batch_set_normals(run.batch, sm->normals));
    CG_TRY(cg_batch_set_numerics(run.batch, sm->numerics));
    CG_TRY(cg_batch_mesh(run.batch, &sm->shape, g.verts, run.vcap, g.idx, run.icap,
                         run.d_results, run.d_totals, sm->stream));
    CG_CUDA(cudaMemcpyAsync(run.h_results, run.d_results, sizeof(cg_job_mesh) * run.jobs.size(),
                            cudaMemcpyDeviceToHost, sm->stream));
    CG_CUDA(cudaMemcpyAsync(run.h_totals, run.d_totals, 3 * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, sm->stream));
    CG_CUDA(cudaEventRecord(run.done, sm->stream));
    return CG_OK;
}

cg_status alloc_gen_buffers(cg_shape_mesh* sm, const Run& run, Generation& g) {
    CG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&g.verts),
                            sizeof(cg_vertex) * (run.vcap ? run.vcap : 1), sm->stream));
    CG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&g.idx),
                            sizeof(uint32_t) * (run.icap ? run.icap : 1), sm->stream));
    return CG_OK;
}

void free_run(Run& run) {
    if (run.batch) cg_batch_destroy(run.batch);
    if (run.d_results) cudaFree(run.d_results);
    if (run.h_results) cudaFreeHost(run.h_results);
    if (run.d_totals) cudaFree(run.d_totals);
    if (run.h_totals) cudaFreeHost(run.h_totals);
    if (run.done) cudaEventDestroy(run.done);
    run = Run{};
}

// Collects a finished run: grows and reruns it once if an output overflowed,
// then hands every job's mesh to the leaf around its span's centre.  A rerun
// goes to the back of the stream, so it waits for the runs queued after
// this one; the queue's order of collection stays the launch order.
cg_status collect(cg_shape_mesh* sm, Run& run, uint32_t* collected) {
    CG_CUDA(cudaEventSynchronize(run.done));
    const uint64_t nv = run.h_totals[0], ni = 6ull * run.h_totals[1];
    if (nv > run.vcap || ni > run.icap) {
        Generation& g = sm->gens[run.gen];
        CG_CUDA(cudaFreeAsync(g.verts, sm->stream));
        CG_CUDA(cudaFreeAsync(g.idx, sm->stream));
        run.vcap = nv;
        run.icap = ni;
        CG_TRY(alloc_gen_buffers(sm, run, g));
        CG_TRY(launch_run(sm, run));
        CG_CUDA(cudaEventSynchronize(run.done));
    }
    Generation& g = sm->gens[run.gen];
    for (size_t j = 0; j < run.jobs.size(); ++j) {
        const cg_span& sp = run.jobs[j].span;
        // SpanExt::center: start + (end - start) / 2 (src/octree/mod.rs:20-22)
        const V3 c = {sp.start[0] + (sp.end[0] - sp.start[0]) / 2.0f,
                      sp.start[1] + (sp.end[1] - sp.start[1]) / 2.0f,
                      sp.start[2] + (sp.end[2] - sp.start[2]) / 2.0f};
        const int32_t i = leaf_around(sm, c);
        if (i < 0) continue;
        Node& n = sm->nodes[i];
        release(sm, n);
        const cg_job_mesh& r = run.h_results[j];
        n.status = 2;
        n.gen = run.gen;
        n.voff = r.vertex_offset;
        n.ioff = r.index_offset;
        n.nv = r.vertices;
        n.ni = r.indices;
        ++g.refs;
        ++*collected;
    }
    if (g.refs == 0) {  // every leaf of the run was split away meanwhile
        cudaFreeAsync(g.verts, sm->stream);
        cudaFreeAsync(g.idx, sm->stream);
        g.verts = nullptr;
        g.idx = nullptr;
    }
    run.inflight = false;
    run.jobs.clear();
    run.gen = -1;
    return CG_OK;
}

uint32_t jobs_in_flight(const cg_shape_mesh* sm) {
    uint32_t n = 0;
    for (uint32_t k : sm->queue) n += (uint32_t)sm->runs[k].jobs.size();
    return n;
}

}  // namespace

extern "C" {

cg_status cg_view_focus_rays(const cg_view* view, uint32_t focus_points, float* origins,
                             float* dirs) {
    if (!view || !origins || !dirs) {
        set_error("bad arguments to cg_view_focus_rays");
        return CG_EINVAL;
    }
    return focus_rays(*view, focus_points, origins, dirs);
}

cg_status cg_shape_mesh_create(int device, const cg_shape* shape, const cg_span* bounds,
                               uint32_t resolution, cg_shape_mesh** out) {
    if (!out || !bounds) {
        set_error("bad arguments to cg_shape_mesh_create");
        return CG_EINVAL;
    }
    *out = nullptr;
    CG_TRY(check_shape(shape));
    if (resolution < 2 || (resolution & (resolution - 1)) || resolution > 256) {
        set_error("resolution must be a power of two in [2, 256]");
        return CG_EINVAL;
    }
    for (int k = 0; k < 3; ++k) {
        if (!(bounds->start[k] < bounds->end[k])) {
            set_error("bounds.start < bounds.end does not hold");
            return CG_EINVAL;
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error("no CUDA device");
        return CG_ENODEV;
    }
    cg_shape_mesh* sm = new (std::nothrow) cg_shape_mesh();
    if (!sm) return CG_ENOMEM;
    sm->device = device;
    sm->shape = *shape;
    sm->sdev = make_shape_dev(*shape);
    sm->res = resolution;
    // Octree::spanning + split of the root and of its eight children (mod.rs:50-56).
    Node root;
    root.span = *bounds;
    sm->nodes.push_back(root);
    split(sm, 0);
    for (int c = 0; c < 8; ++c) split(sm, sm->nodes[0].child + c);
    DevScope g(device);
    const size_t F2 = kFocusPoints * kFocusPoints;
    cg_status st = CG_OK;
    auto ok = [&](cudaError_t e, const char* what) {
        if (st == CG_OK) st = cuda_status(e, what, __FILE__, __LINE__);
    };
    ok(cudaStreamCreateWithFlags(&sm->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ok(cudaStreamCreateWithFlags(&sm->fstream, cudaStreamNonBlocking), "cudaStreamCreate");
    ok(cudaMalloc(&sm->d_rays, 9 * F2 * sizeof(float)), "cudaMalloc");
    ok(cudaMalloc(&sm->d_hit, F2), "cudaMalloc");
    ok(cudaMallocHost(&sm->h_rays, 9 * F2 * sizeof(float)), "cudaMallocHost");
    ok(cudaMallocHost(&sm->h_hit, F2), "cudaMallocHost");
    if (st != CG_OK) {
        cg_shape_mesh_destroy(sm);
        return st;
    }
    *out = sm;
    return CG_OK;
}

void cg_shape_mesh_destroy(cg_shape_mesh* sm) {
    if (!sm) return;
    DevScope g(sm->device);
    if (sm->stream) {
        for (Generation& gen : sm->gens) {
            if (gen.verts) cudaFreeAsync(gen.verts, sm->stream);
            if (gen.idx) cudaFreeAsync(gen.idx, sm->stream);
        }
        cudaStreamSynchronize(sm->stream);
    }
    for (Run& run : sm->runs) free_run(run);
    if (sm->d_rays) cudaFree(sm->d_rays);
    if (sm->d_hit) cudaFree(sm->d_hit);
    if (sm->h_rays) cudaFreeHost(sm->h_rays);
    if (sm->h_hit) cudaFreeHost(sm->h_hit);
    if (sm->fstream) cudaStreamDestroy(sm->fstream);
    if (sm->stream) cudaStreamDestroy(sm->stream);
    delete sm;
}

cg_status cg_shape_mesh_update(cg_shape_mesh* sm, const cg_view* view, uint32_t wait,
                               cg_lod_stats* stats) {
    if (!sm || !view) {
        set_error("bad arguments to cg_shape_mesh_update");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(sm->mu);
    DevScope g(sm->device);
    cg_lod_stats s{};
    // (1) focus rays on the GPU, then the split rule on the host.
    const uint32_t F2 = kFocusPoints * kFocusPoints;
    float* h_org = sm->h_rays;
    float* h_dir = sm->h_rays + 3 * F2;
    float* h_hits = sm->h_rays + 6 * F2;
    CG_TRY(focus_rays(*view, kFocusPoints, h_org, h_dir));
    CG_CUDA(cudaMemcpyAsync(sm->d_rays, sm->h_rays, 6 * F2 * sizeof(float),
                            cudaMemcpyHostToDevice, sm->fstream));
    CG_TRY(launch_march(sm->sdev, sm->d_rays, sm->d_rays + 3 * F2, F2, kFocusSteps, kFocusEpsilon,
                        sm->d_rays + 6 * F2, sm->d_hit, sm->fstream));
    CG_CUDA(cudaMemcpyAsync(h_hits, sm->d_rays + 6 * F2, 3 * F2 * sizeof(float),
                            cudaMemcpyDeviceToHost, sm->fstream));
    CG_CUDA(cudaMemcpyAsync(sm->h_hit, sm->d_hit, F2, cudaMemcpyDeviceToHost, sm->fstream));
    CG_CUDA(cudaStreamSynchronize(sm->fstream));
    sm->focii.clear();
    const V3 cam = {view->position[0], view->position[1], view->position[2]};
    for (uint32_t k = 0; k < F2; ++k) {
        if (!sm->h_hit[k]) continue;
        const V3 focus = {h_hits[3 * k], h_hits[3 * k + 1], h_hits[3 * k + 2]};
        sm->focii.insert(sm->focii.end(), {focus.x, focus.y, focus.z});
        ++s.focii;
        const int32_t i = leaf_around(sm, focus);
        if (i < 0 || sm->nodes[i].status != 2) continue;
        const V3 dv = sub(cam, focus);
        const float dist = std::sqrt(dot(dv, dv));  // MetricSpace::distance
        const cg_span& sp = sm->nodes[i].span;
        const float threshold = 2.0f * std::fabs(sp.end[0] - sp.start[0]);
        if (dist < threshold) {
            split(sm, i);
            ++s.splits;
        }
    }
    // (2) meshes of the finished runs, oldest first (with wait: all of them).
    while (!sm->queue.empty()) {
        Run& run = sm->runs[sm->queue.front()];
        const cudaError_t q = wait ? cudaSuccess : cudaEventQuery(run.done);
        if (q == cudaErrorNotReady) break;  // the later runs are behind it
        if (q != cudaSuccess) return cuda_status(q, "cudaEventQuery", __FILE__, __LINE__);
        CG_TRY(collect(sm, run, &s.collected));
        sm->queue.erase(sm->queue.begin());
    }
    // (3) a job for every empty leaf, in a new run queued behind the ones in
    // flight (its leaves are "requested"); with all kMaxRuns slots in flight
    // the empty leaves wait for a later update.
    std::vector<int32_t> empty;
    for (int32_t i : leaves_in_order(sm))
        if (sm->nodes[i].status == 0) empty.push_back(i);
    if (!empty.empty() && sm->queue.size() < kMaxRuns) {
        uint32_t slot = 0;
        while (sm->runs[slot].inflight) ++slot;
        Run& run = sm->runs[slot];
        run.jobs.clear();
        for (int32_t i : empty) {
            cg_span_job j{};
            j.span = sm->nodes[i].span;
            j.resolution = sm->res;
            run.jobs.push_back(j);
        }
        CG_TRY(fit_batch(sm, run, run.jobs));
        // A res-64 leaf of the Mandelbulb has ~1/16 of its cells on the
        // surface at most; the run grows and repeats once if not.
        const uint64_t r3 = (uint64_t)sm->res * sm->res * sm->res;
        run.vcap = std::max<uint64_t>(4096, empty.size() * (r3 / 16));
        run.icap = 8 * run.vcap;
        sm->gens.push_back(Generation{});
        run.gen = (int32_t)sm->gens.size() - 1;
        CG_TRY(alloc_gen_buffers(sm, run, sm->gens.back()));
        CG_TRY(launch_run(sm, run));
        run.inflight = true;
        sm->queue.push_back(slot);
        for (int32_t i : empty) sm->nodes[i].status = 1;
        s.started = (uint32_t)empty.size();
    }
    s.active = jobs_in_flight(sm);
    s.leaves = (uint32_t)leaves_in_order(sm).size();
    if (stats) *stats = s;
    return CG_OK;
}

cg_status cg_shape_mesh_leaves(cg_shape_mesh* sm, cg_leaf* leaves, uint32_t cap,
                               uint32_t* count) {
    if (!sm || !count || (cap && !leaves)) {
        set_error("bad arguments to cg_shape_mesh_leaves");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(sm->mu);
    const std::vector<int32_t> order = leaves_in_order(sm);
    *count = (uint32_t)order.size();
    for (uint32_t k = 0; k < cap && k < order.size(); ++k) {
        const Node& n = sm->nodes[order[k]];
        cg_leaf& l = leaves[k];
        memset(&l, 0, sizeof l);
        l.span = n.span;
        l.status = n.status;
        l.depth = n.depth;
        if (n.status == 2 && n.gen >= 0) {
            const Generation& gen = sm->gens[n.gen];
            l.vertices = gen.verts + n.voff;
            l.indices = gen.idx + n.ioff;
            l.n_vertices = n.nv;
            l.n_indices = n.ni;
        }
    }
    return CG_OK;
}

cg_status cg_shape_mesh_focii(cg_shape_mesh* sm, float* points, uint32_t cap, uint32_t* count) {
    if (!sm || !count || (cap && !points)) {
        set_error("bad arguments to cg_shape_mesh_focii");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(sm->mu);
    *count = (uint32_t)(sm->focii.size() / 3);
    for (uint32_t k = 0; k < cap && k < *count; ++k)
        for (int c = 0; c < 3; ++c) points[3 * k + c] = sm->focii[3 * k + c];
    return CG_OK;
}

cg_status cg_shape_mesh_set_options(cg_shape_mesh* sm, uint32_t normals, uint32_t numerics) {
    if (!sm || normals > CG_NORMALS_ADJOINT || numerics > CG_NUMERICS_FAST ||
        (normals == CG_NORMALS_ADJOINT && numerics == CG_NUMERICS_FAST)) {
        set_error("bad shape mesh or options (fast numerics with the six-sample normals only)");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(sm->mu);
    sm->normals = normals;
    sm->numerics = numerics;
    return CG_OK;
}

}  // extern "C"
