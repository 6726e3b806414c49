// capi.cu -- implementation of the C ABI declared in include/cantucci_gpu.h:
// argument checks (the reference's assert! panics become CG_EINVAL), span
// set-up in the reference's f32 operation order, the mesher object and its
// device workspace.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <new>

#include "common.cuh"
#include "kernels.cuh"
#include "mesh_rows.cuh"

namespace cg {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const char* get_error() { return g_err; }

int sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 148;
        cache[dev] = n;
    }
    return cache[dev];
}

// R = Rz(c) Ry(b) Rx(a), row-major, computed in double and rounded to f32.
__host__ ShapeDev make_shape_dev(const cg_shape& s) {
    ShapeDev d;
    memset(&d, 0, sizeof d);
    d.kind = s.kind;
    d.power = s.power;
    d.power_f = s.power_f;
    d.max_iters = s.max_iters;
    d.bailout = s.bailout;
    const double ca = cos((double)s.rot[0]), sa = sin((double)s.rot[0]);
    const double cb = cos((double)s.rot[1]), sb = sin((double)s.rot[1]);
    const double cc = cos((double)s.rot[2]), sc = sin((double)s.rot[2]);
    const double m[9] = {cc * cb, cc * sb * sa - sc * ca, cc * sb * ca + sc * sa,
                         sc * cb, sc * sb * sa + cc * ca, sc * sb * ca - cc * sa,
                         -sb,     cb * sa,                cb * ca};
    for (int i = 0; i < 9; ++i) d.m[i] = (float)m[i];
    for (int i = 0; i < 3; ++i) d.center[i] = s.center[i];
    d.radius = s.radius;
    d.rotated = s.rot[0] != 0.0f || s.rot[1] != 0.0f || s.rot[2] != 0.0f;
    return d;
}

// Span widening and grid steps of src/mesh/buffer.rs:64-67,77,101,257, one
// f32 rounding per operation (host code is built with -ffp-contract=off).
SpanSetup setup_span(const cg_span& sp, uint32_t res) {
    SpanSetup su;
    const float rf = (float)res;
    for (int k = 0; k < 3; ++k) {
        const float ov = (sp.end[k] - sp.start[k]) / rf;
        su.start[k] = sp.start[k] + -ov;
        su.end[k] = sp.end[k] + ov;
        su.across[k] = su.end[k] - su.start[k];
        su.step[k] = (su.end[k] - su.start[k]) / rf;
        su.delta[k] = (0.7f * (su.end[k] - su.start[k])) / rf;
    }
    return su;
}

GridDev make_grid(const SpanSetup& su, uint32_t res) {
    GridDev g;
    for (int k = 0; k < 3; ++k) {
        g.start[k] = su.start[k];
        g.across[k] = su.across[k];
    }
    g.inv_res = 1.0f / (float)res;
    g.n = res + 1;
    return g;
}

cg_status check_shape(const cg_shape* s) {
    if (!s) {
        set_error("shape is NULL");
        return CG_EINVAL;
    }
    switch (s->kind) {
    case CG_SHAPE_MANDELBULB:
        if (s->power < 0 || s->power > 255) {
            set_error("Mandelbulb power %d outside the u8 range", s->power);
            return CG_EINVAL;
        }
        if (s->max_iters < 1) {
            set_error("Mandelbulb::new asserts max_iters >= 1");
            return CG_EINVAL;
        }
        return CG_OK;
    case CG_SHAPE_MANDELBULB_POLAR:
        if (s->max_iters < 1) {
            set_error("max_iters must be >= 1");
            return CG_EINVAL;
        }
        return CG_OK;
    case CG_SHAPE_SPHERE:
        return CG_OK;
    default:
        set_error("unknown shape kind %d", s->kind);
        return CG_EINVAL;
    }
}

// generate_for_box's assertions (src/mesh/buffer.rs:35-39) plus
// GridTable::fill_with's size >= 2 (src/util/grid.rs:24); res <= 1024 keeps
// every grid index in 32 bits.
cg_status check_span_res(const cg_span* span, uint32_t res) {
    if (!span) {
        set_error("span is NULL");
        return CG_EINVAL;
    }
    for (int k = 0; k < 3; ++k) {
        if (!(span->start[k] < span->end[k])) {
            set_error("span.start[%d] < span.end[%d] does not hold", k, k);
            return CG_EINVAL;
        }
    }
    if (res < 2 || (res & (res - 1)) != 0 || res > 1024) {
        set_error("resolution %u must be a power of two in [2, 1024]", res);
        return CG_EINVAL;
    }
    return CG_OK;
}

}  // namespace cg

using namespace cg;

// The span-dependent parameters of a mesh, read from device memory by a
// replayed graph.
struct MeshGraphParams {
    GridDev g;
    PlaceParams pp;
};

// What a captured mesh graph depends on besides the span (compared bytewise).
struct MeshGraphKey {
    cg_shape shape;
    uint32_t res, numerics, normals, root_iters, grid_kernel, place_bps;
    const void* work;
    const void* dverts;
    const void* didx;
    uint64_t vcap, icap;
};

struct cg_mesher {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host-output copies overlapping placement
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t fork = nullptr, join = nullptr;  // quads on copy_stream beside placement
    char* work = nullptr;
    size_t work_bytes = 0;
    cg_vertex* dverts = nullptr;
    size_t dverts_cap = 0;
    uint32_t* didx = nullptr;
    size_t didx_cap = 0;
    MeshCounters* hcnt = nullptr;  // pinned
    uint32_t normals = CG_NORMALS_FD;
    uint32_t root_iters = 0;  // CG_CROSSINGS_LERP
    uint32_t placement = CG_PLACEMENT_CENTROID;
    uint32_t numerics = CG_NUMERICS_EXACT;
    DeviceScratch edge_rows, edge_data;  // dual contouring's edge table
    // The device-side mesh captured as a graph (run_mesh): replayed while the
    // key matches, the span going in through the parameter block.
    cudaGraphExec_t gexec = nullptr;
    MeshGraphKey gkey{};
    MeshGraphParams* gparams_dev = nullptr;
    MeshGraphParams* gparams_host = nullptr;  // pinned
    bool graph_broken = false;                // a capture failed: launch directly
    uint32_t last_res = 0;
    MeshWork last_w{};
    std::mutex mu;
};

namespace {

// 1 (default): meshes up to resolution 128 without dual contouring replay a
// graph captured per mesher (cg_set_option "mesh_graphs"; 0: direct
// launches).
std::atomic<int> g_mesh_graphs{1};

// 1 (default): meshers created afterwards give their side stream (quads,
// index copies) the highest stream priority, so its short kernels take
// SMs ahead of the placement's waiting blocks (cg_set_option
// "side_stream_priority"; 0: equal priorities).
std::atomic<int> g_side_priority{1};

PlaceOptions place_options(cg_mesher* m) {
    PlaceOptions o;
    o.analytic_normals = m->normals == CG_NORMALS_ADJOINT;
    o.root_iters = m->root_iters;
    o.qef = m->placement == CG_PLACEMENT_QEF;
    o.numerics = m->numerics;
    o.edge_rows = &m->edge_rows;
    o.edge_data = &m->edge_data;
    return o;
}

cg_status ensure(void** p, size_t* cap, size_t bytes) {
    if (*cap >= bytes && *p) return CG_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    CG_CUDA(cudaMalloc(p, bytes));
    *cap = bytes;
    return CG_OK;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Steps 1-3 into device outputs on m->stream, up to the counters' copy into
// m->hcnt: what a mesh graph replays.  With `dp` the span's grid and
// placement parameters are read from the device block dp (copied there from
// the pinned m->gparams_host first).
cg_status enqueue_mesh(cg_mesher* m, const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                       const MeshWork& w, cg_vertex* dverts, uint64_t vcap, uint32_t* didx,
                       uint64_t icap, MeshGraphParams* dp) {
    cudaStream_t st = m->stream;
    if (dp)
        CG_CUDA(cudaMemcpyAsync(dp, m->gparams_host, sizeof(MeshGraphParams),
                                cudaMemcpyHostToDevice, st));
    CG_CUDA(record_event(m->ev[0], st));
    CG_CUDA(cudaMemsetAsync(w.sgn, 0, (size_t)d.n * d.n * d.W * sizeof(uint32_t), st));
    CG_TRY(launch_de_grid(s, make_grid(su, d.res), w.dists, m->numerics, st, w.sgn, d.W,
                          dp ? &dp->g : nullptr));
    CG_CUDA(record_event(m->ev[1], st));
    const SideStream side = {m->copy_stream, m->fork, m->join};
    PlaceOptions opt = place_options(m);
    opt.pp_dev = dp ? &dp->pp : nullptr;
    CG_TRY(launch_mesh_from_dists(s, su, d, w, dverts, vcap, didx, icap, st, m->ev[2],
                                  /*signs_ready=*/true, opt, &side));
    CG_CUDA(record_event(m->ev[3], st));
    CG_CUDA(cudaMemcpyAsync(m->hcnt, w.counters, sizeof(MeshCounters), cudaMemcpyDeviceToHost, st));
    return CG_OK;
}

// Meshes into the graph kept for this mesher, capturing it first if the key
// changed.  Only up to kGraphMaxRes: there the launches cost about as
// much as the work, while in a large mesh they are negligible and a
// replayed graph loses the side stream's priority (its quads then end 0.2 ms
// after the placement on the 513^3 span instead of under it).  Returns false
// (nothing enqueued) if the mesh is not replayed: larger, dual contouring
// (it reads the edge count back mid-way), or capturing failed.
constexpr uint32_t kGraphMaxRes = 128;

bool graph_sized(const cg_mesher* m, uint32_t res) {
    return g_mesh_graphs.load() && !m->graph_broken && m->placement != CG_PLACEMENT_QEF &&
           res <= kGraphMaxRes;
}

bool launch_mesh_graph(cg_mesher* m, const cg_shape* shape, const ShapeDev& s,
                       const SpanSetup& su, const MeshDims& d, const MeshWork& w,
                       cg_vertex* dverts, uint64_t vcap, uint32_t* didx, uint64_t icap) {
    if (!graph_sized(m, d.res)) return false;
    if (!m->gparams_dev) {
        if (cudaMalloc(&m->gparams_dev, sizeof(MeshGraphParams)) != cudaSuccess ||
            cudaMallocHost(&m->gparams_host, sizeof(MeshGraphParams)) != cudaSuccess) {
            cudaGetLastError();
            m->graph_broken = true;
            return false;
        }
    }
    m->gparams_host->g = make_grid(su, d.res);
    m->gparams_host->pp = place_params(su);
    MeshGraphKey k;
    memset(&k, 0, sizeof k);
    k.shape = *shape;
    k.res = d.res;
    k.numerics = m->numerics;
    k.normals = m->normals;
    k.root_iters = m->root_iters;
    k.grid_kernel = (uint32_t)de_grid_kernel_option();
    k.place_bps = place_blocks_per_sm();
    k.work = m->work;
    k.dverts = dverts;
    k.didx = didx;
    k.vcap = vcap;
    k.icap = icap;
    if (!m->gexec || memcmp(&k, &m->gkey, sizeof k) != 0) {
        if (m->gexec) cudaGraphExecDestroy(m->gexec);
        m->gexec = nullptr;
        cudaStream_t st = m->stream;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            m->graph_broken = true;
            return false;
        }
        const cg_status cs = enqueue_mesh(m, s, su, d, w, dverts, vcap, didx, icap, m->gparams_dev);
        cudaGraph_t gr = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(st, &gr);
        cudaError_t ie = cudaErrorUnknown;
        if (cs == CG_OK && ee == cudaSuccess && gr) ie = cudaGraphInstantiate(&m->gexec, gr, 0);
        if (gr) cudaGraphDestroy(gr);
        if (ie != cudaSuccess) {
            cudaGetLastError();
            m->gexec = nullptr;
            m->graph_broken = true;
            return false;
        }
        m->gkey = k;
    }
    return cudaGraphLaunch(m->gexec, m->stream) == cudaSuccess;
}

// Runs steps 1-3 into device outputs; counts and status land in m->hcnt.
cg_status run_mesh(cg_mesher* m, const cg_span* span, const cg_shape* shape, uint32_t res,
                   cg_vertex* dverts, uint64_t vcap, uint32_t* didx, uint64_t icap,
                   cg_timings* tm) {
    CG_TRY(check_span_res(span, res));
    CG_TRY(check_shape(shape));
    const ShapeDev s = make_shape_dev(*shape);
    const SpanSetup su = setup_span(*span, res);
    const MeshDims d = mesh_dims(res);
    const size_t need = mesh_workspace_layout(res, nullptr, nullptr);
    CG_TRY(ensure(reinterpret_cast<void**>(&m->work), &m->work_bytes, need));
    MeshWork w;
    mesh_workspace_layout(res, m->work, &w);
    if (!launch_mesh_graph(m, shape, s, su, d, w, dverts, vcap, didx, icap))
        CG_TRY(enqueue_mesh(m, s, su, d, w, dverts, vcap, didx, icap, nullptr));
    CG_CUDA(cudaStreamSynchronize(m->stream));
    m->last_res = res;
    m->last_w = w;
    if (tm) {
        float a = 0, b = 0, c = 0;
        CG_CUDA(cudaEventElapsedTime(&a, m->ev[0], m->ev[1]));
        CG_CUDA(cudaEventElapsedTime(&b, m->ev[1], m->ev[2]));
        CG_CUDA(cudaEventElapsedTime(&c, m->ev[2], m->ev[3]));
        tm->first_ms = a;
        tm->second_ms = b;
        tm->third_ms = c;
        tm->vertices = m->hcnt->vertices;
        tm->faces = m->hcnt->quads;
    }
    return CG_OK;
}

// Device address of pinned (page-locked, mapped) host memory, else NULL.
void* mapped_host(void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clear the sticky-free error of an unknown pointer
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Steps 1-3 with host outputs, both pinned: the overlapped pipeline of
// launch_mesh_to_host.  Counts and status land in m->hcnt.
cg_status run_mesh_to_host(cg_mesher* m, const cg_span* span, const cg_shape* shape, uint32_t res,
                           cg_vertex* hverts_dev, uint64_t vcap, uint32_t* hidx, uint64_t icap,
                           cg_timings* tm) {
    CG_TRY(check_span_res(span, res));
    CG_TRY(check_shape(shape));
    const ShapeDev s = make_shape_dev(*shape);
    const SpanSetup su = setup_span(*span, res);
    const MeshDims d = mesh_dims(res);
    const size_t need = mesh_workspace_layout(res, nullptr, nullptr);
    CG_TRY(ensure(reinterpret_cast<void**>(&m->work), &m->work_bytes, need));
    const uint64_t r3 = (uint64_t)res * res * res;
    const uint64_t idev = icap < 18 * r3 ? icap : 18 * r3;
    CG_TRY(ensure(reinterpret_cast<void**>(&m->didx), &m->didx_cap,
                  (idev ? idev : 1) * sizeof(uint32_t)));
    MeshWork w;
    mesh_workspace_layout(res, m->work, &w);
    cudaStream_t st = m->stream;
    CG_CUDA(cudaEventRecord(m->ev[0], st));
    CG_CUDA(cudaMemsetAsync(w.sgn, 0, (size_t)d.n * d.n * d.W * sizeof(uint32_t), st));
    CG_TRY(launch_de_grid(s, make_grid(su, res), w.dists, m->numerics, st, w.sgn, d.W));
    CG_CUDA(cudaEventRecord(m->ev[1], st));
    CG_TRY(launch_mesh_to_host(s, su, d, w, hverts_dev, vcap, m->didx, hidx, idev, st,
                               m->copy_stream, m->ev[2], m->ev[3], m->hcnt, place_options(m)));
    CG_CUDA(cudaEventRecord(m->ev[4], st));
    CG_CUDA(cudaMemcpyAsync(m->hcnt, w.counters, sizeof(MeshCounters), cudaMemcpyDeviceToHost, st));
    CG_CUDA(cudaStreamSynchronize(st));
    CG_CUDA(cudaStreamSynchronize(m->copy_stream));
    if (tm) {
        // The quads ran on the copy stream from ev[2]; ev[3] closes them.
        float a = 0, b = 0, c = 0;
        CG_CUDA(cudaEventElapsedTime(&a, m->ev[0], m->ev[1]));
        CG_CUDA(cudaEventElapsedTime(&b, m->ev[1], m->ev[4]));
        CG_CUDA(cudaEventElapsedTime(&c, m->ev[2], m->ev[3]));
        tm->first_ms = a;
        tm->second_ms = b;  // cells, counts and vertex placement
        tm->third_ms = c;   // quad indices, beside the placement
        tm->vertices = m->hcnt->vertices;
        tm->faces = m->hcnt->quads;
    }
    m->last_res = res;
    m->last_w = w;
    return CG_OK;
}

cg_status finish_status(const MeshCounters& c, uint64_t vcap, uint64_t icap) {
    if (c.status & MESH_LERP_FAIL) {
        set_error("a lerp factor left [0, 1] (src/math.rs:19 panics here)");
        return CG_ELERP;
    }
    if ((uint64_t)c.vertices > vcap || 6ull * c.quads > icap) {
        set_error("output capacity too small: need %u vertices and %llu indices", c.vertices,
                  6ull * c.quads);
        return CG_ECAPACITY;
    }
    return CG_OK;
}

}  // namespace

extern "C" {

int cg_abi_version(void) { return CG_ABI_VERSION; }
const char* cg_last_error(void) { return get_error(); }
uint32_t cg_sizeof_shape(void) { return (uint32_t)sizeof(cg_shape); }
uint32_t cg_sizeof_vertex(void) { return (uint32_t)sizeof(cg_vertex); }

cg_status cg_min_distance_from(const cg_shape* shape, const float* points, uint64_t n, float* out,
                               uint32_t numerics, void* stream) {
    CG_TRY(check_shape(shape));
    if (n && (!points || !out)) {
        set_error("points/out is NULL");
        return CG_EINVAL;
    }
    return launch_de_points(make_shape_dev(*shape), points, n, out, numerics,
                            (cudaStream_t)stream);
}

cg_status cg_contains(const cg_shape* shape, const float* points, uint64_t n, uint8_t* out,
                      void* stream) {
    CG_TRY(check_shape(shape));
    if (n && (!points || !out)) {
        set_error("points/out is NULL");
        return CG_EINVAL;
    }
    return launch_contains(make_shape_dev(*shape), points, n, out, (cudaStream_t)stream);
}

cg_status cg_de_span_grid(const cg_shape* shape, const cg_span* span, uint32_t resolution,
                          float* dists, uint32_t numerics, void* stream) {
    CG_TRY(check_shape(shape));
    CG_TRY(check_span_res(span, resolution));
    if (!dists) {
        set_error("dists is NULL");
        return CG_EINVAL;
    }
    const SpanSetup su = setup_span(*span, resolution);
    return launch_de_grid(make_shape_dev(*shape), make_grid(su, resolution), dists, numerics,
                          (cudaStream_t)stream);
}

cg_status cg_mandelbulb_state(const cg_shape* shape, const float* points, uint64_t n,
                              float* state, void* stream) {
    CG_TRY(check_shape(shape));
    if (shape->kind != CG_SHAPE_MANDELBULB) {
        set_error("cg_mandelbulb_state needs an integer-power Mandelbulb");
        return CG_EINVAL;
    }
    return launch_state(make_shape_dev(*shape), points, n, state, (cudaStream_t)stream);
}

cg_status cg_mesher_create(int device, cg_mesher** out) {
    if (!out) {
        set_error("out is NULL");
        return CG_EINVAL;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        set_error("no CUDA device");
        return CG_ENODEV;
    }
    if (device < 0 || device >= ndev) {
        set_error("device %d out of range", device);
        return CG_EINVAL;
    }
    cg_mesher* m = new (std::nothrow) cg_mesher();
    if (!m) return CG_ENOMEM;
    m->device = device;
    DeviceGuard g(device);
    cg_status st = CG_OK;
    if ((st = cuda_status(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking),
                          "cudaStreamCreate", __FILE__, __LINE__)) != CG_OK) {
        delete m;
        return st;
    }
    for (auto& e : m->ev) cudaEventCreate(&e);
    cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&m->join, cudaEventDisableTiming);
    int prio_lo = 0, prio_hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess) prio_hi = prio_lo = 0;
    if ((st = cuda_status(cudaStreamCreateWithPriority(&m->copy_stream, cudaStreamNonBlocking,
                                                       g_side_priority.load() ? prio_hi : prio_lo),
                          "cudaStreamCreate", __FILE__, __LINE__)) != CG_OK) {
        cg_mesher_destroy(m);
        return st;
    }
    if (cudaMallocHost(reinterpret_cast<void**>(&m->hcnt), sizeof(MeshCounters)) != cudaSuccess) {
        cg_mesher_destroy(m);
        set_error("cudaMallocHost failed");
        return CG_ENOMEM;
    }
    *out = m;
    return CG_OK;
}

void cg_mesher_destroy(cg_mesher* m) {
    if (!m) return;
    DeviceGuard g(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    if (m->work) cudaFree(m->work);
    if (m->dverts) cudaFree(m->dverts);
    if (m->didx) cudaFree(m->didx);
    if (m->hcnt) cudaFreeHost(m->hcnt);
    if (m->gexec) cudaGraphExecDestroy(m->gexec);
    if (m->gparams_dev) cudaFree(m->gparams_dev);
    if (m->gparams_host) cudaFreeHost(m->gparams_host);
    if (m->edge_rows.ptr) cudaFree(m->edge_rows.ptr);
    if (m->edge_data.ptr) cudaFree(m->edge_data.ptr);
    for (auto& e : m->ev)
        if (e) cudaEventDestroy(e);
    if (m->fork) cudaEventDestroy(m->fork);
    if (m->join) cudaEventDestroy(m->join);
    if (m->copy_stream) cudaStreamDestroy(m->copy_stream);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

cg_status cg_mesher_set_normals(cg_mesher* m, uint32_t normals) {
    if (!m || normals > CG_NORMALS_ADJOINT) {
        set_error("bad mesher or normals mode");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(m->mu);
    m->normals = normals;
    return CG_OK;
}

cg_status cg_mesher_set_crossings(cg_mesher* m, uint32_t crossings, uint32_t iters) {
    if (!m || crossings > CG_CROSSINGS_ROOT ||
        (crossings == CG_CROSSINGS_ROOT && (iters < 1 || iters > 16))) {
        set_error("crossings: CG_CROSSINGS_LERP, or CG_CROSSINGS_ROOT with 1..16 iterations");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(m->mu);
    m->root_iters = crossings == CG_CROSSINGS_ROOT ? iters : 0;
    return CG_OK;
}

cg_status cg_mesher_set_numerics(cg_mesher* m, uint32_t numerics) {
    if (!m || numerics > CG_NUMERICS_FAST) {
        set_error("numerics: CG_NUMERICS_EXACT or CG_NUMERICS_FAST");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(m->mu);
    m->numerics = numerics;
    return CG_OK;
}

cg_status cg_mesher_set_placement(cg_mesher* m, uint32_t placement) {
    if (!m || placement > CG_PLACEMENT_QEF) {
        set_error("placement: CG_PLACEMENT_CENTROID or CG_PLACEMENT_QEF");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(m->mu);
    m->placement = placement;
    return CG_OK;
}

cg_status cg_generate_for_box(cg_mesher* m, const cg_span* span, const cg_shape* shape,
                              uint32_t res, cg_vertex* vertices, uint64_t vertex_cap,
                              uint32_t* indices, uint64_t index_cap, uint64_t* n_vertices,
                              uint64_t* n_indices, cg_timings* tm) {
    if (!m) {
        set_error("mesher is NULL");
        return CG_EINVAL;
    }
    if ((vertex_cap && !vertices) || (index_cap && !indices)) {
        set_error("output buffer is NULL");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(m->mu);
    DeviceGuard g(m->device);
    CG_TRY(check_span_res(span, res));
    // Pinned outputs of a mesh too large for a replayed graph: the GPU writes
    // the vertices into them directly and the index copy overlaps the vertex
    // placement.  Smaller meshes (and pageable outputs) are meshed into
    // device staging and copied once the counts are known.
    void* vmap = vertex_cap && !graph_sized(m, res) ? mapped_host(vertices) : nullptr;
    void* imap = vmap && index_cap ? mapped_host(indices) : nullptr;
    if (vmap && imap) {
        CG_TRY(run_mesh_to_host(m, span, shape, res, static_cast<cg_vertex*>(vmap), vertex_cap,
                                static_cast<uint32_t*>(imap), index_cap, tm));
        const MeshCounters c = *m->hcnt;
        if (n_vertices) *n_vertices = c.vertices;
        if (n_indices) *n_indices = 6ull * c.quads;
        return finish_status(c, vertex_cap, index_cap);
    }
    // Device staging sized to min(capacity, the largest possible count).
    const uint64_t r3 = (uint64_t)res * res * res;
    const uint64_t vdev = vertex_cap < r3 ? vertex_cap : r3;
    const uint64_t idev = index_cap < 18 * r3 ? index_cap : 18 * r3;
    CG_TRY(ensure(reinterpret_cast<void**>(&m->dverts), &m->dverts_cap,
                  (vdev ? vdev : 1) * sizeof(cg_vertex)));
    CG_TRY(ensure(reinterpret_cast<void**>(&m->didx), &m->didx_cap,
                  (idev ? idev : 1) * sizeof(uint32_t)));
    CG_TRY(run_mesh(m, span, shape, res, m->dverts, vdev, m->didx, idev, tm));
    const MeshCounters c = *m->hcnt;
    const uint64_t nv = c.vertices, ni = 6ull * c.quads;
    if (n_vertices) *n_vertices = nv;
    if (n_indices) *n_indices = ni;
    const uint64_t cv = nv < vdev ? nv : vdev, ci = ni < idev ? ni : idev;
    if (cv)
        CG_CUDA(cudaMemcpyAsync(vertices, m->dverts, cv * sizeof(cg_vertex), cudaMemcpyDeviceToHost,
                                m->stream));
    if (ci)
        CG_CUDA(cudaMemcpyAsync(indices, m->didx, ci * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                m->stream));
    CG_CUDA(cudaStreamSynchronize(m->stream));
    return finish_status(c, vertex_cap, index_cap);
}

cg_status cg_generate_for_box_device(cg_mesher* m, const cg_span* span, const cg_shape* shape,
                                     uint32_t res, cg_vertex* vertices, uint64_t vertex_cap,
                                     uint32_t* indices, uint64_t index_cap, uint64_t* n_vertices,
                                     uint64_t* n_indices, cg_timings* tm) {
    if (!m) {
        set_error("mesher is NULL");
        return CG_EINVAL;
    }
    if ((vertex_cap && !vertices) || (index_cap && !indices)) {
        set_error("output buffer is NULL");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(m->mu);
    DeviceGuard g(m->device);
    CG_TRY(run_mesh(m, span, shape, res, vertices, vertex_cap, indices, index_cap, tm));
    const MeshCounters c = *m->hcnt;
    if (n_vertices) *n_vertices = c.vertices;
    if (n_indices) *n_indices = 6ull * c.quads;
    return finish_status(c, vertex_cap, index_cap);
}

cg_status cg_mesher_dists(cg_mesher* m, const float** dists, uint32_t* resolution) {
    if (!m || !m->last_res) {
        set_error("no mesh has been generated yet");
        return CG_EINVAL;
    }
    if (dists) *dists = m->last_w.dists;
    if (resolution) *resolution = m->last_res;
    return CG_OK;
}

cg_status cg_mesher_points(cg_mesher* m, uint32_t* points) {
    if (!m || !m->last_res || !points) {
        set_error("no mesh has been generated yet, or points is NULL");
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(m->mu);
    DeviceGuard g(m->device);
    CG_TRY(launch_points_table(mesh_dims(m->last_res), m->last_w, points, m->stream));
    CG_CUDA(cudaStreamSynchronize(m->stream));
    return CG_OK;
}

cg_status cg_set_option(const char* name, int64_t value) {
    if (name && strcmp(name, "de_grid_kernel") == 0 && set_de_grid_kernel((int)value))
        return CG_OK;
    if (name && set_batch_option(name, value)) return CG_OK;
    if (name && set_trace_option(name, value)) return CG_OK;
    if (name && set_place_option(name, value)) return CG_OK;
    if (name && set_adjoint_option(name, value) == 1) return CG_OK;
    if (name && strcmp(name, "mesh_graphs") == 0 && (value == 0 || value == 1)) {
        g_mesh_graphs.store((int)value);
        return CG_OK;
    }
    if (name && strcmp(name, "side_stream_priority") == 0 && (value == 0 || value == 1)) {
        g_side_priority.store((int)value);
        return CG_OK;
    }
    set_error("unknown option or value: %s = %lld", name ? name : "(null)", (long long)value);
    return CG_EINVAL;
}

cg_status cg_debug_oob(uint64_t* count, uint32_t* line, uint32_t reset) {
#ifdef CG_CHECKED
    if (!count || !line) {
        set_error("NULL argument");
        return CG_EINVAL;
    }
    CG_CUDA(cudaDeviceSynchronize());
    *count = 0;
    *line = 0;
    oob_read_mesh(count, line, reset != 0);
    oob_read_de_kernels(count, line, reset != 0);
    oob_read_scan(count, line, reset != 0);
    oob_read_mesh_batch(count, line, reset != 0);
    return CG_OK;
#else
    (void)count;
    (void)line;
    (void)reset;
    set_error("cg_debug_oob: not the bounds-checked build (libcantucci_gpu_checked.so)");
    return CG_EINVAL;
#endif
}

cg_status cg_mesher_stream(cg_mesher* m, void** stream) {
    if (!m || !stream) {
        set_error("NULL argument");
        return CG_EINVAL;
    }
    *stream = (void*)m->stream;
    return CG_OK;
}

cg_status cg_span_grid_work(const cg_shape* shape, const cg_span* span, uint32_t resolution,
                            uint64_t* steps, uint64_t* escapes) {
    CG_TRY(check_shape(shape));
    CG_TRY(check_span_res(span, resolution));
    if (shape->kind != CG_SHAPE_MANDELBULB || !steps || !escapes) {
        set_error("cg_span_grid_work needs an integer-power Mandelbulb and outputs");
        return CG_EINVAL;
    }
    unsigned long long* acc = nullptr;
    CG_CUDA(cudaMalloc(&acc, 2 * sizeof(unsigned long long)));
    unsigned long long h[2] = {0, 0};
    cg_status st = cuda_status(cudaMemset(acc, 0, sizeof h), "cudaMemset", __FILE__, __LINE__);
    if (st == CG_OK)
        st = launch_grid_work(make_shape_dev(*shape), make_grid(setup_span(*span, resolution),
                                                                resolution),
                              acc, nullptr);
    if (st == CG_OK)
        st = cuda_status(cudaMemcpy(h, acc, sizeof h, cudaMemcpyDeviceToHost), "cudaMemcpy",
                         __FILE__, __LINE__);
    cudaFree(acc);
    *steps = h[0];
    *escapes = h[1];
    return st;
}

cg_status cg_march(const cg_shape* shape, const float* origins, const float* dirs, uint64_t n,
                   uint32_t max_steps, float epsilon, float* hits, uint8_t* hit, void* stream) {
    CG_TRY(check_shape(shape));
    if (n && (!origins || !dirs || !hits || !hit)) {
        set_error("NULL buffer");
        return CG_EINVAL;
    }
    return launch_march(make_shape_dev(*shape), origins, dirs, n, max_steps, epsilon, hits, hit,
                        (cudaStream_t)stream);
}

}  // extern "C"
