// trace.cu -- sphere tracing a depth map and its implicit-surface gradient.
//
// The reference's only ray march is ShapeMesh::get_focii
// (src/mesh/mod.rs:229-241: pos += dir * DE, hit when DE < eps); cg_march
// restates it.  Here the same march runs per pixel of a pinhole camera, with
// the hit threshold scaled by the pixel footprint at the ray distance t
// (eps_scale * t * pixel_angle), up to max_steps steps, and returns the depth
// t of every pixel (-1 for a miss).
//
// Backward: at a hit x = o + t d the surface satisfies DE(x; theta) = 0, so
// dt/dtheta = -(dDE/dtheta) / (grad_x DE . d).  The adjoint kernel gives
// both gradients at x; the kernel sums dL/dt * dt/dtheta over pixels for
// theta = (power, three Euler angles).
#include <cmath>
#include <cstring>

#include "adjoint.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace cg {

struct CameraDev {
    float eye[3], right[3], up[3], fwd[3];
    float tan_half, aspect;
    uint32_t width, height;
};

__device__ __forceinline__ void pixel_ray(const CameraDev& c, uint32_t i, float d[3]) {
    const uint32_t px = i % c.width, py = i / c.width;
    const float u = ((px + 0.5f) / c.width * 2.0f - 1.0f) * c.tan_half * c.aspect;
    const float v = (1.0f - (py + 0.5f) / c.height * 2.0f) * c.tan_half;
    float x = c.fwd[0] + u * c.right[0] + v * c.up[0];
    float y = c.fwd[1] + u * c.right[1] + v * c.up[1];
    float z = c.fwd[2] + u * c.right[2] + v * c.up[2];
    const float inv = rsqrtf(x * x + y * y + z * z);
    d[0] = x * inv;
    d[1] = y * inv;
    d[2] = z * inv;
}

template <int M>
__global__ void __launch_bounds__(128) k_trace(ShapeDev s, CameraDev c, uint32_t max_steps,
                                               float eps_scale, float* __restrict__ depth) {
    const uint32_t n = c.width * c.height;
    const float pix = 2.0f * c.tan_half / c.height;  // radians per pixel
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float d[3];
        pixel_ray(c, i, d);
        float t = 0.0f, out = -1.0f;
        for (uint32_t k = 0; k < max_steps; ++k) {
            const float x = c.eye[0] + t * d[0], y = c.eye[1] + t * d[1], z = c.eye[2] + t * d[2];
            const float de = eval<M>(s, x, y, z);
            if (!(de == de)) break;  // NaN: no surface information
            if (de < eps_scale * fmaxf(t, 1e-3f) * pix) {
                out = t;
                break;
            }
            t += de;
            if (t > 10.0f) break;
        }
        depth[i] = out;
    }
}

// The polar estimator one loop iteration at a time (the same operations as
// polar_de, or polar_de_fast with FAST), so that a lane can start a new
// estimate while its warp neighbours are still iterating theirs.
template <bool FAST>
struct PolarIter {
    float qx, qy, qz;  // R^T p
    StepState st;      // z, dr
    float r;
    uint32_t it;

    __device__ __forceinline__ void start(const ShapeDev& s, float px, float py, float pz) {
        rotate_point<FAST>(s, px, py, pz, qx, qy, qz);
        st = {qx, qy, qz, 1.0f};
        r = 0.0f;
        it = 0;
    }
    // One iteration; true when the estimate is complete (escape, or the
    // last iteration ran: r is then the stale |z| of that iteration).
    __device__ __forceinline__ bool advance(const ShapeDev& s) {
        float ri;
        const bool go = FAST ? polar_step_fast(s.power_f, s.bailout, qx, qy, qz, st.x, st.y,
                                               st.z, st.dr, ri)
                             : polar_step(s, qx, qy, qz, st, ri);
        r = ri;
        if (!go) return true;
        return ++it >= s.max_iters;
    }
    __device__ __forceinline__ float value() const {
        if (FAST) return x86_nan(__fdividef(0.5f * __logf(r) * r, st.dr));
        const float ln_r = __fmul_rn(logf(r), r);
        return x86_nan(__fdiv_rn(__fmul_rn(0.5f, ln_r), st.dr));
    }
};

// The same march with a work queue: persistent warps, and a lane whose ray
// is finished takes the next pixel at once (one atomic per warp and refill),
// so a warp no longer waits for its longest ray.  For the polar form the
// lanes advance one estimator iteration per loop trip, so a lane also does
// not wait for the slowest estimate of its warp.  Same depths as k_trace.
template <int M>
__global__ void __launch_bounds__(128) k_trace_queue(ShapeDev s, CameraDev c, uint32_t max_steps,
                                                     float eps_scale, float* __restrict__ depth,
                                                     uint32_t* __restrict__ next) {
    const uint32_t n = c.width * c.height;
    const float pix = 2.0f * c.tan_half / c.height;
    const uint32_t lane = threadIdx.x & 31;
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    uint32_t i = kNone, k = 0;
    bool done = false;
    float d[3] = {0.0f, 0.0f, 0.0f}, t = 0.0f;
    constexpr bool kIter = M == MODE_POLAR || M == MODE_POLAR_FAST;
    PolarIter<M == MODE_POLAR_FAST> pe;
    for (;;) {
        const bool need = !done && i == kNone;
        const unsigned need_mask = __ballot_sync(0xFFFFFFFFu, need);
        if (need_mask) {
            const int leader = __ffs(need_mask) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(next, (uint32_t)__popc(need_mask));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (need) {
                const uint32_t idx = base + __popc(need_mask & ((1u << lane) - 1u));
                if (idx >= n) {
                    done = true;
                } else if (max_steps == 0) {
                    depth[idx] = -1.0f;
                } else {
                    i = idx;
                    pixel_ray(c, i, d);
                    t = 0.0f;
                    k = 0;
                    if (kIter) pe.start(s, c.eye[0], c.eye[1], c.eye[2]);
                }
            }
        }
        if (__all_sync(0xFFFFFFFFu, done)) break;
        if (done || i == kNone) continue;
        float de;
        if (kIter) {
            if (!pe.advance(s)) continue;
            de = pe.value();
        } else {
            de = eval<M>(s, c.eye[0] + t * d[0], c.eye[1] + t * d[1], c.eye[2] + t * d[2]);
        }
        float out = -1.0f;
        bool fin = false;
        if (!(de == de)) {
            fin = true;  // NaN: no surface information
        } else if (de < eps_scale * fmaxf(t, 1e-3f) * pix) {
            out = t;
            fin = true;
        } else {
            t += de;
            fin = t > 10.0f || ++k >= max_steps;
        }
        if (fin) {
            depth[i] = out;
            i = kNone;
        } else if (kIter) {
            pe.start(s, c.eye[0] + t * d[0], c.eye[1] + t * d[1], c.eye[2] + t * d[2]);
        }
    }
}

// Sum over hit pixels of g[i] * dt_i/dtheta; with cap > 0, pixels whose
// |dt_i/dtheta_k| exceeds cap for some k are left out.
__global__ void __launch_bounds__(128) k_trace_backward(ShapeDev s, CameraDev c, Dm3 dm,
                                                        const float* __restrict__ depth,
                                                        const float* __restrict__ g, float cap,
                                                        float* __restrict__ params) {
    extern __shared__ __align__(16) float4 adj_smem[];
    const AdjTape tape = adj_tape(adj_smem, s.max_iters, ADJ_CK);
    const uint32_t n = c.width * c.height;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float t = depth[i], gi = g[i];
        if (!(t > 0.0f) || gi == 0.0f) continue;
        float d[3];
        pixel_ray(c, i, d);
        float o[8];
        polar_de_grad<ADJ_CK>(s, dm.m, c.eye[0] + t * d[0], c.eye[1] + t * d[1],
                              c.eye[2] + t * d[2], tape, o);
        const float dn = o[1] * d[0] + o[2] * d[1] + o[3] * d[2];
        if (!(fabsf(dn) > 1e-6f)) continue;  // grazing ray: no stable depth derivative
        float dt[4];
        bool keep = true;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            dt[k] = -o[4 + k] / dn;
            if (cap > 0.0f && !(fabsf(dt[k]) <= cap)) keep = false;
        }
        if (!keep) continue;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float v = gi * dt[k];
            if (v == v && fabsf(v) < 1e30f) acc[k] += v;
        }
    }
    // per-warp partial sums, added up in a fixed order by k_sum_partials4
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float v = acc[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, off);
        if ((threadIdx.x & 31) == 0) params[4 * w + k] = v;
    }
}

static CameraDev make_camera(const cg_camera& cam) {
    CameraDev c;
    for (int k = 0; k < 3; ++k) {
        c.eye[k] = cam.eye[k];
    }
    // forward = normalize(target - eye); right = normalize(forward x up); up' = right x forward
    double f[3] = {cam.target[0] - cam.eye[0], cam.target[1] - cam.eye[1],
                   cam.target[2] - cam.eye[2]};
    double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& v : f) v /= fl;
    double r[3] = {f[1] * cam.up[2] - f[2] * cam.up[1], f[2] * cam.up[0] - f[0] * cam.up[2],
                   f[0] * cam.up[1] - f[1] * cam.up[0]};
    double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (double& v : r) v /= rl;
    double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    for (int k = 0; k < 3; ++k) {
        c.fwd[k] = (float)f[k];
        c.right[k] = (float)r[k];
        c.up[k] = (float)u[k];
    }
    c.tan_half = (float)tan(0.5 * (double)cam.fov_y);
    c.width = cam.width;
    c.height = cam.height;
    c.aspect = (float)cam.width / (float)cam.height;
    return c;
}

// "trace_kernel": 1 (default) the work-queue march, 0 one pixel per thread.
static int g_trace_kernel = 1;

int set_trace_option(const char* name, int64_t v) {
    if (strcmp(name, "trace_kernel") || v < 0 || v > 1) return 0;
    g_trace_kernel = (int)v;
    return 1;
}

template <int M>
static void launch_trace_queue(const ShapeDev& s, const CameraDev& c, uint32_t max_steps,
                               float eps_scale, float* depth, uint32_t* next, cudaStream_t st) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_queue<M>, 128, 0) !=
            cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    k_trace_queue<M><<<(unsigned)(sm_count() * per_sm), 128, 0, st>>>(s, c, max_steps, eps_scale,
                                                                     depth, next);
}

static cg_status check_camera(const cg_camera* cam) {
    if (!cam || cam->width == 0 || cam->height == 0 || !(cam->fov_y > 0.0f && cam->fov_y < 3.1f) ||
        (uint64_t)cam->width * cam->height > (1ull << 31)) {
        set_error("bad camera");
        return CG_EINVAL;
    }
    return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" {

cg_status cg_trace_depth(const cg_shape* shape, const cg_camera* camera, uint32_t max_steps,
                         float eps_scale, uint32_t numerics, float* depth, void* stream) {
    if (!shape || !depth) {
        set_error("NULL argument");
        return CG_EINVAL;
    }
    CG_TRY(check_camera(camera));
    const ShapeDev s = make_shape_dev(*shape);
    const CameraDev c = make_camera(*camera);
    const uint64_t n = (uint64_t)c.width * c.height;
    cudaStream_t st = (cudaStream_t)stream;
    if (g_trace_kernel == 0) {
        const unsigned G = grid_for(n, 128, 16);
        switch (mode_of(s, numerics)) {
        case MODE_P8: k_trace<MODE_P8><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
        case MODE_INT: k_trace<MODE_INT><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
        case MODE_POLAR: k_trace<MODE_POLAR><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
        case MODE_POLAR_FAST:
            k_trace<MODE_POLAR_FAST><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth);
            break;
        case MODE_P8_FAST:
            k_trace<MODE_P8_FAST><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth);
            break;
        case MODE_INT_POLY:
            k_trace<MODE_INT_POLY><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth);
            break;
        default: k_trace<MODE_SPHERE><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
        }
        CG_CHECK_LAUNCH("k_trace");
        return CG_OK;
    }
    // the work queue's counter: the first word of the thread's scratch buffer
    float* scratch = nullptr;
    CG_TRY(acquire_partials(4, st, &scratch));
    uint32_t* next = reinterpret_cast<uint32_t*>(scratch);
    const cudaError_t ze = cudaMemsetAsync(next, 0, sizeof(uint32_t), st);
    if (ze != cudaSuccess) {  // give the scratch buffer back before reporting
        const cg_status rr = release_partials(scratch, st);
        CG_CUDA(ze);
        return rr;
    }
    switch (mode_of(s, numerics)) {
    case MODE_P8: launch_trace_queue<MODE_P8>(s, c, max_steps, eps_scale, depth, next, st); break;
    case MODE_INT: launch_trace_queue<MODE_INT>(s, c, max_steps, eps_scale, depth, next, st); break;
    case MODE_POLAR: launch_trace_queue<MODE_POLAR>(s, c, max_steps, eps_scale, depth, next, st); break;
    case MODE_POLAR_FAST:
        launch_trace_queue<MODE_POLAR_FAST>(s, c, max_steps, eps_scale, depth, next, st);
        break;
    case MODE_P8_FAST:
        launch_trace_queue<MODE_P8_FAST>(s, c, max_steps, eps_scale, depth, next, st);
        break;
    case MODE_INT_POLY:
        launch_trace_queue<MODE_INT_POLY>(s, c, max_steps, eps_scale, depth, next, st);
        break;
    default: launch_trace_queue<MODE_SPHERE>(s, c, max_steps, eps_scale, depth, next, st); break;
    }
    const cudaError_t le = cudaGetLastError();
    CG_TRY(release_partials(scratch, st));
    CG_CUDA(le);
    return CG_OK;
}

cg_status cg_trace_backward_capped(const cg_shape* shape, const cg_camera* camera,
                                   const float* depth, const float* grad_depth, float cap,
                                   float* grad_params, void* stream);

cg_status cg_trace_backward(const cg_shape* shape, const cg_camera* camera, const float* depth,
                            const float* grad_depth, float* grad_params, void* stream) {
    return cg_trace_backward_capped(shape, camera, depth, grad_depth, 0.0f, grad_params, stream);
}

cg_status cg_trace_backward_capped(const cg_shape* shape, const cg_camera* camera,
                                   const float* depth, const float* grad_depth, float cap,
                                   float* grad_params, void* stream) {
    if (!shape || shape->kind != CG_SHAPE_MANDELBULB_POLAR || !depth || !grad_depth ||
        !grad_params) {
        set_error("cg_trace_backward needs the polar shape and device buffers");
        return CG_EINVAL;
    }
    if (shape->max_iters < 1 || shape->max_iters > ADJ_MAX_ITERS) {
        set_error("cg_trace_backward supports 1 <= max_iters <= %d", ADJ_MAX_ITERS);
        return CG_EINVAL;
    }
    if (!(cap >= 0.0f)) {
        set_error("cg_trace_backward_capped: cap must be >= 0 (0: no cap)");
        return CG_EINVAL;
    }
    CG_TRY(check_camera(camera));
    const ShapeDev s = make_shape_dev(*shape);
    const CameraDev c = make_camera(*camera);
    const Dm3 dm = rotation_derivatives(*shape);
    cudaStream_t st = (cudaStream_t)stream;
    CG_CUDA(cudaMemsetAsync(grad_params, 0, 4 * sizeof(float), st));
    const uint64_t n = (uint64_t)c.width * c.height;
    unsigned G = 0;
    size_t smem = 0;
    CG_TRY(adj_launch_shape(k_trace_backward, shape->max_iters, ADJ_CK, n, &G, &smem));
    const uint32_t nwarps = G * 4;
    float* partial = nullptr;
    CG_TRY(acquire_partials((size_t)nwarps * 4, st, &partial));
    k_trace_backward<<<G, 128, smem, st>>>(s, c, dm, depth, grad_depth, cap, partial);
    cg_status rs = cuda_status(cudaGetLastError(), "k_trace_backward", __FILE__, __LINE__);
    if (rs == CG_OK) rs = launch_sum_partials4(partial, nwarps, grad_params, st);
    const cg_status rr = release_partials(partial, st);
    return rs == CG_OK ? rr : rs;
}

}  // extern "C"
