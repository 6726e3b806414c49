// adjoint.cu -- point kernels of the estimator's gradient (the adjoint in
// adjoint.cuh and its forward-mode twin), its batch vector-Jacobian product
// (the autograd backward), and the six-evaluation central-difference
// gradient they replace.
#include <cmath>
#include <cstring>

#include "adjoint.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "point_io.cuh"
#include "qef.cuh"

namespace cg {

// One point's 8 outputs: two 16-byte stores when `out` is 16-byte aligned.
__device__ __forceinline__ void store8(float* __restrict__ out, uint64_t i, const float (&o)[8]) {
    float* dst = out + 8 * i;
    if ((((uintptr_t)out) & 15u) == 0) {
        reinterpret_cast<float4*>(dst)[0] = make_float4(o[0], o[1], o[2], o[3]);
        reinterpret_cast<float4*>(dst)[1] = make_float4(o[4], o[5], o[6], o[7]);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) dst[k] = o[k];
    }
}

// The reverse-mode gradient of each point; the tape is the dynamic shared
// memory (adj_tape_bytes(max_iters, CK, blockDim.x) bytes).
template <int CK, bool FASTREC>
__global__ void __launch_bounds__(128) k_de_grad(ShapeDev s, Dm3 dm, const float* __restrict__ pts,
                                                 uint64_t n, float* __restrict__ out) {
    extern __shared__ __align__(16) float4 adj_smem[];
    __shared__ __align__(16) float stage[4][96];
    const AdjTape tape = adj_tape(adj_smem, s.max_iters, CK);
    const WarpWalk w = warp_walk();
    for (uint64_t base = w.first; base < n; base += w.stride) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (!load_point_warp(pts, n, base, stage[threadIdx.x >> 5], x, y, z)) continue;
        float o[8];
        polar_de_grad<CK, FASTREC>(s, dm.m, x, y, z, tape, o);
        store8(out, base + (threadIdx.x & 31), o);
    }
}

template <int T, bool FAST>
__global__ void __launch_bounds__(128) k_de_grad_tangent(ShapeDev s, Dm3 dm,
                                                         const float* __restrict__ pts, uint64_t n,
                                                         float* __restrict__ out) {
    __shared__ __align__(16) float stage[4][96];
    const WarpWalk w = warp_walk();
    for (uint64_t base = w.first; base < n; base += w.stride) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (!load_point_warp(pts, n, base, stage[threadIdx.x >> 5], x, y, z)) continue;
        float o[8];
        polar_de_tangent<T, true, FAST>(s, dm.m, x, y, z, o);
        store8(out, base + (threadIdx.x & 31), o);
    }
}

// DE and dDE/dp of any shape (shape_gradient), one 16-byte store per point
// when `out` is 16-byte aligned.  The DE is the estimator's, bit for bit
// (for integer powers other than 8 one more estimator call gives it).
template <int M>
__global__ void __launch_bounds__(128) k_de_spatial_grad(ShapeDev s, const float* __restrict__ pts,
                                                         uint64_t n, float* __restrict__ out) {
    __shared__ __align__(16) float stage[4][96];
    const WarpWalk w = warp_walk();
    const bool vec = (((uintptr_t)out) & 15u) == 0;
    for (uint64_t base = w.first; base < n; base += w.stride) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (!load_point_warp(pts, n, base, stage[threadIdx.x >> 5], x, y, z)) continue;
        float g[4];
        shape_gradient<M>(s, x, y, z, g);
        if constexpr (M == MODE_INT) g[0] = eval<M>(s, x, y, z);  // the estimator's bits
        float* dst = out + 4 * (base + (threadIdx.x & 31));
        if (vec) {
            *reinterpret_cast<float4*>(dst) = make_float4(g[0], g[1], g[2], g[3]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) dst[k] = g[k];
        }
    }
}

// Vector-Jacobian product of a batch: g[i] * dDE/dp into grad_points (n x 3)
// and, per warp, the sum over its points of g[i] * dDE/d(power, euler) into
// partial[4 w .. 4 w + 3] (added up by k_sum_partials4 in a fixed order, so
// the result does not depend on scheduling).
__global__ void __launch_bounds__(128) k_de_vjp(ShapeDev s, Dm3 dm, const float* __restrict__ pts,
                                                const float* __restrict__ g, uint64_t n,
                                                float* __restrict__ gp, float* __restrict__ params) {
    extern __shared__ __align__(16) float4 adj_smem[];
    const AdjTape tape = adj_tape(adj_smem, s.max_iters, ADJ_CK);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float o[8];
        polar_de_grad<ADJ_CK>(s, dm.m, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], tape, o);
        const float gi = g[i];
        if (gp) {
            gp[3 * i] = gi * o[1];
            gp[3 * i + 1] = gi * o[2];
            gp[3 * i + 2] = gi * o[3];
        }
        if (gi != 0.0f) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float v = gi * o[4 + k];
                if (v == v) acc[k] += v;  // skip NaN (degenerate points)
            }
        }
    }
    if (params) {
        const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float v = acc[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
            if ((threadIdx.x & 31) == 0) params[4 * w + k] = v;
        }
    }
}

// params[k] += the sum over warps w < nwarps of partial[4 w + k], in a fixed
// order (one block: strided sequential sums of one 16-byte load per warp,
// then a fixed tree).  `partial` is 16-byte aligned.
__global__ void __launch_bounds__(256) k_sum_partials4(const float* __restrict__ partial,
                                                       uint32_t nwarps, float* __restrict__ params) {
    __shared__ float sh[4][256];
    const float4* p4 = reinterpret_cast<const float4*>(partial);
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (uint32_t w = threadIdx.x; w < nwarps; w += 256) {
        const float4 q = p4[w];
        v.x += q.x;
        v.y += q.y;
        v.z += q.z;
        v.w += q.w;
    }
    sh[0][threadIdx.x] = v.x;
    sh[1][threadIdx.x] = v.y;
    sh[2][threadIdx.x] = v.z;
    sh[3][threadIdx.x] = v.w;
    __syncthreads();
    for (uint32_t half = 128; half > 0; half >>= 1) {
        if (threadIdx.x < half)
#pragma unroll
            for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + half];
        __syncthreads();
    }
    if (threadIdx.x < 4) params[threadIdx.x] += sh[threadIdx.x][0];
}

// The calling thread's partials buffer on the current device, grown as
// needed and reused across calls.  A call waits on `st` (not on the host)
// for the previous call's use of the buffer, whatever its stream, and
// release_partials() marks the end of its own use.  While `st` is being
// captured into a graph, a stream-ordered allocation takes its place (it
// becomes a node of the graph; an event from outside the capture could
// not be waited on).
namespace {
struct PartialBuf {
    int device = -1;
    float* p = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    ~PartialBuf() {
        if (p) cudaFree(p);  // errors at process exit are of no consequence
        if (done) cudaEventDestroy(done);
    }
};
thread_local PartialBuf t_partials[16];
}  // namespace

static bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

cg_status acquire_partials(size_t floats, cudaStream_t st, float** out) {
    if (capturing(st)) {
        CG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(out), floats * sizeof(float), st));
        return CG_OK;
    }
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 16) {
        set_error("device ordinal %d out of range", dev);
        return CG_EINVAL;
    }
    PartialBuf& b = t_partials[dev];
    if (!b.done) CG_CUDA(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming));
    else CG_CUDA(cudaStreamWaitEvent(st, b.done, 0));
    if (b.cap < floats) {
        CG_CUDA(cudaEventSynchronize(b.done));  // the old buffer is idle before it goes
        if (b.p) CG_CUDA(cudaFree(b.p));
        b.p = nullptr;
        b.cap = 0;
        CG_CUDA(cudaMalloc(&b.p, floats * sizeof(float)));
        b.cap = floats;
    }
    *out = b.p;
    return CG_OK;
}

cg_status release_partials(float* partial, cudaStream_t st) {
    if (capturing(st)) {
        CG_CUDA(cudaFreeAsync(partial, st));
        return CG_OK;
    }
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    CG_CUDA(cudaEventRecord(t_partials[dev].done, st));
    return CG_OK;
}

cg_status launch_sum_partials4(const float* partial, uint32_t nwarps, float* params,
                               cudaStream_t st) {
    k_sum_partials4<<<1, 256, 0, st>>>(partial, nwarps, params);
    CG_CHECK_LAUNCH("k_sum_partials4");
    return CG_OK;
}

// Central-difference gradient with six estimator evaluations per point
// (the normal of src/mesh/buffer.rs:256-266 with step h, divided by 2h).
template <int M>
__global__ void __launch_bounds__(128) k_fd_grad(ShapeDev s, const float* __restrict__ pts,
                                                 uint64_t n, float h, float* __restrict__ out) {
    __shared__ __align__(16) float stage[4][96];
    const WarpWalk w = warp_walk();
    for (uint64_t base = w.first; base < n; base += w.stride) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (!load_point_warp(pts, n, base, stage[threadIdx.x >> 5], x, y, z)) continue;
        const uint64_t i = base + (threadIdx.x & 31);
        float g[3];
#pragma unroll 1
        for (int a = 0; a < 3; ++a) {
            const float hx = a == 0 ? h : 0.0f, hy = a == 1 ? h : 0.0f, hz = a == 2 ? h : 0.0f;
            const float dp = eval<M>(s, x + hx, y + hy, z + hz);
            const float dm = eval<M>(s, x - hx, y - hy, z - hz);
            g[a] = (dp - dm) / (2.0f * h);
        }
        out[3 * i] = g[0];
        out[3 * i + 1] = g[1];
        out[3 * i + 2] = g[2];
    }
}

Dm3 rotation_derivatives(const cg_shape& c) {
    Dm3 gs;
    const double a = c.rot[0], b = c.rot[1], g = c.rot[2];
    const double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cc = cos(g), sc = sin(g);
    const double d0[9] = {0, cc * sb * ca + sc * sa, -cc * sb * sa + sc * ca,
                          0, sc * sb * ca - cc * sa, -sc * sb * sa - cc * ca,
                          0, cb * ca,                -cb * sa};
    const double d1[9] = {-cc * sb, cc * cb * sa, cc * cb * ca,
                          -sc * sb, sc * cb * sa, sc * cb * ca,
                          -cb,      -sb * sa,     -sb * ca};
    const double d2[9] = {-sc * cb, -sc * sb * sa - cc * ca, -sc * sb * ca + cc * sa,
                          cc * cb,  cc * sb * sa - sc * ca,  cc * sb * ca + sc * sa,
                          0,        0,                       0};
    for (int i = 0; i < 9; ++i) {
        gs.m[i] = (float)d0[i];
        gs.m[9 + i] = (float)d1[i];
        gs.m[18 + i] = (float)d2[i];
    }
    return gs;
}

static cg_status check_grad_shape(const cg_shape* shape) {
    if (!shape || shape->kind != CG_SHAPE_MANDELBULB_POLAR) {
        set_error("the adjoint is defined on the real-power polar Mandelbulb (kind 2)");
        return CG_EINVAL;
    }
    if (shape->max_iters < 1 || shape->max_iters > ADJ_MAX_ITERS) {
        set_error("adjoint supports 1 <= max_iters <= %d", ADJ_MAX_ITERS);
        return CG_EINVAL;
    }
    return CG_OK;
}

// "adjoint_ck": the checkpoint interval of cg_de_grad (5 default, 4 or 8);
// every interval gives the same outputs.  "adjoint_recompute": 0 (default)
// recomputes segments with the exact arithmetic, 1 with the fast polar
// arithmetic (from exact checkpoints; the DE column is exact either way).
static int g_adjoint_ck = ADJ_CK;
static int g_adjoint_fastrec = 0;

int set_adjoint_option(const char* name, int64_t v) {
    if (std::strcmp(name, "adjoint_ck") == 0) {
        if (v != 4 && v != 5 && v != 8) return 0;
        g_adjoint_ck = (int)v;
        return 1;
    }
    if (std::strcmp(name, "adjoint_recompute") == 0) {
        if (v != 0 && v != 1) return 0;
        g_adjoint_fastrec = (int)v;
        return 1;
    }
    return -1;
}

template <int CK, bool FR>
static cg_status launch_de_grad(const ShapeDev& sd, const Dm3& dm, uint32_t max_iters,
                                const float* points, uint64_t n, float* out, cudaStream_t st) {
    unsigned G = 0;
    size_t smem = 0;
    CG_TRY(adj_launch_shape(k_de_grad<CK, FR>, max_iters, CK, n, &G, &smem));
    k_de_grad<CK, FR><<<G, 128, smem, st>>>(sd, dm, points, n, out);
    CG_CHECK_LAUNCH("k_de_grad");
    return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" {

cg_status cg_de_grad(const cg_shape* shape, const float* points, uint64_t n, float* out,
                     void* stream) {
    CG_TRY(check_grad_shape(shape));
    if (n && (!points || !out)) {
        set_error("NULL buffer");
        return CG_EINVAL;
    }
    if (!n) return CG_OK;
    const ShapeDev sd = make_shape_dev(*shape);
    const Dm3 dm = rotation_derivatives(*shape);
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t N = shape->max_iters;
    const bool fr = g_adjoint_fastrec != 0;
    switch (g_adjoint_ck) {
    case 4:
        return fr ? launch_de_grad<4, true>(sd, dm, N, points, n, out, st)
                  : launch_de_grad<4, false>(sd, dm, N, points, n, out, st);
    case 8:
        return fr ? launch_de_grad<8, true>(sd, dm, N, points, n, out, st)
                  : launch_de_grad<8, false>(sd, dm, N, points, n, out, st);
    default:
        return fr ? launch_de_grad<ADJ_CK, true>(sd, dm, N, points, n, out, st)
                  : launch_de_grad<ADJ_CK, false>(sd, dm, N, points, n, out, st);
    }
}

cg_status cg_de_grad_tangent(const cg_shape* shape, const float* points, uint64_t n,
                             uint32_t flags, float* out, void* stream) {
    if (!shape || shape->kind != CG_SHAPE_MANDELBULB_POLAR || shape->max_iters < 1) {
        set_error("the gradient is defined on the real-power polar Mandelbulb (kind 2)");
        return CG_EINVAL;
    }
    if (n && (!points || !out)) {
        set_error("NULL buffer");
        return CG_EINVAL;
    }
    if (!n) return CG_OK;
    const unsigned G = grid_for(n, 128, 16);
    cudaStream_t st = (cudaStream_t)stream;
    if (flags & ~3u) {
        set_error("cg_de_grad_tangent flags: CG_GRAD_POWER | CG_GRAD_FAST");
        return CG_EINVAL;
    }
    const ShapeDev sd = make_shape_dev(*shape);
    const Dm3 dm = rotation_derivatives(*shape);
    switch (flags) {
    case 0: k_de_grad_tangent<3, false><<<G, 128, 0, st>>>(sd, dm, points, n, out); break;
    case CG_GRAD_POWER: k_de_grad_tangent<4, false><<<G, 128, 0, st>>>(sd, dm, points, n, out); break;
    case CG_GRAD_FAST: k_de_grad_tangent<3, true><<<G, 128, 0, st>>>(sd, dm, points, n, out); break;
    default: k_de_grad_tangent<4, true><<<G, 128, 0, st>>>(sd, dm, points, n, out); break;
    }
    CG_CHECK_LAUNCH("k_de_grad_tangent");
    return CG_OK;
}

cg_status cg_de_spatial_grad(const cg_shape* shape, const float* points, uint64_t n, float* out,
                             void* stream) {
    CG_TRY(check_shape(shape));
    if (n && (!points || !out)) {
        set_error("NULL buffer");
        return CG_EINVAL;
    }
    if (!n) return CG_OK;
    const ShapeDev sd = make_shape_dev(*shape);
    const unsigned G = grid_for(n, 128, 16);
    cudaStream_t st = (cudaStream_t)stream;
    switch (mode_of(sd, CG_NUMERICS_EXACT)) {
    case MODE_P8: k_de_spatial_grad<MODE_P8><<<G, 128, 0, st>>>(sd, points, n, out); break;
    case MODE_INT: k_de_spatial_grad<MODE_INT><<<G, 128, 0, st>>>(sd, points, n, out); break;
    case MODE_POLAR: k_de_spatial_grad<MODE_POLAR><<<G, 128, 0, st>>>(sd, points, n, out); break;
    default: k_de_spatial_grad<MODE_SPHERE><<<G, 128, 0, st>>>(sd, points, n, out); break;
    }
    CG_CHECK_LAUNCH("k_de_spatial_grad");
    return CG_OK;
}

cg_status cg_de_backward(const cg_shape* shape, const float* points, const float* grad_out,
                         uint64_t n, float* grad_points, float* grad_params, void* stream) {
    CG_TRY(check_grad_shape(shape));
    if (n && (!points || !grad_out)) {
        set_error("NULL buffer");
        return CG_EINVAL;
    }
    cudaStream_t st = (cudaStream_t)stream;
    if (grad_params) CG_CUDA(cudaMemsetAsync(grad_params, 0, 4 * sizeof(float), st));
    if (!n) return CG_OK;
    unsigned G = 0;
    size_t smem = 0;
    CG_TRY(adj_launch_shape(k_de_vjp, shape->max_iters, ADJ_CK, n, &G, &smem));
    const uint32_t nwarps = G * 4;
    float* partial = nullptr;
    if (grad_params) CG_TRY(acquire_partials((size_t)nwarps * 4, st, &partial));
    k_de_vjp<<<G, 128, smem, st>>>(make_shape_dev(*shape), rotation_derivatives(*shape), points,
                                   grad_out, n, grad_points, partial);
    cg_status rs = cuda_status(cudaGetLastError(), "k_de_vjp", __FILE__, __LINE__);
    if (rs == CG_OK && partial) rs = launch_sum_partials4(partial, nwarps, grad_params, st);
    if (partial) {
        const cg_status rr = release_partials(partial, st);
        if (rs == CG_OK) rs = rr;
    }
    return rs;
}

cg_status cg_fd_grad(const cg_shape* shape, const float* points, uint64_t n, float h, float* out,
                     void* stream) {
    if (!shape || (n && (!points || !out)) || !(h > 0.0f)) {
        set_error("bad arguments to cg_fd_grad");
        return CG_EINVAL;
    }
    if (!n) return CG_OK;
    const ShapeDev s = make_shape_dev(*shape);
    const unsigned G = grid_for(n, 128, 16);
    cudaStream_t st = (cudaStream_t)stream;
    switch (mode_of(s, CG_NUMERICS_EXACT)) {
    case MODE_P8: k_fd_grad<MODE_P8><<<G, 128, 0, st>>>(s, points, n, h, out); break;
    case MODE_INT: k_fd_grad<MODE_INT><<<G, 128, 0, st>>>(s, points, n, h, out); break;
    case MODE_POLAR: k_fd_grad<MODE_POLAR><<<G, 128, 0, st>>>(s, points, n, h, out); break;
    default: k_fd_grad<MODE_SPHERE><<<G, 128, 0, st>>>(s, points, n, h, out); break;
    }
    CG_CHECK_LAUNCH("k_fd_grad");
    return CG_OK;
}

}  // extern "C"
