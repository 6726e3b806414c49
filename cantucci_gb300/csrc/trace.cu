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

// Sum over hit pixels of g[i] * dt_i/dtheta.
__global__ void __launch_bounds__(128) k_trace_backward(ShapeDev s, CameraDev c, Dm3 dm,
                                                        const float* __restrict__ depth,
                                                        const float* __restrict__ g,
                                                        float* __restrict__ params) {
    const uint32_t n = c.width * c.height;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float t = depth[i], gi = g[i];
        if (!(t > 0.0f) || gi == 0.0f) continue;
        float d[3];
        pixel_ray(c, i, d);
        float o[8];
        polar_de_grad(s, dm.m, c.eye[0] + t * d[0], c.eye[1] + t * d[1], c.eye[2] + t * d[2], o);
        const float dn = o[1] * d[0] + o[2] * d[1] + o[3] * d[2];
        if (!(fabsf(dn) > 1e-6f)) continue;  // grazing ray: no stable depth derivative
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float v = -gi * o[4 + k] / dn;
            if (v == v && fabsf(v) < 1e30f) acc[k] += v;
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float v = acc[k];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, off);
        if ((threadIdx.x & 31) == 0 && v != 0.0f) atomicAdd(&params[k], v);
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
                         float eps_scale, float* depth, void* stream) {
    if (!shape || !depth) {
        set_error("NULL argument");
        return CG_EINVAL;
    }
    CG_TRY(check_camera(camera));
    const ShapeDev s = make_shape_dev(*shape);
    const CameraDev c = make_camera(*camera);
    const uint64_t n = (uint64_t)c.width * c.height;
    const unsigned G = grid_for(n, 128, 16);
    cudaStream_t st = (cudaStream_t)stream;
    switch (mode_of(s, CG_NUMERICS_EXACT)) {
    case MODE_P8: k_trace<MODE_P8><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
    case MODE_INT: k_trace<MODE_INT><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
    case MODE_POLAR: k_trace<MODE_POLAR><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
    default: k_trace<MODE_SPHERE><<<G, 128, 0, st>>>(s, c, max_steps, eps_scale, depth); break;
    }
    CG_CHECK_LAUNCH("k_trace");
    return CG_OK;
}

cg_status cg_trace_backward(const cg_shape* shape, const cg_camera* camera, const float* depth,
                            const float* grad_depth, float* grad_params, void* stream) {
    if (!shape || shape->kind != CG_SHAPE_MANDELBULB_POLAR || !depth || !grad_depth ||
        !grad_params) {
        set_error("cg_trace_backward needs the polar shape and device buffers");
        return CG_EINVAL;
    }
    CG_TRY(check_camera(camera));
    const ShapeDev s = make_shape_dev(*shape);
    const CameraDev c = make_camera(*camera);
    const Dm3 dm = rotation_derivatives(*shape);
    cudaStream_t st = (cudaStream_t)stream;
    CG_CUDA(cudaMemsetAsync(grad_params, 0, 4 * sizeof(float), st));
    const uint64_t n = (uint64_t)c.width * c.height;
    k_trace_backward<<<grid_for(n, 128, 16), 128, 0, st>>>(s, c, dm, depth, grad_depth,
                                                            grad_params);
    CG_CHECK_LAUNCH("k_trace_backward");
    return CG_OK;
}

}  // extern "C"
