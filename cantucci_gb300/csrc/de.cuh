// de.cuh -- device-side distance estimators.
//
// Exact numerics restate Mandelbulb::min_distance_from
// (src/shape/mandelbulb.rs:59-79) with one IEEE round-to-nearest operation per
// source operation, in source order: __fmul_rn/__fadd_rn/__fsub_rn are never
// contracted into FMA, and __fdiv_rn/__fsqrt_rn are correctly rounded, so the
// loop state (z, r, dr) is bit-identical to the reference's SSE f32 loop.
// Only the final ln (glibc logf vs CUDA logf) and, off the P=8 path, the
// trigonometric functions may differ in the last bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "cantucci_gpu.h"

namespace cg {

// Shape parameters in the form the kernels use (rotation matrix precomputed).
struct ShapeDev {
    int32_t kind;
    int32_t power;
    float power_f;
    uint32_t max_iters;
    float bailout;
    float m[9];        // row-major R; the DE is evaluated at R^T p
    float center[3];
    float radius;
};

__host__ ShapeDev make_shape_dev(const cg_shape& s);

// x86-64 SSE turns an invalid operation into the negative default NaN
// 0xFFC00000 and propagates NaN operands, so every NaN the reference's DE can
// return has its sign bit set (f32::is_sign_positive is false).  CUDA's
// canonical NaN is positive; outputs are mapped to the x86 pattern.
__device__ __forceinline__ float x86_nan(float v) {
    return (v != v) ? __uint_as_float(0xFFC00000u) : v;
}

struct Exact {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
};

// Vec3::magnitude with SSE4.1 (mandelbulb.rs:412-418): dpps sums the lane
// products as (x*x + y*y) + z*z.
template <class O>
__device__ __forceinline__ float magnitude(float x, float y, float z) {
    return O::sqrt(O::add(O::add(O::mul(x, x), O::mul(y, y)), O::mul(z, z)));
}

// Vec3::is_on_z_axis (mandelbulb.rs:421-426).
__device__ __forceinline__ bool on_z_axis(float x, float y) {
    return ((__float_as_uint(x) | __float_as_uint(y)) & 0x7FFFFFFFu) == 0u;
}

// f32::powi with a constant exponent: square-and-multiply, low bit first, as
// LLVM expands llvm.powi (x^7 = (x * x^2) * x^4).
template <class O>
__device__ __forceinline__ float powi(float x, int32_t n) {
    if (n == 0) return 1.0f;
    const bool neg = n < 0;
    uint32_t m = neg ? (uint32_t)(-n) : (uint32_t)n;
    float res = 0.0f, cur = x;
    bool have = false;
    for (;;) {
        if (m & 1u) {
            res = have ? O::mul(res, cur) : cur;
            have = true;
        }
        m >>= 1;
        if (!m) break;
        cur = O::mul(cur, cur);
    }
    return neg ? O::div(1.0f, res) : res;
}

// rotate_inner_p8_scalar (mandelbulb.rs:148-200), every operation in source order.
template <class O>
__device__ __forceinline__ void rotate_p8(float x, float y, float z, float& ox, float& oy,
                                          float& oz) {
    const float x2 = O::mul(x, x), x4 = O::mul(x2, x2), x6 = O::mul(x4, x2), x8 = O::mul(x4, x4);
    const float y2 = O::mul(y, y), y4 = O::mul(y2, y2), y6 = O::mul(y4, y2), y8 = O::mul(y4, y4);
    const float z2 = O::mul(z, z), z4 = O::mul(z2, z2), z6 = O::mul(z4, z2), z8 = O::mul(z4, z4);
    const float rxy2 = O::add(x2, y2);
    const float rxy4 = O::mul(rxy2, rxy2);
    const float rxy6 = O::mul(rxy2, rxy4);
    const float rxy8 = O::mul(rxy4, rxy4);
    // a = 1 + (z8 - 28 z6 rxy2 + 70 z4 rxy4 - 28 z2 rxy6) / rxy8
    const float num = O::sub(O::add(O::sub(z8, O::mul(O::mul(28.0f, z6), rxy2)),
                                    O::mul(O::mul(70.0f, z4), rxy4)),
                             O::mul(O::mul(28.0f, z2), rxy6));
    const float a = O::add(1.0f, O::div(num, rxy8));
    // a * (x8 - 28 x6 y2 + 70 x4 y4 - 28 x2 y6 - y8)
    const float X = O::sub(O::sub(O::add(O::sub(x8, O::mul(O::mul(28.0f, x6), y2)),
                                         O::mul(O::mul(70.0f, x4), y4)),
                                  O::mul(O::mul(28.0f, x2), y6)),
                           y8);
    ox = O::mul(a, X);
    // 8 a x y (x6 - 7 x4 y2 + 7 x2 y4 - y6)
    const float Y = O::sub(O::add(O::sub(x6, O::mul(O::mul(7.0f, x4), y2)),
                                  O::mul(O::mul(7.0f, x2), y4)),
                           y6);
    oy = O::mul(O::mul(O::mul(O::mul(8.0f, a), x), y), Y);
    // 8 z sqrt(rxy2) (z2 - rxy2) (z4 - 6 z2 rxy2 + rxy4)
    const float Z = O::add(O::sub(z4, O::mul(O::mul(6.0f, z2), rxy2)), rxy4);
    oz = O::mul(O::mul(O::mul(O::mul(8.0f, z), O::sqrt(rxy2)), O::sub(z2, rxy2)), Z);
}

// rotate_on_z_axis (mandelbulb.rs:114-126).
template <class O>
__device__ __noinline__ void rotate_axis(int32_t P, float x, float y, float z, float& ox,
                                         float& oy, float& oz) {
    const float old_radius = magnitude<O>(x, y, z);
    float theta = acosf(O::div(z, old_radius));
    const float new_radius = powi<O>(old_radius, P);
    theta = O::mul(theta, (float)P);
    ox = 0.0f;
    oy = 0.0f;
    oz = O::mul(new_radius, cosf(theta));
}

// rotate_inner_px_generic (mandelbulb.rs:128-146).
template <class O>
__device__ __forceinline__ void rotate_generic(int32_t P, float x, float y, float z, float& ox,
                                               float& oy, float& oz) {
    const float old_radius = magnitude<O>(x, y, z);
    float theta = acosf(O::div(z, old_radius));
    float phi = atan2f(y, x);
    const float new_radius = powi<O>(old_radius, P);
    theta = O::mul(theta, (float)P);
    phi = O::mul(phi, (float)P);
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    ox = O::mul(O::mul(st, cp), new_radius);
    oy = O::mul(O::mul(sp, st), new_radius);
    oz = O::mul(ct, new_radius);
}

struct MbState {
    float r, dr;
    uint32_t steps, escaped;
};

// Mandelbulb::min_distance_from (mandelbulb.rs:59-79) for power P (P8 = true
// selects the polynomial at compile time).  `r` is stale when the loop runs
// out: it is |z| at the start of the last iteration.
template <class O, bool P8>
__device__ __forceinline__ float mandelbulb_de(int32_t P, uint32_t max_iters, float bailout,
                                               float px, float py, float pz,
                                               MbState* st = nullptr) {
    float zx = px, zy = py, zz = pz;
    float dr = 1.0f;
    float r = 0.0f;
    const float Pf = (float)P;
    uint32_t steps = 0, esc = 0;
    for (uint32_t i = 0; i < max_iters; ++i) {
        r = magnitude<O>(zx, zy, zz);
        if (r > bailout) {
            esc = 1;
            break;
        }
        dr = O::add(O::mul(O::mul(powi<O>(r, P - 1), Pf), dr), 1.0f);
        float nx, ny, nz;
        if (on_z_axis(zx, zy)) {
            rotate_axis<O>(P, zx, zy, zz, nx, ny, nz);
        } else if (P8) {
            rotate_p8<O>(zx, zy, zz, nx, ny, nz);
        } else {
            rotate_generic<O>(P, zx, zy, zz, nx, ny, nz);
        }
        zx = O::add(nx, px);
        zy = O::add(ny, py);
        zz = O::add(nz, pz);
        ++steps;
    }
    if (st) {
        st->r = r;
        st->dr = dr;
        st->steps = steps;
        st->escaped = esc;
    }
    const float ln_r = O::mul(logf(r), r);
    return x86_nan(O::div(O::mul(0.5f, ln_r), dr));
}

// Polar form of src/shape/mandelbulb.frag:1-39 with a real power, evaluated
// at q = R^T p.  GLSL length() is taken as sqrt((x*x + y*y) + z*z).
__device__ __forceinline__ float polar_de(const ShapeDev& s, float px, float py, float pz) {
    const float qx = __fadd_rn(__fadd_rn(__fmul_rn(s.m[0], px), __fmul_rn(s.m[3], py)), __fmul_rn(s.m[6], pz));
    const float qy = __fadd_rn(__fadd_rn(__fmul_rn(s.m[1], px), __fmul_rn(s.m[4], py)), __fmul_rn(s.m[7], pz));
    const float qz = __fadd_rn(__fadd_rn(__fmul_rn(s.m[2], px), __fmul_rn(s.m[5], py)), __fmul_rn(s.m[8], pz));
    const float P = s.power_f;
    float zx = qx, zy = qy, zz = qz, dr = 1.0f, r = 0.0f;
    for (uint32_t i = 0; i < s.max_iters; ++i) {
        r = magnitude<Exact>(zx, zy, zz);
        if (r > s.bailout) break;
        float theta = acosf(__fdiv_rn(zz, r));
        float phi = atan2f(zy, zx);
        dr = __fadd_rn(__fmul_rn(__fmul_rn(powf(r, __fsub_rn(P, 1.0f)), P), dr), 1.0f);
        const float zr = powf(r, P);
        theta = __fmul_rn(theta, P);
        phi = __fmul_rn(phi, P);
        float st, ct, sp, cp;
        sincosf(theta, &st, &ct);
        sincosf(phi, &sp, &cp);
        zx = __fadd_rn(__fmul_rn(zr, __fmul_rn(st, cp)), qx);
        zy = __fadd_rn(__fmul_rn(zr, __fmul_rn(sp, st)), qy);
        zz = __fadd_rn(__fmul_rn(zr, ct), qz);
    }
    const float ln_r = __fmul_rn(logf(r), r);
    return x86_nan(__fdiv_rn(__fmul_rn(0.5f, ln_r), dr));
}

// Sphere::min_distance_from (src/shape/sphere.rs:33-35).
__device__ __forceinline__ float sphere_de(const ShapeDev& s, float x, float y, float z) {
    const float dx = __fsub_rn(s.center[0], x);
    const float dy = __fsub_rn(s.center[1], y);
    const float dz = __fsub_rn(s.center[2], z);
    return __fsub_rn(magnitude<Exact>(dx, dy, dz), s.radius);
}

// One exact DE evaluation for any shape kind.
__device__ __forceinline__ float shape_de(const ShapeDev& s, float x, float y, float z) {
    if (s.kind == CG_SHAPE_SPHERE) return sphere_de(s, x, y, z);
    if (s.kind == CG_SHAPE_MANDELBULB_POLAR) return polar_de(s, x, y, z);
    if (s.power == 8) return mandelbulb_de<Exact, true>(8, s.max_iters, s.bailout, x, y, z);
    return mandelbulb_de<Exact, false>(s.power, s.max_iters, s.bailout, x, y, z);
}

}  // namespace cg
