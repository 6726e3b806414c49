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
    int32_t rotated;   // 0 when all three Euler angles are 0: q = p exactly
};

__host__ ShapeDev make_shape_dev(const cg_shape& s);

// x86-64 SSE turns an invalid operation into the negative default NaN
// 0xFFC00000 and propagates NaN operands, so every NaN the reference's DE can
// return has its sign bit set (f32::is_sign_positive is false).  CUDA's
// canonical NaN is positive; outputs are mapped to the x86 pattern.
__device__ __forceinline__ float x86_nan(float v) {
    return (v != v) ? __uint_as_float(0xFFC00000u) : v;
}

// q = R^T p for the polar form, one rounding per operation, sums left to
// right (FMA = true: the contracted form of the fast paths).  Without a
// rotation q = p, as in src/shape/mandelbulb.frag, which applies none: signed
// zeros and non-finite coordinates pass unchanged.
template <bool FMA = false>
__device__ __forceinline__ void rotate_point(const ShapeDev& s, float px, float py, float pz,
                                             float& qx, float& qy, float& qz) {
    if (!s.rotated) {
        qx = px;
        qy = py;
        qz = pz;
    } else if (FMA) {
        qx = fmaf(s.m[0], px, fmaf(s.m[3], py, s.m[6] * pz));
        qy = fmaf(s.m[1], px, fmaf(s.m[4], py, s.m[7] * pz));
        qz = fmaf(s.m[2], px, fmaf(s.m[5], py, s.m[8] * pz));
    } else {
        qx = __fadd_rn(__fadd_rn(__fmul_rn(s.m[0], px), __fmul_rn(s.m[3], py)), __fmul_rn(s.m[6], pz));
        qy = __fadd_rn(__fadd_rn(__fmul_rn(s.m[1], px), __fmul_rn(s.m[4], py)), __fmul_rn(s.m[7], pz));
        qz = __fadd_rn(__fadd_rn(__fmul_rn(s.m[2], px), __fmul_rn(s.m[5], py)), __fmul_rn(s.m[8], pz));
    }
}

struct Exact {
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float sqrt(float a) { return __fsqrt_rn(a); }
};

// Plain float operations (the compiler may contract them).
struct Fast {
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
    static __device__ __forceinline__ float div(float a, float b) { return a / b; }
    static __device__ __forceinline__ float sqrt(float a) { return sqrtf(a); }
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

// rotate_on_z_axis (mandelbulb.rs:114-126): x' = y' = 0, and z' as returned.
// Out of line (the path is rare) and with no reference parameters, so the
// call needs no stack slots in the hot loop.
template <class O>
__device__ __noinline__ float rotate_axis_z(int32_t P, float x, float y, float z) {
    const float old_radius = magnitude<O>(x, y, z);
    float theta = acosf(O::div(z, old_radius));
    const float new_radius = powi<O>(old_radius, P);
    theta = O::mul(theta, (float)P);
    return O::mul(new_radius, cosf(theta));
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

// One iteration of Mandelbulb::min_distance_from's loop (mandelbulb.rs:
// 63-75): r = |z|; false if r > bailout (escape), else dr and z advance.
template <class O, bool P8>
__device__ __forceinline__ bool mandelbulb_step(int32_t P, float Pf, float bailout, float px,
                                                float py, float pz, float& zx, float& zy,
                                                float& zz, float& dr, float& r) {
    r = magnitude<O>(zx, zy, zz);
    if (r > bailout) return false;
    dr = O::add(O::mul(O::mul(powi<O>(r, P - 1), Pf), dr), 1.0f);
    float nx, ny, nz;
    if (on_z_axis(zx, zy)) {
        nx = 0.0f;
        ny = 0.0f;
        nz = rotate_axis_z<O>(P, zx, zy, zz);
    } else if (P8) {
        rotate_p8<O>(zx, zy, zz, nx, ny, nz);
    } else {
        rotate_generic<O>(P, zx, zy, zz, nx, ny, nz);
    }
    zx = O::add(nx, px);
    zy = O::add(ny, py);
    zz = O::add(nz, pz);
    return true;
}

// Mandelbulb::min_distance_from (mandelbulb.rs:59-79) for power P (P8 = true
// selects the polynomial at compile time).  `r` is stale when the loop runs
// out: it is |z| at the start of the last iteration.  FIXED > 0 is a
// compile-time max_iters: the loop is unrolled, which drops the trip-count
// test from every iteration (same operations, same bits).
template <class O, bool P8, int FIXED = 0, bool NAN_EXIT = false>
__device__ __forceinline__ float mandelbulb_de(int32_t P, uint32_t max_iters, float bailout,
                                               float px, float py, float pz,
                                               MbState* st = nullptr) {
    float zx = px, zy = py, zz = pz;
    float dr = 1.0f;
    float r = 0.0f;
    const float Pf = (float)P;
    uint32_t steps = 0, esc = 0;
    if constexpr (FIXED > 0) {
#pragma unroll
        for (int i = 0; i < FIXED; ++i) {
            if (!mandelbulb_step<O, P8>(P, Pf, bailout, px, py, pz, zx, zy, zz, dr, r)) {
                esc = 1;
                break;
            }
            ++steps;
            // NAN_EXIT: once |z| is NaN every later iterate is NaN (each
            // component of the next z takes a NaN operand), r stays NaN,
            // nothing escapes, and the distance is NaN whatever the
            // remaining steps do.  The origin gets there in its second step
            // (acos(0/0) on the z axis) and would otherwise run all its steps
            // through the division's and square root's special-case paths,
            // which sets the time of a small grid; stop there.  Only for
            // callers that want the distance alone (the loop state differs).
            if constexpr (NAN_EXIT)
                if (i == 1 && r != r) break;
        }
    } else {
        for (uint32_t i = 0; i < max_iters; ++i) {
            if (!mandelbulb_step<O, P8>(P, Pf, bailout, px, py, pz, zx, zy, zz, dr, r)) {
                esc = 1;
                break;
            }
            ++steps;
        }
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

// ---- two points per thread with packed IEEE instructions ----------------
//
// sm_100+ executes add/sub/mul/fma.rn.f32x2 on a pair of f32 lanes in one
// instruction, each lane rounded like the scalar .rn operation.  ptxas
// (CUDA 13.0, sm_103a) however fuses a packed multiply whose only use is a
// packed add or subtract into a single fused multiply-add -- one rounding
// instead of the reference's two -- even with .rn and --fmad=false; it
// leaves fma.rn.f32x2(q, -1, c) alone.  So every sum that has a single-use
// product p as an operand is written as c - q with q = -p formed exactly (a
// negated constant factor: round-to-nearest is symmetric in sign) and
// evaluated as fma(q, -1, c), which rounds exactly like c + p.  Products
// that feed several operations (x^2, y^2, z^2, x^6, z^4, rxy^4) keep plain
// adds.  Division and square root stay scalar (__fdiv_rn / __fsqrt_rn).
typedef unsigned long long u64;

struct X2 {
    static __device__ __forceinline__ u64 pk(float a, float b) {
        u64 r;
        asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
        return r;
    }
    static __device__ __forceinline__ void up(u64 v, float& a, float& b) {
        asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    }
    static __device__ __forceinline__ u64 splat(float c) { return pk(c, c); }
    static __device__ __forceinline__ u64 mul(u64 a, u64 b) {
        u64 d;
        asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
        return d;
    }
    static __device__ __forceinline__ u64 add(u64 a, u64 b) {
        u64 d;
        asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
        return d;
    }
    static __device__ __forceinline__ u64 sub(u64 a, u64 b) {
        u64 d;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
        return d;
    }
    // c - q, one rounding, for a q that is a single-use product.
    static __device__ __forceinline__ u64 rsub(u64 c, u64 q) {
        u64 d;
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(q), "l"(splat(-1.0f)), "l"(c));
        return d;
    }
    static __device__ __forceinline__ u64 div(u64 a, u64 b) {
        float a0, a1, b0, b1;
        up(a, a0, a1);
        up(b, b0, b1);
        return pk(__fdiv_rn(a0, b0), __fdiv_rn(a1, b1));
    }
    static __device__ __forceinline__ u64 sqrt(u64 a) {
        float a0, a1;
        up(a, a0, a1);
        return pk(__fsqrt_rn(a0), __fsqrt_rn(a1));
    }
};

// rotate_inner_p8_scalar (mandelbulb.rs:148-200) on two points at once,
// returning the NEGATED result (-x', -y', -z') so that the caller's "+ p"
// can be a fusion-proof subtraction.  x2 = x*x, y2 = y*y, z2 = z*z are
// passed in (they are also the magnitude's products); rxy2 = x2 + y2.
__device__ __forceinline__ void rotate_p8_x2_neg(u64 x, u64 y, u64 z, u64 x2, u64 y2, u64 z2,
                                                 u64 rxy2, u64& nox, u64& noy, u64& noz) {
    typedef X2 O;
    const u64 c28 = O::splat(28.0f), m70 = O::splat(-70.0f), c7 = O::splat(7.0f);
    const u64 m7 = O::splat(-7.0f), m8 = O::splat(-8.0f), c6 = O::splat(6.0f);
    const u64 x4 = O::mul(x2, x2), x6 = O::mul(x4, x2), x8 = O::mul(x4, x4);
    const u64 y4 = O::mul(y2, y2), y6 = O::mul(y4, y2), y8 = O::mul(y4, y4);
    const u64 z4 = O::mul(z2, z2), z6 = O::mul(z4, z2), z8 = O::mul(z4, z4);
    const u64 rxy4 = O::mul(rxy2, rxy2);
    const u64 rxy6 = O::mul(rxy2, rxy4);
    const u64 rxy8 = O::mul(rxy4, rxy4);
    // num = ((z8 - (28 z6) rxy2) + (70 z4) rxy4) - (28 z2) rxy6
    const u64 num = O::rsub(O::rsub(O::rsub(z8, O::mul(O::mul(c28, z6), rxy2)),
                                    O::mul(O::mul(m70, z4), rxy4)),
                            O::mul(O::mul(c28, z2), rxy6));
    const u64 q = O::div(num, rxy8);
    const u64 a = O::add(O::splat(1.0f), q);    // 1 + q
    const u64 na = O::sub(O::splat(-1.0f), q);  // -(1 + q), exactly
    // X = (((x8 - (28 x6) y2) + (70 x4) y4) - (28 x2) y6) - y8
    const u64 X = O::rsub(O::rsub(O::rsub(O::rsub(x8, O::mul(O::mul(c28, x6), y2)),
                                          O::mul(O::mul(m70, x4), y4)),
                                  O::mul(O::mul(c28, x2), y6)),
                          y8);
    nox = O::mul(na, X);
    // Y = ((x6 - (7 x4) y2) + (7 x2) y4) - y6
    const u64 Y = O::rsub(O::rsub(O::rsub(x6, O::mul(O::mul(c7, x4), y2)),
                                  O::mul(O::mul(m7, x2), y4)),
                          y6);
    noy = O::mul(O::mul(O::mul(O::mul(m8, a), x), y), Y);
    // Z = (z4 - (6 z2) rxy2) + rxy4
    const u64 Z = O::add(O::rsub(z4, O::mul(O::mul(c6, z2), rxy2)), rxy4);
    noz = O::mul(O::mul(O::mul(O::mul(m8, z), O::sqrt(rxy2)), O::sub(z2, rxy2)), Z);
}

// Mandelbulb<8>::min_distance_from for points A and B together.  A lane
// whose point has escaped (or is inactive) keeps iterating in lock-step with
// garbage that is never read; its r and dr were captured when it stopped.
__device__ __forceinline__ void mandelbulb_p8_x2(uint32_t max_iters, float bailout, bool liveA,
                                                 bool liveB, float pxA, float pyA, float pzA,
                                                 float pxB, float pyB, float pzB, float& dA,
                                                 float& dB) {
    typedef X2 O;
    const u64 px = O::pk(pxA, pxB), py = O::pk(pyA, pyB), pz = O::pk(pzA, pzB);
    const u64 c1 = O::splat(1.0f), m8 = O::splat(-8.0f);
    u64 zx = px, zy = py, zz = pz, dr = c1;
    float rA = 0.0f, rB = 0.0f, drA = 1.0f, drB = 1.0f;
    bool aA = liveA, aB = liveB;
    for (uint32_t i = 0; i < max_iters; ++i) {
        const u64 x2 = O::mul(zx, zx), y2 = O::mul(zy, zy), z2 = O::mul(zz, zz);
        const u64 rxy2 = O::add(x2, y2);
        const u64 m2 = O::add(rxy2, z2);  // Vec3::magnitude: (x*x + y*y) + z*z
        float mA, mB, d0, d1;
        O::up(m2, mA, mB);
        O::up(dr, d0, d1);
        if (aA) {
            rA = __fsqrt_rn(mA);
            if (rA > bailout) {
                aA = false;
                drA = d0;
            }
        }
        if (aB) {
            rB = __fsqrt_rn(mB);
            if (rB > bailout) {
                aB = false;
                drB = d1;
            }
        }
        if (!(aA || aB)) break;
        const u64 r = O::pk(rA, rB);
        const u64 r2 = O::mul(r, r), r4 = O::mul(r2, r2);
        const u64 r7 = O::mul(O::mul(r, r2), r4);  // powi(r, 7): (r * r^2) * r^4
        dr = O::rsub(c1, O::mul(O::mul(r7, m8), dr));  // ((r^7 * 8) * dr) + 1
        u64 nx, ny, nz;
        rotate_p8_x2_neg(zx, zy, zz, x2, y2, z2, rxy2, nx, ny, nz);
        float xA, xB, yA, yB;
        O::up(zx, xA, xB);
        O::up(zy, yA, yB);
        if ((aA && on_z_axis(xA, yA)) || (aB && on_z_axis(xB, yB))) {
            float zA, zB, oxA, oxB, oyA, oyB, ozA, ozB;
            O::up(zz, zA, zB);
            O::up(nx, oxA, oxB);
            O::up(ny, oyA, oyB);
            O::up(nz, ozA, ozB);
            if (aA && on_z_axis(xA, yA)) {  // negated outputs: -(0), -(0), -z'
                oxA = -0.0f;
                oyA = -0.0f;
                ozA = -rotate_axis_z<Exact>(8, xA, yA, zA);
            }
            if (aB && on_z_axis(xB, yB)) {
                oxB = -0.0f;
                oyB = -0.0f;
                ozB = -rotate_axis_z<Exact>(8, xB, yB, zB);
            }
            nx = O::pk(oxA, oxB);
            ny = O::pk(oyA, oyB);
            nz = O::pk(ozA, ozB);
        }
        zx = O::rsub(px, nx);  // rotate(z) + p
        zy = O::rsub(py, ny);
        zz = O::rsub(pz, nz);
    }
    float d0, d1;
    O::up(dr, d0, d1);
    if (aA) drA = d0;
    if (aB) drB = d1;
    dA = x86_nan(__fdiv_rn(__fmul_rn(0.5f, __fmul_rn(logf(rA), rA)), drA));
    dB = x86_nan(__fdiv_rn(__fmul_rn(0.5f, __fmul_rn(logf(rB), rB)), drB));
}

// Polar form of src/shape/mandelbulb.frag:1-39 with a real power, evaluated
// at q = R^T p.  GLSL length() is taken as sqrt((x*x + y*y) + z*z).
__device__ __forceinline__ float polar_de(const ShapeDev& s, float px, float py, float pz) {
    float qx, qy, qz;
    rotate_point(s, px, py, pz, qx, qy, qz);
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

// FMA-contracted P=8 Mandelbulb (CG_NUMERICS_FAST).  Same polynomial as
// rotate_p8 but regrouped for fused multiply-adds and approximate division
// and square root; its loop state is not bit-identical to the reference.
__device__ __forceinline__ float fast_sqrt(float x) {
    return x > 0.0f ? x * rsqrtf(x) : 0.0f;
}

__device__ __forceinline__ bool p8_fast_step(float bailout, float px, float py, float pz,
                                             float& zx, float& zy, float& zz, float& dr,
                                             float& r) {
    const float r2 = fmaf(zx, zx, fmaf(zy, zy, zz * zz));
    r = fast_sqrt(r2);
    if (r > bailout) return false;
    const float rr2 = r * r, rr4 = rr2 * rr2;
    dr = fmaf(rr4 * rr2 * r * 8.0f, dr, 1.0f);
    const float x = zx, y = zy, z = zz;
    const float x2 = x * x, y2 = y * y, z2 = z * z;
    const float y4 = y2 * y2;
    const float rxy2 = x2 + y2;
    const float rxy4 = rxy2 * rxy2;
    // num = z8 - 28 z6 rxy2 + 70 z4 rxy4 - 28 z2 rxy6 (Horner in z2)
    const float num = fmaf(fmaf(fmaf(z2 - 28.0f * rxy2, z2, 70.0f * rxy4), z2,
                                -28.0f * rxy4 * rxy2), z2, 0.0f);
    const float a = 1.0f + __fdividef(num, rxy4 * rxy4);
    const float X = fmaf(fmaf(fmaf(x2 - 28.0f * y2, x2, 70.0f * y4), x2, -28.0f * y4 * y2),
                         x2, -y4 * y4);
    const float Y = fmaf(fmaf(x2 - 7.0f * y2, x2, 7.0f * y4), x2, -y4 * y2);
    const float Z = fmaf(z2 - 6.0f * rxy2, z2, rxy4);
    zx = fmaf(a, X, px);
    zy = fmaf(8.0f * a * x * y, Y, py);
    zz = fmaf(8.0f * z * fast_sqrt(rxy2) * (z2 - rxy2), Z, pz);
    return true;
}

// FIXED > 0: a compile-time max_iters, the loop unrolled.
template <int FIXED = 0>
__device__ __forceinline__ float mandelbulb_p8_fast(uint32_t max_iters, float bailout, float px,
                                                    float py, float pz) {
    float zx = px, zy = py, zz = pz, dr = 1.0f, r = 0.0f;
    if constexpr (FIXED > 0) {
#pragma unroll
        for (int i = 0; i < FIXED; ++i)
            if (!p8_fast_step(bailout, px, py, pz, zx, zy, zz, dr, r)) break;
    } else {
        for (uint32_t i = 0; i < max_iters; ++i)
            if (!p8_fast_step(bailout, px, py, pz, zx, zy, zz, dr, r)) break;
    }
    return x86_nan(__fdividef(0.5f * __logf(r) * r, dr));
}

// Integer power P >= 1 of the complex number (re, im), square-and-multiply.
__device__ __forceinline__ void cpow_int(float re, float im, int32_t P, float& ore, float& oim) {
    float rr = 1.0f, ri = 0.0f, br = re, bi = im;
    uint32_t m = (uint32_t)P;
    while (m) {
        if (m & 1u) {
            const float t = fmaf(rr, br, -ri * bi);
            ri = fmaf(rr, bi, ri * br);
            rr = t;
        }
        m >>= 1;
        if (m) {
            const float t = fmaf(br, br, -bi * bi);
            bi = 2.0f * br * bi;
            br = t;
        }
    }
    ore = rr;
    oim = ri;
}

// Trig-free form of rotate_inner_px_generic (mandelbulb.rs:128-146) for an
// integer power P (CG_NUMERICS_FAST): with theta = acos(z / r) and
// phi = atan2(y, x), the unit complex numbers a = (z + i rho) / r and
// b = (x + i y) / rho (rho = |(x, y)|) have arguments theta and phi, so
//   cos(P theta) + i sin(P theta) = a^P,   cos(P phi) + i sin(P phi) = b^P,
// and x' = r^P Im(a^P) Re(b^P), y' = r^P Im(a^P) Im(b^P), z' = r^P Re(a^P):
// two square-and-multiply complex powers instead of acos, atan2 and two
// sincos.  On the z axis (x = y = 0, rotate_on_z_axis) b is undefined and
// x' = y' = 0, z' = r^P Re(a^P) as before.  Not bit-faithful to the
// reference's libm path (which is not bit-reproducible itself).
__device__ __forceinline__ float mandelbulb_int_poly(int32_t P, uint32_t max_iters, float bailout,
                                                     float px, float py, float pz) {
    float zx = px, zy = py, zz = pz, dr = 1.0f, r = 0.0f;
    const float Pf = (float)P;
    for (uint32_t i = 0; i < max_iters; ++i) {
        const float r2 = fmaf(zx, zx, fmaf(zy, zy, zz * zz));
        r = sqrtf(r2);
        if (r > bailout) break;
        const float rp1 = powi<Fast>(r, P - 1);
        dr = fmaf(rp1 * Pf, dr, 1.0f);
        const float rho2 = fmaf(zx, zx, zy * zy);
        const float rho = sqrtf(rho2);
        const float inv_r = 1.0f / r;
        float ar, ai;
        cpow_int(zz * inv_r, rho * inv_r, P, ar, ai);
        const float rP = rp1 * r;
        float nx = 0.0f, ny = 0.0f;
        if (rho > 0.0f) {
            const float inv_rho = 1.0f / rho;
            float br, bi;
            cpow_int(zx * inv_rho, zy * inv_rho, P, br, bi);
            const float k = rP * ai;
            nx = k * br;
            ny = k * bi;
        }
        zx = nx + px;
        zy = ny + py;
        zz = fmaf(rP, ar, pz);
    }
    return x86_nan(0.5f * logf(r) * r / dr);
}

// ---- fast polar form (CG_NUMERICS_FAST) ----------------------------------
//
// The polar estimator with approximate transcendentals, for marching: one
// branch-free arctangent instead of acosf and atan2f (theta = atan2(rho, z)
// equals acos(z / r) for r = |(rho, z)|), powers as exp2(P log2 r), and sin /
// cos after reduction to [-pi, pi] from the SFU.

// atan(t), t in [0, 1]: t * p(t^2) with p of degree 7, fitted to atan(t)/t on
// Chebyshev nodes by iteratively reweighted least squares (Lawson's
// near-minimax method); |error| < 2e-7 when evaluated in f32.
__device__ __forceinline__ float atan01(float t) {
    const float u = t * t;
    float p = -4.780781455e-03f;
    p = fmaf(p, u, 2.455833741e-02f);
    p = fmaf(p, u, -5.990651995e-02f);
    p = fmaf(p, u, 9.942895174e-02f);
    p = fmaf(p, u, -1.402947456e-01f);
    p = fmaf(p, u, 1.997138709e-01f);
    p = fmaf(p, u, -3.333209455e-01f);
    p = fmaf(p, u, 9.999999404e-01f);
    return t * p;
}

// atan2(y, x) by octant folding into atan01: selects, no branches.
__device__ __forceinline__ float atan2_fast(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    float r = atan01(mx > 0.0f ? __fdividef(mn, mx) : 0.0f);
    r = ay > ax ? 1.57079633f - r : r;
    r = x < 0.0f ? 3.14159265f - r : r;
    return copysignf(r, y);
}

// sin and cos of x (|x| up to a few hundred): reduce by 2 pi, then the SFU.
__device__ __forceinline__ void sincos_fast(float x, float* sn, float* cs) {
    const float k = rintf(x * 0.159154943f);
    __sincosf(fmaf(-k, 6.28318531f, x), sn, cs);
}

// One iteration of the polar loop (polar_step's contract, fast numerics).
__device__ __forceinline__ bool polar_step_fast(float P, float bailout, float qx, float qy, float qz,
                                                float& x, float& y, float& z, float& dr, float& r) {
    const float rho2 = fmaf(x, x, y * y);
    r = sqrtf(fmaf(z, z, rho2));
    if (r > bailout) return false;
    const float theta = atan2_fast(sqrtf(rho2), z) * P;
    const float phi = atan2_fast(y, x) * P;
    const float lr = __log2f(r);
    const float zr = exp2f(P * lr);
    dr = fmaf(exp2f((P - 1.0f) * lr) * P, dr, 1.0f);
    float sn, cs, sp, cp;
    sincos_fast(theta, &sn, &cs);
    sincos_fast(phi, &sp, &cp);
    x = fmaf(zr, sn * cp, qx);
    y = fmaf(zr, sp * sn, qy);
    z = fmaf(zr, cs, qz);
    return true;
}

__device__ __forceinline__ float polar_de_fast(const ShapeDev& s, float px, float py, float pz) {
    float qx, qy, qz;
    rotate_point<true>(s, px, py, pz, qx, qy, qz);
    float x = qx, y = qy, z = qz, dr = 1.0f, r = 0.0f;
    for (uint32_t i = 0; i < s.max_iters; ++i)
        if (!polar_step_fast(s.power_f, s.bailout, qx, qy, qz, x, y, z, dr, r)) break;
    return x86_nan(__fdividef(0.5f * __logf(r) * r, dr));
}

// Kernel modes.
enum Mode {
    MODE_P8 = 0,
    MODE_INT = 1,
    MODE_POLAR = 2,
    MODE_SPHERE = 3,
    MODE_P8_FAST = 4,
    MODE_INT_POLY = 5,
    MODE_POLAR_FAST = 6,
    // MODE_P8 with max_iters == 15 (the reference's default), the loop
    // unrolled at compile time; chosen at launch (p8_unrolled) by the grid
    // and point kernels, never returned by mode_of.
    MODE_P8_IT15 = 7,
    MODE_P8_FAST_IT15 = 8  // MODE_P8_FAST likewise
};

// NAN_EXIT: the unrolled P=8 loop stops at a NaN second step (same bits).
template <int M, bool NAN_EXIT = false>
__device__ __forceinline__ float eval(const ShapeDev& s, float x, float y, float z) {
    if (M == MODE_P8) return mandelbulb_de<Exact, true>(8, s.max_iters, s.bailout, x, y, z);
    if (M == MODE_P8_IT15)
        return mandelbulb_de<Exact, true, 15, NAN_EXIT>(8, 15, s.bailout, x, y, z);
    if (M == MODE_INT) return mandelbulb_de<Exact, false>(s.power, s.max_iters, s.bailout, x, y, z);
    if (M == MODE_POLAR) return polar_de(s, x, y, z);
    if (M == MODE_SPHERE) return sphere_de(s, x, y, z);
    if (M == MODE_INT_POLY) return mandelbulb_int_poly(s.power, s.max_iters, s.bailout, x, y, z);
    if (M == MODE_POLAR_FAST) return polar_de_fast(s, x, y, z);
    if (M == MODE_P8_FAST_IT15) return mandelbulb_p8_fast<15>(15, s.bailout, x, y, z);
    return mandelbulb_p8_fast(s.max_iters, s.bailout, x, y, z);
}


// MODE_P8 / MODE_P8_FAST or, for max_iters 15, their unrolled twins.
__host__ __forceinline__ bool p8_unrolled(const ShapeDev& s) { return s.max_iters == 15; }

// Kernel mode of a shape (integer P=8 takes the polynomial).
__host__ __device__ __forceinline__ int mode_of(const ShapeDev& s, uint32_t numerics) {
    if (s.kind == CG_SHAPE_SPHERE) return MODE_SPHERE;
    if (s.kind == CG_SHAPE_MANDELBULB_POLAR)
        return numerics == CG_NUMERICS_FAST ? MODE_POLAR_FAST : MODE_POLAR;
    if (s.power == 8) return numerics == CG_NUMERICS_FAST ? MODE_P8_FAST : MODE_P8;
    return numerics == CG_NUMERICS_FAST && s.power >= 1 ? MODE_INT_POLY : MODE_INT;
}

}  // namespace cg
