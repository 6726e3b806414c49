// adjoint.cuh -- reverse-mode gradient of the real-power polar estimator
// (src/shape/mandelbulb.frag:1-39, rotated), shared by the point kernels
// (adjoint.cu) and the depth-map backward (trace.cu); and its forward-mode
// twin polar_de_tangent (end of file), also used for analytic mesh normals
// (mesh_rows.cuh).
//
// For the polar loop one thread returns, per point,
//   DE, dDE/dp (3), dDE/dpower, dDE/d(euler angles) (3).
// It is the adjoint of the forward loop, not a finite difference: the
// forward pass keeps a checkpoint of (z, dr) every CK steps and the step
// records of its last segment in a per-thread tape in shared memory (never
// in HBM or local memory); the backward pass walks the segments from last to
// first, recomputes each earlier segment's iterates from its checkpoint and
// back-propagates through them.  Work is one forward pass, the recompute of
// all steps but the last segment's, and one backward pass.
//
// Per step k (z_k -> z_{k+1} = r^P u(P theta, P phi) + q, dr_{k+1} =
// r^(P-1) P dr_k + 1, r = |z_k|, theta = acos(z_z / r), phi = atan2(y, x)):
//   q_bar     += z_bar
//   g_zr       = z_bar . u,   g_th = zr (z_bar . du/dtheta'),  g_ph = zr (z_bar . du/dphi')
//   r_bar     += g_zr P zr / r + dr_bar P dr (P - 1) r^(P-1) / r
//   P_bar     += g_zr zr ln r + g_th theta + g_ph phi + dr_bar dr r^(P-1) (1 + P ln r)
//   dr_bar     = dr_bar P r^(P-1)
//   z_bar      = r_bar z / r + P g_th grad(theta) + P g_ph grad(phi)
// The final DE = 0.5 r ln r / dr seeds r_bar = 0.5 (ln r + 1) / dr and
// dr_bar = -DE / dr on the z whose |z| is the returned r (the escaping
// iterate, or the stale one of the last step when the loop runs out).
#pragma once

#include <cmath>

#include "common.cuh"
#include "de.cuh"

namespace cg {

constexpr int ADJ_CK = 5;          // default checkpoint interval (steps)
constexpr int ADJ_MAX_ITERS = 64;  // the longest loop a tape is sized for

// dR/d(angle k) for k = a, b, c, row-major, 3 x 9 floats.
struct Dm3 {
    float m[27];
};
Dm3 rotation_derivatives(const cg_shape& c);

struct StepState {
    float x, y, z, dr;
};

// One forward step of the polar loop from (z, dr); returns false on escape
// (r > bailout).  r is always returned.
__device__ __forceinline__ bool polar_step(const ShapeDev& s, float qx, float qy, float qz,
                                           StepState& st, float& r) {
    r = magnitude<Exact>(st.x, st.y, st.z);
    if (r > s.bailout) return false;
    const float P = s.power_f;
    float theta = acosf(__fdiv_rn(st.z, r));
    float phi = atan2f(st.y, st.x);
    st.dr = __fadd_rn(__fmul_rn(__fmul_rn(powf(r, __fsub_rn(P, 1.0f)), P), st.dr), 1.0f);
    const float zr = powf(r, P);
    theta = __fmul_rn(theta, P);
    phi = __fmul_rn(phi, P);
    float sn, cs, sp, cp;
    sincosf(theta, &sn, &cs);
    sincosf(phi, &sp, &cp);
    st.x = __fadd_rn(__fmul_rn(zr, __fmul_rn(sn, cp)), qx);
    st.y = __fadd_rn(__fmul_rn(zr, __fmul_rn(sp, sn)), qy);
    st.z = __fadd_rn(__fmul_rn(zr, cs), qz);
    return true;
}

// A step's input and the values its forward computation produces.
struct StepDeriv {
    float x, y, z, dr;       // z_k, dr_k
    float r, theta, phi;     // |z_k|, acos(z/r), atan2(y, x)
    float t1, zr;            // r^(P-1), r^P
    float sn, cs, sp, cp;    // sin/cos of P theta and P phi
};
constexpr int STEP_FIELDS = 13;

// The step from `st` with |z| = r (not an escape), recorded into `d`: the
// same operations as polar_step, so the iterate is bit-identical.
__device__ __forceinline__ void polar_step_rec(const ShapeDev& s, float qx, float qy, float qz,
                                               float r, StepState& st, StepDeriv& d) {
    d.x = st.x;
    d.y = st.y;
    d.z = st.z;
    d.dr = st.dr;
    d.r = r;
    const float P = s.power_f;
    d.theta = acosf(__fdiv_rn(st.z, r));
    d.phi = atan2f(st.y, st.x);
    d.t1 = powf(r, __fsub_rn(P, 1.0f));
    st.dr = __fadd_rn(__fmul_rn(__fmul_rn(d.t1, P), st.dr), 1.0f);
    d.zr = powf(r, P);
    sincosf(__fmul_rn(d.theta, P), &d.sn, &d.cs);
    sincosf(__fmul_rn(d.phi, P), &d.sp, &d.cp);
    st.x = __fadd_rn(__fmul_rn(d.zr, __fmul_rn(d.sn, d.cp)), qx);
    st.y = __fadd_rn(__fmul_rn(d.zr, __fmul_rn(d.sp, d.sn)), qy);
    st.z = __fadd_rn(__fmul_rn(d.zr, d.cs), qz);
}

// The same step in the fast polar arithmetic (polar_step_fast: one
// branch-free arctangent per angle, SFU powers and sin/cos), recorded.  For
// recomputing a segment from an exact checkpoint: its iterates stay within
// the fast arithmetic's error of the exact ones over the few steps of a
// segment.
__device__ __forceinline__ void polar_step_rec_fast(float P, float qx, float qy, float qz,
                                                    StepState& st, StepDeriv& d) {
    d.x = st.x;
    d.y = st.y;
    d.z = st.z;
    d.dr = st.dr;
    const float rho2 = fmaf(st.x, st.x, st.y * st.y);
    d.r = sqrtf(fmaf(st.z, st.z, rho2));
    d.theta = atan2_fast(sqrtf(rho2), st.z);
    d.phi = atan2_fast(st.y, st.x);
    const float lr = __log2f(d.r);
    d.zr = exp2f(P * lr);
    d.t1 = exp2f((P - 1.0f) * lr);
    st.dr = fmaf(d.t1 * P, st.dr, 1.0f);
    sincos_fast(d.theta * P, &d.sn, &d.cs);
    sincos_fast(d.phi * P, &d.sp, &d.cp);
    st.x = fmaf(d.zr, d.sn * d.cp, qx);
    st.y = fmaf(d.zr, d.sp * d.sn, qy);
    st.z = fmaf(d.zr, d.cs, qz);
}

// 1/x from the hardware estimate and one Newton step (within an ulp).
__device__ __forceinline__ float rcp_nr(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return fmaf(fmaf(-x, y, 1.0f), y, y);
}

// A thread's tape in shared memory: the (z, dr) checkpoint of every CK-th
// step and the records of one segment of CK steps, field-major
// ([slot][field][thread]) so that a warp's accesses fall in distinct banks.
// Shared memory takes run-time slot indices without spilling to local
// memory.  Bytes per block: adj_tape_bytes.
struct AdjTape {
    float4* ck;
    float* seg;
    uint32_t tid, nth;
};

__host__ __device__ constexpr size_t adj_tape_bytes(uint32_t max_iters, int ck, uint32_t nth) {
    return ((size_t)((max_iters + ck - 1) / ck) * 16u + (size_t)STEP_FIELDS * ck * 4u) * nth;
}

__device__ __forceinline__ AdjTape adj_tape(void* smem, uint32_t max_iters, int ck) {
    AdjTape t;
    t.tid = threadIdx.x;
    t.nth = blockDim.x;
    t.ck = reinterpret_cast<float4*>(smem);
    t.seg = reinterpret_cast<float*>(t.ck + (size_t)((max_iters + ck - 1) / ck) * blockDim.x);
    return t;
}

__device__ __forceinline__ void tape_put_ck(const AdjTape& t, uint32_t j, const StepState& st) {
    t.ck[(size_t)j * t.nth + t.tid] = make_float4(st.x, st.y, st.z, st.dr);
}

__device__ __forceinline__ StepState tape_get_ck(const AdjTape& t, uint32_t j) {
    const float4 v = t.ck[(size_t)j * t.nth + t.tid];
    return StepState{v.x, v.y, v.z, v.w};
}

__device__ __forceinline__ void tape_put(const AdjTape& t, uint32_t slot, const StepDeriv& d) {
    float* b = t.seg + (size_t)slot * STEP_FIELDS * t.nth + t.tid;
    const uint32_t n = t.nth;
    b[0] = d.x; b[n] = d.y; b[2 * n] = d.z; b[3 * n] = d.dr; b[4 * n] = d.r;
    b[5 * n] = d.theta; b[6 * n] = d.phi; b[7 * n] = d.t1; b[8 * n] = d.zr;
    b[9 * n] = d.sn; b[10 * n] = d.cs; b[11 * n] = d.sp; b[12 * n] = d.cp;
}

__device__ __forceinline__ StepDeriv tape_get(const AdjTape& t, uint32_t slot) {
    const float* b = t.seg + (size_t)slot * STEP_FIELDS * t.nth + t.tid;
    const uint32_t n = t.nth;
    return StepDeriv{b[0], b[n], b[2 * n], b[3 * n], b[4 * n], b[5 * n], b[6 * n],
                     b[7 * n], b[8 * n], b[9 * n], b[10 * n], b[11 * n], b[12 * n]};
}

// Launch shape of a kernel with a per-thread tape: block 128, dynamic shared
// memory for the tape (opting in above 48 KB), and a grid of the blocks
// that fit on the GPU at once (the kernels walk their points grid-stride).
template <class Kernel>
cg_status adj_launch_shape(Kernel kernel, uint32_t max_iters, int ck, uint64_t n,
                           unsigned* grid, size_t* smem) {
    *smem = adj_tape_bytes(max_iters, ck, 128);
    if (*smem > 48 * 1024)
        CG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)*smem));
    int per_sm = 0;
    CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, *smem));
    *grid = grid_for(n, 128, (unsigned)(per_sm > 0 ? per_sm : 1));
    return CG_OK;
}

// Backward through one recorded step (the step formulas at the top of this
// file).  `stale` adds the seed of the returned r when the loop ran out and
// this is its last step.
__device__ __forceinline__ void polar_back_step(float P, const StepDeriv& z, bool stale,
                                                float r_seed, float& zbx, float& zby, float& zbz,
                                                float& drb, float& qbx, float& qby, float& qbz,
                                                float& Pb) {
    qbx += zbx;  // the "+ q" of this step
    qby += zby;
    qbz += zbz;
    const float inv_r = rcp_nr(z.r);
    const float rho2 = z.x * z.x + z.y * z.y;
    const float lnr = __logf(z.r);
    const float g_zr = zbx * (z.sn * z.cp) + zby * (z.sn * z.sp) + zbz * z.cs;
    const float g_th = z.zr * (zbx * (z.cs * z.cp) + zby * (z.cs * z.sp) - zbz * z.sn);
    const float g_ph = z.zr * z.sn * (zby * z.cp - zbx * z.sp);
    float rb = g_zr * P * z.t1 + drb * P * z.dr * (P - 1.0f) * z.t1 * inv_r;
    if (stale) rb += r_seed;
    Pb += g_zr * z.zr * lnr + g_th * z.theta + g_ph * z.phi + drb * z.dr * z.t1 * (1.0f + P * lnr);
    drb = drb * P * z.t1;
    const float thb = P * g_th, phb = P * g_ph;
    const float rbr = rb * inv_r;
    float gx = rbr * z.x, gy = rbr * z.y, gz = rbr * z.z;
    if (rho2 > 1e-30f) {
        const float inv_rho = rsqrtf(rho2);
        const float rho = rho2 * inv_rho;
        const float inv_rho2 = inv_rho * inv_rho;
        const float inv_r2 = inv_r * inv_r;
        const float k = thb * z.z * inv_r2 * inv_rho;
        gx += k * z.x - phb * z.y * inv_rho2;
        gy += k * z.y + phb * z.x * inv_rho2;
        gz += -thb * rho * inv_r2;
    }
    zbx = gx;
    zby = gy;
    zbz = gz;
}

// DE and its gradient with respect to p, the power and the Euler angles
// (out[0..7]) by reverse mode over `tape` (adj_tape, sized for
// s.max_iters <= ADJ_MAX_ITERS).  The forward pass keeps a checkpoint every
// CK steps and the records of its last segment; the backward pass walks the
// segments from last to first, recomputing every segment but the last from
// its checkpoint (FASTREC: in the fast polar arithmetic).
template <int CK = ADJ_CK, bool FASTREC = false>
__device__ __forceinline__ void polar_de_grad(const ShapeDev& s, const float* __restrict__ dm,
                                              float px, float py, float pz, const AdjTape& tape,
                                              float* out) {
    float qx, qy, qz;
    rotate_point(s, px, py, pz, qx, qy, qz);
    const float P = s.power_f;
    const uint32_t N = s.max_iters;

    // Forward: checkpoints, and every step recorded in its segment slot.
    StepState st = {qx, qy, qz, 1.0f};
    float r = 0.0f;
    uint32_t K = 0;
    bool escaped = false;
    for (uint32_t i = 0; i < N; ++i) {
        if (i % CK == 0) tape_put_ck(tape, i / CK, st);
        const float ri = magnitude<Exact>(st.x, st.y, st.z);
        r = ri;
        if (ri > s.bailout) {
            escaped = true;
            break;
        }
        StepDeriv d;
        polar_step_rec(s, qx, qy, qz, ri, st, d);
        tape_put(tape, i % CK, d);
        ++K;
    }
    // st = z_K (escaped) or z_N; r = |z_K| (escaped) or |z_{N-1}| (stale).
    const float dr_fin = st.dr;
    const float ln_r = logf(r);
    const float de = __fdiv_rn(__fmul_rn(0.5f, __fmul_rn(ln_r, r)), dr_fin);
    float r_seed = 0.5f * (ln_r + 1.0f) / dr_fin;
    float drb = -de / dr_fin;
    float zbx = 0.0f, zby = 0.0f, zbz = 0.0f;
    if (escaped && r > 0.0f) {
        const float k = r_seed / r;
        zbx = k * st.x;
        zby = k * st.y;
        zbz = k * st.z;
        r_seed = 0.0f;
    }
    float qbx = 0.0f, qby = 0.0f, qbz = 0.0f, Pb = 0.0f;

    // Backward, segment by segment; the last segment's records are the
    // forward pass's own.
    if (K > 0) {
        const uint32_t last = (K - 1) / CK;
        for (int j = (int)last; j >= 0; --j) {
            const uint32_t k0 = (uint32_t)j * CK;
            const uint32_t k1 = min(k0 + CK, K);
            if ((uint32_t)j != last) {
                StepState t = tape_get_ck(tape, (uint32_t)j);
                for (uint32_t k = k0; k < k1; ++k) {
                    StepDeriv d;
                    if (FASTREC)
                        polar_step_rec_fast(P, qx, qy, qz, t, d);
                    else
                        polar_step_rec(s, qx, qy, qz, magnitude<Exact>(t.x, t.y, t.z), t, d);
                    tape_put(tape, k - k0, d);
                }
            }
            for (int k = (int)k1 - 1; k >= (int)k0; --k) {
                const StepDeriv d = tape_get(tape, (uint32_t)k - k0);
                polar_back_step(P, d, !escaped && (uint32_t)k + 1 == N, r_seed, zbx, zby, zbz,
                                drb, qbx, qby, qbz, Pb);
            }
        }
    }
    // z_0 = q.
    qbx += zbx;
    qby += zby;
    qbz += zbz;
    out[0] = x86_nan(de);
    // dDE/dp = R q_bar (q = R^T p).
    out[1] = s.m[0] * qbx + s.m[1] * qby + s.m[2] * qbz;
    out[2] = s.m[3] * qbx + s.m[4] * qby + s.m[5] * qbz;
    out[3] = s.m[6] * qbx + s.m[7] * qby + s.m[8] * qbz;
    out[4] = Pb;
    for (int a = 0; a < 3; ++a) {
        const float* d = dm + 9 * a;
        // dq/d(angle) = (dR/d(angle))^T p
        const float dqx = d[0] * px + d[3] * py + d[6] * pz;
        const float dqy = d[1] * px + d[4] * py + d[7] * pz;
        const float dqz = d[2] * px + d[5] * py + d[8] * pz;
        out[5 + a] = qbx * dqx + qby * dqy + qbz * dqz;
    }
}

// Forward (tangent) mode of the same loop: one pass carries the derivative
// of (z, dr) along T directions next to the iterate -- dq = e_x, e_y, e_z
// and, with T = 4, d(power) -- so nothing is stored or recomputed.  The
// loop state and DE are those of polar_de (same exact operations); the
// tangent updates use contracted arithmetic.  Per step and direction:
//   r'   = (z . z') / r
//   th'  = (z_z (x x' + y y') / rho - rho z_z') / r^2,  ph' = (x y' - y x') / rho^2
//   zr'  = P r^(P-1) r' (+ r^P ln r P')
//   Z'   = zr' u + zr ((P th' + th P') du/dTh + (P ph' + ph P') du/dPh) + q'
//   dr'' = P (P-1) r^(P-2) dr r' + P r^(P-1) dr' (+ r^(P-1) dr (1 + P ln r) P')
// and at the end DE' = 0.5 (ln r + 1) r' / dr - DE dr' / dr (the quotient
// rule on DE = 0.5 r ln r / dr).  Outputs as polar_de_grad; with T = 3 there
// is no power direction and out[4] = 0 (the rotation derivatives need only
// the three point directions).  Work: one forward pass plus T tangent
// updates of ~30 operations per step, against polar_de_grad's two forward
// passes plus one backward step.
template <int T, bool Rot = true, bool FAST = false>
__device__ __forceinline__ void polar_de_tangent(const ShapeDev& s, const float* __restrict__ dm,
                                                 float px, float py, float pz, float* out) {
    float qx, qy, qz;
    rotate_point<FAST>(s, px, py, pz, qx, qy, qz);
    const float P = s.power_f;
    float zx = qx, zy = qy, zz = qz, dr = 1.0f, r = 0.0f;
    // tangents: direction k has (tx, ty, tz, tdr); dq_k = e_k for k < 3
    float tx[T], ty[T], tz[T], tdr[T], tr[T];
#pragma unroll
    for (int k = 0; k < T; ++k) {
        tx[k] = k == 0 ? 1.0f : 0.0f;
        ty[k] = k == 1 ? 1.0f : 0.0f;
        tz[k] = k == 2 ? 1.0f : 0.0f;
        tdr[k] = 0.0f;
        tr[k] = 0.0f;
    }
    for (uint32_t i = 0; i < s.max_iters; ++i) {
        const float rho2 = zx * zx + zy * zy;
        r = FAST ? sqrtf(fmaf(zz, zz, rho2)) : magnitude<Exact>(zx, zy, zz);
        const float inv_r = 1.0f / r;
#pragma unroll
        for (int k = 0; k < T; ++k) tr[k] = (zx * tx[k] + zy * ty[k] + zz * tz[k]) * inv_r;
        if (r > s.bailout) break;
        const float rho = sqrtf(rho2);
        float theta, phi, t1, zr, sn, cs, sp, cp;
        const float dr_old = dr;
        if (FAST) {  // polar_step_fast's arithmetic
            theta = atan2_fast(rho, zz);
            phi = atan2_fast(zy, zx);
            const float lr = __log2f(r);
            zr = exp2f(P * lr);
            t1 = exp2f((P - 1.0f) * lr);
            dr = fmaf(t1 * P, dr, 1.0f);
            sincos_fast(theta * P, &sn, &cs);
            sincos_fast(phi * P, &sp, &cp);
        } else {
            theta = acosf(__fdiv_rn(zz, r));
            phi = atan2f(zy, zx);
            t1 = powf(r, __fsub_rn(P, 1.0f));
            dr = __fadd_rn(__fmul_rn(__fmul_rn(t1, P), dr), 1.0f);
            zr = powf(r, P);
            sincosf(__fmul_rn(theta, P), &sn, &cs);
            sincosf(__fmul_rn(phi, P), &sp, &cp);
        }
        // shared factors of the tangent step
        const bool off_axis = rho > 1e-30f;
        const float inv_rho = off_axis ? 1.0f / rho : 0.0f;
        const float inv_rho2 = off_axis ? 1.0f / rho2 : 0.0f;
        const float inv_r2 = inv_r * inv_r;
        const float Pt1 = P * t1;
        const float k_dr = Pt1 * (P - 1.0f) * inv_r * dr_old;  // d(dr')/dr
        // u and its derivatives, scaled by zr
        const float ux = sn * cp, uy = sp * sn, uz = cs;
        const float ax = zr * cs * cp, ay = zr * sp * cs, az = -zr * sn;  // zr du/dTh
        const float bx = -zr * sn * sp, by = zr * cp * sn;                // zr du/dPh
        float lnr = 0.0f;
        if (T == 4) lnr = FAST ? __logf(r) : logf(r);
#pragma unroll
        for (int k = 0; k < T; ++k) {
            const float th_t = (zz * (zx * tx[k] + zy * ty[k]) * inv_rho - rho * tz[k]) * inv_r2;
            const float ph_t = (zx * ty[k] - zy * tx[k]) * inv_rho2;
            float zr_t = Pt1 * tr[k];
            float Th_t = P * th_t, Ph_t = P * ph_t;
            float dr_t = k_dr * tr[k] + Pt1 * tdr[k];
            if (T == 4 && k == 3) {  // the power direction
                zr_t += zr * lnr;
                Th_t += theta;
                Ph_t += phi;
                dr_t += t1 * dr_old * (1.0f + P * lnr);
            }
            tx[k] = zr_t * ux + Th_t * ax + Ph_t * bx + (k == 0 ? 1.0f : 0.0f);
            ty[k] = zr_t * uy + Th_t * ay + Ph_t * by + (k == 1 ? 1.0f : 0.0f);
            tz[k] = zr_t * uz + Th_t * az + (k == 2 ? 1.0f : 0.0f);
            tdr[k] = dr_t;
        }
        if (FAST) {
            zx = fmaf(zr, sn * cp, qx);
            zy = fmaf(zr, sp * sn, qy);
            zz = fmaf(zr, cs, qz);
        } else {
            zx = __fadd_rn(__fmul_rn(zr, __fmul_rn(sn, cp)), qx);
            zy = __fadd_rn(__fmul_rn(zr, __fmul_rn(sp, sn)), qy);
            zz = __fadd_rn(__fmul_rn(zr, cs), qz);
        }
    }
    // tr holds r' of the returned r: the escaping iterate's, or the stale
    // one of the last step when the loop runs out (tdr is then dr_N's).
    const float ln_r = FAST ? __logf(r) : logf(r);
    const float de = FAST ? __fdividef(0.5f * ln_r * r, dr)
                          : __fdiv_rn(__fmul_rn(0.5f, __fmul_rn(ln_r, r)), dr);
    const float c_r = 0.5f * (ln_r + 1.0f) / dr, c_dr = -de / dr;
    float g[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < T; ++k) g[k] = c_r * tr[k] + c_dr * tdr[k];
    out[0] = x86_nan(de);
    out[1] = s.m[0] * g[0] + s.m[1] * g[1] + s.m[2] * g[2];
    out[2] = s.m[3] * g[0] + s.m[4] * g[1] + s.m[5] * g[2];
    out[3] = s.m[6] * g[0] + s.m[7] * g[1] + s.m[8] * g[2];
    out[4] = g[3];
    if constexpr (Rot) {  // without Rot: out[0..4] only (dm unused)
        for (int a = 0; a < 3; ++a) {
            const float* d = dm + 9 * a;
            const float dqx = d[0] * px + d[3] * py + d[6] * pz;
            const float dqy = d[1] * px + d[4] * py + d[7] * pz;
            const float dqz = d[2] * px + d[5] * py + d[8] * pz;
            out[5 + a] = g[0] * dqx + g[1] * dqy + g[2] * dqz;
        }
    }
}

}  // namespace cg
