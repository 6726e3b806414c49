/*
 * oracle.c -- CPU restatement of cantucci's Mandelbulb distance estimator,
 * span mesher and march loop.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path (tests/, smoke(),
 * bench.py's CPU baseline).  Nothing in the shipped package uses it.
 *
 * Build: see oracle/build.py (gcc -O3 -ffp-contract=off -fno-fast-math).
 * Contraction must stay off: Rust never fuses a*b+c, so every product and sum
 * below is rounded to f32 on its own, in the order the reference writes it.
 *
 * Parity: pinned bit for bit to the reference's own Rust source, translated
 * into C++ by oracle/rust_build.py; see oracle.h.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------ */
/* small helpers                                                       */
/* ------------------------------------------------------------------ */

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* f32::is_sign_positive: the sign bit, NaN included (used by the mesher,
 * src/mesh/buffer.rs:131-135,195,299). */
static inline int sign_positive(float f) { return (f2u(f) >> 31) == 0; }

/* x86-64 SSE returns the "default NaN" 0xFFC00000 (sign bit set) for an
 * invalid operation (0/0, inf-inf, ...) and propagates the NaN operand's bits
 * otherwise, so every NaN the reference can produce here is sign-negative.
 * aarch64's default NaN is sign-positive; outputs are mapped to the x86 bit
 * pattern so that the oracle means the same thing on both hosts. */
static inline float x86_nan(float v) { return isnan(v) ? u2f(0xFFC00000u) : v; }

static double now_ms(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec * 1e3 + (double)ts.tv_nsec * 1e-6;
}

/* ---- parallel for: dynamic chunks over [0, n) (mirrors a thread pool) ---- */
typedef void (*range_fn)(void* ctx, uint64_t begin, uint64_t end);
typedef struct {
    range_fn fn;
    void* ctx;
    uint64_t n, chunk;
    uint64_t next;
} pfor_state;

static void* pfor_worker(void* arg) {
    pfor_state* st = (pfor_state*)arg;
    for (;;) {
        uint64_t b = __atomic_fetch_add(&st->next, st->chunk, __ATOMIC_RELAXED);
        if (b >= st->n) break;
        uint64_t e = b + st->chunk;
        if (e > st->n) e = st->n;
        st->fn(st->ctx, b, e);
    }
    return NULL;
}

static void parallel_for(uint64_t n, uint64_t chunk, int nthreads, range_fn fn, void* ctx) {
    if (n == 0) return;
    if (chunk == 0) chunk = 1;
    if (nthreads <= 1 || n <= chunk) {
        fn(ctx, 0, n);
        return;
    }
    if (nthreads > 256) nthreads = 256;
    pfor_state st = {fn, ctx, n, chunk, 0};
    pthread_t th[256];
    int started = 0;
    for (int t = 1; t < nthreads; t++) {
        if (pthread_create(&th[started], NULL, pfor_worker, &st) == 0) started++;
    }
    pfor_worker(&st);
    for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* Mandelbulb<P>, f32, reference semantics                             */
/* ------------------------------------------------------------------ */

/* Vec3::magnitude with SSE4.1 (src/shape/mandelbulb.rs:412-418):
 * _mm_dp_ps(v, v, 0x71) sums lane products as (x*x + y*y) + (z*z + 0), then
 * _mm_sqrt_ss. */
static inline float mag_dpps(float x, float y, float z) {
    float s = (x * x + y * y) + z * z;
    return sqrtf(s);
}

/* Vec3::is_on_z_axis (mandelbulb.rs:421-426): x and y both +-0. */
static inline int on_z_axis(float x, float y) {
    return ((f2u(x) | f2u(y)) & 0x7FFFFFFFu) == 0;
}

/* f32::powi with a constant exponent: LLVM expands llvm.powi into
 * square-and-multiply, low bit first (x^7 = (x * x^2) * x^4).  Used by
 * mandelbulb.rs:73,121,136. */
static inline float powi_f(float x, int32_t n) {
    if (n == 0) return 1.0f;
    int neg = n < 0;
    uint32_t m = neg ? (uint32_t)(-(int64_t)n) : (uint32_t)n;
    float res = 0.0f, cur = x;
    int have = 0;
    for (;;) {
        if (m & 1u) {
            res = have ? res * cur : cur;
            have = 1;
        }
        m >>= 1;
        if (!m) break;
        cur = cur * cur;
    }
    return neg ? 1.0f / res : res;
}

/* rotate_inner_p8_scalar (mandelbulb.rs:148-200), operation order as written. */
static inline void rotate_p8(float x, float y, float z, float* ox, float* oy, float* oz) {
    float x2 = x * x, x4 = x2 * x2, x6 = x4 * x2, x8 = x4 * x4;
    float y2 = y * y, y4 = y2 * y2, y6 = y4 * y2, y8 = y4 * y4;
    float z2 = z * z, z4 = z2 * z2, z6 = z4 * z2, z8 = z4 * z4;
    float rxy2 = x2 + y2;
    float rxy4 = rxy2 * rxy2;
    float rxy6 = rxy2 * rxy4;
    float rxy8 = rxy4 * rxy4;
    float a = 1.0f + (((z8 - 28.0f * z6 * rxy2) + 70.0f * z4 * rxy4) - 28.0f * z2 * rxy6) / rxy8;
    *ox = a * ((((x8 - 28.0f * x6 * y2) + 70.0f * x4 * y4) - 28.0f * x2 * y6) - y8);
    *oy = 8.0f * a * x * y * (((x6 - 7.0f * x4 * y2) + 7.0f * x2 * y4) - y6);
    *oz = 8.0f * z * sqrtf(rxy2) * (z2 - rxy2) * ((z4 - 6.0f * z2 * rxy2) + rxy4);
}

/* rotate_inner_px_generic (mandelbulb.rs:128-146). */
static inline void rotate_generic(uint32_t P, float x, float y, float z,
                                  float* ox, float* oy, float* oz) {
    float old_radius = mag_dpps(x, y, z);
    float theta = acosf(z / old_radius);
    float phi = atan2f(y, x);
    float new_radius = powi_f(old_radius, (int32_t)P);
    theta = theta * (float)P;
    phi = phi * (float)P;
    float vx = sinf(theta) * cosf(phi);
    float vy = sinf(phi) * sinf(theta);
    float vz = cosf(theta);
    /* f32 * Vec3 -> Vec3 * f32: lane-wise products */
    *ox = vx * new_radius;
    *oy = vy * new_radius;
    *oz = vz * new_radius;
}

/* rotate_on_z_axis (mandelbulb.rs:114-126). */
static inline void rotate_axis(uint32_t P, float x, float y, float z,
                               float* ox, float* oy, float* oz) {
    float old_radius = mag_dpps(x, y, z);
    float theta = acosf(z / old_radius);
    float new_radius = powi_f(old_radius, (int32_t)P);
    theta = theta * (float)P;
    *ox = 0.0f;
    *oy = 0.0f;
    *oz = new_radius * cosf(theta);
}

/* rotate (mandelbulb.rs:97-112). */
static inline void rotate_int(uint32_t P, float x, float y, float z,
                              float* ox, float* oy, float* oz) {
    if (on_z_axis(x, y)) {
        rotate_axis(P, x, y, z, ox, oy, oz);
    } else if (P == 8) {
        rotate_p8(x, y, z, ox, oy, oz);
    } else {
        rotate_generic(P, x, y, z, ox, oy, oz);
    }
}

/* Mandelbulb::min_distance_from (mandelbulb.rs:59-79).  `r` is stale when the
 * loop runs out: it is |z| from the start of the last iteration. */
static float mb_de_int(uint32_t P, uint64_t max_iters, float bailout,
                       float px, float py, float pz,
                       float* r_out, float* dr_out, uint32_t* steps_out, uint32_t* esc_out) {
    float zx = px, zy = py, zz = pz;
    float dr = 1.0f;
    float r = 0.0f;
    uint32_t steps = 0, esc = 0;
    for (uint64_t i = 0; i < max_iters; i++) {
        r = mag_dpps(zx, zy, zz);
        if (r > bailout) {
            esc = 1;
            break;
        }
        dr = powi_f(r, (int32_t)P - 1) * (float)P * dr + 1.0f;
        float nx, ny, nz;
        rotate_int(P, zx, zy, zz, &nx, &ny, &nz);
        zx = nx + px;
        zy = ny + py;
        zz = nz + pz;
        steps++;
    }
    if (r_out) *r_out = r;
    if (dr_out) *dr_out = dr;
    if (steps_out) *steps_out = steps;
    if (esc_out) *esc_out = esc;
    float ln_r = logf(r) * r;
    return 0.5f * ln_r / dr;
}

/* ------------------------------------------------------------------ */
/* rotation (new: not in the reference)                                */
/* ------------------------------------------------------------------ */

static void rot_matrix_d(const double e[3], double m[9]) {
    double ca = cos(e[0]), sa = sin(e[0]);
    double cb = cos(e[1]), sb = sin(e[1]);
    double cc = cos(e[2]), sc = sin(e[2]);
    /* R = Rz(c) * Ry(b) * Rx(a), row-major */
    m[0] = cc * cb;
    m[1] = cc * sb * sa - sc * ca;
    m[2] = cc * sb * ca + sc * sa;
    m[3] = sc * cb;
    m[4] = sc * sb * sa + cc * ca;
    m[5] = sc * sb * ca - cc * sa;
    m[6] = -sb;
    m[7] = cb * sa;
    m[8] = cb * ca;
}

/* dR/d(angle k), row-major. */
static void rot_matrix_dd(const double e[3], int k, double m[9]) {
    double ca = cos(e[0]), sa = sin(e[0]);
    double cb = cos(e[1]), sb = sin(e[1]);
    double cc = cos(e[2]), sc = sin(e[2]);
    if (k == 0) {
        m[0] = 0;
        m[1] = cc * sb * ca + sc * sa;
        m[2] = -cc * sb * sa + sc * ca;
        m[3] = 0;
        m[4] = sc * sb * ca - cc * sa;
        m[5] = -sc * sb * sa - cc * ca;
        m[6] = 0;
        m[7] = cb * ca;
        m[8] = -cb * sa;
    } else if (k == 1) {
        m[0] = -cc * sb;
        m[1] = cc * cb * sa;
        m[2] = cc * cb * ca;
        m[3] = -sc * sb;
        m[4] = sc * cb * sa;
        m[5] = sc * cb * ca;
        m[6] = -cb;
        m[7] = -sb * sa;
        m[8] = -sb * ca;
    } else {
        m[0] = -sc * cb;
        m[1] = -sc * sb * sa - cc * ca;
        m[2] = -sc * sb * ca + cc * sa;
        m[3] = cc * cb;
        m[4] = cc * sb * sa - sc * ca;
        m[5] = cc * sb * ca + sc * sa;
        m[6] = 0;
        m[7] = 0;
        m[8] = 0;
    }
}

void orc_rotation_matrix(const float euler[3], float m[9]) {
    double e[3] = {euler[0], euler[1], euler[2]}, md[9];
    rot_matrix_d(e, md);
    for (int i = 0; i < 9; i++) m[i] = (float)md[i];
}

/* Whether the polar form has a rotation.  Without one the point enters the
 * estimator unchanged, as in src/shape/mandelbulb.frag (which has no
 * rotation): a product with the identity would turn -0 into +0 and an
 * infinite coordinate into NaN. */
static inline int rotated(const orc_shape* s) {
    return s->rot[0] != 0.0f || s->rot[1] != 0.0f || s->rot[2] != 0.0f;
}

/* q = R^T p in f32, sums left to right. */
static inline void rot_apply_t(const float m[9], float px, float py, float pz,
                               float* qx, float* qy, float* qz) {
    *qx = (m[0] * px + m[3] * py) + m[6] * pz;
    *qy = (m[1] * px + m[4] * py) + m[7] * pz;
    *qz = (m[2] * px + m[5] * py) + m[8] * pz;
}

/* Polar form of src/shape/mandelbulb.frag:1-39 with a real power, f32 libm.
 * GLSL length() is taken as sqrt((x*x + y*y) + z*z). */
static float polar_de_f32(const orc_shape* s, const float m[9], float px, float py, float pz,
                          uint32_t* steps_out) {
    float qx = px, qy = py, qz = pz;
    if (rotated(s)) rot_apply_t(m, px, py, pz, &qx, &qy, &qz);
    const float P = s->power_f;
    float zx = qx, zy = qy, zz = qz, dr = 1.0f, r = 0.0f;
    uint32_t steps = 0;
    for (uint32_t i = 0; i < s->max_iters; i++) {
        r = sqrtf((zx * zx + zy * zy) + zz * zz);
        if (r > s->bailout) break;
        float theta = acosf(zz / r);
        float phi = atan2f(zy, zx);
        dr = powf(r, P - 1.0f) * P * dr + 1.0f;
        float zr = powf(r, P);
        theta = theta * P;
        phi = phi * P;
        float st = sinf(theta), ct = cosf(theta), sp = sinf(phi), cp = cosf(phi);
        zx = zr * (st * cp) + qx;
        zy = zr * (sp * st) + qy;
        zz = zr * ct + qz;
        steps++;
    }
    if (steps_out) *steps_out = steps;
    float ln_r = logf(r) * r;
    return 0.5f * ln_r / dr;
}

/* Sphere::min_distance_from (src/shape/sphere.rs:33-35): cgmath magnitude =
 * sqrt((x*x + y*y) + z*z). */
static inline float sphere_de(const orc_shape* s, float x, float y, float z) {
    float dx = s->center[0] - x, dy = s->center[1] - y, dz = s->center[2] - z;
    return sqrtf((dx * dx + dy * dy) + dz * dz) - s->radius;
}

/* One DE evaluation; `m` is the rotation matrix for the polar form. */
static inline float de_f32(const orc_shape* s, const float m[9], float x, float y, float z) {
    switch (s->kind) {
    case ORC_SPHERE:
        return sphere_de(s, x, y, z);
    case ORC_MANDELBULB_POLAR:
        return x86_nan(polar_de_f32(s, m, x, y, z, NULL));
    default:
        return x86_nan(mb_de_int((uint32_t)s->power, s->max_iters, s->bailout, x, y, z,
                                 NULL, NULL, NULL, NULL));
    }
}

float orc_min_distance_from(const orc_shape* s, float x, float y, float z) {
    float m[9];
    orc_rotation_matrix(s->rot, m);
    return de_f32(s, m, x, y, z);
}

/* Shape::contains (src/shape/mod.rs:78-80) and Sphere's override (sphere.rs:24-26). */
int orc_contains(const orc_shape* s, float x, float y, float z) {
    if (s->kind == ORC_SPHERE) {
        float dx = s->center[0] - x, dy = s->center[1] - y, dz = s->center[2] - z;
        return ((dx * dx + dy * dy) + dz * dz) <= s->radius * s->radius;
    }
    return orc_min_distance_from(s, x, y, z) < 0.0f;
}

void orc_mandelbulb_state(const orc_shape* s, float x, float y, float z,
                          float* r, float* dr, uint32_t* steps, uint32_t* escaped) {
    mb_de_int((uint32_t)s->power, s->max_iters, s->bailout, x, y, z, r, dr, steps, escaped);
}

typedef struct {
    const orc_shape* s;
    float m[9];
    const float* pts;
    float* out;
    uint64_t* steps;
    uint64_t* esc;
    pthread_mutex_t mu;
} batch_ctx;

static void batch_range(void* vctx, uint64_t b, uint64_t e) {
    batch_ctx* c = (batch_ctx*)vctx;
    for (uint64_t i = b; i < e; i++)
        c->out[i] = de_f32(c->s, c->m, c->pts[3 * i], c->pts[3 * i + 1], c->pts[3 * i + 2]);
}

void orc_batch_min_distance_from(const orc_shape* s, const float* pts, uint64_t n,
                                 float* out, int nthreads) {
    batch_ctx c;
    memset(&c, 0, sizeof c);
    c.s = s;
    c.pts = pts;
    c.out = out;
    orc_rotation_matrix(s->rot, c.m);
    parallel_for(n, 4096, nthreads, batch_range, &c);
}

static void steps_range(void* vctx, uint64_t b, uint64_t e) {
    batch_ctx* c = (batch_ctx*)vctx;
    uint64_t st = 0, es = 0;
    for (uint64_t i = b; i < e; i++) {
        uint32_t k = 0, q = 0;
        if (c->s->kind == ORC_MANDELBULB_POLAR) {
            polar_de_f32(c->s, c->m, c->pts[3 * i], c->pts[3 * i + 1], c->pts[3 * i + 2], &k);
            q = k < c->s->max_iters;
        } else {
            mb_de_int((uint32_t)c->s->power, c->s->max_iters, c->s->bailout, c->pts[3 * i],
                      c->pts[3 * i + 1], c->pts[3 * i + 2], NULL, NULL, &k, &q);
        }
        st += k;
        es += q;
    }
    pthread_mutex_lock(&c->mu);
    *c->steps += st;
    *c->esc += es;
    pthread_mutex_unlock(&c->mu);
}

void orc_batch_steps(const orc_shape* s, const float* pts, uint64_t n,
                     uint64_t* steps_total, uint64_t* escaped_total, int nthreads) {
    batch_ctx c;
    memset(&c, 0, sizeof c);
    c.s = s;
    c.pts = pts;
    *steps_total = 0;
    *escaped_total = 0;
    c.steps = steps_total;
    c.esc = escaped_total;
    pthread_mutex_init(&c.mu, NULL);
    orc_rotation_matrix(s->rot, c.m);
    parallel_for(n, 4096, nthreads, steps_range, &c);
    pthread_mutex_destroy(&c.mu);
}

/* ------------------------------------------------------------------ */
/* FP64                                                                */
/* ------------------------------------------------------------------ */

static inline double powi_d(double x, int32_t n) {
    if (n == 0) return 1.0;
    int neg = n < 0;
    uint32_t m = neg ? (uint32_t)(-(int64_t)n) : (uint32_t)n;
    double res = 0.0, cur = x;
    int have = 0;
    for (;;) {
        if (m & 1u) {
            res = have ? res * cur : cur;
            have = 1;
        }
        m >>= 1;
        if (!m) break;
        cur = cur * cur;
    }
    return neg ? 1.0 / res : res;
}

static double mb_de_int_d(uint32_t P, uint64_t max_iters, double bailout,
                          double px, double py, double pz, uint32_t* steps_out) {
    double zx = px, zy = py, zz = pz, dr = 1.0, r = 0.0;
    uint32_t steps = 0;
    for (uint64_t i = 0; i < max_iters; i++) {
        r = sqrt((zx * zx + zy * zy) + zz * zz);
        if (r > bailout) break;
        dr = powi_d(r, (int32_t)P - 1) * (double)P * dr + 1.0;
        double nx, ny, nz;
        if (zx == 0.0 && zy == 0.0) {
            double th = acos(zz / r) * (double)P;
            nx = 0.0;
            ny = 0.0;
            nz = powi_d(r, (int32_t)P) * cos(th);
        } else if (P == 8) {
            double x = zx, y = zy, z = zz;
            double x2 = x * x, x4 = x2 * x2, x6 = x4 * x2, x8 = x4 * x4;
            double y2 = y * y, y4 = y2 * y2, y6 = y4 * y2, y8 = y4 * y4;
            double z2 = z * z, z4 = z2 * z2, z6 = z4 * z2, z8 = z4 * z4;
            double rxy2 = x2 + y2, rxy4 = rxy2 * rxy2, rxy6 = rxy2 * rxy4, rxy8 = rxy4 * rxy4;
            double a = 1.0 + (((z8 - 28.0 * z6 * rxy2) + 70.0 * z4 * rxy4) - 28.0 * z2 * rxy6) / rxy8;
            nx = a * ((((x8 - 28.0 * x6 * y2) + 70.0 * x4 * y4) - 28.0 * x2 * y6) - y8);
            ny = 8.0 * a * x * y * (((x6 - 7.0 * x4 * y2) + 7.0 * x2 * y4) - y6);
            nz = 8.0 * z * sqrt(rxy2) * (z2 - rxy2) * ((z4 - 6.0 * z2 * rxy2) + rxy4);
        } else {
            double th = acos(zz / r) * (double)P, ph = atan2(zy, zx) * (double)P;
            double nr = powi_d(r, (int32_t)P);
            nx = nr * (sin(th) * cos(ph));
            ny = nr * (sin(ph) * sin(th));
            nz = nr * cos(th);
        }
        zx = nx + px;
        zy = ny + py;
        zz = nz + pz;
        steps++;
    }
    if (steps_out) *steps_out = steps;
    return 0.5 * (log(r) * r) / dr;
}

static double polar_de_d(const orc_shape* s, const double m[9], double px, double py, double pz,
                         uint32_t* steps_out) {
    double qx = px, qy = py, qz = pz;
    if (rotated(s)) {
        qx = m[0] * px + m[3] * py + m[6] * pz;
        qy = m[1] * px + m[4] * py + m[7] * pz;
        qz = m[2] * px + m[5] * py + m[8] * pz;
    }
    const double P = s->power_f;
    double zx = qx, zy = qy, zz = qz, dr = 1.0, r = 0.0;
    uint32_t steps = 0;
    for (uint32_t i = 0; i < s->max_iters; i++) {
        r = sqrt(zx * zx + zy * zy + zz * zz);
        if (r > (double)s->bailout) break;
        double th = acos(zz / r), ph = atan2(zy, zx);
        dr = pow(r, P - 1.0) * P * dr + 1.0;
        double zr = pow(r, P);
        th *= P;
        ph *= P;
        zx = zr * sin(th) * cos(ph) + qx;
        zy = zr * sin(ph) * sin(th) + qy;
        zz = zr * cos(th) + qz;
        steps++;
    }
    if (steps_out) *steps_out = steps;
    return 0.5 * log(r) * r / dr;
}

static inline double de_f64_m(const orc_shape* s, const double m[9], double x, double y, double z,
                              uint32_t* steps) {
    switch (s->kind) {
    case ORC_SPHERE: {
        double dx = s->center[0] - x, dy = s->center[1] - y, dz = s->center[2] - z;
        if (steps) *steps = 0;
        return sqrt(dx * dx + dy * dy + dz * dz) - s->radius;
    }
    case ORC_MANDELBULB_POLAR:
        return polar_de_d(s, m, x, y, z, steps);
    default:
        return mb_de_int_d((uint32_t)s->power, s->max_iters, s->bailout, x, y, z, steps);
    }
}

static void shape_rot_d(const orc_shape* s, double m[9]) {
    double e[3] = {s->rot[0], s->rot[1], s->rot[2]};
    rot_matrix_d(e, m);
}

double orc_de_f64(const orc_shape* s, double x, double y, double z) {
    double m[9];
    shape_rot_d(s, m);
    return de_f64_m(s, m, x, y, z, NULL);
}

typedef struct {
    const orc_shape* s;
    double m[9];
    const float* pts;
    double* out;
    uint32_t* steps;
} batch64_ctx;

static void batch64_range(void* vctx, uint64_t b, uint64_t e) {
    batch64_ctx* c = (batch64_ctx*)vctx;
    for (uint64_t i = b; i < e; i++) {
        uint32_t k = 0;
        c->out[i] = de_f64_m(c->s, c->m, c->pts[3 * i], c->pts[3 * i + 1], c->pts[3 * i + 2], &k);
        if (c->steps) c->steps[i] = k;
    }
}

void orc_batch_de_f64(const orc_shape* s, const float* pts, uint64_t n, double* out,
                      uint32_t* steps_out, int nthreads) {
    batch64_ctx c = {s, {0}, pts, out, steps_out};
    shape_rot_d(s, c.m);
    parallel_for(n, 2048, nthreads, batch64_range, &c);
}

/* ---- FP64 forward mode (dual numbers, 4 tangents: q.x, q.y, q.z, power) ---- */
#define NT 4
typedef struct { double v; double d[NT]; } dual;

static inline dual dc(double v) { dual r; r.v = v; for (int i = 0; i < NT; i++) r.d[i] = 0; return r; }
static inline dual dadd(dual a, dual b) { dual r; r.v = a.v + b.v; for (int i = 0; i < NT; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
static inline dual dsub(dual a, dual b) { dual r; r.v = a.v - b.v; for (int i = 0; i < NT; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
static inline dual dmul(dual a, dual b) { dual r; r.v = a.v * b.v; for (int i = 0; i < NT; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
static inline dual ddiv(dual a, dual b) { dual r; r.v = a.v / b.v; for (int i = 0; i < NT; i++) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v); return r; }
static inline dual dsqrt(dual a) { dual r; r.v = sqrt(a.v); for (int i = 0; i < NT; i++) r.d[i] = a.d[i] / (2.0 * r.v); return r; }
static inline dual dlog(dual a) { dual r; r.v = log(a.v); for (int i = 0; i < NT; i++) r.d[i] = a.d[i] / a.v; return r; }
static inline dual dacos(dual a) { dual r; r.v = acos(a.v); double k = -1.0 / sqrt(1.0 - a.v * a.v); for (int i = 0; i < NT; i++) r.d[i] = k * a.d[i]; return r; }
static inline dual datan2(dual y, dual x) {
    dual r; r.v = atan2(y.v, x.v);
    double q = x.v * x.v + y.v * y.v;
    for (int i = 0; i < NT; i++) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) / q;
    return r;
}
static inline dual dsin(dual a) { dual r; r.v = sin(a.v); double k = cos(a.v); for (int i = 0; i < NT; i++) r.d[i] = k * a.d[i]; return r; }
static inline dual dcos(dual a) { dual r; r.v = cos(a.v); double k = -sin(a.v); for (int i = 0; i < NT; i++) r.d[i] = k * a.d[i]; return r; }
static inline dual dpow(dual b, dual e) {
    dual r; r.v = pow(b.v, e.v);
    double lb = log(b.v);
    for (int i = 0; i < NT; i++) r.d[i] = r.v * (e.d[i] * lb + e.v * b.d[i] / b.v);
    return r;
}

/* Polar-form DE in duals at q (shape frame); power P as a variable. */
static dual polar_de_dual(double qx0, double qy0, double qz0, double P0,
                          uint32_t max_iters, double bailout) {
    dual qx = dc(qx0), qy = dc(qy0), qz = dc(qz0), P = dc(P0);
    qx.d[0] = 1;
    qy.d[1] = 1;
    qz.d[2] = 1;
    P.d[3] = 1;
    dual zx = qx, zy = qy, zz = qz, dr = dc(1.0), r = dc(0.0);
    dual one = dc(1.0);
    for (uint32_t i = 0; i < max_iters; i++) {
        r = dsqrt(dadd(dadd(dmul(zx, zx), dmul(zy, zy)), dmul(zz, zz)));
        if (r.v > bailout) break;
        dual th = dacos(ddiv(zz, r));
        dual ph = datan2(zy, zx);
        dr = dadd(dmul(dmul(dpow(r, dsub(P, one)), P), dr), one);
        dual zr = dpow(r, P);
        th = dmul(th, P);
        ph = dmul(ph, P);
        dual st = dsin(th), ct = dcos(th), sp = dsin(ph), cp = dcos(ph);
        zx = dadd(dmul(zr, dmul(st, cp)), qx);
        zy = dadd(dmul(zr, dmul(sp, st)), qy);
        zz = dadd(dmul(zr, ct), qz);
    }
    dual half = dc(0.5);
    return ddiv(dmul(half, dmul(dlog(r), r)), dr);
}

/* Mandelbulb<P> (integer power, reference code paths) in duals: tangents
 * d[0..2] on p; d[3] on the power where it enters continuously (the trig and
 * z-axis paths).  The P=8 polynomial (mandelbulb.rs:148-200) has no power
 * parameter, so its d[3] is NaN.  Note that this polynomial is not the polar
 * map: it computes x' = a*(Re((x+iy)^8) - 2 y^8), y' = a*Im((x+iy)^8),
 * z' = r^8 sin(8 theta), a*rxy^8 = r^8 cos(8 theta). */
static dual mb_de_int_dual(uint32_t P, uint64_t max_iters, double bailout,
                           double px0, double py0, double pz0) {
    dual px = dc(px0), py = dc(py0), pz = dc(pz0), one = dc(1.0);
    px.d[0] = 1;
    py.d[1] = 1;
    pz.d[2] = 1;
    dual Pd = dc((double)P);
    if (P != 8) Pd.d[3] = 1.0;
    else Pd.d[3] = 0.0;
    dual zx = px, zy = py, zz = pz, dr = dc(1.0), r = dc(0.0);
    int used_poly = 0;
    for (uint64_t i = 0; i < max_iters; i++) {
        r = dsqrt(dadd(dadd(dmul(zx, zx), dmul(zy, zy)), dmul(zz, zz)));
        if (r.v > bailout) break;
        dr = dadd(dmul(dmul(dpow(r, dsub(Pd, one)), Pd), dr), one);
        dual nx, ny, nz;
        if (zx.v == 0.0 && zy.v == 0.0) {
            dual th = dmul(dacos(ddiv(zz, r)), Pd);
            nx = dc(0.0);
            ny = dc(0.0);
            nz = dmul(dpow(r, Pd), dcos(th));
        } else if (P == 8) {
            used_poly = 1;
            dual x = zx, y = zy, z = zz;
            dual x2 = dmul(x, x), x4 = dmul(x2, x2), x6 = dmul(x4, x2), x8 = dmul(x4, x4);
            dual y2 = dmul(y, y), y4 = dmul(y2, y2), y6 = dmul(y4, y2), y8 = dmul(y4, y4);
            dual z2 = dmul(z, z), z4 = dmul(z2, z2), z6 = dmul(z4, z2), z8 = dmul(z4, z4);
            dual rxy2 = dadd(x2, y2), rxy4 = dmul(rxy2, rxy2), rxy6 = dmul(rxy2, rxy4),
                 rxy8 = dmul(rxy4, rxy4);
            dual num = dsub(dadd(dsub(z8, dmul(dmul(dc(28), z6), rxy2)), dmul(dmul(dc(70), z4), rxy4)),
                            dmul(dmul(dc(28), z2), rxy6));
            dual a = dadd(one, ddiv(num, rxy8));
            dual X = dsub(dsub(dadd(dsub(x8, dmul(dmul(dc(28), x6), y2)), dmul(dmul(dc(70), x4), y4)),
                               dmul(dmul(dc(28), x2), y6)), y8);
            nx = dmul(a, X);
            dual Y = dsub(dadd(dsub(x6, dmul(dmul(dc(7), x4), y2)), dmul(dmul(dc(7), x2), y4)), y6);
            ny = dmul(dmul(dmul(dmul(dc(8), a), x), y), Y);
            dual Z = dadd(dsub(z4, dmul(dmul(dc(6), z2), rxy2)), rxy4);
            nz = dmul(dmul(dmul(dmul(dc(8), z), dsqrt(rxy2)), dsub(z2, rxy2)), Z);
        } else {
            dual th = dmul(dacos(ddiv(zz, r)), Pd);
            dual ph = dmul(datan2(zy, zx), Pd);
            dual nr = dpow(r, Pd);
            nx = dmul(dmul(dsin(th), dcos(ph)), nr);
            ny = dmul(dmul(dsin(ph), dsin(th)), nr);
            nz = dmul(dcos(th), nr);
        }
        zx = dadd(nx, px);
        zy = dadd(ny, py);
        zz = dadd(nz, pz);
    }
    dual out = ddiv(dmul(dc(0.5), dmul(dlog(r), r)), dr);
    if (used_poly) out.d[3] = NAN;
    return out;
}

static void de_grad_f64_m(const orc_shape* s, const double m[9], double px, double py, double pz,
                          double out[8]) {
    for (int i = 0; i < 8; i++) out[i] = 0.0;
    if (s->kind == ORC_SPHERE) {
        double dx = px - s->center[0], dy = py - s->center[1], dz = pz - s->center[2];
        double n = sqrt(dx * dx + dy * dy + dz * dz);
        out[0] = n - s->radius;
        out[1] = dx / n;
        out[2] = dy / n;
        out[3] = dz / n;
        return;
    }
    if (s->kind == ORC_MANDELBULB) {
        dual d = mb_de_int_dual((uint32_t)s->power, s->max_iters, s->bailout, px, py, pz);
        out[0] = d.v;
        out[1] = d.d[0];
        out[2] = d.d[1];
        out[3] = d.d[2];
        out[4] = d.d[3];
        return;
    }
    double qx = px, qy = py, qz = pz;
    if (rotated(s)) {
        qx = m[0] * px + m[3] * py + m[6] * pz;
        qy = m[1] * px + m[4] * py + m[7] * pz;
        qz = m[2] * px + m[5] * py + m[8] * pz;
    }
    double P = s->kind == ORC_MANDELBULB_POLAR ? (double)s->power_f : (double)s->power;
    dual d = polar_de_dual(qx, qy, qz, P, s->max_iters, s->bailout);
    out[0] = d.v;
    /* grad_p = R grad_q */
    for (int j = 0; j < 3; j++)
        out[1 + j] = m[3 * j + 0] * d.d[0] + m[3 * j + 1] * d.d[1] + m[3 * j + 2] * d.d[2];
    out[4] = d.d[3];
    double e[3] = {s->rot[0], s->rot[1], s->rot[2]};
    for (int k = 0; k < 3; k++) {
        double dm[9];
        rot_matrix_dd(e, k, dm);
        /* dq/dk = (dR/dk)^T p */
        double dqx = dm[0] * px + dm[3] * py + dm[6] * pz;
        double dqy = dm[1] * px + dm[4] * py + dm[7] * pz;
        double dqz = dm[2] * px + dm[5] * py + dm[8] * pz;
        out[5 + k] = d.d[0] * dqx + d.d[1] * dqy + d.d[2] * dqz;
    }
}

void orc_de_grad_f64(const orc_shape* s, double x, double y, double z, double out[8]) {
    double m[9];
    shape_rot_d(s, m);
    de_grad_f64_m(s, m, x, y, z, out);
}

typedef struct {
    const orc_shape* s;
    double m[9];
    const float* pts;
    double* out;
} grad_ctx;

static void grad_range(void* vctx, uint64_t b, uint64_t e) {
    grad_ctx* c = (grad_ctx*)vctx;
    for (uint64_t i = b; i < e; i++)
        de_grad_f64_m(c->s, c->m, c->pts[3 * i], c->pts[3 * i + 1], c->pts[3 * i + 2], c->out + 8 * i);
}

void orc_batch_de_grad_f64(const orc_shape* s, const float* pts, uint64_t n, double* out,
                           int nthreads) {
    grad_ctx c = {s, {0}, pts, out};
    shape_rot_d(s, c.m);
    parallel_for(n, 512, nthreads, grad_range, &c);
}

/* ------------------------------------------------------------------ */
/* naive surface nets (src/mesh/buffer.rs:58-391)                      */
/* ------------------------------------------------------------------ */

typedef struct {
    const orc_shape* s;
    float m[9];
    uint32_t res, N;           /* N = res + 1 corners per axis */
    float start[3];            /* expanded span start */
    float across[3];           /* expanded span end - start */
    float step[3];
    float delta[3];            /* FD normal offset */
    float* dists;
    uint8_t* surf;
    uint32_t* points;
    orc_vertex* verts;
    uint64_t vcap;
    int lerp_fail;
    uint64_t* row_quads;       /* quads per x-slab */
    uint32_t* idx;
    uint64_t icap;
    uint64_t* slab_off;
} mesh_ctx;

#define DIDX(c, x, y, z) (((uint64_t)(x) * (c)->N + (y)) * (c)->N + (z))
#define CIDX(c, x, y, z) (((uint64_t)(x) * (c)->res + (y)) * (c)->res + (z))

/* Step 1 (buffer.rs:77-83): p = start + across (*) (v / res), v = (x, y, z). */
static void mesh_step1(void* vctx, uint64_t b, uint64_t e) {
    mesh_ctx* c = (mesh_ctx*)vctx;
    const float rf = (float)c->res;
    for (uint64_t i = b; i < e; i++) {
        uint32_t z = (uint32_t)(i % c->N);
        uint32_t y = (uint32_t)((i / c->N) % c->N);
        uint32_t x = (uint32_t)(i / ((uint64_t)c->N * c->N));
        float vx = (float)x / rf, vy = (float)y / rf, vz = (float)z / rf;
        float px = c->start[0] + c->across[0] * vx;
        float py = c->start[1] + c->across[1] * vy;
        float pz = c->start[2] + c->across[2] * vz;
        c->dists[i] = de_f32(c->s, c->m, px, py, pz);
    }
}

/* Step 2a (buffer.rs:116-147): a cell is on the surface iff the sign bits of
 * its 8 corners differ. */
static void mesh_surface(void* vctx, uint64_t b, uint64_t e) {
    mesh_ctx* c = (mesh_ctx*)vctx;
    for (uint64_t i = b; i < e; i++) {
        uint32_t z = (uint32_t)(i % c->res);
        uint32_t y = (uint32_t)((i / c->res) % c->res);
        uint32_t x = (uint32_t)(i / ((uint64_t)c->res * c->res));
        int first = sign_positive(c->dists[DIDX(c, x, y, z)]);
        int same = 1;
        for (int k = 1; k < 8 && same; k++) {
            uint32_t dx = (k >> 2) & 1, dy = (k >> 1) & 1, dz = k & 1;
            if (sign_positive(c->dists[DIDX(c, x + dx, y + dy, z + dz)]) != first) same = 0;
        }
        c->surf[i] = (uint8_t)!same;
    }
}

static const uint8_t EDGES[12][2] = {
    {0, 4}, {1, 5}, {2, 6}, {3, 7},   /* x edges */
    {0, 2}, {1, 3}, {4, 6}, {5, 7},   /* y edges */
    {0, 1}, {2, 3}, {4, 5}, {6, 7},   /* z edges */
};

/* Step 2b (buffer.rs:149-274): centroid of the edge crossings, DE at the
 * vertex and the central-difference normal. */
static void mesh_vertices(void* vctx, uint64_t b, uint64_t e) {
    mesh_ctx* c = (mesh_ctx*)vctx;
    for (uint64_t i = b; i < e; i++) {
        if (!c->surf[i]) continue;
        uint32_t id = c->points[i];
        uint32_t z = (uint32_t)(i % c->res);
        uint32_t y = (uint32_t)((i / c->res) % c->res);
        uint32_t x = (uint32_t)(i / ((uint64_t)c->res * c->res));
        float d[8];
        for (int k = 0; k < 8; k++)
            d[k] = c->dists[DIDX(c, x + ((k >> 2) & 1), y + ((k >> 1) & 1), z + (k & 1))];
        /* p0 = start + (x, y, z) (*) step */
        float p0x = c->start[0] + (float)x * c->step[0];
        float p0y = c->start[1] + (float)y * c->step[1];
        float p0z = c->start[2] + (float)z * c->step[2];
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        uint32_t count = 0;
        for (int k = 0; k < 12; k++) {
            int from = EDGES[k][0], to = EDGES[k][1];
            if (sign_positive(d[from]) == sign_positive(d[to])) continue;
            float df, dt;
            if (d[from] < 0.0f) {
                df = d[from];
                dt = d[to];
            } else {
                df = -d[from];
                dt = -d[to];
            }
            float w;
            if (dt == df) {
                w = 0.5f;
            } else {
                float delta = dt - df;
                w = (df + delta) / delta;
            }
            /* math::lerp asserts 0 <= t <= 1 (src/math.rs:19) */
            if (!(w >= 0.0f && w <= 1.0f)) {
                __atomic_store_n(&c->lerp_fail, 1, __ATOMIC_RELAXED);
                w = 0.0f;
            }
            float ax = p0x + (((from >> 2) & 1) ? c->step[0] : 0.0f);
            float ay = p0y + (((from >> 1) & 1) ? c->step[1] : 0.0f);
            float az = p0z + ((from & 1) ? c->step[2] : 0.0f);
            float bx = p0x + (((to >> 2) & 1) ? c->step[0] : 0.0f);
            float by = p0y + (((to >> 1) & 1) ? c->step[1] : 0.0f);
            float bz = p0z + ((to & 1) ? c->step[2] : 0.0f);
            /* Point3::lerp: self * (1 - t) + other * t (src/math.rs:45-49) */
            float omt = 1.0f - w;
            float qx = ax * omt + bx * w;
            float qy = ay * omt + by * w;
            float qz = az * omt + bz * w;
            sx = sx + qx;
            sy = sy + qy;
            sz = sz + qz;
            count++;
        }
        float cf = (float)count;
        float vx = 0.0f + sx / cf, vy = 0.0f + sy / cf, vz = 0.0f + sz / cf;
        float dist_p = de_f32(c->s, c->m, vx, vy, vz);
        const float dx = c->delta[0], dy = c->delta[1], dz = c->delta[2];
        /* p + unit * delta = p + (delta, +0, +0); p + unit * -delta = p + (-delta, -0, -0) */
        float nx = de_f32(c->s, c->m, vx + dx, vy + 0.0f, vz + 0.0f) -
                   de_f32(c->s, c->m, vx + -dx, vy + -0.0f, vz + -0.0f);
        float ny = de_f32(c->s, c->m, vx + 0.0f, vy + dy, vz + 0.0f) -
                   de_f32(c->s, c->m, vx + -0.0f, vy + -dy, vz + -0.0f);
        float nz = de_f32(c->s, c->m, vx + 0.0f, vy + 0.0f, vz + dz) -
                   de_f32(c->s, c->m, vx + -0.0f, vy + -0.0f, vz + -dz);
        /* cgmath normalize: v * (1 / sqrt((x*x + y*y) + z*z)) */
        float inv = 1.0f / sqrtf((nx * nx + ny * ny) + nz * nz);
        if (id < c->vcap) {
            orc_vertex* v = &c->verts[id];
            v->position[0] = vx;
            v->position[1] = vy;
            v->position[2] = vz;
            v->normal[0] = nx * inv;
            v->normal[1] = ny * inv;
            v->normal[2] = nz * inv;
            v->distance_from_surface = dist_p;
        }
    }
}

/* Step 3 (buffer.rs:288-372), done per x-slab: pass 0 counts, pass 1 writes. */
static uint64_t quads_slab(mesh_ctx* c, uint32_t x, uint32_t* out, uint64_t cap, uint64_t off) {
    uint64_t n = 0;
    const uint32_t R = c->res;
    for (uint32_t y = 0; y < R; y++) {
        for (uint32_t z = 0; z < R; z++) {
            float d0 = c->dists[DIDX(c, x, y, z)];
            int base = sign_positive(d0);
            int neg = d0 < 0.0f;
            uint32_t q[6];
            int have;
            /* +x */
            have = 0;
            if (y > 0 && z > 0 && base != sign_positive(c->dists[DIDX(c, x + 1, y, z)])) {
                uint32_t v0 = c->points[CIDX(c, x, y - 1, z - 1)];
                uint32_t v1 = c->points[CIDX(c, x, y - 1, z)];
                uint32_t v2 = c->points[CIDX(c, x, y, z - 1)];
                uint32_t v3 = c->points[CIDX(c, x, y, z)];
                if (neg) { q[0] = v0; q[1] = v2; q[2] = v1; q[3] = v1; q[4] = v2; q[5] = v3; }
                else     { q[0] = v0; q[1] = v1; q[2] = v2; q[3] = v1; q[4] = v3; q[5] = v2; }
                have = 1;
            }
            if (have) {
                if (out) for (int k = 0; k < 6; k++) if (off + n + k < cap) out[off + n + k] = q[k];
                n += 6;
            }
            /* +y */
            have = 0;
            if (x > 0 && z > 0 && base != sign_positive(c->dists[DIDX(c, x, y + 1, z)])) {
                uint32_t v0 = c->points[CIDX(c, x - 1, y, z - 1)];
                uint32_t v1 = c->points[CIDX(c, x - 1, y, z)];
                uint32_t v2 = c->points[CIDX(c, x, y, z - 1)];
                uint32_t v3 = c->points[CIDX(c, x, y, z)];
                if (neg) { q[0] = v0; q[1] = v1; q[2] = v2; q[3] = v1; q[4] = v3; q[5] = v2; }
                else     { q[0] = v0; q[1] = v2; q[2] = v1; q[3] = v1; q[4] = v2; q[5] = v3; }
                have = 1;
            }
            if (have) {
                if (out) for (int k = 0; k < 6; k++) if (off + n + k < cap) out[off + n + k] = q[k];
                n += 6;
            }
            /* +z */
            have = 0;
            if (x > 0 && y > 0 && base != sign_positive(c->dists[DIDX(c, x, y, z + 1)])) {
                uint32_t v0 = c->points[CIDX(c, x - 1, y - 1, z)];
                uint32_t v1 = c->points[CIDX(c, x - 1, y, z)];
                uint32_t v2 = c->points[CIDX(c, x, y - 1, z)];
                uint32_t v3 = c->points[CIDX(c, x, y, z)];
                if (neg) { q[0] = v0; q[1] = v2; q[2] = v1; q[3] = v1; q[4] = v2; q[5] = v3; }
                else     { q[0] = v0; q[1] = v1; q[2] = v2; q[3] = v1; q[4] = v3; q[5] = v2; }
                have = 1;
            }
            if (have) {
                if (out) for (int k = 0; k < 6; k++) if (off + n + k < cap) out[off + n + k] = q[k];
                n += 6;
            }
        }
    }
    return n;
}

static void mesh_quads_count(void* vctx, uint64_t b, uint64_t e) {
    mesh_ctx* c = (mesh_ctx*)vctx;
    for (uint64_t x = b; x < e; x++) c->row_quads[x] = quads_slab(c, (uint32_t)x, NULL, 0, 0);
}

static void mesh_quads_write(void* vctx, uint64_t b, uint64_t e) {
    mesh_ctx* c = (mesh_ctx*)vctx;
    for (uint64_t x = b; x < e; x++) quads_slab(c, (uint32_t)x, c->idx, c->icap, c->slab_off[x]);
}

static int is_pow2(uint32_t v) { return v && !(v & (v - 1)); }

/* generate_for_box, or with `dists_in` steps 2 and 3 only, on those corner
 * distances instead of step 1's. */
static int generate_impl(const orc_shape* s, const float span[6], uint32_t res, int nthreads,
                         const float* dists_in, float* dists_out, uint32_t* points_out,
                         orc_vertex* verts, uint64_t vcap, uint32_t* idx, uint64_t icap,
                         uint64_t* nv, uint64_t* ni, double timings_ms[3]) {
    /* generate_for_box asserts (buffer.rs:35-39); GridTable::fill_with(res)
     * asserts res >= 2 (src/util/grid.rs:24). */
    if (!(span[0] < span[3] && span[1] < span[4] && span[2] < span[5])) return ORC_EINVAL;
    if (!is_pow2(res) || res < 2) return ORC_EINVAL;
    if (s->kind == ORC_MANDELBULB && (s->max_iters < 1 || s->power < 1 || s->power > 255))
        return ORC_EINVAL;

    mesh_ctx c;
    memset(&c, 0, sizeof c);
    c.s = s;
    orc_rotation_matrix(s->rot, c.m);
    c.res = res;
    c.N = res + 1;
    const float rf = (float)res;
    /* span expanded by one cell on each side (buffer.rs:64-67) */
    float ov[3], st[3], en[3];
    for (int k = 0; k < 3; k++) {
        ov[k] = (span[3 + k] - span[k]) / rf;
        st[k] = span[k] + -ov[k];
        en[k] = span[3 + k] + ov[k];
        c.start[k] = st[k];
        c.across[k] = en[k] - st[k];
        c.step[k] = (en[k] - st[k]) / rf;
        c.delta[k] = (0.7f * (en[k] - st[k])) / rf;
    }
    const uint64_t ncorner = (uint64_t)c.N * c.N * c.N;
    const uint64_t ncell = (uint64_t)res * res * res;

    c.dists = dists_in ? (float*)dists_in
                       : (dists_out ? dists_out : (float*)malloc(ncorner * sizeof(float)));
    c.surf = (uint8_t*)malloc(ncell);
    c.points = points_out ? points_out : (uint32_t*)malloc(ncell * sizeof(uint32_t));
    c.row_quads = (uint64_t*)calloc(res, sizeof(uint64_t));
    c.slab_off = (uint64_t*)calloc(res + 1, sizeof(uint64_t));

    double t0 = now_ms();
    if (!dists_in) parallel_for(ncorner, 4096, nthreads, mesh_step1, &c);
    double t1 = now_ms();

    parallel_for(ncell, 1 << 16, nthreads, mesh_surface, &c);
    uint64_t v = 0;
    for (uint64_t i = 0; i < ncell; i++) c.points[i] = c.surf[i] ? (uint32_t)v++ : 0xFFFFFFFFu;
    c.verts = verts;
    c.vcap = verts ? vcap : 0;
    parallel_for(ncell, 4096, nthreads, mesh_vertices, &c);
    double t2 = now_ms();

    parallel_for(res, 1, nthreads, mesh_quads_count, &c);
    uint64_t q = 0;
    for (uint32_t x = 0; x < res; x++) {
        c.slab_off[x] = q;
        q += c.row_quads[x];
    }
    c.idx = idx;
    c.icap = idx ? icap : 0;
    if (idx) parallel_for(res, 1, nthreads, mesh_quads_write, &c);
    double t3 = now_ms();

    if (timings_ms) {
        timings_ms[0] = t1 - t0;
        timings_ms[1] = t2 - t1;
        timings_ms[2] = t3 - t2;
    }
    *nv = v;
    *ni = q;
    int rc = ORC_OK;
    if (c.lerp_fail) rc = ORC_ELERP;
    else if ((verts && v > vcap) || (idx && q > icap)) rc = ORC_ECAPACITY;

    if (!dists_in && !dists_out) free(c.dists);
    if (!points_out) free(c.points);
    free(c.surf);
    free(c.row_quads);
    free(c.slab_off);
    return rc;
}

int orc_generate_for_box(const orc_shape* s, const float span[6], uint32_t res, int nthreads,
                         float* dists_out, uint32_t* points_out,
                         orc_vertex* verts, uint64_t vcap, uint32_t* idx, uint64_t icap,
                         uint64_t* nv, uint64_t* ni, double timings_ms[3]) {
    return generate_impl(s, span, res, nthreads, NULL, dists_out, points_out, verts, vcap, idx,
                         icap, nv, ni, timings_ms);
}

int orc_mesh_from_dists(const orc_shape* s, const float span[6], uint32_t res, int nthreads,
                        const float* dists, uint32_t* points_out, orc_vertex* verts,
                        uint64_t vcap, uint32_t* idx, uint64_t icap, uint64_t* nv, uint64_t* ni) {
    if (!dists) return ORC_EINVAL;
    return generate_impl(s, span, res, nthreads, dists, NULL, points_out, verts, vcap, idx, icap,
                         nv, ni, NULL);
}

/* ------------------------------------------------------------------ */
/* march loop of ShapeMesh::get_focii (src/mesh/mod.rs:229-241)        */
/* ------------------------------------------------------------------ */

typedef struct {
    const orc_shape* s;
    float m[9];
    const float* o;
    const float* d;
    uint32_t max_steps;
    float eps;
    float* hits;
    uint8_t* hit;
} march_ctx;

static void march_range(void* vctx, uint64_t b, uint64_t e) {
    march_ctx* c = (march_ctx*)vctx;
    for (uint64_t i = b; i < e; i++) {
        float px = c->o[3 * i], py = c->o[3 * i + 1], pz = c->o[3 * i + 2];
        const float dx = c->d[3 * i], dy = c->d[3 * i + 1], dz = c->d[3 * i + 2];
        uint8_t h = 0;
        for (uint32_t k = 0; k < c->max_steps; k++) {
            float dist = de_f32(c->s, c->m, px, py, pz);
            px += dx * dist;
            py += dy * dist;
            pz += dz * dist;
            if (dist < c->eps) {
                h = 1;
                break;
            }
        }
        c->hits[3 * i] = px;
        c->hits[3 * i + 1] = py;
        c->hits[3 * i + 2] = pz;
        c->hit[i] = h;
    }
}

void orc_march(const orc_shape* s, const float* origins, const float* dirs, uint64_t n,
               uint32_t max_steps, float epsilon, float* hits, uint8_t* hit, int nthreads) {
    march_ctx c = {s, {0}, origins, dirs, max_steps, epsilon, hits, hit};
    orc_rotation_matrix(s->rot, c.m);
    parallel_for(n, 64, nthreads, march_range, &c);
}

/* create_spans (src/octree/mod.rs:315-329): centre = start + (end - start) / 2. */
void orc_create_spans(const float p[6], float ch[8 * 6]) {
    float s[3] = {p[0], p[1], p[2]}, e[3] = {p[3], p[4], p[5]}, c[3];
    for (int k = 0; k < 3; k++) c[k] = s[k] + (e[k] - s[k]) / 2.0f;
    /* child i: bit 2 -> x upper half, bit 1 -> y, bit 0 -> z */
    for (int i = 0; i < 8; i++) {
        int hx = (i >> 2) & 1, hy = (i >> 1) & 1, hz = i & 1;
        float* o = ch + 6 * i;
        o[0] = hx ? c[0] : s[0];
        o[1] = hy ? c[1] : s[1];
        o[2] = hz ? c[2] : s[2];
        o[3] = hx ? e[0] : c[0];
        o[4] = hy ? e[1] : c[1];
        o[5] = hz ? e[2] : c[2];
    }
}

uint32_t orc_sizeof_shape(void) { return (uint32_t)sizeof(orc_shape); }
uint32_t orc_sizeof_vertex(void) { return (uint32_t)sizeof(orc_vertex); }

/* Loop state for a batch: out[4 i + 0..3] = r, dr, steps (bits), escaped (bits). */
typedef struct {
    const orc_shape* s;
    const float* pts;
    float* out;
} state_ctx;

static void state_range(void* vctx, uint64_t b, uint64_t e) {
    state_ctx* c = (state_ctx*)vctx;
    for (uint64_t i = b; i < e; i++) {
        float r, dr;
        uint32_t k, q;
        mb_de_int((uint32_t)c->s->power, c->s->max_iters, c->s->bailout, c->pts[3 * i],
                  c->pts[3 * i + 1], c->pts[3 * i + 2], &r, &dr, &k, &q);
        c->out[4 * i] = r;
        c->out[4 * i + 1] = dr;
        c->out[4 * i + 2] = u2f(k);
        c->out[4 * i + 3] = u2f(q);
    }
}

void orc_batch_state(const orc_shape* s, const float* pts, uint64_t n, float* out, int nthreads) {
    state_ctx c = {s, pts, out};
    parallel_for(n, 4096, nthreads, state_range, &c);
}
