/*
 * oracle.h -- CPU restatement of cantucci's Mandelbulb distance estimator and
 * naive-surface-nets span mesher.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path: it
 * is loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg, and by nothing else.  The product (cantucci_gb300/) never
 * links, loads or calls it.
 *
 * Parity status: pinned to the reference's own source.  The reference
 * (Rust, nightly, x86-64 SSE4.1 only) has no unit tests and no golden
 * vectors, and no Rust toolchain exists here, so its source text is compiled
 * another way.  Every formula below follows the cited reference line in
 * operation order and rounding (f32, no contraction, glibc libm where Rust
 * std calls libm), and:
 *   - the integer-power estimator (the P=8 polynomial, the generic-trig and
 *     z-axis paths), the sphere and the whole mesher give the same bits as
 *     the reference's Rust source translated mechanically into C++ by
 *     oracle/rust_build.py (fixture tests/golden/rust_ref.npz); at a point
 *     with a NaN coordinate only NaN-ness is defined (the NaN an SSE
 *     operation with two NaN operands returns depends on the operand order
 *     the compiler picks);
 *   - the polar and sphere estimators give the same bits as the reference's
 *     own shader source (src/shape/mandelbulb.frag, src/shape/shape.frag)
 *     compiled as C++ by oracle/ref_build.py (tests/golden/shader_de.npz).
 * tests/golden/golden.npz (tests/golden/make_golden.py) holds this oracle's
 * outputs on x86-64; tests/test_rust_pin.py checks it against the pin.
 */
#ifndef CANTUCCI_ORACLE_H
#define CANTUCCI_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_MANDELBULB = 0,        /* Mandelbulb<const P: u8> (src/shape/mandelbulb.rs:13) */
    ORC_SPHERE = 1,            /* Sphere (src/shape/sphere.rs:5) */
    ORC_MANDELBULB_POLAR = 2   /* float-power polar form (src/shape/mandelbulb.frag:1-39) + Euler rotation */
};

/* Same layout as cg_shape in include/cantucci_gpu.h (48 bytes). */
typedef struct {
    int32_t kind;
    int32_t power;       /* integer power P of Mandelbulb<P> */
    float power_f;       /* real power of the polar form */
    uint32_t max_iters;
    float bailout;
    float rot[3];        /* Euler angles (a, b, c): R = Rz(c) Ry(b) Rx(a); DE(p) = DE0(R^T p) */
    float center[3];     /* Sphere centre */
    float radius;        /* Sphere radius */
} orc_shape;

/* Vertex of src/mesh/mod.rs:257-261, #[repr(C)], 28 bytes. */
typedef struct {
    float position[3];
    float normal[3];
    float distance_from_surface;
} orc_vertex;

/* ---- distance estimator, f32 reference semantics ---- */
float orc_min_distance_from(const orc_shape* s, float x, float y, float z);
int orc_contains(const orc_shape* s, float x, float y, float z);
/* Loop state of Mandelbulb::min_distance_from at exit: r (stale |z|, see
 * mandelbulb.rs:65-75), dr, number of rotate steps, escaped flag. */
void orc_mandelbulb_state(const orc_shape* s, float x, float y, float z,
                          float* r, float* dr, uint32_t* steps, uint32_t* escaped);
/* Batch of the above: out[4 i + 0..3] = r, dr, steps (u32 bits), escaped (u32 bits). */
void orc_batch_state(const orc_shape* s, const float* pts, uint64_t n, float* out, int nthreads);
void orc_batch_min_distance_from(const orc_shape* s, const float* pts, uint64_t n,
                                 float* out, int nthreads);
/* Sum over points of the rotate steps and escapes (for the flop count). */
void orc_batch_steps(const orc_shape* s, const float* pts, uint64_t n,
                     uint64_t* steps_total, uint64_t* escaped_total, int nthreads);

/* ---- distance estimator, FP64 ---- */
double orc_de_f64(const orc_shape* s, double x, double y, double z);
void orc_batch_de_f64(const orc_shape* s, const float* pts, uint64_t n, double* out,
                      uint32_t* steps_out, int nthreads);
/* FP64 forward-mode gradient (dual numbers) of the same code path as the f32 DE:
 * out[0] = DE, out[1..3] = dDE/dp, out[4] = dDE/dpower, out[5..7] = dDE/d(euler). */
void orc_de_grad_f64(const orc_shape* s, double x, double y, double z, double out[8]);
void orc_batch_de_grad_f64(const orc_shape* s, const float* pts, uint64_t n, double* out,
                           int nthreads);

/* ---- span mesher: MeshBuffer::generate_for_box (src/mesh/buffer.rs:30-391) ---- */
enum { ORC_OK = 0, ORC_EINVAL = 1, ORC_ECAPACITY = 2, ORC_ELERP = 3 };
int orc_generate_for_box(const orc_shape* s, const float span[6], uint32_t res, int nthreads,
                         float* dists, uint32_t* points,
                         orc_vertex* verts, uint64_t vcap, uint32_t* idx, uint64_t icap,
                         uint64_t* nv, uint64_t* ni, double timings_ms[3]);

/* Steps 2 and 3 of the same mesher (buffer.rs:85-372) on GIVEN corner
 * distances `dists` ((res+1)^3 floats, GridTable order) instead of step 1's:
 * the surface cells, vertex positions and quads follow from the distances
 * alone, so a mesher fed the same distances must place the same bits. */
int orc_mesh_from_dists(const orc_shape* s, const float span[6], uint32_t res, int nthreads,
                        const float* dists, uint32_t* points, orc_vertex* verts, uint64_t vcap,
                        uint32_t* idx, uint64_t icap, uint64_t* nv, uint64_t* ni);

/* ---- sphere tracing: ShapeMesh::get_focii march loop (src/mesh/mod.rs:229-241) ---- */
void orc_march(const orc_shape* s, const float* origins, const float* dirs, uint64_t n,
               uint32_t max_steps, float epsilon, float* hits, uint8_t* hit, int nthreads);

/* ---- octree child spans: create_spans (src/octree/mod.rs:315-329) ---- */
void orc_create_spans(const float parent[6], float children[8 * 6]);

/* Rotation matrix used by the polar form: row-major R (float), computed in double. */
void orc_rotation_matrix(const float euler[3], float m[9]);

/* Sizes of the structs, for the Python loader's layout check. */
uint32_t orc_sizeof_shape(void);
uint32_t orc_sizeof_vertex(void);

#ifdef __cplusplus
}
#endif
#endif
