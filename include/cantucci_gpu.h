/*
 * cantucci_gpu.h -- C ABI of the GB300 (sm_103a) Mandelbulb distance
 * estimator, span mesher and sphere tracer.
 *
 * Every function is `extern "C"`, takes plain pointers and sizes, and returns
 * a cg_status.  Pointers documented as "device" are CUDA device pointers on
 * the current device; `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Reference citations are file:line in
 * LukasKalbertodt/cantucci; each entry point names the Rust interface it
 * replaces.  Where the reference panics (assert!, lerp factor outside [0,1])
 * these functions return an error status instead.
 *
 * Thread safety: the stateless entry points (cg_min_distance_from,
 * cg_contains, cg_de_span_grid, cg_march, ...) may be called from any number
 * of host threads.  A cg_mesher serialises its own calls with an internal
 * mutex; give each worker thread its own mesher for concurrency (the
 * reference runs generate_for_box from a thread pool, src/mesh/mod.rs:141).
 */
#ifndef CANTUCCI_GPU_H
#define CANTUCCI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CG_ABI_VERSION 1

typedef enum cg_status {
    CG_OK = 0,
    CG_EINVAL = 1,     /* invalid argument (the reference asserts and panics) */
    CG_ECAPACITY = 2,  /* an output buffer is too small; required counts are reported */
    CG_ELERP = 3,      /* a lerp factor left [0,1] (src/math.rs:19 panics there) */
    CG_ECUDA = 4,      /* a CUDA call failed; see cg_last_error() */
    CG_ENOMEM = 5,     /* device allocation failed */
    CG_ETIMEOUT = 6,   /* a device-side wait hit its iteration limit */
    CG_ENODEV = 7      /* no CUDA device */
} cg_status;

/* Shape kinds. */
enum {
    CG_SHAPE_MANDELBULB = 0,       /* Mandelbulb<const P: u8> (src/shape/mandelbulb.rs:13-91) */
    CG_SHAPE_SPHERE = 1,           /* Sphere (src/shape/sphere.rs:5-52) */
    CG_SHAPE_MANDELBULB_POLAR = 2  /* real-power polar form (src/shape/mandelbulb.frag:1-39) + rotation */
};

/* Numerics of the distance estimator. */
enum {
    CG_NUMERICS_EXACT = 0,  /* IEEE f32, reference operation order: bit-identical loop state */
    CG_NUMERICS_FAST = 1    /* not bit-faithful: P=8 FMA-contracted with approximate div/sqrt;
                               other integer powers trig-free (complex powers, no acos/atan2/
                               sin/cos); the polar form with a branch-free arctangent, SFU
                               powers and sin/cos */
};

/* Normals of the mesher. */
enum {
    CG_NORMALS_FD = 0,      /* six central differences, as buffer.rs:256-266 */
    CG_NORMALS_ADJOINT = 1  /* analytic dDE/dp, one forward-mode pass per vertex instead of
                               six extra estimator calls; any shape (new) */
};

/* Edge crossings of the mesher. */
enum {
    CG_CROSSINGS_LERP = 0,  /* distance-weighted lerp of the corners, as buffer.rs:187-250 */
    CG_CROSSINGS_ROOT = 1   /* the DE's root along the edge, regula falsi (new; issue #1) */
};

/* Where a surface cell's vertex goes (cg_mesher_set_placement). */
enum {
    CG_PLACEMENT_CENTROID = 0, /* centroid of the edge crossings: naive surface nets,
                                  buffer.rs:149-252 */
    CG_PLACEMENT_QEF = 1       /* dual contouring: minimiser of the squared distances to the
                                  tangent planes at the crossings, buffer.rs:53-54 (new; issue #2) */
};

/* A shape; 48 bytes.  `power`/`max_iters`/`bailout` are Mandelbulb's fields
 * (src/shape/mandelbulb.rs:13-16; the reference's u64 max_iters fits u32 here). */
typedef struct cg_shape {
    int32_t kind;
    int32_t power;       /* integer power P, 1..255 (Mandelbulb<const P: u8>) */
    float power_f;       /* real power of the polar form */
    uint32_t max_iters;  /* >= 1 (mandelbulb.rs:20) */
    float bailout;
    float rot[3];        /* Euler angles (a,b,c), R = Rz(c) Ry(b) Rx(a), DE(p) = DE0(R^T p) */
    float center[3];     /* Sphere centre */
    float radius;        /* Sphere radius */
} cg_shape;

/* octree::Span = Range<Point3<f32>> (src/octree/mod.rs:13). */
typedef struct cg_span {
    float start[3];
    float end[3];
} cg_span;

/* mesh::Vertex, #[repr(C)], 28 bytes (src/mesh/mod.rs:255-261). */
typedef struct cg_vertex {
    float position[3];
    float normal[3];
    float distance_from_surface;
} cg_vertex;

/* mesh::buffer::Timings (src/mesh/buffer.rs:398-405): stage times in ms. */
typedef struct cg_timings {
    float first_ms;   /* step 1: distances at every corner */
    float second_ms;  /* step 2: surface cells, vertices, normals */
    float third_ms;   /* step 3: quad indices (built beside step 2's vertex placement on
                         the GPU: this is the part that outlasts the placement) */
    uint32_t vertices;
    uint32_t faces;
} cg_timings;

/* ---- library ---------------------------------------------------------- */

/* CG_ABI_VERSION of the loaded library. */
int cg_abi_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char* cg_last_error(void);
/* sizeof(cg_shape), sizeof(cg_vertex): layout check for foreign callers. */
uint32_t cg_sizeof_shape(void);
uint32_t cg_sizeof_vertex(void);

/* ---- distance estimator ----------------------------------------------- */

/* Shape::batch_min_distance_from (src/shape/mod.rs:89; per point
 * Mandelbulb::min_distance_from, src/shape/mandelbulb.rs:59-79).
 * points: device, n x 3 floats (Point3<f32> layout); out: device, n floats. */
cg_status cg_min_distance_from(const cg_shape* shape, const float* points, uint64_t n,
                               float* out, uint32_t numerics, void* stream);

/* Shape::contains (src/shape/mod.rs:78-80; Sphere override
 * src/shape/sphere.rs:24-26).  out: device, n bytes of 0/1. */
cg_status cg_contains(const cg_shape* shape, const float* points, uint64_t n, uint8_t* out,
                      void* stream);

/* Step 1 of naive_surface_nets (src/mesh/buffer.rs:63-83): the span is
 * widened by one cell per side and the DE is evaluated at all (res+1)^3
 * corners.  dists: device, (res+1)^3 floats, x-major, z fastest
 * (GridTable layout, src/util/grid.rs:45-48). */
cg_status cg_de_span_grid(const cg_shape* shape, const cg_span* span, uint32_t resolution,
                          float* dists, uint32_t numerics, void* stream);

/* Mandelbulb loop state at exit, for bit-level parity tests: stale r, dr,
 * rotate steps (uint32 stored as float bits) and escape flag per point.
 * state: device, n x 4 floats. */
cg_status cg_mandelbulb_state(const cg_shape* shape, const float* points, uint64_t n,
                              float* state, void* stream);

/* ---- span mesher -------------------------------------------------------- */

typedef struct cg_mesher cg_mesher;

/* A mesher owns a stream, events and a grow-only device workspace. */
cg_status cg_mesher_create(int device, cg_mesher** out);
void cg_mesher_destroy(cg_mesher* mesher);
/* Select the normals (CG_NORMALS_FD default).  With CG_NORMALS_ADJOINT each
 * vertex's normal is the normalised gradient of the DE there, one
 * forward-mode pass (for Mandelbulb<8> the reference's polynomial,
 * mandelbulb.rs:148-200, in dual numbers); vertex positions, DE values and
 * indices are unchanged, only the normals differ from the reference's
 * six-sample difference. */
cg_status cg_mesher_set_normals(cg_mesher* mesher, uint32_t normals);
/* Select the edge crossings (CG_CROSSINGS_LERP default).  CG_CROSSINGS_ROOT
 * refines each crossing with `iters` (1..16) Illinois steps on the DE along
 * the edge (iters extra estimator calls per crossing edge), the experiment
 * buffer.rs:178-186 suggests; the cell table and index list are unchanged,
 * vertex positions (and so their DE and normals) move onto the surface. */
cg_status cg_mesher_set_crossings(cg_mesher* mesher, uint32_t crossings, uint32_t iters);
/* Select the vertex placement (CG_PLACEMENT_CENTROID default).  With
 * CG_PLACEMENT_QEF each surface cell's vertex minimises sum_i (n_i . (x -
 * p_i))^2 over the crossings p_i (lerped or root-found, as selected) and the
 * unit gradients n_i of the DE there (one forward-mode pass per crossing),
 * by a truncated pseudo-inverse (eigenvalues below 1% of the largest
 * dropped) around the crossings' mass point, clamped to the cell.  The cell
 * table and index list are unchanged; the DE and normal are evaluated at
 * the new position.  Any shape. */
cg_status cg_mesher_set_placement(cg_mesher* mesher, uint32_t placement);
/* Select the estimator's numerics for the whole mesh (CG_NUMERICS_EXACT
 * default: the reference's bits).  CG_NUMERICS_FAST meshes with the fast
 * estimator (see the enum): the corner signs near the surface, and so the
 * cell set, may differ from the reference's.  Only with the default
 * normals, crossings and placement; a mesh with another option set fails
 * with CG_EINVAL. */
cg_status cg_mesher_set_numerics(cg_mesher* mesher, uint32_t numerics);

/* MeshBuffer::generate_for_box (src/mesh/buffer.rs:30-42) into HOST buffers.
 * Writes min(count, cap) items; if a count exceeds its capacity the call
 * returns CG_ECAPACITY with *n_vertices / *n_indices set to the required
 * counts.  timings may be NULL.  Page-locked (cudaHostAlloc / pinned)
 * outputs of meshes above resolution 128 are written by the GPU itself: the
 * vertices by the placement kernel, the indices by a copy beside it (a
 * kernel when both buffers are 16-byte aligned).  Smaller meshes and
 * pageable outputs are meshed into device staging and copied. */
cg_status cg_generate_for_box(cg_mesher* mesher, const cg_span* span, const cg_shape* shape,
                              uint32_t resolution, cg_vertex* vertices, uint64_t vertex_cap,
                              uint32_t* indices, uint64_t index_cap, uint64_t* n_vertices,
                              uint64_t* n_indices, cg_timings* timings);

/* Same, with DEVICE output buffers; the mesh stays on the GPU (replaces the
 * host round trip before MeshView::new, src/mesh/view.rs:23-41). */
cg_status cg_generate_for_box_device(cg_mesher* mesher, const cg_span* span,
                                     const cg_shape* shape, uint32_t resolution,
                                     cg_vertex* vertices, uint64_t vertex_cap, uint32_t* indices,
                                     uint64_t index_cap, uint64_t* n_vertices,
                                     uint64_t* n_indices, cg_timings* timings);

/* generate_for_box for callers that must not allocate device memory:
 * engines whose own allocator owns all device memory, and per-frame LOD
 * loops that cannot take cudaMalloc's synchronisation.  No counterpart in the
 * reference (which allocates Vecs per call).  Uses a fixed 3 MiB __device__
 * workspace inside the library instead of a cg_mesher, so resolution is
 * limited to 64 (cantucci's leaf resolution, src/mesh/mod.rs:133); larger
 * values return CG_EINVAL, and spans and shapes are checked as
 * cg_generate_for_box checks them.  Every GPU that loads the library holds
 * the 3 MiB until exit.  The first call on a device looks the workspace up
 * (cudaGetSymbolAddress) and should come before any stream capture; the
 * address is kept for the life of the device's primary context (after a
 * cudaDeviceReset, load the library anew).  All calls share the workspace:
 * calls that overlap on the GPU race, so serialise them.  Asynchronous on
 * `stream`: counts (DEVICE, 3 x uint32: vertices, quads, status bit 0 = a
 * lerp factor left [0,1], where the reference panics) and the mesh are valid
 * once the stream reaches this point.  The mesh is cut at the capacities:
 * min(counts[0], vertex_cap) vertices and min(6 counts[1], index_cap)
 * indices are written, nothing beyond, and the call still returns CG_OK, so
 * the caller compares counts[0] with vertex_cap and 6 counts[1] with
 * index_cap (and tests bit 0 of counts[2]) before using the mesh. */
cg_status cg_generate_for_box_noalloc(const cg_span* span, const cg_shape* shape,
                                      uint32_t resolution, cg_vertex* vertices,
                                      uint64_t vertex_cap, uint32_t* indices, uint64_t index_cap,
                                      uint32_t* counts, void* stream);

/* Device pointer of the last mesh's corner distances (GridTable `dists` of
 * buffer.rs:78, (res+1)^3 floats), valid until the mesher's next call. */
cg_status cg_mesher_dists(cg_mesher* mesher, const float** dists, uint32_t* resolution);

/* Expands the last mesh's cell -> vertex-id table (GridTable `points` of
 * buffer.rs:113: 0xFFFFFFFF off the surface) into `points`, a DEVICE buffer
 * of res^3 uint32, on the mesher's stream (synchronised before return). */
cg_status cg_mesher_points(cg_mesher* mesher, uint32_t* points);

/* ---- batched meshing ---------------------------------------------------- */

/* One octree leaf to mesh: generate_for_box(&span, shape, resolution). */
typedef struct cg_span_job {
    cg_span span;
    uint32_t resolution;
    uint32_t reserved;
} cg_span_job;

/* Where one span's mesh landed in the batch outputs.  Its indices refer to
 * its own vertices (0-based), exactly as that span's MeshBuffer would. */
typedef struct cg_job_mesh {
    uint64_t vertex_offset;
    uint64_t index_offset;
    uint32_t vertices;
    uint32_t indices;
} cg_job_mesh;

typedef struct cg_batch cg_batch;

/* Plans a batch of spans: the GPU form of ShapeMesh::update's thread pool,
 * which runs one MeshBuffer::generate_for_box job per empty octree leaf
 * (src/mesh/mod.rs:129-161).  Validates every job like generate_for_box
 * (CG_EINVAL naming the job), uploads the span table and allocates the
 * workspace, with room for `vertex_cap` vertices in total.  jobs: HOST. */
cg_status cg_batch_create(int device, const cg_span_job* jobs, uint32_t n_jobs,
                          uint64_t vertex_cap, cg_batch** out);
void cg_batch_destroy(cg_batch* batch);

/* Meshes every span of the batch: one persistent step-1 kernel pulling work
 * from an atomic queue, then steps 2-3 over all spans.  Asynchronous on
 * `stream`, no allocation, no host synchronisation (capturable).  DEVICE
 * outputs: vertices / indices (written up to their capacities), results
 * (n_jobs entries), totals (3 x uint32: vertices, quads, status bit 0 = a
 * lerp factor left [0,1] in some span). */
cg_status cg_batch_mesh(cg_batch* batch, const cg_shape* shape, cg_vertex* vertices,
                        uint64_t vertex_cap, uint32_t* indices, uint64_t index_cap,
                        cg_job_mesh* results, uint32_t* totals, void* stream);

/* Same, replayed from a CUDA graph: the first call (and any call whose
 * arguments or batch options differ from the last) captures cg_batch_mesh
 * into a graph; later calls launch that graph on `stream`. */
cg_status cg_batch_mesh_graph(cg_batch* batch, const cg_shape* shape, cg_vertex* vertices,
                              uint64_t vertex_cap, uint32_t* indices, uint64_t index_cap,
                              cg_job_mesh* results, uint32_t* totals, void* stream);

/* Device pointer of job `job`'s corner distances after a cg_batch_mesh. */
cg_status cg_batch_dists(cg_batch* batch, uint32_t job, const float** dists);

/* Replaces the batch's job list without reallocating, for a caller that
 * meshes a new set of leaves every frame (ShapeMesh::update's job fan-out,
 * src/mesh/mod.rs:125-161).  The list must fit the workspace the batch was
 * created with (no more jobs, corners, sign words, cell words or cell rows),
 * else CG_ECAPACITY; jobs are validated like cg_batch_create's.  The batch
 * must be idle (no cg_batch_mesh of it still running).  jobs: HOST. */
cg_status cg_batch_set_jobs(cg_batch* batch, const cg_span_job* jobs, uint32_t n_jobs);

/* Launch shapes of one batch (no reference counterpart: the reference's
 * thread pool has no such knobs).  None of them changes any output bit.
 *   de_block       threads per block of the persistent step-1 kernel
 *                  (power of two, 64..512; the grid is every block that fits
 *                  on the GPU at once)
 *   de_chunk       step-1 work items a warp takes from the queue per grab
 *                  (1..4096)
 *   brick_min_res  spans with resolution >= this are walked in runs of eight
 *                  2x4x4 corner bricks along z per work item (one sign word
 *                  per row), smaller ones in runs of 32 corners
 *   place_block    threads per block of vertex placement (64, 128, 256) */
typedef struct cg_batch_tuning {
    uint32_t de_block;
    uint32_t de_chunk;
    uint32_t brick_min_res;
    uint32_t place_block;
} cg_batch_tuning;

/* Normals and numerics of the batch's meshes, as cg_mesher_set_normals /
 * cg_mesher_set_numerics for one span (defaults CG_NORMALS_FD and
 * CG_NUMERICS_EXACT, the reference's; CG_NUMERICS_FAST only with the
 * six-sample normals, else cg_batch_mesh fails with CG_EINVAL).  A captured
 * graph is captured again after a change. */
cg_status cg_batch_set_normals(cg_batch* batch, uint32_t normals);
cg_status cg_batch_set_numerics(cg_batch* batch, uint32_t numerics);
cg_status cg_batch_get_tuning(const cg_batch* batch, cg_batch_tuning* tuning);
/* Validates (CG_EINVAL) and applies; re-uploads the span table when
 * brick_min_res changes (synchronous).  Not during a cg_batch_mesh capture. */
cg_status cg_batch_set_tuning(cg_batch* batch, const cg_batch_tuning* tuning);

/* The batch's autotuner: times cg_batch_mesh with these arguments (one
 * untimed run, then the best of `reps` runs, CUDA events on `stream`) over
 * candidate launch shapes by coordinate descent -- brick_min_res in
 * {8, 16, 32, 64, never}, de_block in {128, 256, 512}, de_chunk in
 * {4, 16, 64, 256}, place_block in {64, 128, 256} -- keeps a change only if
 * it is 3% faster, applies the winner to the batch and returns it with its
 * time.  Synchronous; the outputs hold a valid mesh afterwards. */
cg_status cg_batch_autotune(cg_batch* batch, const cg_shape* shape, cg_vertex* vertices,
                            uint64_t vertex_cap, uint32_t* indices, uint64_t index_cap,
                            cg_job_mesh* results, uint32_t* totals, void* stream, uint32_t reps,
                            cg_batch_tuning* best, float* best_ms);

/* ---- sphere tracing ----------------------------------------------------- */

/* March loop of ShapeMesh::get_focii (src/mesh/mod.rs:229-241): for each ray
 * pos += dir * DE(pos) up to max_steps times, hit when DE < epsilon.
 * origins, dirs, hits: device n x 3 floats; hit: device n bytes. */
cg_status cg_march(const cg_shape* shape, const float* origins, const float* dirs, uint64_t n,
                   uint32_t max_steps, float epsilon, float* hits, uint8_t* hit,
                   void* stream);

/* ---- level of detail: ShapeMesh ------------------------------------------ */

/* The camera of src/camera.rs:14-19,175-189: position, look direction
 * (normalised by the callee), vertical field of view (radians), aspect ratio
 * (width / height), near and far plane; up is (0, 0, 1). */
typedef struct cg_view {
    float position[3];
    float direction[3];
    float fov_y;
    float aspect;
    float near_plane;
    float far_plane;
} cg_view;

/* The rays of ShapeMesh::get_focii (src/mesh/mod.rs:205-243): the centres
 * of a focus_points x focus_points grid on the near plane (iter::square
 * order: x outer, y inner, src/util/iter.rs:54-88), moved to world space by
 * the inverse view transform; each ray starts at the camera position.
 * Host arithmetic only (needs no GPU).  origins, dirs: HOST, n^2 x 3 floats. */
cg_status cg_view_focus_rays(const cg_view* view, uint32_t focus_points, float* origins,
                             float* dirs);

typedef struct cg_shape_mesh cg_shape_mesh;

/* ShapeMesh::new (src/mesh/mod.rs:45-78): an octree spanning `bounds` (the
 * shape's bounding_box) with its first two levels split, i.e. 64 empty
 * leaves; leaves are meshed at `resolution` (64 in the reference). */
cg_status cg_shape_mesh_create(int device, const cg_shape* shape, const cg_span* bounds,
                               uint32_t resolution, cg_shape_mesh** out);
void cg_shape_mesh_destroy(cg_shape_mesh* sm);

typedef struct cg_lod_stats {
    uint32_t focii;      /* focus rays that hit the surface */
    uint32_t splits;     /* ready leaves split by this update */
    uint32_t collected;  /* meshes that became ready in this update */
    uint32_t started;    /* mesh jobs started by this update */
    uint32_t active;     /* jobs in flight after this update */
    uint32_t leaves;     /* leaves of the octree after this update */
} cg_lod_stats;

/* ShapeMesh::update (src/mesh/mod.rs:82-178), in the reference's order:
 * (1) the 5 x 5 focus rays are marched on the GPU (100 steps, hit when
 *     DE < 1e-6) and every READY leaf around a hit closer to the camera than
 *     twice the leaf's width is split into eight empty leaves;
 * (2) the meshes of the runs that have finished (with wait != 0, of all
 *     runs, after waiting for them) become ready, each in the leaf around
 *     its span's centre; runs are collected in the order they started;
 * (3) every empty leaf becomes a job: all of them are meshed by one batched
 *     persistent launch chain (the thread pool's generate_for_box jobs),
 *     asynchronously, queued behind the runs still in flight (at most four
 *     runs at a time; beyond that the empty leaves wait for a later
 *     update); those leaves are "requested" until a later update collects
 *     them.
 * stats may be NULL. */
cg_status cg_shape_mesh_update(cg_shape_mesh* sm, const cg_view* view, uint32_t wait,
                               cg_lod_stats* stats);

/* A leaf of the octree.  status: 0 empty, 1 requested, 2 ready.  vertices /
 * indices: DEVICE pointers to the leaf's mesh while ready (NULL otherwise),
 * valid until the next cg_shape_mesh_update or destroy; its indices refer to
 * its own vertices, as the leaf's MeshBuffer would. */
typedef struct cg_leaf {
    cg_span span;
    uint32_t status;
    uint32_t depth;
    const cg_vertex* vertices;
    const uint32_t* indices;
    uint32_t n_vertices;
    uint32_t n_indices;
} cg_leaf;

/* The leaves in the reference's traversal order (Octree::iter pops a stack
 * and pushes children 0..7, src/octree/iter.rs:24-33).  Writes
 * min(count, cap) entries; *count = the number of leaves.  leaves: HOST. */
cg_status cg_shape_mesh_leaves(cg_shape_mesh* sm, cg_leaf* leaves, uint32_t cap,
                               uint32_t* count);

/* The focus points of the last update: hits only, in ray order.  points:
 * HOST, cap x 3 floats; *count = the number of hits. */
cg_status cg_shape_mesh_focii(cg_shape_mesh* sm, float* points, uint32_t cap, uint32_t* count);
/* Normals and numerics of the leaves meshed from the next update on (see
 * cg_batch_set_normals / cg_batch_set_numerics). */
cg_status cg_shape_mesh_set_options(cg_shape_mesh* sm, uint32_t normals, uint32_t numerics);

/* A pinhole camera: eye looking at target, `up` hint, vertical field of view
 * fov_y (radians), width x height pixels (row-major, row 0 at the top). */
typedef struct cg_camera {
    float eye[3];
    float target[3];
    float up[3];
    float fov_y;
    uint32_t width;
    uint32_t height;
} cg_camera;

/* Depth map by sphere tracing every pixel's ray: the march of
 * ShapeMesh::get_focii (src/mesh/mod.rs:229-241) per pixel, hit when
 * DE < eps_scale * t * (pixel angle), at most max_steps steps.  numerics:
 * CG_NUMERICS_EXACT, or CG_NUMERICS_FAST (for the polar form: one branch-free
 * arctangent, SFU powers and sin/cos).
 * depth: device, width*height floats, ray distance t or -1 for a miss. */
cg_status cg_trace_depth(const cg_shape* shape, const cg_camera* camera, uint32_t max_steps,
                         float eps_scale, uint32_t numerics, float* depth, void* stream);

/* Implicit-surface backward of cg_trace_depth for the polar shape: at a hit
 * x = eye + t d, DE(x; theta) = 0 gives dt/dtheta = -(dDE/dtheta) /
 * (grad_x DE . d).  Sums grad_depth[i] * dt_i/d(power, a, b, c) over hit
 * pixels into grad_params (device, 4 floats; per-warp partial sums added in
 * a fixed order, so the result is reproducible).  No reference counterpart.
 * The partial sums (and cg_trace_depth's work-queue counter) live in a
 * scratch buffer of the calling host thread: a call's GPU work waits for
 * the previous call's use of it, on whichever stream that ran.  While
 * `stream` is being captured into a CUDA graph, the call allocates its own
 * (a stream-ordered allocation, captured as a graph node). */
cg_status cg_trace_backward(const cg_shape* shape, const cg_camera* camera, const float* depth,
                            const float* grad_depth, float* grad_params, void* stream);

/* cg_trace_backward with outlier rejection, for fitting (no reference
 * counterpart).  A hit pixel whose depth derivative |dt/dtheta_k| exceeds
 * `cap` for any of the four parameters is left out of the sum.  On the
 * fractal a small share of pixels (a tenth at cap 2 on the power-8.3 map)
 * carry derivatives of 10^2..10^6: the exact derivative of the f32
 * estimator along an orbit that the iteration's chaos makes arbitrarily
 * steep, while the depth itself changes by a small, finite amount over any
 * step an optimiser takes.  Their sum swamps the rest and points away from
 * the finite-difference gradient of the loss; without them it agrees with
 * it (cosine ~0.95).  cap = 0 keeps every pixel, as cg_trace_backward does. */
cg_status cg_trace_backward_capped(const cg_shape* shape, const cg_camera* camera,
                                   const float* depth, const float* grad_depth, float cap,
                                   float* grad_params, void* stream);

/* ---- gradients ---------------------------------------------------------- */

/* Forward + reverse-mode adjoint of the real-power polar estimator
 * (kind CG_SHAPE_MANDELBULB_POLAR, src/shape/mandelbulb.frag:1-39, rotated).
 * No reference counterpart: it replaces the six extra estimator calls of the
 * central-difference normal (src/mesh/buffer.rs:256-266) and gives the
 * parameter gradients for fitting.  Iterates are recomputed from
 * checkpoints, never stored.  max_iters <= 64.
 * out: device, n x 8 floats: DE, dDE/dx, dDE/dy, dDE/dz, dDE/dpower,
 * dDE/da, dDE/db, dDE/dc (Euler angles). */
cg_status cg_de_grad(const cg_shape* shape, const float* points, uint64_t n, float* out,
                     void* stream);

/* The same derivatives in forward (tangent) mode: one pass carries d/dq
 * along x, y, z (and, with CG_GRAD_POWER in flags, d/dpower) next to the
 * iterate, so there is no recompute.  Same out layout as cg_de_grad; without
 * CG_GRAD_POWER, out[4] (dDE/dpower) is 0 and the rest is computed.  With
 * CG_GRAD_FAST the iteration uses the fast polar estimator's arithmetic
 * (CG_NUMERICS_FAST).  Any max_iters >= 1.  No reference counterpart. */
enum { CG_GRAD_POWER = 1, CG_GRAD_FAST = 2 };
cg_status cg_de_grad_tangent(const cg_shape* shape, const float* points, uint64_t n,
                             uint32_t flags, float* out, void* stream);

/* DE and its spatial gradient for any shape, one forward-mode pass per
 * point (the gradient dual contouring uses).  out: device, n x 4 floats:
 * DE (the estimator's, bit for bit), dDE/dx, dDE/dy, dDE/dz.  Mandelbulb
 * P = 8 differentiates rotate_inner_p8_scalar (mandelbulb.rs:148-200) as
 * written; other integer powers the equal polar map; Sphere (p - c) /
 * |p - c|.  No reference counterpart. */
cg_status cg_de_spatial_grad(const cg_shape* shape, const float* points, uint64_t n, float* out,
                             void* stream);

/* Backward of DE over a batch (the autograd.Function backward): given the
 * upstream gradient g (device, n floats), writes g[i] * dDE/dp_i to
 * grad_points (device n x 3, may be NULL) and the sums over i of
 * g[i] * dDE/d(power, a, b, c) to grad_params (device, 4 floats, may be NULL;
 * summed in a fixed order, so the result is reproducible).  Its partial sums
 * use the calling thread's scratch buffer, as cg_trace_backward's do. */
cg_status cg_de_backward(const cg_shape* shape, const float* points, const float* grad_out,
                         uint64_t n, float* grad_points, float* grad_params, void* stream);

/* Central-difference gradient with six estimator calls per point and step h
 * (the normal of src/mesh/buffer.rs:256-266, scaled by 1/2h), any shape.
 * out: device, n x 3 floats. */
cg_status cg_fd_grad(const cg_shape* shape, const float* points, uint64_t n, float h, float* out,
                     void* stream);

/* ---- measurement -------------------------------------------------------- */

/* Process-wide tuning knobs.  "de_grid_kernel": 0 auto, 1 one corner per
 * thread in GridTable order, 2 2x4x4 bricks per warp, 3 (P=8 only) one
 * 4x4x4 brick per warp, two corners per thread with packed f32x2 arithmetic.
 * "place_blocks_per_sm" (1..1024, default 128): the vertex placement's grid.
 * "side_stream_priority" (1 default, or 0): whether meshers created
 * afterwards run their quads and copies on a highest-priority stream.
 * "trace_kernel": 1 work-queue march (default), 0 one pixel per thread.
 * "mesh_graphs" (1 default, or 0): meshes up to resolution 128 (other than
 * dual contouring) replay a CUDA graph the mesher captured for that
 * resolution, shape and option set, the span going in as a parameter block.
 * None of these changes an output bit.  "batch_block", "batch_chunk",
 * "batch_brick_min_res", "batch_place_block": the cg_batch_tuning that
 * batches created afterwards start with (defaults 256, 4, 8, 128). */
cg_status cg_set_option(const char* name, int64_t value);

/* The bounds-checked build (libcantucci_gpu_checked.so, built with
 * -DCG_CHECKED): the number of out-of-range array accesses the mesh path's
 * kernels skipped since the last reset, and the source line of the first
 * (0 if none).  Synchronises the device; reset != 0 clears the counts.  In
 * the normal build it fails with CG_EINVAL. */
cg_status cg_debug_oob(uint64_t* count, uint32_t* line, uint32_t reset);

/* The cudaStream_t (as void*) the mesher launches on, so a caller can time
 * its calls with CUDA events on that stream. */
cg_status cg_mesher_stream(cg_mesher* mesher, void** stream);

/* Work actually done by step 1 on a span grid (the same loop as
 * cg_de_span_grid): total rotate steps and escapes over the (res+1)^3
 * corners of an integer-power Mandelbulb.  Synchronous. */
cg_status cg_span_grid_work(const cg_shape* shape, const cg_span* span, uint32_t resolution,
                            uint64_t* steps, uint64_t* escapes);


#ifdef __cplusplus
}
#endif
#endif
