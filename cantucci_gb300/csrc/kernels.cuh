// kernels.cuh -- declarations shared between the kernel translation units
// and the C ABI implementation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "cantucci_gpu.h"
#include "de.cuh"

namespace cg {

// A span grid after the one-cell widening of src/mesh/buffer.rs:64-67.
struct GridDev {
    float start[3];   // widened span start
    float across[3];  // widened span end - start
    float inv_res;    // 1 / res (exact: res is a power of two)
    uint32_t n;       // res + 1 corners per axis
};

// Host-side span set-up, in the reference's f32 operation order.
struct SpanSetup {
    float start[3], end[3];  // widened span
    float across[3];         // end - start (buffer.rs:77)
    float step[3];           // (end - start) / res (buffer.rs:101)
    float delta[3];          // 0.7 * (end - start) / res (buffer.rs:257)
};
SpanSetup setup_span(const cg_span& span, uint32_t res);
GridDev make_grid(const SpanSetup& su, uint32_t res);

cg_status launch_de_points(const ShapeDev& s, const float* pts, uint64_t n, float* out,
                           uint32_t numerics, cudaStream_t st);
// Batched-mesher knobs: "batch_chunk", "batch_block", "batch_brick_min_res".
int set_batch_option(const char* name, int64_t v);

// Step-1 kernel variants (cg_set_option "de_grid_kernel").
enum { DE_GRID_AUTO = 0, DE_GRID_LINEAR = 1, DE_GRID_BRICK = 2, DE_GRID_PACKED = 3 };
#ifdef CG_CHECKED
// Out-of-range counters of each checked translation unit (common.cuh).
void oob_read_mesh(uint64_t* count, uint32_t* line, bool reset);
void oob_read_de_kernels(uint64_t* count, uint32_t* line, bool reset);
void oob_read_scan(uint64_t* count, uint32_t* line, bool reset);
void oob_read_mesh_batch(uint64_t* count, uint32_t* line, bool reset);
#endif
int set_de_grid_kernel(int v);
int de_grid_kernel_option();
uint32_t place_blocks_per_sm();

// Step 1 on a span grid.  With `sgn` (zeroed, (res+1)^2 rows x W words) the
// kernel also packs is_sign_positive of every corner into sign words.
// With `gp` the kernels take the grid from device memory instead of `g`
// (which still fixes the launch shape): a captured graph then serves every
// span of the same resolution.
cg_status launch_de_grid(const ShapeDev& s, const GridDev& g, float* out, uint32_t numerics,
                         cudaStream_t st, uint32_t* sgn = nullptr, uint32_t W = 0,
                         const GridDev* gp = nullptr);
cg_status launch_grid_work(const ShapeDev& s, const GridDev& g, unsigned long long* acc,
                           cudaStream_t st);
cg_status launch_state(const ShapeDev& s, const float* pts, uint64_t n, float* out,
                       cudaStream_t st);
cg_status launch_contains(const ShapeDev& s, const float* pts, uint64_t n, uint8_t* out,
                          cudaStream_t st);
cg_status launch_march(const ShapeDev& s, const float* org, const float* dir, uint64_t n,
                       uint32_t max_steps, float eps, float* hits, uint8_t* hit, cudaStream_t st);
// cg_set_option knobs of the depth-map march (trace.cu).
int set_trace_option(const char* name, int64_t v);
int set_place_option(const char* name, int64_t v);
// cg_set_option knob of the reverse-mode gradient (adjoint.cu): 1 if taken.
int set_adjoint_option(const char* name, int64_t v);
// Shape argument checks of the C ABI (kind, power, max_iters).
cg_status check_shape(const cg_shape* s);
// Span and resolution checks of the meshing entry points (capi.cu).
cg_status check_span_res(const cg_span* span, uint32_t res);

// Counters the mesher kernels write on the device.
struct MeshCounters {
    uint32_t vertices;  // surface cells
    uint32_t quads;     // faces
    uint32_t status;    // bit 0: a lerp factor left [0,1]
    uint32_t edges;     // sign-changing corner edges (dual contouring's edge table)
};
enum : uint32_t { MESH_LERP_FAIL = 1u };

// Device workspace of one span mesh (sizes from mesh_workspace_layout).
struct MeshWork {
    float* dists;        // (res+1)^3 corner distances
    uint32_t* sgn;       // sign words: (res+1)^2 rows x W words
    uint32_t* cellbits;  // surface-cell words: res^2 rows x Wc words
    uint32_t* wordoff;   // vertices before each cell word, within its row
    uint32_t* rowcnt;    // vertices per cell row
    uint32_t* rowoff;    // exclusive scan of rowcnt
    uint32_t* quadcnt;   // quads per corner row
    uint32_t* quadoff;   // exclusive scan of quadcnt
    uint32_t* cellidx;   // cell index of each vertex (capacity res^3)
    uint32_t* scratch;   // scan block sums
    MeshCounters* counters;
};

struct MeshDims {
    uint32_t res, n, W, Wc;
};
MeshDims mesh_dims(uint32_t res);
// Byte size of a workspace for `res`; fills `w` with offsets from `base`.
size_t mesh_workspace_layout(uint32_t res, char* base, MeshWork* w);

struct PlaceParams;  // mesh_rows.cuh

// A grow-only device buffer owned by the caller.
struct DeviceScratch {
    void* ptr = nullptr;
    size_t bytes = 0;
};
cg_status grow_scratch(DeviceScratch* b, size_t bytes);

// Vertex placement options of the span mesher; the defaults are the
// reference's placement.  analytic_normals replaces the
// six-sample normal by the forward-mode gradient; root_iters > 0 places edge
// crossings at the DE's root along each edge; qef places the vertex at the
// dual-contouring minimiser of the crossings' tangent planes.
// With qef the crossings go into an edge table first (one crossing and
// gradient per sign-changing edge, shared by the edge's cells): its per-row
// part lives in edge_rows, its per-edge part in edge_data; both are
// required with qef.
struct PlaceOptions {
    bool analytic_normals = false;
    uint32_t root_iters = 0;
    bool qef = false;
    uint32_t numerics = CG_NUMERICS_EXACT;  // FAST: with none of the options above
    const PlaceParams* pp_dev = nullptr;    // placement parameters in device memory (graphs)
    DeviceScratch* edge_rows = nullptr;
    DeviceScratch* edge_data = nullptr;
};

// Steps 2 and 3 of naive_surface_nets on a filled `dists` grid (and, with
// signs_ready, filled sign words).  Output arrays are written only up to
// their capacity; counts land in w.counters.
// A second stream and a fork / join event pair: with it the quad indices
// are built concurrently with the vertex placement.
struct SideStream {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};
cg_status launch_mesh_from_dists(const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                                 const MeshWork& w, cg_vertex* verts, uint64_t vcap,
                                 uint32_t* idx, uint64_t icap, cudaStream_t st,
                                 cudaEvent_t ev_after_vertices, bool signs_ready,
                                 const PlaceOptions& opt = PlaceOptions(),
                                 const SideStream* side = nullptr);

// The same steps for a mesh whose outputs go to host memory, reordered so
// the transfers overlap the vertex placement: surface cells and both counts
// first (read back: ev_counts is synchronised), then the quad indices into
// `dev_idx` and their copy to `host_idx` on `copy_st` (ev_quads marks the
// end of the indices), while on `st` k_place stores the vertices straight
// into `host_verts`.  Both host buffers are pinned and passed by their
// device-mapped addresses.
cg_status launch_mesh_to_host(const ShapeDev& s, const SpanSetup& su, const MeshDims& d,
                              const MeshWork& w, cg_vertex* host_verts, uint64_t vcap,
                              uint32_t* dev_idx, uint32_t* host_idx, uint64_t icap,
                              cudaStream_t st, cudaStream_t copy_st, cudaEvent_t ev_counts,
                              cudaEvent_t ev_quads, MeshCounters* hcnt,
                              const PlaceOptions& opt);

// Cell -> vertex id table of the last mesh (0xFFFFFFFF off the surface).
cg_status launch_points_table(const MeshDims& d, const MeshWork& w, uint32_t* points,
                              cudaStream_t st);

// Exclusive scan of n uint32 (n <= 16M); the total goes to *total.
cg_status launch_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                                uint32_t* total, cudaStream_t st);
size_t scan_scratch_words(uint32_t n);
// params[k] += the sum over nwarps per-warp partials partial[4 w + k], in a
// fixed order (deterministic parameter gradients).
cg_status launch_sum_partials4(const float* partial, uint32_t nwarps, float* params,
                               cudaStream_t st);
// The calling thread's scratch buffer (at least `floats` words, 16-byte
// aligned: per-warp partial sums, a work-queue counter) for work enqueued
// on `st`; release_partials(p, st) after the last launch that uses it.
cg_status acquire_partials(size_t floats, cudaStream_t st, float** out);
cg_status release_partials(float* partial, cudaStream_t st);

}  // namespace cg
