// noalloc.cu -- span meshing without any device allocation.
//
// Some callers cannot call cudaMalloc at the point where they mesh a span:
//   * engines and frameworks whose own caching allocator has already reserved
//     the device memory and forbids other allocations after start-up;
//   * real-time loops (a renderer's per-frame LOD update, as cantucci's
//     ShapeMesh::update is) that must not hit the implicit device
//     synchronisation and latency spikes of cudaMalloc/cudaFree.
// For them, cg_generate_for_box_noalloc meshes one span of at most
// NOALLOC_MAX_RES cells per axis -- the resolution cantucci uses for every
// octree leaf (RESOLUTION = 64, src/mesh/mod.rs:133) -- using a workspace in a
// file-scope __device__ array instead of a cg_mesher's heap workspace.  The
// caller still provides the output buffers.
//
// The array is part of the module image: every GPU that loads this library
// holds NOALLOC_SCRATCH_BYTES of it until the process exits.  In host code
// the symbol is only a stand-in, not a device address; the device address is
// looked up with cudaGetSymbolAddress, once per device, on the first call
// made with that device current.  That first call should therefore come
// before any stream capture.  The address is valid for the life of the
// device's primary context: a cudaDeviceReset unloads the module, and the
// cached address then no longer names the array.  All calls share the one
// array: two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.
// Everything the kernels read before writing (the mesh counters) is cleared
// by each call.
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

namespace cg {

constexpr uint32_t NOALLOC_MAX_RES = 64;
constexpr size_t NOALLOC_SCRATCH_BYTES = 3u << 20;  // 3 MiB; res 64 needs about 2.3 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
cg_status noalloc_scratch(char** out) {
    int dev = -1;
    CG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) {
        set_error("device %d out of range for the no-allocation workspace", dev);
        return CG_EINVAL;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        CG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = p;
    }
    *out = static_cast<char*>(g_noalloc_ptr[dev]);
    return CG_OK;
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" cg_status cg_generate_for_box_noalloc(const cg_span* span, const cg_shape* shape,
                                                 uint32_t resolution, cg_vertex* vertices,
                                                 uint64_t vertex_cap, uint32_t* indices,
                                                 uint64_t index_cap, uint32_t* counts,
                                                 void* stream) {
    if (!span || !shape || !counts || (vertex_cap && !vertices) || (index_cap && !indices)) {
        set_error("NULL argument");
        return CG_EINVAL;
    }
    // the allocating entry point's checks, then the fixed workspace's cap
    CG_TRY(check_span_res(span, resolution));
    CG_TRY(check_shape(shape));
    if (resolution > NOALLOC_MAX_RES) {
        set_error("cg_generate_for_box_noalloc: resolution %u must be a power of two in [2, %u] "
                  "(its fixed workspace is %zu bytes)",
                  resolution, NOALLOC_MAX_RES, NOALLOC_SCRATCH_BYTES);
        return CG_EINVAL;
    }
    const size_t need = mesh_workspace_layout(resolution, nullptr, nullptr);
    if (need > NOALLOC_SCRATCH_BYTES) {
        set_error("workspace of %zu bytes exceeds the fixed %zu", need, NOALLOC_SCRATCH_BYTES);
        return CG_EINVAL;
    }
    char* base = nullptr;
    CG_TRY(noalloc_scratch(&base));
    MeshWork w;
    mesh_workspace_layout(resolution, base, &w);
    const ShapeDev s = make_shape_dev(*shape);
    const SpanSetup su = setup_span(*span, resolution);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // Step 1 writes every corner; the sign words are then packed by their own
    // kernel, which writes every word, so no stale scratch is read.
    CG_TRY(launch_de_grid(s, make_grid(su, resolution), w.dists, CG_NUMERICS_EXACT, st));
    CG_TRY(launch_mesh_from_dists(s, su, mesh_dims(resolution), w, vertices, vertex_cap, indices,
                                  index_cap, st, nullptr, /*signs_ready=*/false));
    CG_CUDA(cudaMemcpyAsync(counts, w.counters, 3 * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                            st));
    return CG_OK;
}
