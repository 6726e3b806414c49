// common.cuh -- error plumbing and launch helpers shared by the kernels.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "cantucci_gpu.h"

namespace cg {

// Last error message of this host thread (cg_last_error()).
void set_error(const char* fmt, ...);
const char* get_error();

inline cg_status cuda_status(cudaError_t e, const char* what, const char* file, int line) {
    if (e == cudaSuccess) return CG_OK;
    set_error("%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? CG_ENOMEM : CG_ECUDA;
}

#define CG_CUDA(call)                                                              \
    do {                                                                           \
        cg_status _st = ::cg::cuda_status((call), #call, __FILE__, __LINE__);      \
        if (_st != CG_OK) return _st;                                              \
    } while (0)

#define CG_CHECK_LAUNCH(name) CG_CUDA(cudaGetLastError())

#define CG_TRY(expr)                                                               \
    do {                                                                           \
        cg_status _st = (expr);                                                    \
        if (_st != CG_OK) return _st;                                              \
    } while (0)

// Array accesses of the mesh path: CG_AT(p, i, n) is p[i] for an array of n
// elements.  In the checked build (-DCG_CHECKED, libcantucci_gpu_checked.so)
// an index at or past n is not performed: the access goes to a scratch
// slot, and the translation unit's counters record it (how many, and the
// source line of the first).  cg_debug_oob() reads and clears them.  No
// trap, so the context stays usable.
#ifdef CG_CHECKED
static __device__ unsigned long long cg_oob_count;
static __device__ unsigned int cg_oob_line;
static __device__ unsigned long long cg_oob_sink[8];

template <class T>
__device__ __forceinline__ T* checked_at(T* p, uint64_t i, uint64_t n, unsigned line) {
    if (i < n) return p + i;
    atomicAdd(&cg_oob_count, 1ull);
    atomicCAS(&cg_oob_line, 0u, line);
    return reinterpret_cast<T*>(cg_oob_sink);
}
#define CG_AT(p, i, n) (*::cg::checked_at((p), (uint64_t)(i), (uint64_t)(n), __LINE__))

// One per translation unit with checked accesses: reads (and with `reset`
// clears) that unit's counters.
#define CG_OOB_READER(name)                                                              \
    void oob_read_##name(uint64_t* count, uint32_t* line, bool reset) {                  \
        unsigned long long c = 0;                                                        \
        unsigned int l = 0;                                                              \
        cudaMemcpyFromSymbol(&c, cg_oob_count, sizeof c);                                \
        cudaMemcpyFromSymbol(&l, cg_oob_line, sizeof l);                                 \
        *count += c;                                                                     \
        if (!*line) *line = l;                                                           \
        if (reset) {                                                                     \
            c = 0;                                                                       \
            l = 0;                                                                       \
            cudaMemcpyToSymbol(cg_oob_count, &c, sizeof c);                              \
            cudaMemcpyToSymbol(cg_oob_line, &l, sizeof l);                               \
        }                                                                                \
    }
#else
#define CG_AT(p, i, n) ((p)[i])
#define CG_OOB_READER(name)
#endif

// Number of SMs of the current device (cached per device).
int sm_count();

// A timing event: while `st` is being captured into a graph, recorded as an
// event node of the graph (so it times the replay), else recorded now.
inline cudaError_t record_event(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
        return cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
    return cudaEventRecord(ev, st);
}

// Grid size for a grid-stride kernel: enough blocks to fill every SM
// `per_sm` times, never more than the work needs.
inline unsigned grid_for(uint64_t n, unsigned block, unsigned per_sm) {
    uint64_t need = (n + block - 1) / block;
    uint64_t cap = (uint64_t)sm_count() * per_sm;
    if (need < 1) need = 1;
    return (unsigned)(need < cap ? need : cap);
}

// Exclusive scan of one value per thread across the CTA (blockDim.x a
// multiple of 32, at most 1024; warp_sums holds 33 words of shared memory);
// the CTA total goes to `total`.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums,
                                                         uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? warp_sums[lane] : 0;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) warp_sums[lane] = wi - w;  // exclusive warp offsets
        if (lane == nw - 1) warp_sums[32] = wi;   // CTA total
    }
    __syncthreads();
    const uint32_t res = warp_sums[warp] + inc - v;
    total = warp_sums[32];
    __syncthreads();
    return res;
}

}  // namespace cg
