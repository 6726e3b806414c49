// point_io.cuh -- warp-cooperative point loads for the per-point kernels.
//
// Points are Point3<f32> triples (12 bytes), so one point per lane is a
// strided 4-byte access.  A warp instead takes 32 consecutive points: 384
// bytes = 24 float4 loads by lanes 0..23 into shared memory, then each lane
// reads its own x, y, z from there (stride 3 words: no bank conflicts).
// Tails and unaligned bases fall back to scalar loads.
#pragma once

#include <cstdint>

namespace cg {

// Loop bounds of a warp-uniform walk over groups of 32 consecutive points.
struct WarpWalk {
    uint64_t first, stride;
};

__device__ __forceinline__ WarpWalk warp_walk() {
    const uint32_t wid = threadIdx.x >> 5;
    return {((uint64_t)blockIdx.x * blockDim.x) + 32ull * wid, (uint64_t)gridDim.x * blockDim.x};
}

// Loads points [base, base + 32) (those below n) into `stage` (96 floats,
// 16-byte aligned) and returns this lane's point.  Call from all 32 lanes.
__device__ __forceinline__ bool load_point_warp(const float* __restrict__ pts, uint64_t n,
                                                uint64_t base, float* __restrict__ stage,
                                                float& x, float& y, float& z) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t left = n - base;
    const uint32_t cnt = left < 32 ? (uint32_t)left : 32u;
    const float* src = pts + 3 * base;
    if (cnt == 32 && (((uintptr_t)src) & 15u) == 0) {
        if (lane < 24)
            reinterpret_cast<float4*>(stage)[lane] = reinterpret_cast<const float4*>(src)[lane];
    } else {
        for (uint32_t i = lane; i < 3 * cnt; i += 32) stage[i] = src[i];
    }
    __syncwarp();
    const bool live = lane < cnt;
    if (live) {
        x = stage[3 * lane];
        y = stage[3 * lane + 1];
        z = stage[3 * lane + 2];
    }
    __syncwarp();
    return live;
}

}  // namespace cg
