// scan.cu -- device-wide exclusive prefix sum of uint32 counts, used to turn
// per-row surface-cell and quad counts into vertex and index offsets in the
// reference's cube() order (src/util/iter.rs:31-51).
//
// Three launches: per-tile sums, one-CTA scan of the tile sums, per-tile scan
// plus offset; one launch when the counts fit one tile.  Tiles are 4096
// counts (1024 threads x 4), so one top-level CTA covers 4096 tiles = 16M
// counts, enough for res^2 rows at res <= 1024.
#include "common.cuh"
#include "kernels.cuh"

namespace cg {

CG_OOB_READER(scan)

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ in,
                                                              uint32_t n,
                                                              uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t ws[33];
    const uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += CG_AT(in, base + k, n);
    uint32_t total;
    block_exclusive_scan(s, ws, total);
    if (threadIdx.x == 0) CG_AT(tile_sums, blockIdx.x, gridDim.x) = total;
}

// One CTA: exclusive scan of the tile sums in place, total to *total.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_top(uint32_t* __restrict__ tile_sums,
                                                           uint32_t ntiles,
                                                           uint32_t* __restrict__ total) {
    __shared__ uint32_t ws[33];
    const uint32_t base = threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < ntiles) ? CG_AT(tile_sums, base + k, ntiles) : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t off = block_exclusive_scan(s, ws, tot);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < ntiles) CG_AT(tile_sums, base + k, ntiles) = off;
        off += v[k];
    }
    if (threadIdx.x == 0) *total = tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const uint32_t* __restrict__ in,
                                                            uint32_t n,
                                                            const uint32_t* __restrict__ tile_off,
                                                            uint32_t* __restrict__ out) {
    __shared__ uint32_t ws[33];
    const uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < n) ? CG_AT(in, base + k, n) : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t off = block_exclusive_scan(s, ws, tot) + tile_off[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) CG_AT(out, base + k, n) = off;
        off += v[k];
    }
}

// n <= SCAN_TILE (rows of a span up to res 64): the whole scan in one CTA.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile(const uint32_t* __restrict__ in,
                                                            uint32_t n, uint32_t* __restrict__ out,
                                                            uint32_t* __restrict__ total) {
    __shared__ uint32_t ws[33];
    const uint32_t base = threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < n) ? CG_AT(in, base + k, n) : 0;
        s += v[k];
    }
    uint32_t tot;
    uint32_t off = block_exclusive_scan(s, ws, tot);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) CG_AT(out, base + k, n) = off;
        off += v[k];
    }
    if (threadIdx.x == 0) *total = tot;
}

size_t scan_scratch_words(uint32_t n) {
    return (n + SCAN_TILE - 1) / SCAN_TILE + 1;
}

cg_status launch_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                                uint32_t* total, cudaStream_t st) {
    const uint32_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (ntiles > SCAN_TILE) {
        set_error("exclusive scan of %u counts exceeds the %u-count limit", n,
                  SCAN_TILE * SCAN_TILE);
        return CG_EINVAL;
    }
    if (n == 0) {
        CG_CUDA(cudaMemsetAsync(total, 0, sizeof(uint32_t), st));
        return CG_OK;
    }
    if (ntiles == 1) {
        k_scan_tile<<<1, SCAN_THREADS, 0, st>>>(in, n, out, total);
        CG_CHECK_LAUNCH("k_scan_tile");
        return CG_OK;
    }
    k_scan_reduce<<<ntiles, SCAN_THREADS, 0, st>>>(in, n, scratch);
    CG_CHECK_LAUNCH("k_scan_reduce");
    k_scan_top<<<1, SCAN_THREADS, 0, st>>>(scratch, ntiles, total);
    CG_CHECK_LAUNCH("k_scan_top");
    k_scan_down<<<ntiles, SCAN_THREADS, 0, st>>>(in, n, scratch, out);
    CG_CHECK_LAUNCH("k_scan_down");
    return CG_OK;
}

}  // namespace cg
