// de_kernels.cu -- distance-estimator kernels: point batches, span grids,
// contains, loop-state dumps and the get_focii march loop.
#include <cmath>

#include "common.cuh"
#include "de.cuh"
#include "kernels.cuh"
#include "point_io.cuh"

namespace cg {

CG_OOB_READER(de_kernels)

template <int M>
__global__ void __launch_bounds__(256) k_de_points(ShapeDev s, const float* __restrict__ pts,
                                                   uint64_t n, float* __restrict__ out) {
    __shared__ __align__(16) float stage[8][96];
    const WarpWalk w = warp_walk();
    for (uint64_t base = w.first; base < n; base += w.stride) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (load_point_warp(pts, n, base, stage[threadIdx.x >> 5], x, y, z))
            out[base + (threadIdx.x & 31)] = eval<M>(s, x, y, z);
    }
}

// Corner (x, y, z) of a span grid: p = start + across * (v / res)
// (src/mesh/buffer.rs:79-80).  v / res is exact for a power-of-two res, so it
// is formed as v * inv_res.
__device__ __forceinline__ void grid_point(const GridDev& g, uint32_t i, float& px, float& py,
                                           float& pz) {
    const uint32_t z = i % g.n;
    const uint32_t xy = i / g.n;
    const uint32_t y = xy % g.n;
    const uint32_t x = xy / g.n;
    px = __fadd_rn(g.start[0], __fmul_rn(g.across[0], __fmul_rn((float)x, g.inv_res)));
    py = __fadd_rn(g.start[1], __fmul_rn(g.across[1], __fmul_rn((float)y, g.inv_res)));
    pz = __fadd_rn(g.start[2], __fmul_rn(g.across[2], __fmul_rn((float)z, g.inv_res)));
}

__device__ __forceinline__ float grid_coord(const GridDev& g, int k, uint32_t v) {
    return __fadd_rn(g.start[k], __fmul_rn(g.across[k], __fmul_rn((float)v, g.inv_res)));
}

// Small grids: one corner per thread in linear (GridTable) order.  With
// `sgn`, also sets bit z%32 of sign word (x, y, z/32) for positive corners.
template <int M>
__global__ void __launch_bounds__(256) k_de_grid(ShapeDev s, GridDev g, float* __restrict__ out,
                                                 uint32_t* __restrict__ sgn, uint32_t W,
                                                 const GridDev* __restrict__ gp) {
    if (gp) g = *gp;
    const uint32_t total = g.n * g.n * g.n;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        float x, y, z;
        grid_point(g, i, x, y, z);
        const float d = eval<M, true>(s, x, y, z);
        CG_AT(out, i, total) = d;
        if (sgn && !(__float_as_uint(d) >> 31)) {
            const uint32_t zi = i % g.n, row = i / g.n;
            atomicOr(&CG_AT(sgn, row * W + (zi >> 5), (uint64_t)g.n * g.n * W), 1u << (zi & 31));
        }
    }
}

// Large grids: each warp evaluates 2x4x4 bricks of corners (x, y, z), which
// keeps the escape counts of a warp's lanes close (89% lane efficiency on the
// 513^3 span vs 75% for 32 corners along z).  A work unit is a run of
// `group` bricks along z.  With group 8 (grids with work for several waves)
// the unit covers 32 consecutive distances of each of its 8 (x, y) rows
// (whole 128-byte lines) and, with `sgn`, exactly one sign word per row:
// one ballot per brick gives the signs, the z-lane-0 thread of each row
// collects its row's 4 bits per brick and stores the finished word once (no
// atomics; every word is written, padding bits 0).  With group 1 (smaller
// grids, where 8-brick units would leave SMs idle) each brick's 4 bits go
// into the word with atomicOr (sgn zeroed first).
template <int M>
__global__ void __launch_bounds__(256) k_de_grid_brick(ShapeDev s, GridDev g,
                                                       float* __restrict__ out,
                                                       uint32_t* __restrict__ sgn, uint32_t W,
                                                       uint32_t group,
                                                       const GridDev* __restrict__ gp) {
    if (gp) g = *gp;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t n = g.n;
    const uint32_t BX = (n + 1) >> 1, BY = (n + 3) >> 2, BZ = (n + 3) >> 2;
    const uint32_t GZ = (BZ + group - 1) / group;  // units along z
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t dx = lane >> 4, dy = (lane >> 2) & 3, dz = lane & 3;
    // Unit (bx, by, gz), advanced by the grid stride in the same mixed radix.
    const uint32_t u0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t gz = u0 % GZ, by = (u0 / GZ) % BY, bx = u0 / (GZ * BY);
    const uint32_t sz = nwarps % GZ, sy = (nwarps / GZ) % BY, sx = nwarps / (GZ * BY);
    for (; bx < BX;) {
        const uint32_t x = 2 * bx + dx, y = 4 * by + dy;
        const bool row_ok = x < n && y < n;
        const float px = grid_coord(g, 0, x), py = grid_coord(g, 1, y);
        const uint32_t bz0 = gz * group, bz_end = min(bz0 + group, BZ);
        uint32_t word = 0;
        for (uint32_t bz = bz0; bz < bz_end; ++bz) {
            const uint32_t z = 4 * bz + dz;
            bool pos = false;
            if (row_ok && z < n) {
                const float d = eval<M>(s, px, py, grid_coord(g, 2, z));
                CG_AT(out, ((size_t)x * n + y) * n + z, (uint64_t)n * n * n) = d;
                pos = (__float_as_uint(d) >> 31) == 0u;
            }
            if (sgn) {
                const uint32_t b = __ballot_sync(0xFFFFFFFFu, pos);
                word |= ((b >> (lane & ~3u)) & 0xFu) << ((4 * bz) & 31);
            }
        }
        if (sgn && dz == 0 && row_ok) {
            uint32_t* wp = &CG_AT(sgn, (x * n + y) * W + ((4 * bz0) >> 5), (uint64_t)n * n * W);
            if (group == 8) *wp = word;
            else if (word) atomicOr(wp, word);
        }
        gz += sz;
        uint32_t carry = 0;
        if (gz >= GZ) {
            gz -= GZ;
            carry = 1;
        }
        by += sy + carry;
        carry = 0;
        if (by >= BY) {
            by -= BY;
            carry = 1;
        }
        bx += sx + carry;
    }
}

__global__ void __launch_bounds__(256) k_state(ShapeDev s, const float* __restrict__ pts,
                                               uint64_t n, float4* __restrict__ out) {
    __shared__ __align__(16) float stage[8][96];
    const WarpWalk w = warp_walk();
    for (uint64_t base = w.first; base < n; base += w.stride) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (!load_point_warp(pts, n, base, stage[threadIdx.x >> 5], x, y, z)) continue;
        MbState st;
        if (s.power == 8)
            mandelbulb_de<Exact, true>(8, s.max_iters, s.bailout, x, y, z, &st);
        else
            mandelbulb_de<Exact, false>(s.power, s.max_iters, s.bailout, x, y, z, &st);
        out[base + (threadIdx.x & 31)] =
            make_float4(st.r, st.dr, __uint_as_float(st.steps), __uint_as_float(st.escaped));
    }
}

// Shape::contains (src/shape/mod.rs:78-80); Sphere overrides it with
// |c - p|^2 <= r^2 (src/shape/sphere.rs:24-26).
__global__ void __launch_bounds__(256) k_contains(ShapeDev s, const float* __restrict__ pts,
                                                  uint64_t n, uint8_t* __restrict__ out) {
    __shared__ __align__(16) float stage[8][96];
    const WarpWalk w = warp_walk();
    for (uint64_t base = w.first; base < n; base += w.stride) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (!load_point_warp(pts, n, base, stage[threadIdx.x >> 5], x, y, z)) continue;
        const uint64_t i = base + (threadIdx.x & 31);
        bool in;
        if (s.kind == CG_SHAPE_SPHERE) {
            const float dx = __fsub_rn(s.center[0], x), dy = __fsub_rn(s.center[1], y),
                        dz = __fsub_rn(s.center[2], z);
            const float m2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                       __fmul_rn(dz, dz));
            in = m2 <= __fmul_rn(s.radius, s.radius);
        } else {
            in = shape_de(s, x, y, z) < 0.0f;
        }
        out[i] = in ? 1 : 0;
    }
}

// March loop of ShapeMesh::get_focii (src/mesh/mod.rs:229-241).
__global__ void k_march(ShapeDev s, const float* __restrict__ org, const float* __restrict__ dir,
                        uint64_t n, uint32_t max_steps, float eps, float* __restrict__ hits,
                        uint8_t* __restrict__ hit) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float px = org[3 * i], py = org[3 * i + 1], pz = org[3 * i + 2];
        const float dx = dir[3 * i], dy = dir[3 * i + 1], dz = dir[3 * i + 2];
        uint8_t h = 0;
        for (uint32_t k = 0; k < max_steps; ++k) {
            const float d = shape_de(s, px, py, pz);
            px = __fadd_rn(px, __fmul_rn(dx, d));
            py = __fadd_rn(py, __fmul_rn(dy, d));
            pz = __fadd_rn(pz, __fmul_rn(dz, d));
            if (d < eps) {
                h = 1;
                break;
            }
        }
        hits[3 * i] = px;
        hits[3 * i + 1] = py;
        hits[3 * i + 2] = pz;
        hit[i] = h;
    }
}

// Rotate steps and escapes over a span grid (same loop as k_de_grid).
template <bool P8>
__global__ void __launch_bounds__(256) k_grid_work(ShapeDev s, GridDev g,
                                                   unsigned long long* __restrict__ acc) {
    const uint32_t total = g.n * g.n * g.n;
    unsigned long long steps = 0, esc = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += gridDim.x * blockDim.x) {
        float x, y, z;
        grid_point(g, i, x, y, z);
        MbState st;
        mandelbulb_de<Exact, P8>(s.power, s.max_iters, s.bailout, x, y, z, &st);
        steps += st.steps;
        esc += st.escaped;
    }
    for (int o = 16; o > 0; o >>= 1) {
        steps += __shfl_down_sync(0xFFFFFFFFu, steps, o);
        esc += __shfl_down_sync(0xFFFFFFFFu, esc, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], steps);
        atomicAdd(&acc[1], esc);
    }
}

cg_status launch_grid_work(const ShapeDev& s, const GridDev& g, unsigned long long* acc,
                           cudaStream_t st) {
    const uint64_t total = (uint64_t)g.n * g.n * g.n;
    const unsigned B = 256, G = grid_for(total, B, 16);
    if (s.power == 8)
        k_grid_work<true><<<G, B, 0, st>>>(s, g, acc);
    else
        k_grid_work<false><<<G, B, 0, st>>>(s, g, acc);
    CG_CHECK_LAUNCH("k_grid_work");
    return CG_OK;
}


cg_status launch_de_points(const ShapeDev& s, const float* pts, uint64_t n, float* out,
                           uint32_t numerics, cudaStream_t st) {
    if (n == 0) return CG_OK;
    const unsigned B = 256, G = grid_for(n, B, 16);
    switch (mode_of(s, numerics)) {
    case MODE_P8:
        if (p8_unrolled(s)) k_de_points<MODE_P8_IT15><<<G, B, 0, st>>>(s, pts, n, out);
        else k_de_points<MODE_P8><<<G, B, 0, st>>>(s, pts, n, out);
        break;
    case MODE_INT: k_de_points<MODE_INT><<<G, B, 0, st>>>(s, pts, n, out); break;
    case MODE_POLAR: k_de_points<MODE_POLAR><<<G, B, 0, st>>>(s, pts, n, out); break;
    case MODE_SPHERE: k_de_points<MODE_SPHERE><<<G, B, 0, st>>>(s, pts, n, out); break;
    case MODE_INT_POLY: k_de_points<MODE_INT_POLY><<<G, B, 0, st>>>(s, pts, n, out); break;
    case MODE_POLAR_FAST: k_de_points<MODE_POLAR_FAST><<<G, B, 0, st>>>(s, pts, n, out); break;
    default:
        if (p8_unrolled(s)) k_de_points<MODE_P8_FAST_IT15><<<G, B, 0, st>>>(s, pts, n, out);
        else k_de_points<MODE_P8_FAST><<<G, B, 0, st>>>(s, pts, n, out);
        break;
    }
    CG_CHECK_LAUNCH("k_de_points");
    return CG_OK;
}

// P=8 exact, two corners per thread with packed f32x2 instructions: each
// warp evaluates a 4x4x4 brick, lane (dx, dy, dz) taking corners (x, y, z)
// and (x + 2, y, z).  With `sgn` the four z-lanes of each (x, y) row OR their
// sign bits with two shuffles and one lane sets them with atomicOr (sgn must
// be zeroed first).
__global__ void __launch_bounds__(256) k_de_grid_p8x2(ShapeDev s, GridDev g,
                                                      float* __restrict__ out,
                                                      uint32_t* __restrict__ sgn, uint32_t W,
                                                      const GridDev* __restrict__ gp) {
    if (gp) g = *gp;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t n = g.n;
    const uint32_t B4 = (n + 3) >> 2;
    const uint32_t bricks = B4 * B4 * B4;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t dx = lane >> 4, dy = (lane >> 2) & 3, dz = lane & 3;
    for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < bricks; b += nwarps) {
        const uint32_t bz = b % B4, t = b / B4, by = t % B4, bx = t / B4;
        const uint32_t xA = 4 * bx + dx, xB = xA + 2, y = 4 * by + dy, z = 4 * bz + dz;
        const bool inYZ = y < n && z < n;
        const bool liveA = inYZ && xA < n, liveB = inYZ && xB < n;
        const float py = grid_coord(g, 1, y), pz = grid_coord(g, 2, z);
        float dA = 0.0f, dB = 0.0f;
        // Both lanes always iterate a real corner (an inactive lane repeats
        // the other's), so no code path sees a lane that is known to be idle.
        const float pxA = grid_coord(g, 0, liveA ? xA : xB);
        const float pxB = grid_coord(g, 0, liveB ? xB : xA);
        if (liveA || liveB)
            mandelbulb_p8_x2(s.max_iters, s.bailout, true, true, pxA, py, pz, pxB, py, pz, dA, dB);
        uint32_t bitA = 0, bitB = 0;
        if (liveA) {
            out[((size_t)xA * n + y) * n + z] = dA;
            bitA = (__float_as_uint(dA) >> 31) ? 0u : (1u << (z & 31));
        }
        if (liveB) {
            out[((size_t)xB * n + y) * n + z] = dB;
            bitB = (__float_as_uint(dB) >> 31) ? 0u : (1u << (z & 31));
        }
        if (sgn) {
            bitA |= __shfl_xor_sync(0xFFFFFFFFu, bitA, 1);
            bitA |= __shfl_xor_sync(0xFFFFFFFFu, bitA, 2);
            bitB |= __shfl_xor_sync(0xFFFFFFFFu, bitB, 1);
            bitB |= __shfl_xor_sync(0xFFFFFFFFu, bitB, 2);
            if (dz == 0 && bitA) atomicOr(&sgn[(xA * n + y) * W + (z >> 5)], bitA);
            if (dz == 0 && bitB) atomicOr(&sgn[(xB * n + y) * W + (z >> 5)], bitB);
        }
    }
}

// Kernel choice for step 1 (cg_set_option "de_grid_kernel").
static int g_de_grid_kernel = DE_GRID_AUTO;

int de_grid_kernel_option() { return g_de_grid_kernel; }

int set_de_grid_kernel(int v) {
    if (v < DE_GRID_AUTO || v > DE_GRID_PACKED) return 0;
    g_de_grid_kernel = v;
    return 1;
}

template <int M>
static void launch_grid_mode(const ShapeDev& s, const GridDev& g, float* out, uint32_t* sgn,
                             uint32_t W, cudaStream_t st, const GridDev* gp) {
    const unsigned B = 256;
    int k = g_de_grid_kernel;
    // Up to 65^3 corners (res 64, cantucci's leaves) one corner per thread:
    // a warp's DE chain is then the whole time (about 12 us for one
    // 15-iteration evaluation at low occupancy), and the linear kernel's 45
    // registers (5 resident blocks per SM) fit the grid in fewer waves than
    // the bricks' 72 (3 blocks): 19.6 against 23.5 us for the res-64 grid.
    if (k == DE_GRID_AUTO) k = g.n > 65 ? DE_GRID_BRICK : DE_GRID_LINEAR;
    if (k == DE_GRID_PACKED && (M == MODE_P8 || M == MODE_P8_IT15)) {
        const uint64_t b4 = (g.n + 3) >> 2;
        k_de_grid_p8x2<<<grid_for(b4 * b4 * b4 * 32, B, 8), B, 0, st>>>(s, g, out, sgn, W, gp);
    } else if (k != DE_GRID_LINEAR) {
        // 8-brick units when they make at least four waves of resident warps
        // (8 blocks of 256 threads per SM), single bricks otherwise.
        const uint64_t rows = (uint64_t)((g.n + 1) >> 1) * ((g.n + 3) >> 2);
        const uint64_t bz = (g.n + 3) >> 2;
        const uint64_t units8 = rows * ((bz + 7) / 8);
        const uint32_t group = units8 >= 4ull * sm_count() * 8 * (B / 32) ? 8u : 1u;
        const uint64_t units = rows * ((bz + group - 1) / group);
        k_de_grid_brick<M><<<grid_for(units * 32, B, 8), B, 0, st>>>(s, g, out, sgn, W, group, gp);
    } else {
        const uint64_t total = (uint64_t)g.n * g.n * g.n;
        k_de_grid<M><<<grid_for(total, B, 8), B, 0, st>>>(s, g, out, sgn, W, gp);
    }
}

cg_status launch_de_grid(const ShapeDev& s, const GridDev& g, float* out, uint32_t numerics,
                         cudaStream_t st, uint32_t* sgn, uint32_t W, const GridDev* gp) {
    switch (mode_of(s, numerics)) {
    case MODE_P8:
        if (p8_unrolled(s)) launch_grid_mode<MODE_P8_IT15>(s, g, out, sgn, W, st, gp);
        else launch_grid_mode<MODE_P8>(s, g, out, sgn, W, st, gp);
        break;
    case MODE_INT: launch_grid_mode<MODE_INT>(s, g, out, sgn, W, st, gp); break;
    case MODE_POLAR: launch_grid_mode<MODE_POLAR>(s, g, out, sgn, W, st, gp); break;
    case MODE_SPHERE: launch_grid_mode<MODE_SPHERE>(s, g, out, sgn, W, st, gp); break;
    case MODE_INT_POLY: launch_grid_mode<MODE_INT_POLY>(s, g, out, sgn, W, st, gp); break;
    case MODE_POLAR_FAST: launch_grid_mode<MODE_POLAR_FAST>(s, g, out, sgn, W, st, gp); break;
    default:
        if (p8_unrolled(s)) launch_grid_mode<MODE_P8_FAST_IT15>(s, g, out, sgn, W, st, gp);
        else launch_grid_mode<MODE_P8_FAST>(s, g, out, sgn, W, st, gp);
        break;
    }
    CG_CHECK_LAUNCH("k_de_grid");
    return CG_OK;
}

cg_status launch_state(const ShapeDev& s, const float* pts, uint64_t n, float* out,
                       cudaStream_t st) {
    if (n == 0) return CG_OK;
    const unsigned B = 256, G = grid_for(n, B, 16);
    k_state<<<G, B, 0, st>>>(s, pts, n, reinterpret_cast<float4*>(out));
    CG_CHECK_LAUNCH("k_state");
    return CG_OK;
}

cg_status launch_contains(const ShapeDev& s, const float* pts, uint64_t n, uint8_t* out,
                          cudaStream_t st) {
    if (n == 0) return CG_OK;
    const unsigned B = 256, G = grid_for(n, B, 16);
    k_contains<<<G, B, 0, st>>>(s, pts, n, out);
    CG_CHECK_LAUNCH("k_contains");
    return CG_OK;
}

cg_status launch_march(const ShapeDev& s, const float* org, const float* dir, uint64_t n,
                       uint32_t max_steps, float eps, float* hits, uint8_t* hit, cudaStream_t st) {
    if (n == 0) return CG_OK;
    const unsigned B = 128, G = grid_for(n, B, 16);
    k_march<<<G, B, 0, st>>>(s, org, dir, n, max_steps, eps, hits, hit);
    CG_CHECK_LAUNCH("k_march");
    return CG_OK;
}

}  // namespace cg
