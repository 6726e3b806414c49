// leaf_pool.cpp -- the reference's call pattern for meshing octree leaves,
// as a native thread pool: ShapeMesh::update hands every empty leaf to a
// ThreadPool worker, which calls MeshBuffer::generate_for_box(span, shape, 64)
// into freshly owned Vecs (src/mesh/mod.rs:58-63,129-148).  Here T std::threads
// each own a cg_mesher and call the blocking cg_generate_for_box per leaf into
// pageable std::vectors (or, for comparison, pinned or device buffers).
// Benchmark instrumentation for bench.py; not part of the C ABI.
//
//   cg_leaf_pool <spans.f32> <pageable|pinned|device> <rounds> <T> [<T> ...]
//
// spans.f32 holds n x 6 floats (start xyz, end xyz).  Prints one JSON object
// per thread count: leaves/s and ms per leaf over `rounds` passes over all
// leaves, after one untimed pass.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "cantucci_gpu.h"

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s spans.f32 pageable|pinned|device rounds T...\n", argv[0]);
        return 2;
    }
    std::vector<cg_span> leaves;
    {
        FILE* f = std::fopen(argv[1], "rb");
        if (!f) return 2;
        float b[6];
        while (std::fread(b, sizeof(float), 6, f) == 6) {
            cg_span s;
            std::memcpy(s.start, b, 3 * sizeof(float));
            std::memcpy(s.end, b + 3, 3 * sizeof(float));
            leaves.push_back(s);
        }
        std::fclose(f);
    }
    const char* mode = argv[2];
    const int rounds = std::atoi(argv[3]);
    if (leaves.empty() || rounds < 1) return 2;
    cg_shape sh;
    std::memset(&sh, 0, sizeof sh);
    sh.kind = CG_SHAPE_MANDELBULB;
    sh.power = 8;
    sh.power_f = 8.0f;
    sh.max_iters = 15;
    sh.bailout = 2.5f;
    const uint32_t res = 64;
    const uint64_t vcap = (uint64_t)res * res * res / 4, icap = 18ull * res * res * res / 4;
    for (int a = 4; a < argc; ++a) {
        const int T = std::atoi(argv[a]);
        if (T < 1) return 2;
        std::vector<cg_mesher*> ms(T, nullptr);
        std::vector<std::vector<cg_vertex>> vb(T);
        std::vector<std::vector<uint32_t>> ib(T);
        std::vector<void*> ov(T, nullptr), oi(T, nullptr);
        for (int t = 0; t < T; ++t) {
            if (cg_mesher_create(0, &ms[t]) != CG_OK) return 1;
            if (!std::strcmp(mode, "pinned")) {
                if (cudaMallocHost(&ov[t], vcap * sizeof(cg_vertex)) != cudaSuccess ||
                    cudaMallocHost(&oi[t], icap * sizeof(uint32_t)) != cudaSuccess)
                    return 1;
            } else if (!std::strcmp(mode, "device")) {
                if (cudaMalloc(&ov[t], vcap * sizeof(cg_vertex)) != cudaSuccess ||
                    cudaMalloc(&oi[t], icap * sizeof(uint32_t)) != cudaSuccess)
                    return 1;
            } else {
                vb[t].resize(vcap);
                ib[t].resize(icap);
                ov[t] = vb[t].data();
                oi[t] = ib[t].data();
            }
        }
        std::atomic<int> failed{0};
        std::atomic<uint64_t> verts{0};
        auto work = [&](int t, int passes) {
            uint64_t v = 0;
            for (int p = 0; p < passes; ++p) {
                for (size_t j = t; j < leaves.size(); j += T) {
                    uint64_t nv = 0, ni = 0;
                    const cg_status st =
                        !std::strcmp(mode, "device")
                            ? cg_generate_for_box_device(ms[t], &leaves[j], &sh, res,
                                                         (cg_vertex*)ov[t], vcap, (uint32_t*)oi[t],
                                                         icap, &nv, &ni, nullptr)
                            : cg_generate_for_box(ms[t], &leaves[j], &sh, res, (cg_vertex*)ov[t],
                                                  vcap, (uint32_t*)oi[t], icap, &nv, &ni,
                                                  nullptr);
                    if (st != CG_OK && st != CG_ELERP) failed++;
                    v += nv;
                }
            }
            verts += v;
        };
        {
            std::vector<std::thread> th;
            for (int t = 0; t < T; ++t) th.emplace_back(work, t, 1);
            for (auto& x : th) x.join();
        }
        verts = 0;
        const auto t0 = std::chrono::steady_clock::now();
        {
            std::vector<std::thread> th;
            for (int t = 0; t < T; ++t) th.emplace_back(work, t, rounds);
            for (auto& x : th) x.join();
        }
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        const double n = (double)rounds * leaves.size();
        std::printf("{\"mode\": \"%s\", \"threads\": %d, \"leaves_per_s\": %.1f, "
                    "\"ms_per_leaf\": %.4f, \"vertices_per_pass\": %llu, \"failed\": %d}\n",
                    mode, T, n / s, 1e3 * s / n, (unsigned long long)(verts / rounds),
                    failed.load());
        std::fflush(stdout);
        for (int t = 0; t < T; ++t) {
            if (!std::strcmp(mode, "pinned")) {
                cudaFreeHost(ov[t]);
                cudaFreeHost(oi[t]);
            } else if (!std::strcmp(mode, "device")) {
                cudaFree(ov[t]);
                cudaFree(oi[t]);
            }
            cg_mesher_destroy(ms[t]);
        }
    }
    return 0;
}
