// Drives the C++ mirror (include/cantucci_gpu.hpp) the way cantucci's mesh
// thread pool drives MeshBuffer::generate_for_box, and writes what it got.
//   mirror_main <out_dir>  ->  <out_dir>/indices.u32, vertices.f32, de.f32, summary.txt
#include <cstdio>
#include <string>
#include <vector>

#include "cantucci_gpu.hpp"

using namespace cantucci;

static void write(const std::string& path, const void* p, size_t bytes) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    fwrite(p, 1, bytes, f);
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: mirror_main <out_dir>\n");
        return 2;
    }
    const std::string out = argv[1];
    const auto shape = Mandelbulb<8>::classic(15, 2.5f);
    const Span span = shape.bounding_box();
    auto [buf, t] = MeshBuffer::generate_for_box(span, shape, 64);
    write(out + "/indices.u32", buf.indices.data(), buf.indices.size() * 4);
    write(out + "/vertices.f32", buf.vertices.data(), buf.vertices.size() * sizeof(Vertex));

    const std::vector<Point3> pts = {{-0.73772496f, -0.002343091f, -0.7382717f},
                                     {-0.7484558f, -0.8255949f, -0.0026540023f},
                                     {0.0f, 0.0f, 0.0f}};
    const std::vector<float> de = shape.batch_min_distance_from(pts);
    write(out + "/de.f32", de.data(), de.size() * 4);

    int panicked = 0;
    try {  // a reversed span panics in the reference (buffer.rs:35)
        MeshBuffer::generate_for_box({{0, 0, 0}, {-1, 1, 1}}, shape, 8);
    } catch (const Panic& p) {
        panicked = p.status == CG_EINVAL;
    }
    const auto children = create_spans(span);

    // ShapeMesh: two updates from afar mesh the 64 initial leaves; a camera
    // near the surface then splits some of them.
    ShapeMesh lod(shape, 32);
    Camera far_cam;
    far_cam.position = {0.0f, -30.0f, 0.0f};
    lod.update(far_cam, true);
    const cg_lod_stats s2 = lod.update(far_cam, true);
    Camera near_cam;
    near_cam.position = {0.05f, -1.45f, 0.1f};
    near_cam.direction = {0.0f, 1.0f, 0.05f};
    const cg_lod_stats s3 = lod.update(near_cam, true);
    size_t ready = 0;
    for (const auto& l : lod.leaves()) ready += l.status == 2;

    FILE* f = fopen((out + "/summary.txt").c_str(), "w");
    fprintf(f, "%zu %zu %u %u %d %.7g %d %u %u %u %zu\n", buf.vertices.size(), buf.indices.size(),
            t.vertices, t.faces, panicked, children[3].start.y,
            (int)Sphere({0, 0, 0}, 1.0f).contains({0.5f, 0, 0}), s2.collected, s3.splits,
            s3.leaves, ready);
    fclose(f);
    return 0;
}
