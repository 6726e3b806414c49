// cantucci_gpu.hpp -- header-only C++ mirror of cantucci's Shape / Span /
// MeshBuffer API over the C ABI of cantucci_gpu.h.
//
// Names, argument meaning and failure behaviour follow the Rust reference:
//   trait Shape            src/shape/mod.rs:24-105
//   Mandelbulb<const P>    src/shape/mandelbulb.rs:13-91
//   Sphere                 src/shape/sphere.rs:5-52
//   Span, create_spans     src/octree/mod.rs:13-32,315-329
//   MeshBuffer, Timings    src/mesh/buffer.rs:24-42,395-433
//   Vertex                 src/mesh/mod.rs:255-261 (== cg_vertex)
//   Camera, Projection     src/camera.rs:14-190 (the fields the mesher needs)
//   ShapeMesh              src/mesh/mod.rs:24-243 (update; leaves instead of draw)
// Where the reference panics (assert!, lerp outside [0,1]) these throw
// cantucci::Panic.  Link with -lcantucci_gpu -lcudart.
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "cantucci_gpu.h"

namespace cantucci {

struct Panic : std::runtime_error {
    cg_status status;
    Panic(cg_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(cg_status s) {
    if (s != CG_OK) throw Panic(s, std::string("cantucci_gpu: ") + cg_last_error());
}

struct Point3 {
    float x, y, z;
};

using Vertex = cg_vertex;

// octree::Span = Range<Point3<f32>>.
struct Span {
    Point3 start, end;

    // SpanExt::center: start + (end - start) / 2
    Point3 center() const {
        return {start.x + (end.x - start.x) / 2.0f, start.y + (end.y - start.y) / 2.0f,
                start.z + (end.z - start.z) / 2.0f};
    }
    // SpanExt::contains: half-open box test
    bool contains(Point3 p) const {
        return start.x <= p.x && start.y <= p.y && start.z <= p.z && p.x < end.x &&
               p.y < end.y && p.z < end.z;
    }
    cg_span to_c() const { return {{start.x, start.y, start.z}, {end.x, end.y, end.z}}; }
};

// create_spans: the 8 children in Octnode order (bit 2 = upper x half,
// bit 1 = upper y half, bit 0 = upper z half).
inline std::array<Span, 8> create_spans(const Span& p) {
    const Point3 c = p.center();
    std::array<Span, 8> out;
    for (int i = 0; i < 8; ++i) {
        const bool hx = (i >> 2) & 1, hy = (i >> 1) & 1, hz = i & 1;
        out[i].start = {hx ? c.x : p.start.x, hy ? c.y : p.start.y, hz ? c.z : p.start.z};
        out[i].end = {hx ? p.end.x : c.x, hy ? p.end.y : c.y, hz ? p.end.z : c.z};
    }
    return out;
}

// trait Shape, evaluated on the GPU.
class Shape {
public:
    virtual ~Shape() = default;
    virtual cg_shape to_cg_shape() const = 0;
    virtual Span bounding_box() const = 0;

    // Shape::batch_min_distance_from (host points in, host distances out).
    std::vector<float> batch_min_distance_from(const std::vector<Point3>& points) const {
        std::vector<float> out(points.size());
        if (points.empty()) return out;
        float* dp = nullptr;
        float* dd = nullptr;
        const size_t n = points.size();
        if (cudaMalloc(&dp, n * sizeof(Point3)) != cudaSuccess ||
            cudaMalloc(&dd, n * sizeof(float)) != cudaSuccess) {
            cudaFree(dp);
            throw Panic(CG_ENOMEM, "cudaMalloc failed");
        }
        const cg_shape s = to_cg_shape();
        cudaMemcpy(dp, points.data(), n * sizeof(Point3), cudaMemcpyHostToDevice);
        const cg_status st = cg_min_distance_from(&s, dp, n, dd, CG_NUMERICS_EXACT, nullptr);
        if (st == CG_OK) cudaMemcpy(out.data(), dd, n * sizeof(float), cudaMemcpyDeviceToHost);
        cudaFree(dp);
        cudaFree(dd);
        check(st);
        return out;
    }
    float min_distance_from(Point3 p) const { return batch_min_distance_from({p})[0]; }
    // Shape::contains: min_distance_from(p) < 0 (Sphere overrides, as in the reference).
    virtual bool contains(Point3 p) const { return min_distance_from(p) < 0.0f; }
};

template <uint8_t P>
class Mandelbulb : public Shape {
public:
    Mandelbulb(uint64_t max_iters, float bailout) : max_iters_(max_iters), bailout_(bailout) {
        if (max_iters < 1) throw Panic(CG_EINVAL, "assertion failed: max_iters >= 1");
    }
    static Mandelbulb classic(uint64_t max_iters, float bailout) {
        static_assert(P == 8, "classic() is Mandelbulb<8>");
        return Mandelbulb(max_iters, bailout);
    }
    cg_shape to_cg_shape() const override {
        cg_shape s{};
        s.kind = CG_SHAPE_MANDELBULB;
        s.power = P;
        s.power_f = (float)P;
        s.max_iters = (uint32_t)max_iters_;
        s.bailout = bailout_;
        return s;
    }
    Span bounding_box() const override { return {{-1.2f, -1.2f, -1.2f}, {1.2f, 1.2f, 1.2f}}; }

private:
    uint64_t max_iters_;
    float bailout_;
};

class Sphere : public Shape {
public:
    Sphere(Point3 center, float radius) : c_(center), r_(radius) {}
    cg_shape to_cg_shape() const override {
        cg_shape s{};
        s.kind = CG_SHAPE_SPHERE;
        s.max_iters = 1;
        s.center[0] = c_.x;
        s.center[1] = c_.y;
        s.center[2] = c_.z;
        s.radius = r_;
        return s;
    }
    Span bounding_box() const override {
        return {{c_.x + -r_, c_.y + -r_, c_.z + -r_}, {c_.x + r_, c_.y + r_, c_.z + r_}};
    }
    bool contains(Point3 p) const override {
        const float dx = c_.x - p.x, dy = c_.y - p.y, dz = c_.z - p.z;
        return (dx * dx + dy * dy) + dz * dz <= r_ * r_;
    }

private:
    Point3 c_;
    float r_;
};

// mesh::buffer::Timings: stage times in milliseconds.
struct Timings {
    double first = 0, second = 0, third = 0;
    uint32_t vertices = 0, faces = 0;
    Timings operator+(const Timings& o) const {
        return {first + o.first, second + o.second, third + o.third, vertices + o.vertices,
                faces + o.faces};
    }
};

// One cg_mesher per thread (stream + grow-only workspace).
class Mesher {
public:
    explicit Mesher(int device = 0) { check(cg_mesher_create(device, &m_)); }
    ~Mesher() { cg_mesher_destroy(m_); }
    Mesher(const Mesher&) = delete;
    Mesher& operator=(const Mesher&) = delete;
    cg_mesher* get() const { return m_; }

    // CG_NORMALS_FD (the reference's) or CG_NORMALS_ADJOINT (analytic, any shape).
    void set_normals(uint32_t normals) { check(cg_mesher_set_normals(m_, normals)); }
    // CG_CROSSINGS_LERP (the reference's) or CG_CROSSINGS_ROOT with 1..16 steps.
    void set_crossings(uint32_t crossings, uint32_t iters = 4) {
        check(cg_mesher_set_crossings(m_, crossings, iters));
    }
    // CG_PLACEMENT_CENTROID (the reference's) or CG_PLACEMENT_QEF (dual contouring).
    void set_placement(uint32_t placement) { check(cg_mesher_set_placement(m_, placement)); }
    // CG_NUMERICS_EXACT (the reference's bits) or CG_NUMERICS_FAST.
    void set_numerics(uint32_t numerics) { check(cg_mesher_set_numerics(m_, numerics)); }

    static Mesher& for_this_thread() {
        thread_local Mesher m(0);
        return m;
    }

private:
    cg_mesher* m_ = nullptr;
};

struct MeshBuffer {
    std::vector<Vertex> vertices;
    std::vector<uint32_t> indices;

    // MeshBuffer::generate_for_box on the GPU.  Capacity is sized in two
    // phases: CG_ECAPACITY returns the counts and the call is repeated.
    static std::pair<MeshBuffer, Timings> generate_for_box(const Span& span, const Shape& shape,
                                                           uint32_t resolution,
                                                           Mesher& mesher = Mesher::for_this_thread()) {
        const cg_span cs = span.to_c();
        const cg_shape sh = shape.to_cg_shape();
        const uint64_t r3 = (uint64_t)resolution * resolution * resolution;
        MeshBuffer b;
        b.vertices.resize(r3 / 8 + 64);
        b.indices.resize(6 * (r3 / 8 + 64));
        uint64_t nv = 0, ni = 0;
        cg_timings t{};
        for (int attempt = 0; attempt < 2; ++attempt) {
            const cg_status st = cg_generate_for_box(mesher.get(), &cs, &sh, resolution,
                                                     b.vertices.data(), b.vertices.size(),
                                                     b.indices.data(), b.indices.size(), &nv, &ni,
                                                     &t);
            if (st == CG_ECAPACITY && attempt == 0) {
                b.vertices.resize(nv);
                b.indices.resize(ni);
                continue;
            }
            check(st);
            break;
        }
        b.vertices.resize(nv);
        b.indices.resize(ni);
        return {std::move(b), Timings{t.first_ms, t.second_ms, t.third_ms, t.vertices, t.faces}};
    }
};

// Camera + Projection: position, look direction (normalised by the library),
// vertical field of view in radians, aspect ratio, near and far plane.
struct Camera {
    Point3 position{0.0f, -2.5f, 0.0f};
    Point3 direction{0.0f, 1.0f, 0.0f};
    float fov = 1.0471976f;  // 60 degrees
    float aspect_ratio = 1.0f;
    float near_plane = 0.01f, far_plane = 100.0f;

    cg_view to_c() const {
        cg_view v{};
        v.position[0] = position.x;
        v.position[1] = position.y;
        v.position[2] = position.z;
        v.direction[0] = direction.x;
        v.direction[1] = direction.y;
        v.direction[2] = direction.z;
        v.fov_y = fov;
        v.aspect = aspect_ratio;
        v.near_plane = near_plane;
        v.far_plane = far_plane;
        return v;
    }
};

// ShapeMesh: the octree of meshed leaves, refined around the camera's focus
// points; all jobs of an update are one batched GPU run.
class ShapeMesh {
public:
    struct Leaf {
        Span span;
        uint32_t status;  // 0 empty, 1 requested, 2 ready
        uint32_t depth;
        const Vertex* vertices;  // device memory, valid until the next update
        const uint32_t* indices;
        uint32_t n_vertices, n_indices;
    };

    explicit ShapeMesh(const Shape& shape, uint32_t resolution = 64, int device = 0) {
        const cg_shape s = shape.to_cg_shape();
        const cg_span b = shape.bounding_box().to_c();
        check(cg_shape_mesh_create(device, &s, &b, resolution, &sm_));
    }
    ~ShapeMesh() { cg_shape_mesh_destroy(sm_); }
    ShapeMesh(const ShapeMesh&) = delete;
    ShapeMesh& operator=(const ShapeMesh&) = delete;

    // CG_NORMALS_FD / CG_NORMALS_ADJOINT and CG_NUMERICS_EXACT / CG_NUMERICS_FAST
    // for the leaves meshed from the next update on.
    void set_options(uint32_t normals, uint32_t numerics) {
        check(cg_shape_mesh_set_options(sm_, normals, numerics));
    }

    // ShapeMesh::update; wait = block for the jobs started by earlier updates.
    cg_lod_stats update(const Camera& camera, bool wait = false) {
        const cg_view v = camera.to_c();
        cg_lod_stats st{};
        check(cg_shape_mesh_update(sm_, &v, wait ? 1u : 0u, &st));
        return st;
    }

    // The leaves in Octree::iter order.
    std::vector<Leaf> leaves() const {
        uint32_t n = 0;
        check(cg_shape_mesh_leaves(sm_, nullptr, 0, &n));
        std::vector<cg_leaf> raw(n);
        check(cg_shape_mesh_leaves(sm_, raw.data(), n, &n));
        std::vector<Leaf> out;
        out.reserve(n);
        for (const cg_leaf& l : raw)
            out.push_back({{{l.span.start[0], l.span.start[1], l.span.start[2]},
                            {l.span.end[0], l.span.end[1], l.span.end[2]}},
                           l.status, l.depth, l.vertices, l.indices, l.n_vertices, l.n_indices});
        return out;
    }

private:
    cg_shape_mesh* sm_ = nullptr;
};

}  // namespace cantucci
