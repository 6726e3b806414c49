"""Python mirror of cantucci's Shape / Span / MeshBuffer API over the C ABI.

Names, argument meaning and error behaviour follow the Rust reference:
  Shape (src/shape/mod.rs:24-105), Mandelbulb (src/shape/mandelbulb.rs:13-91),
  Sphere (src/shape/sphere.rs:5-52), Span / create_spans
  (src/octree/mod.rs:13-32,315-329), MeshBuffer::generate_for_box and Timings
  (src/mesh/buffer.rs:24-42,395-433), Vertex (src/mesh/mod.rs:255-261).
Where the reference panics, these raise CantucciError (or AssertionError for
the constructor asserts).  Device arrays are torch CUDA tensors; host arrays
are numpy.  All compute runs in libcantucci_gpu.so; there is no CPU path.
"""
import ctypes as C
import threading

import numpy as np

from . import _ffi
from ._ffi import CantucciError, VERTEX_DTYPE, check, load

__all__ = ["Span", "create_spans", "Shape", "Mandelbulb", "MandelbulbPolar", "Sphere",
           "MeshBuffer", "Timings", "Mesher", "CantucciError", "VERTEX_DTYPE", "march"]


def _torch():
    import torch
    return torch


def _stream_ptr(device=None):
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class Span:
    """octree::Span = Range<Point3<f32>> (src/octree/mod.rs:13)."""

    def __init__(self, start, end):
        self.start = np.asarray(start, np.float32).reshape(3).copy()
        self.end = np.asarray(end, np.float32).reshape(3).copy()

    def center(self):
        """SpanExt::center (src/octree/mod.rs:21-23): start + (end - start) / 2."""
        return self.start + (self.end - self.start) / np.float32(2.0)

    def contains(self, p):
        """SpanExt::contains (src/octree/mod.rs:25-31): half-open box test."""
        p = np.asarray(p, np.float32)
        return bool(np.all(self.start <= p) and np.all(p < self.end))

    def to_c(self):
        s = _ffi.CgSpan()
        for k in range(3):
            s.start[k] = float(self.start[k])
            s.end[k] = float(self.end[k])
        return s

    def __repr__(self):
        return "Span(%s .. %s)" % (self.start.tolist(), self.end.tolist())


def create_spans(parent: Span):
    """create_spans (src/octree/mod.rs:315-329): the 8 children in Octnode order."""
    s, e = parent.start, parent.end
    c = s + (e - s) / np.float32(2.0)
    out = []
    for i in range(8):
        hx, hy, hz = (i >> 2) & 1, (i >> 1) & 1, i & 1
        lo = np.array([c[0] if hx else s[0], c[1] if hy else s[1], c[2] if hz else s[2]], np.float32)
        hi = np.array([e[0] if hx else c[0], e[1] if hy else c[1], e[2] if hz else c[2]], np.float32)
        out.append(Span(lo, hi))
    return out


class Shape:
    """trait Shape (src/shape/mod.rs:24-105), evaluated on the GPU."""

    numerics = _ffi.CG_NUMERICS_EXACT

    def _cshape(self) -> _ffi.CgShape:
        raise NotImplementedError

    def bounding_box(self) -> Span:
        raise NotImplementedError

    def batch_min_distance_from(self, points):
        """Shape::batch_min_distance_from (src/shape/mod.rs:89).

        `points` is an (n, 3) float32 CUDA tensor (result: CUDA tensor) or a
        host array (result: numpy array)."""
        torch = _torch()
        lib = load()
        on_dev = isinstance(points, torch.Tensor) and points.is_cuda
        pts = points if on_dev else torch.as_tensor(np.ascontiguousarray(points, np.float32))
        pts = pts.reshape(-1, 3).to(device="cuda" if not on_dev else pts.device,
                                    dtype=torch.float32).contiguous()
        out = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
        with torch.cuda.device(pts.device):
            check(lib.cg_min_distance_from(C.byref(self._cshape()), C.c_void_p(pts.data_ptr()),
                                           pts.shape[0], C.c_void_p(out.data_ptr()),
                                           self.numerics, _stream_ptr(pts.device)))
        return out if on_dev else out.cpu().numpy()

    def min_distance_from(self, p) -> float:
        """Shape::min_distance_from (src/shape/mod.rs:37) for one point."""
        return float(self.batch_min_distance_from(np.asarray(p, np.float32).reshape(1, 3))[0])

    def batch_contains(self, points):
        """Shape::contains (src/shape/mod.rs:78-80) for many points (bool)."""
        torch = _torch()
        lib = load()
        on_dev = isinstance(points, torch.Tensor) and points.is_cuda
        pts = points if on_dev else torch.as_tensor(np.ascontiguousarray(points, np.float32))
        pts = pts.reshape(-1, 3).to(device="cuda" if not on_dev else pts.device,
                                    dtype=torch.float32).contiguous()
        out = torch.empty(pts.shape[0], dtype=torch.uint8, device=pts.device)
        with torch.cuda.device(pts.device):
            check(lib.cg_contains(C.byref(self._cshape()), C.c_void_p(pts.data_ptr()),
                                  pts.shape[0], C.c_void_p(out.data_ptr()),
                                  _stream_ptr(pts.device)))
        res = out.bool()
        return res if on_dev else res.cpu().numpy()

    def contains(self, p) -> bool:
        return bool(self.batch_contains(np.asarray(p, np.float32).reshape(1, 3))[0])

    def span_grid(self, span: Span, resolution: int, out=None):
        """Step 1 of naive_surface_nets (src/mesh/buffer.rs:63-83) as a
        (res+1)^3 CUDA tensor."""
        torch = _torch()
        n = resolution + 1
        if out is None:
            out = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
        check(load().cg_de_span_grid(C.byref(self._cshape()), C.byref(span.to_c()), resolution,
                                     C.c_void_p(out.data_ptr()), self.numerics,
                                     _stream_ptr(out.device)))
        return out


class Mandelbulb(Shape):
    """Mandelbulb<const P: u8> (src/shape/mandelbulb.rs:13-91)."""

    def __init__(self, power: int = 8, max_iters: int = 15, bailout: float = 2.5):
        # Mandelbulb::new asserts max_iters >= 1 (mandelbulb.rs:20).
        assert max_iters >= 1
        assert 0 <= int(power) <= 255, "P is a u8"
        self.power = int(power)
        self.max_iters = int(max_iters)
        self.bailout = float(np.float32(bailout))

    @classmethod
    def classic(cls, max_iters: int, bailout: float) -> "Mandelbulb":
        """Mandelbulb::<8>::classic (mandelbulb.rs:29-33)."""
        return cls(8, max_iters, bailout)

    def bounding_box(self) -> Span:
        # mandelbulb.rs:53-57
        return Span([-1.2, -1.2, -1.2], [1.2, 1.2, 1.2])

    def fast(self) -> "Mandelbulb":
        """Same shape with fast numerics (not bit-faithful): P=8 FMA-contracted
        with approximate division and square root, other integer powers
        through the trig-free complex-power form."""
        m = Mandelbulb(self.power, self.max_iters, self.bailout)
        m.numerics = _ffi.CG_NUMERICS_FAST
        return m

    def _cshape(self):
        s = _ffi.CgShape()
        s.kind = _ffi.CG_SHAPE_MANDELBULB
        s.power = self.power
        s.power_f = float(self.power)
        s.max_iters = self.max_iters
        s.bailout = self.bailout
        return s

    def __repr__(self):
        return "Mandelbulb<%d>(max_iters=%d, bailout=%g)" % (self.power, self.max_iters,
                                                             self.bailout)


class MandelbulbPolar(Shape):
    """Real-power polar Mandelbulb of src/shape/mandelbulb.frag:1-39, rotated
    by Euler angles (a, b, c): DE(p) = DE0(R^T p), R = Rz(c) Ry(b) Rx(a)."""

    def __init__(self, power: float = 8.0, max_iters: int = 15, bailout: float = 2.5,
                 rotation=(0.0, 0.0, 0.0)):
        assert max_iters >= 1
        self.power = float(np.float32(power))
        self.max_iters = int(max_iters)
        self.bailout = float(np.float32(bailout))
        self.rotation = tuple(float(np.float32(r)) for r in rotation)

    def bounding_box(self) -> Span:
        return Span([-1.2, -1.2, -1.2], [1.2, 1.2, 1.2])

    def fast(self) -> "MandelbulbPolar":
        """Same shape with fast numerics: one branch-free arctangent instead
        of acos and atan2, powers as exp2(P log2 r), SFU sin/cos."""
        m = MandelbulbPolar(self.power, self.max_iters, self.bailout, self.rotation)
        m.numerics = _ffi.CG_NUMERICS_FAST
        return m

    def _cshape(self):
        s = _ffi.CgShape()
        s.kind = _ffi.CG_SHAPE_MANDELBULB_POLAR
        s.power = int(round(self.power))
        s.power_f = self.power
        s.max_iters = self.max_iters
        s.bailout = self.bailout
        for k in range(3):
            s.rot[k] = self.rotation[k]
        return s


class Sphere(Shape):
    """Sphere (src/shape/sphere.rs:5-52)."""

    def __init__(self, center=(0.0, 0.0, 0.0), radius: float = 1.0):
        self.center = np.asarray(center, np.float32).reshape(3).copy()
        self.radius = float(np.float32(radius))

    def bounding_box(self) -> Span:
        r = np.float32(self.radius)
        return Span(self.center + -r, self.center + r)

    def _cshape(self):
        s = _ffi.CgShape()
        s.kind = _ffi.CG_SHAPE_SPHERE
        s.max_iters = 1
        for k in range(3):
            s.center[k] = float(self.center[k])
        s.radius = self.radius
        return s


class Timings:
    """mesh::buffer::Timings (src/mesh/buffer.rs:398-433); stage times in ms."""

    def __init__(self, first=0.0, second=0.0, third=0.0, vertices=0, faces=0):
        self.first, self.second, self.third = first, second, third
        self.vertices, self.faces = vertices, faces

    def __add__(self, o):
        return Timings(self.first + o.first, self.second + o.second, self.third + o.third,
                       self.vertices + o.vertices, self.faces + o.faces)

    def __str__(self):
        return "%9.3fms (%9.3fms, %9.3fms, %9.3fms) => [%6d verts, %6d faces]" % (
            self.first + self.second + self.third, self.first, self.second, self.third,
            self.vertices, self.faces)


class Mesher:
    """Owns a cg_mesher: a CUDA stream, events and a grow-only workspace."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.cg_mesher_create(device, C.byref(h)))
        self.handle = h
        self.device = device
        self.last_status = _ffi.CG_OK

    def close(self):
        if self.handle:
            self._lib.cg_mesher_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_normals(self, mode: str):
        """"fd": the reference's six-sample central difference (default);
        "analytic": the forward-mode gradient, one pass per vertex (any
        shape)."""
        modes = {"fd": _ffi.CG_NORMALS_FD, "analytic": _ffi.CG_NORMALS_ADJOINT}
        check(self._lib.cg_mesher_set_normals(self.handle, modes[mode]))

    def set_crossings(self, mode: str, iters: int = 4):
        """"lerp": the reference's distance-weighted corner lerp (default);
        "root": each crossing at the DE's root along its edge, `iters`
        regula falsi steps (same cells and indices, vertices on the surface)."""
        modes = {"lerp": _ffi.CG_CROSSINGS_LERP, "root": _ffi.CG_CROSSINGS_ROOT}
        check(self._lib.cg_mesher_set_crossings(self.handle, modes[mode], int(iters)))

    def set_placement(self, mode: str):
        """"centroid": the crossings' centroid, naive surface nets (default);
        "qef": dual contouring -- the minimiser of the squared distances to
        the tangent planes at the crossings, clamped to the cell (same cells
        and indices)."""
        modes = {"centroid": _ffi.CG_PLACEMENT_CENTROID, "qef": _ffi.CG_PLACEMENT_QEF}
        check(self._lib.cg_mesher_set_placement(self.handle, modes[mode]))

    def set_numerics(self, mode: str):
        """"exact": the reference's bits (default); "fast": the fast estimator
        for the whole mesh (cells near the surface may differ; default
        normals, crossings and placement only)."""
        modes = {"exact": _ffi.CG_NUMERICS_EXACT, "fast": _ffi.CG_NUMERICS_FAST}
        check(self._lib.cg_mesher_set_numerics(self.handle, modes[mode]))

    def generate(self, span: Span, shape: Shape, resolution: int, vertex_cap=None,
                 index_cap=None, vertices=None, indices=None, strict: bool = True):
        """Mesh into host numpy arrays (pinned torch tensors also accepted).

        With strict=False a CG_ELERP status (a lerp factor outside [0,1],
        where the reference panics) is returned instead of raised; the mesh
        is complete and uses factor 0 on the offending edges."""
        r3 = resolution ** 3
        if vertices is None:
            vertex_cap = r3 if vertex_cap is None else vertex_cap
            vertices = np.empty(vertex_cap, VERTEX_DTYPE)
        if indices is None:
            index_cap = 18 * r3 if index_cap is None else index_cap
            indices = np.empty(index_cap, np.uint32)
        vptr, vcap = _host_ptr(vertices, VERTEX_DTYPE.itemsize)
        iptr, icap = _host_ptr(indices, 4)
        nv, ni = C.c_uint64(), C.c_uint64()
        tm = _ffi.CgTimings()
        st = self._lib.cg_generate_for_box(self.handle, C.byref(span.to_c()),
                                           C.byref(shape._cshape()), resolution, vptr, vcap,
                                           iptr, icap, C.byref(nv), C.byref(ni), C.byref(tm))
        if strict or st != _ffi.CG_ELERP:
            check(st)
        self.last_status = st
        return vertices, indices, nv.value, ni.value, tm

    def generate_device(self, span: Span, shape: Shape, resolution: int, vertices, indices,
                        strict: bool = True):
        """Mesh into CUDA tensors: vertices (cap, 7) float32, indices (cap,) int32/uint32."""
        nv, ni = C.c_uint64(), C.c_uint64()
        tm = _ffi.CgTimings()
        st = self._lib.cg_generate_for_box_device(
            self.handle, C.byref(span.to_c()), C.byref(shape._cshape()), resolution,
            C.c_void_p(vertices.data_ptr()), vertices.shape[0], C.c_void_p(indices.data_ptr()),
            indices.numel(), C.byref(nv), C.byref(ni), C.byref(tm))
        if strict or st != _ffi.CG_ELERP:
            check(st)
        self.last_status = st
        return nv.value, ni.value, tm

    def last_dists(self):
        """The last mesh's corner distances as a CUDA tensor copy."""
        torch = _torch()
        p, r = C.c_void_p(), C.c_uint32()
        check(self._lib.cg_mesher_dists(self.handle, C.byref(p), C.byref(r)))
        n = r.value + 1
        torch.cuda.synchronize(self.device)
        view = torch.as_tensor(_DeviceView(p.value, (n, n, n), "<f4"),
                               device="cuda:%d" % self.device)
        return view.clone()

    def last_points(self):
        """The last mesh's cell -> vertex id table as an int64 CUDA tensor
        (0xFFFFFFFF = off the surface)."""
        torch = _torch()
        p, r = C.c_void_p(), C.c_uint32()
        check(self._lib.cg_mesher_dists(self.handle, C.byref(p), C.byref(r)))
        res = r.value
        out = torch.empty(res ** 3, dtype=torch.int32, device="cuda:%d" % self.device)
        check(self._lib.cg_mesher_points(self.handle, C.c_void_p(out.data_ptr())))
        return (out.to(torch.int64) & 0xFFFFFFFF).reshape(res, res, res)


class _DeviceView:
    """Zero-copy view of library-owned device memory (CUDA array interface)."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (ptr, False), "version": 2}


def _host_ptr(arr, itemsize):
    torch = _torch()
    if isinstance(arr, torch.Tensor):
        return C.c_void_p(arr.data_ptr()), arr.numel() * arr.element_size() // itemsize
    return C.c_void_p(arr.ctypes.data), arr.nbytes // itemsize


_tls = threading.local()


def _default_mesher() -> Mesher:
    m = getattr(_tls, "mesher", None)
    if m is None:
        torch = _torch()
        m = Mesher(torch.cuda.current_device())
        _tls.mesher = m
    return m


class MeshBuffer:
    """MeshBuffer (src/mesh/buffer.rs:24-27): vertices (Vertex records) and
    u32 triangle indices."""

    def __init__(self, vertices, indices):
        self.vertices = vertices
        self.indices = indices

    @staticmethod
    def generate_for_box(span: Span, shape: Shape, resolution: int, mesher: Mesher = None):
        """MeshBuffer::generate_for_box (src/mesh/buffer.rs:30-42) on the GPU.

        Panics of the reference (reversed span, resolution not a power of two,
        lerp factor outside [0,1]) raise CantucciError."""
        m = mesher or _default_mesher()
        verts, idx, nv, ni, tm = m.generate(span, shape, resolution)
        t = Timings(tm.first_ms, tm.second_ms, tm.third_ms, tm.vertices, tm.faces)
        return MeshBuffer(verts[:nv].copy(), idx[:ni].copy()), t


def march(shape: Shape, origins, dirs, max_steps: int = 100, epsilon: float = 1e-6):
    """March loop of ShapeMesh::get_focii (src/mesh/mod.rs:229-241) for a
    batch of rays; returns (hit points, hit flags) as host arrays."""
    torch = _torch()
    o = torch.as_tensor(np.ascontiguousarray(origins, np.float32)).reshape(-1, 3).cuda()
    d = torch.as_tensor(np.ascontiguousarray(dirs, np.float32)).reshape(-1, 3).cuda()
    hits = torch.empty_like(o)
    hit = torch.empty(o.shape[0], dtype=torch.uint8, device=o.device)
    check(load().cg_march(C.byref(shape._cshape()), C.c_void_p(o.data_ptr()),
                          C.c_void_p(d.data_ptr()), o.shape[0], max_steps, epsilon,
                          C.c_void_p(hits.data_ptr()), C.c_void_p(hit.data_ptr()),
                          _stream_ptr(o.device)))
    return hits.cpu().numpy(), hit.bool().cpu().numpy()
