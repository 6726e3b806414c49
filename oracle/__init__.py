"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the GPU product never does.  See oracle.h for what is restated
and how far parity is pinned.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

ORC_MANDELBULB = 0
ORC_SPHERE = 1
ORC_MANDELBULB_POLAR = 2

ORC_OK, ORC_EINVAL, ORC_ECAPACITY, ORC_ELERP = 0, 1, 2, 3


class Shape(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("power", C.c_int32),
        ("power_f", C.c_float),
        ("max_iters", C.c_uint32),
        ("bailout", C.c_float),
        ("rot", C.c_float * 3),
        ("center", C.c_float * 3),
        ("radius", C.c_float),
    ]


VERTEX_DTYPE = np.dtype([("position", "<f4", (3,)), ("normal", "<f4", (3,)),
                         ("distance_from_surface", "<f4")])

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        f32p = C.POINTER(C.c_float)
        f64p = C.POINTER(C.c_double)
        u32p = C.POINTER(C.c_uint32)
        u64p = C.POINTER(C.c_uint64)
        sp = C.POINTER(Shape)
        L.orc_min_distance_from.argtypes = [sp, C.c_float, C.c_float, C.c_float]
        L.orc_min_distance_from.restype = C.c_float
        L.orc_contains.argtypes = [sp, C.c_float, C.c_float, C.c_float]
        L.orc_contains.restype = C.c_int
        L.orc_mandelbulb_state.argtypes = [sp, C.c_float, C.c_float, C.c_float, f32p, f32p, u32p, u32p]
        L.orc_batch_min_distance_from.argtypes = [sp, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int]
        L.orc_batch_state.argtypes = [sp, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int]
        L.orc_batch_steps.argtypes = [sp, C.c_void_p, C.c_uint64, u64p, u64p, C.c_int]
        L.orc_de_f64.argtypes = [sp, C.c_double, C.c_double, C.c_double]
        L.orc_de_f64.restype = C.c_double
        L.orc_batch_de_f64.argtypes = [sp, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_de_grad_f64.argtypes = [sp, C.c_double, C.c_double, C.c_double, f64p]
        L.orc_batch_de_grad_f64.argtypes = [sp, C.c_void_p, C.c_uint64, C.c_void_p, C.c_int]
        L.orc_generate_for_box.argtypes = [sp, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                           C.c_uint64, u64p, u64p, C.c_void_p]
        L.orc_generate_for_box.restype = C.c_int
        L.orc_mesh_from_dists.argtypes = [sp, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p,
                                          C.c_uint64, u64p, u64p]
        L.orc_mesh_from_dists.restype = C.c_int
        L.orc_march.argtypes = [sp, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_float,
                                C.c_void_p, C.c_void_p, C.c_int]
        L.orc_create_spans.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_rotation_matrix.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_sizeof_shape.restype = C.c_uint32
        L.orc_sizeof_vertex.restype = C.c_uint32
        assert L.orc_sizeof_shape() == C.sizeof(Shape)
        assert L.orc_sizeof_vertex() == VERTEX_DTYPE.itemsize == 28
        _lib = L
    return _lib


_ref_lib = None


def ref_shader():
    """The reference's own estimator shaders compiled as C++
    (oracle/ref_build.py), or None where neither the reference tree nor an
    earlier build is present."""
    global _ref_lib
    if _ref_lib is None:
        from . import ref_build
        path = ref_build.build()
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_shader_count.restype = C.c_int
        L.ref_shader_de.argtypes = [C.c_int, C.c_void_p, C.c_uint64, C.c_void_p]
        assert L.ref_shader_count() == len(ref_build.CONFIGS)
        _ref_lib = L
    return _ref_lib


def ref_shader_de(config: int, points) -> np.ndarray:
    """shape_de() of ref_build.CONFIGS[config] at each point (float32)."""
    L = ref_shader()
    pts = _f32(points).reshape(-1, 3)
    out = np.empty(len(pts), np.float32)
    L.ref_shader_de(config, pts.ctypes.data, len(pts), out.ctypes.data)
    return out


class RustRefShape(C.Structure):
    """rustref_shape of oracle/rust_build.py's C entry points."""
    _fields_ = [("kind", C.c_int32), ("power", C.c_int32), ("max_iters", C.c_uint64),
                ("bailout", C.c_float), ("center", C.c_float * 3), ("radius", C.c_float)]


RR_OK, RR_ASSERT, RR_CAPACITY, RR_LERP, RR_INDEX, RR_EINVAL = 0, 1, 2, 3, 4, 5
_rust_lib = None


def rust_ref():
    """The reference's own Rust source for the estimator and the mesher,
    translated into C++ by oracle/rust_build.py, or None where neither the
    reference tree nor an earlier build is present."""
    global _rust_lib
    if _rust_lib is None:
        from . import rust_build
        try:
            path = rust_build.build()
        except Exception:  # no compiler for the x86-only source (e.g. an Arm host)
            path = rust_build.LIB if os.path.exists(rust_build.LIB) else None
        if path is None:
            return None
        try:
            L = C.CDLL(path)
        except OSError:  # built on another architecture
            return None
        sp = C.POINTER(RustRefShape)
        L.rustref_de.argtypes = [sp, C.c_void_p, C.c_uint64, C.c_void_p]
        L.rustref_contains.argtypes = [sp, C.c_void_p, C.c_uint64, C.c_void_p]
        L.rustref_generate_for_box.argtypes = [sp, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64,
                                               C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64),
                                               C.POINTER(C.c_uint64), C.c_void_p, C.c_void_p]
        _rust_lib = L
    return _rust_lib


def _rust_shape(shape: Shape) -> RustRefShape:
    r = RustRefShape()
    if shape.kind == ORC_SPHERE:
        r.kind = 1
        for i in range(3):
            r.center[i] = shape.center[i]
        r.radius = shape.radius
    elif shape.kind == ORC_MANDELBULB:
        r.kind = 0
        r.power = shape.power
        r.max_iters = shape.max_iters
        r.bailout = shape.bailout
    else:
        raise ValueError("the reference's Rust source has integer-power Mandelbulbs and Spheres")
    return r


def rust_ref_de(shape: Shape, points) -> np.ndarray:
    """Shape::min_distance_from of the translated reference at each point."""
    pts = _f32(points).reshape(-1, 3)
    out = np.empty(len(pts), np.float32)
    rc = rust_ref().rustref_de(C.byref(_rust_shape(shape)), pts.ctypes.data, len(pts),
                               out.ctypes.data)
    if rc != RR_OK:
        raise RuntimeError("rustref_de failed with %d" % rc)
    return out


def rust_ref_contains(shape: Shape, points) -> np.ndarray:
    pts = _f32(points).reshape(-1, 3)
    out = np.empty(len(pts), np.uint8)
    rc = rust_ref().rustref_contains(C.byref(_rust_shape(shape)), pts.ctypes.data, len(pts),
                                     out.ctypes.data)
    if rc != RR_OK:
        raise RuntimeError("rustref_contains failed with %d" % rc)
    return out.astype(bool)


def rust_ref_generate_for_box(shape: Shape, span, res: int, vcap=None, icap=None):
    """MeshBuffer::generate_for_box of the translated reference.  Returns
    dict(rc, nv, ni, vertices, indices, dists, points); rc RR_LERP means the
    reference panics in lerp (dists and points are still filled)."""
    sp = _f32(span).reshape(6)
    N = res + 1
    vcap = res ** 3 if vcap is None else vcap
    icap = 18 * res ** 3 if icap is None else icap
    verts = np.empty(vcap, VERTEX_DTYPE)
    idx = np.empty(icap, np.uint32)
    dists = np.full(N ** 3, np.nan, np.float32)
    points = np.zeros(res ** 3, np.uint32)
    nv, ni = C.c_uint64(), C.c_uint64()
    rc = rust_ref().rustref_generate_for_box(C.byref(_rust_shape(shape)), sp.ctypes.data, res,
                                             verts.ctypes.data, vcap, idx.ctypes.data, icap,
                                             C.byref(nv), C.byref(ni), dists.ctypes.data,
                                             points.ctypes.data)
    out = dict(rc=rc, nv=nv.value, ni=ni.value, dists=dists.reshape(N, N, N),
               points=points.reshape(res, res, res))
    if rc == RR_OK:
        out["vertices"] = verts[:nv.value].copy()
        out["indices"] = idx[:ni.value].copy()
    return out


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def mandelbulb(power=8, max_iters=15, bailout=2.5) -> Shape:
    s = Shape()
    s.kind = ORC_MANDELBULB
    s.power = int(power)
    s.power_f = float(power)
    s.max_iters = int(max_iters)
    s.bailout = float(bailout)
    return s


def mandelbulb_polar(power=8.0, max_iters=15, bailout=2.5, rot=(0.0, 0.0, 0.0)) -> Shape:
    s = Shape()
    s.kind = ORC_MANDELBULB_POLAR
    s.power = int(round(power))
    s.power_f = float(power)
    s.max_iters = int(max_iters)
    s.bailout = float(bailout)
    for i in range(3):
        s.rot[i] = float(rot[i])
    return s


def sphere(center=(0.0, 0.0, 0.0), radius=1.0) -> Shape:
    s = Shape()
    s.kind = ORC_SPHERE
    for i in range(3):
        s.center[i] = float(center[i])
    s.radius = float(radius)
    return s


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def min_distance_from(shape: Shape, points, nthreads=None) -> np.ndarray:
    pts = _f32(points).reshape(-1, 3)
    out = np.empty(len(pts), np.float32)
    lib().orc_batch_min_distance_from(C.byref(shape), pts.ctypes.data, len(pts), out.ctypes.data,
                                      nthreads or default_threads())
    return out


def contains(shape: Shape, x, y, z) -> bool:
    return bool(lib().orc_contains(C.byref(shape), float(x), float(y), float(z)))


def state(shape: Shape, p):
    r, dr = C.c_float(), C.c_float()
    k, e = C.c_uint32(), C.c_uint32()
    lib().orc_mandelbulb_state(C.byref(shape), float(p[0]), float(p[1]), float(p[2]),
                               C.byref(r), C.byref(dr), C.byref(k), C.byref(e))
    return r.value, dr.value, k.value, e.value


def batch_state(shape: Shape, points, nthreads=None) -> np.ndarray:
    """(n, 4) float32: r, dr, steps (uint32 bits), escaped (uint32 bits)."""
    pts = _f32(points).reshape(-1, 3)
    out = np.empty((len(pts), 4), np.float32)
    lib().orc_batch_state(C.byref(shape), pts.ctypes.data, len(pts), out.ctypes.data,
                          nthreads or default_threads())
    return out


def steps_total(shape: Shape, points, nthreads=None):
    pts = _f32(points).reshape(-1, 3)
    st, es = C.c_uint64(), C.c_uint64()
    lib().orc_batch_steps(C.byref(shape), pts.ctypes.data, len(pts), C.byref(st), C.byref(es),
                          nthreads or default_threads())
    return st.value, es.value


def de_f64(shape: Shape, points, nthreads=None, with_steps=False):
    pts = _f32(points).reshape(-1, 3)
    out = np.empty(len(pts), np.float64)
    steps = np.empty(len(pts), np.uint32) if with_steps else None
    lib().orc_batch_de_f64(C.byref(shape), pts.ctypes.data, len(pts), out.ctypes.data,
                           steps.ctypes.data if with_steps else None,
                           nthreads or default_threads())
    return (out, steps) if with_steps else out


def de_grad_f64(shape: Shape, points, nthreads=None) -> np.ndarray:
    """(n, 8): DE, dDE/dp (3), dDE/dpower, dDE/d(euler) (3)."""
    pts = _f32(points).reshape(-1, 3)
    out = np.empty((len(pts), 8), np.float64)
    lib().orc_batch_de_grad_f64(C.byref(shape), pts.ctypes.data, len(pts), out.ctypes.data,
                                nthreads or default_threads())
    return out


def generate_for_box(shape: Shape, span, res: int, nthreads=None, want_grids=False,
                     vcap=None, icap=None):
    """Returns dict(rc, vertices, indices, dists, points, timings_ms)."""
    sp = _f32(span).reshape(6)
    N = res + 1
    dists = np.empty(N ** 3, np.float32) if want_grids else None
    points = np.empty(res ** 3, np.uint32) if want_grids else None
    vcap = res ** 3 if vcap is None else vcap
    icap = 18 * res ** 3 if icap is None else icap
    verts = np.empty(vcap, VERTEX_DTYPE)
    idx = np.empty(icap, np.uint32)
    nv, ni = C.c_uint64(), C.c_uint64()
    tm = (C.c_double * 3)()
    rc = lib().orc_generate_for_box(
        C.byref(shape), sp.ctypes.data, res, nthreads or default_threads(),
        dists.ctypes.data if want_grids else None, points.ctypes.data if want_grids else None,
        verts.ctypes.data, vcap, idx.ctypes.data, icap, C.byref(nv), C.byref(ni), tm)
    out = dict(rc=rc, nv=nv.value, ni=ni.value, timings_ms=list(tm))
    if rc in (ORC_OK, ORC_ELERP):
        out["vertices"] = verts[:nv.value].copy()
        out["indices"] = idx[:ni.value].copy()
    if want_grids:
        out["dists"] = dists.reshape(N, N, N)
        out["points"] = points.reshape(res, res, res)
    return out


def mesh_from_dists(shape: Shape, span, res: int, dists, nthreads=None, vcap=None, icap=None):
    """Steps 2-3 of generate_for_box on the given (res+1)^3 corner distances.
    Returns dict(rc, nv, ni, vertices, indices, points)."""
    sp = _f32(span).reshape(6)
    d = _f32(dists).reshape(-1)
    assert d.size == (res + 1) ** 3
    points = np.empty(res ** 3, np.uint32)
    vcap = res ** 3 if vcap is None else vcap
    icap = 18 * res ** 3 if icap is None else icap
    verts = np.empty(vcap, VERTEX_DTYPE)
    idx = np.empty(icap, np.uint32)
    nv, ni = C.c_uint64(), C.c_uint64()
    rc = lib().orc_mesh_from_dists(C.byref(shape), sp.ctypes.data, res,
                                   nthreads or default_threads(), d.ctypes.data,
                                   points.ctypes.data, verts.ctypes.data, vcap, idx.ctypes.data,
                                   icap, C.byref(nv), C.byref(ni))
    return dict(rc=rc, nv=nv.value, ni=ni.value, vertices=verts[:nv.value].copy(),
                indices=idx[:ni.value].copy(), points=points.reshape(res, res, res))


def march(shape: Shape, origins, dirs, max_steps=100, epsilon=1e-6, nthreads=None):
    o = _f32(origins).reshape(-1, 3)
    d = _f32(dirs).reshape(-1, 3)
    hits = np.empty_like(o)
    hit = np.empty(len(o), np.uint8)
    lib().orc_march(C.byref(shape), o.ctypes.data, d.ctypes.data, len(o), max_steps, epsilon,
                    hits.ctypes.data, hit.ctypes.data, nthreads or default_threads())
    return hits, hit.astype(bool)


def create_spans(parent):
    p = _f32(parent).reshape(6)
    out = np.empty((8, 6), np.float32)
    lib().orc_create_spans(p.ctypes.data, out.ctypes.data)
    return out


def rotation_matrix(euler):
    e = _f32(euler).reshape(3)
    m = np.empty(9, np.float32)
    lib().orc_rotation_matrix(e.ctypes.data, m.ctypes.data)
    return m.reshape(3, 3)
