"""ctypes binding of the C ABI in include/cantucci_gpu.h.

The library is built in-tree (cantucci_gb300/_lib/libcantucci_gpu.so).
There is no fallback: if it is missing or fails to load, every call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# CANTUCCI_GPU_LIB names another build of the same ABI to load instead (the
# bounds-checked libcantucci_gpu_checked.so in its tests).
LIB_PATH = os.environ.get("CANTUCCI_GPU_LIB") or os.path.join(HERE, "_lib", "libcantucci_gpu.so")

CG_OK, CG_EINVAL, CG_ECAPACITY, CG_ELERP, CG_ECUDA, CG_ENOMEM, CG_ETIMEOUT, CG_ENODEV = range(8)
STATUS_NAMES = {0: "CG_OK", 1: "CG_EINVAL", 2: "CG_ECAPACITY", 3: "CG_ELERP", 4: "CG_ECUDA",
                5: "CG_ENOMEM", 6: "CG_ETIMEOUT", 7: "CG_ENODEV"}

CG_SHAPE_MANDELBULB, CG_SHAPE_SPHERE, CG_SHAPE_MANDELBULB_POLAR = 0, 1, 2
CG_NUMERICS_EXACT, CG_NUMERICS_FAST = 0, 1
CG_NORMALS_FD, CG_NORMALS_ADJOINT = 0, 1
CG_CROSSINGS_LERP, CG_CROSSINGS_ROOT = 0, 1
CG_PLACEMENT_CENTROID, CG_PLACEMENT_QEF = 0, 1


class CgShape(C.Structure):
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


class CgSpan(C.Structure):
    _fields_ = [("start", C.c_float * 3), ("end", C.c_float * 3)]


class CgTimings(C.Structure):
    _fields_ = [("first_ms", C.c_float), ("second_ms", C.c_float), ("third_ms", C.c_float),
                ("vertices", C.c_uint32), ("faces", C.c_uint32)]


class CgCamera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_y", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class CgSpanJob(C.Structure):
    _fields_ = [("span", CgSpan), ("resolution", C.c_uint32), ("reserved", C.c_uint32)]


class CgJobMesh(C.Structure):
    _fields_ = [("vertex_offset", C.c_uint64), ("index_offset", C.c_uint64),
                ("vertices", C.c_uint32), ("indices", C.c_uint32)]


class CgView(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("direction", C.c_float * 3), ("fov_y", C.c_float),
                ("aspect", C.c_float), ("near_plane", C.c_float), ("far_plane", C.c_float)]


class CgLodStats(C.Structure):
    _fields_ = [("focii", C.c_uint32), ("splits", C.c_uint32), ("collected", C.c_uint32),
                ("started", C.c_uint32), ("active", C.c_uint32), ("leaves", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class CgLeaf(C.Structure):
    _fields_ = [("span", CgSpan), ("status", C.c_uint32), ("depth", C.c_uint32),
                ("vertices", C.c_void_p), ("indices", C.c_void_p), ("n_vertices", C.c_uint32),
                ("n_indices", C.c_uint32)]


class CgBatchTuning(C.Structure):
    _fields_ = [("de_block", C.c_uint32), ("de_chunk", C.c_uint32),
                ("brick_min_res", C.c_uint32), ("place_block", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


VERTEX_DTYPE = np.dtype([("position", "<f4", (3,)), ("normal", "<f4", (3,)),
                         ("distance_from_surface", "<f4")])

# Every symbol include/cantucci_gpu.h declares: (name, restype, argtypes).
_vp, _u32, _u64, _f32, _i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int
_shp, _spp, _tmp = C.POINTER(CgShape), C.POINTER(CgSpan), C.POINTER(CgTimings)
SIGNATURES = [
    ("cg_abi_version", _i32, []),
    ("cg_last_error", C.c_char_p, []),
    ("cg_sizeof_shape", _u32, []),
    ("cg_sizeof_vertex", _u32, []),
    ("cg_min_distance_from", _i32, [_shp, _vp, _u64, _vp, _u32, _vp]),
    ("cg_contains", _i32, [_shp, _vp, _u64, _vp, _vp]),
    ("cg_de_span_grid", _i32, [_shp, _spp, _u32, _vp, _u32, _vp]),
    ("cg_mandelbulb_state", _i32, [_shp, _vp, _u64, _vp, _vp]),
    ("cg_mesher_create", _i32, [_i32, C.POINTER(_vp)]),
    ("cg_mesher_destroy", None, [_vp]),
    ("cg_mesher_set_normals", _i32, [_vp, _u32]),
    ("cg_mesher_set_crossings", _i32, [_vp, _u32, _u32]),
    ("cg_mesher_set_placement", _i32, [_vp, _u32]),
    ("cg_mesher_set_numerics", _i32, [_vp, _u32]),
    ("cg_generate_for_box", _i32, [_vp, _spp, _shp, _u32, _vp, _u64, _vp, _u64,
                                   C.POINTER(_u64), C.POINTER(_u64), _tmp]),
    ("cg_generate_for_box_device", _i32, [_vp, _spp, _shp, _u32, _vp, _u64, _vp, _u64,
                                          C.POINTER(_u64), C.POINTER(_u64), _tmp]),
    ("cg_generate_for_box_noalloc", _i32, [_spp, _shp, _u32, _vp, _u64, _vp, _u64, _vp, _vp]),
    ("cg_mesher_dists", _i32, [_vp, C.POINTER(_vp), C.POINTER(_u32)]),
    ("cg_mesher_points", _i32, [_vp, _vp]),
    ("cg_batch_create", _i32, [_i32, _vp, _u32, _u64, C.POINTER(_vp)]),
    ("cg_batch_destroy", None, [_vp]),
    ("cg_batch_mesh", _i32, [_vp, _shp, _vp, _u64, _vp, _u64, _vp, _vp, _vp]),
    ("cg_batch_mesh_graph", _i32, [_vp, _shp, _vp, _u64, _vp, _u64, _vp, _vp, _vp]),
    ("cg_batch_dists", _i32, [_vp, _u32, C.POINTER(_vp)]),
    ("cg_batch_set_jobs", _i32, [_vp, _vp, _u32]),
    ("cg_view_focus_rays", _i32, [C.POINTER(CgView), _u32, _vp, _vp]),
    ("cg_shape_mesh_create", _i32, [_i32, _shp, _spp, _u32, C.POINTER(_vp)]),
    ("cg_shape_mesh_destroy", None, [_vp]),
    ("cg_shape_mesh_update", _i32, [_vp, C.POINTER(CgView), _u32, C.POINTER(CgLodStats)]),
    ("cg_shape_mesh_leaves", _i32, [_vp, C.POINTER(CgLeaf), _u32, C.POINTER(_u32)]),
    ("cg_shape_mesh_focii", _i32, [_vp, _vp, _u32, C.POINTER(_u32)]),
    ("cg_batch_get_tuning", _i32, [_vp, C.POINTER(CgBatchTuning)]),
    ("cg_batch_set_tuning", _i32, [_vp, C.POINTER(CgBatchTuning)]),
    ("cg_batch_set_normals", _i32, [_vp, _u32]),
    ("cg_batch_set_numerics", _i32, [_vp, _u32]),
    ("cg_shape_mesh_set_options", _i32, [_vp, _u32, _u32]),
    ("cg_debug_oob", _i32, [C.POINTER(_u64), C.POINTER(_u32), _u32]),
    ("cg_batch_autotune", _i32, [_vp, _shp, _vp, _u64, _vp, _u64, _vp, _vp, _vp, _u32,
                                 C.POINTER(CgBatchTuning), C.POINTER(_f32)]),
    ("cg_march", _i32, [_shp, _vp, _vp, _u64, _u32, _f32, _vp, _vp, _vp]),
    ("cg_trace_depth", _i32, [_shp, C.c_void_p, _u32, _f32, _u32, _vp, _vp]),
    ("cg_trace_backward", _i32, [_shp, C.c_void_p, _vp, _vp, _vp, _vp]),
    ("cg_trace_backward_capped", _i32, [_shp, C.c_void_p, _vp, _vp, _f32, _vp, _vp]),
    ("cg_de_grad", _i32, [_shp, _vp, _u64, _vp, _vp]),
    ("cg_de_grad_tangent", _i32, [_shp, _vp, _u64, _u32, _vp, _vp]),
    ("cg_de_spatial_grad", _i32, [_shp, _vp, _u64, _vp, _vp]),
    ("cg_de_backward", _i32, [_shp, _vp, _vp, _u64, _vp, _vp, _vp]),
    ("cg_fd_grad", _i32, [_shp, _vp, _u64, _f32, _vp, _vp]),
    ("cg_set_option", _i32, [C.c_char_p, C.c_int64]),
    ("cg_mesher_stream", _i32, [_vp, C.POINTER(_vp)]),
    ("cg_span_grid_work", _i32, [_shp, _spp, _u32, C.POINTER(_u64), C.POINTER(_u64)]),
]

_lib = None


class CantucciError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcantucci_gpu.so is not built; run "
                              "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.cg_sizeof_shape() != C.sizeof(CgShape) or L.cg_sizeof_vertex() != VERTEX_DTYPE.itemsize:
            raise ImportError("cantucci_gpu ABI layout mismatch")
        _lib = L
    return _lib


def check(status: int):
    if status != CG_OK:
        raise CantucciError(status, load().cg_last_error().decode(errors="replace"))
    return status
