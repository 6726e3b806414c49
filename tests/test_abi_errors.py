"""Invalid arguments come back as a status, never as a crash (no GPU needed:
every call here is rejected before any device work)."""
import ctypes as C

import pytest


@pytest.fixture(scope="module")
def L():
    from cantucci_gb300 import _ffi, build
    build.build()
    return _ffi.load()


def test_null_handles_and_buffers(L):
    from cantucci_gb300 import _ffi
    EINVAL = _ffi.CG_EINVAL
    shape = _ffi.CgShape()
    shape.kind = _ffi.CG_SHAPE_MANDELBULB
    shape.power, shape.max_iters, shape.bailout = 8, 15, 2.5
    span = _ffi.CgSpan((C.c_float * 3)(-1, -1, -1), (C.c_float * 3)(1, 1, 1))
    n = C.c_uint64()
    u32 = C.c_uint32()
    assert L.cg_generate_for_box(None, C.byref(span), C.byref(shape), 8, None, 0, None, 0,
                                 C.byref(n), C.byref(n), None) == EINVAL
    assert L.cg_generate_for_box_device(None, C.byref(span), C.byref(shape), 8, None, 0, None,
                                        0, C.byref(n), C.byref(n), None) == EINVAL
    assert L.cg_mesher_set_normals(None, 0) == EINVAL
    assert L.cg_mesher_set_crossings(None, 0, 0) == EINVAL
    assert L.cg_mesher_dists(None, None, None) == EINVAL
    assert L.cg_batch_mesh(None, C.byref(shape), None, 0, None, 0, None, None, None) == EINVAL
    assert L.cg_batch_set_jobs(None, None, 0) == EINVAL
    assert L.cg_batch_get_tuning(None, None) == EINVAL
    assert L.cg_batch_set_tuning(None, None) == EINVAL
    assert L.cg_batch_autotune(None, C.byref(shape), None, 0, None, 0, None, None, None, 1,
                               None, None) == EINVAL
    assert L.cg_shape_mesh_update(None, None, 0, None) == EINVAL
    assert L.cg_shape_mesh_leaves(None, None, 0, C.byref(u32)) == EINVAL
    assert L.cg_shape_mesh_focii(None, None, 0, C.byref(u32)) == EINVAL
    assert L.cg_mesher_stream(None, None) == EINVAL
    # destroy functions accept NULL
    L.cg_mesher_destroy(None)
    L.cg_batch_destroy(None)
    L.cg_shape_mesh_destroy(None)


def test_bad_shapes_and_spans(L):
    from cantucci_gb300 import _ffi
    EINVAL = _ffi.CG_EINVAL
    shape = _ffi.CgShape()
    shape.kind = 7  # unknown
    assert L.cg_min_distance_from(C.byref(shape), None, 0, None, 0, None) == EINVAL
    shape.kind = _ffi.CG_SHAPE_MANDELBULB
    shape.power, shape.max_iters = 300, 15  # not a u8
    assert L.cg_min_distance_from(C.byref(shape), None, 0, None, 0, None) == EINVAL
    shape.power, shape.max_iters = 8, 0  # Mandelbulb::new asserts max_iters >= 1
    assert L.cg_contains(C.byref(shape), None, 0, None, None) == EINVAL
    shape.max_iters = 15
    # gradients need the polar form
    assert L.cg_de_grad(C.byref(shape), None, 4, None, None) == EINVAL
    assert L.cg_de_grad_tangent(C.byref(shape), None, 4, 1, None, None) == EINVAL
    # reversed span / non-power-of-two resolution (buffer.rs:35-39)
    bad = _ffi.CgSpan((C.c_float * 3)(1, 0, 0), (C.c_float * 3)(-1, 1, 1))
    ok = _ffi.CgSpan((C.c_float * 3)(-1, -1, -1), (C.c_float * 3)(1, 1, 1))
    assert L.cg_de_span_grid(C.byref(shape), C.byref(bad), 8, None, 0, None) == EINVAL
    assert L.cg_de_span_grid(C.byref(shape), C.byref(ok), 12, None, 0, None) == EINVAL
    job = _ffi.CgSpanJob(bad, 8, 0)
    h = C.c_void_p()
    assert L.cg_batch_create(0, C.byref(job), 1, 64, C.byref(h)) == EINVAL
    job = _ffi.CgSpanJob(ok, 3, 0)
    assert L.cg_batch_create(0, C.byref(job), 1, 64, C.byref(h)) == EINVAL
    assert L.cg_shape_mesh_create(0, C.byref(shape), C.byref(ok), 48, C.byref(h)) == EINVAL
    assert L.cg_shape_mesh_create(0, C.byref(shape), C.byref(bad), 64, C.byref(h)) == EINVAL
    assert L.cg_set_option(b"no_such_option", 1) == EINVAL
    assert L.cg_set_option(b"batch_block", 96) == EINVAL
    assert L.cg_set_option(b"trace_kernel", 2) == EINVAL
    assert b"" != L.cg_last_error()
