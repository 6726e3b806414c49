"""Host side of the level-of-detail driver (no GPU): the focus rays the
library computes for a camera against the oracle's restatement of
camera.rs + cgmath, and the oracle's octree model itself."""
import math

import numpy as np
import pytest


CAMERAS = [
    dict(position=(0.0, -2.5, 0.0), direction=(0.0, 1.0, 0.0), fov=math.radians(60), aspect=1.0,
         near=0.01),
    dict(position=(1.3, -0.7, 0.4), direction=(-1.0, 0.5, -0.2), fov=math.radians(45),
         aspect=16 / 9, near=0.05),
    dict(position=(0.1, 0.2, 1.9), direction=(0.05, -0.1, -1.0), fov=math.radians(80),
         aspect=0.75, near=0.001),
]


@pytest.fixture(scope="module")
def lib_loaded():
    from cantucci_gb300 import build
    build.build()


@pytest.mark.parametrize("cam", CAMERAS)
def test_focus_rays_match_oracle(lib_loaded, cam):
    from cantucci_gb300 import lod
    from oracle import lod as olod
    c = lod.Camera(cam["position"], cam["direction"], cam["fov"], cam["aspect"], cam["near"])
    org, d = lod.focus_rays(c, 5)
    oorg, od = olod.focus_rays(cam["position"], cam["direction"], cam["fov"], cam["aspect"],
                               cam["near"], 5)
    np.testing.assert_array_equal(org, oorg)
    # tan() of the library and numpy may differ in the last bit
    np.testing.assert_allclose(d, od, rtol=0, atol=3e-7)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    # iter::square order: x outer, y inner -> the middle ray looks along the view direction
    mid = d[12]
    want = np.asarray(cam["direction"], np.float64)
    assert np.dot(mid, want / np.linalg.norm(want)) > 0.999999


def test_focus_rays_reject_bad_view(lib_loaded):
    import ctypes as C
    from cantucci_gb300 import _ffi, lod
    o = np.zeros((25, 3), np.float32)
    for bad in [lod.Camera(direction=(0, 0, 0)), lod.Camera(fov=0.0), lod.Camera(near=0.0)]:
        st = _ffi.load().cg_view_focus_rays(C.byref(bad.to_c()), 5, o.ctypes.data, o.ctypes.data)
        assert st == _ffi.CG_EINVAL


def test_model_tree_starts_with_64_leaves():
    from oracle import lod as olod
    t = olod.Octree([-1.2, -1.2, -1.2, 1.2, 1.2, 1.2])
    leaves = t.leaves()
    assert len(leaves) == 64 and all(t.depth[i] == 2 for i in leaves)
    # the leaves tile the root: volumes add up, and each centre finds its own leaf
    vol = sum(np.prod(t.span[i][3:] - t.span[i][:3]) for i in leaves)
    assert abs(vol - 2.4 ** 3) < 1e-4
    for i in leaves:
        c = t.span[i][:3] + (t.span[i][3:] - t.span[i][:3]) / np.float32(2)
        assert t.leaf_around(c) == i
    # Octree::iter pops the last pushed child first: the first leaf is the (+x,+y,+z) corner
    assert np.all(t.span[leaves[0]][3:] == np.float32(1.2))
    assert np.all(t.span[leaves[-1]][:3] == np.float32(-1.2))


def test_model_split_rule():
    from oracle import lod as olod
    t = olod.Octree([-1.2, -1.2, -1.2, 1.2, 1.2, 1.2])
    t.request_empty()
    t.finish_requested()
    # a focus 0.5 from the camera splits its 0.6-wide leaf (threshold 1.2);
    # one 1.5 away does not
    cam = np.array([0.0, -1.5, 0.1], np.float32)
    near = cam + np.array([0, 0.5, 0], np.float32)
    far = np.array([0.9, -0.3, 0.9], np.float32)
    assert t.split_near(cam, [near, far]) == 1
    assert len(t.leaves()) == 71
    # the new leaves are empty: a second focus in them splits nothing
    assert t.split_near(cam, [near]) == 0
