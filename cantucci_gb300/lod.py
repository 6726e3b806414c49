"""Level of detail: the GPU form of cantucci's ShapeMesh (src/mesh/mod.rs).

    cam = Camera(position=(0, -2.5, 0), direction=(0, 1, 0))
    sm = ShapeMesh(Mandelbulb(8, 15, 2.5))     # octree of 64 empty leaves
    sm.update(cam, wait=True)                  # focus rays, splits, one batched mesh run
    for leaf in sm.leaves():                   # Octree::iter order
        if leaf.ready:
            vertices, indices = leaf.mesh()    # that leaf's MeshBuffer

Each update marches the 5 x 5 focus rays on the GPU, splits every ready leaf
around a focus point closer than twice its width, collects the last batched
run, and meshes every empty leaf in one batched run (cg_shape_mesh_update).
"""
import ctypes as C
import math

import numpy as np

from . import _ffi
from ._ffi import check, load

EMPTY, REQUESTED, READY = 0, 1, 2


class Camera:
    """Camera + Projection (src/camera.rs:14-19,138-150): position, look
    direction, vertical field of view (radians), aspect ratio, near and far
    plane; the up vector is +z."""

    def __init__(self, position=(0.0, -2.5, 0.0), direction=(0.0, 1.0, 0.0),
                 fov=math.radians(60.0), aspect=1.0, near=0.01, far=100.0):
        self.position = tuple(float(v) for v in position)
        self.direction = tuple(float(v) for v in direction)
        self.fov, self.aspect, self.near, self.far = float(fov), float(aspect), float(near), \
            float(far)

    def to_c(self) -> _ffi.CgView:
        v = _ffi.CgView()
        for k in range(3):
            v.position[k] = self.position[k]
            v.direction[k] = self.direction[k]
        v.fov_y, v.aspect, v.near_plane, v.far_plane = self.fov, self.aspect, self.near, self.far
        return v


def focus_rays(camera: Camera, focus_points: int = 5):
    """(origins, dirs), each (focus_points^2, 3) float32: the rays of
    ShapeMesh::get_focii, computed by the library on the host."""
    n = focus_points * focus_points
    org = np.empty((n, 3), np.float32)
    d = np.empty((n, 3), np.float32)
    check(load().cg_view_focus_rays(C.byref(camera.to_c()), focus_points,
                                    org.ctypes.data, d.ctypes.data))
    return org, d


class Leaf:
    def __init__(self, c: _ffi.CgLeaf):
        self.start = np.array(c.span.start[:], np.float32)
        self.end = np.array(c.span.end[:], np.float32)
        self.status = int(c.status)
        self.depth = int(c.depth)
        self._v, self._i = c.vertices, c.indices
        self.n_vertices, self.n_indices = int(c.n_vertices), int(c.n_indices)

    @property
    def ready(self) -> bool:
        return self.status == READY

    def mesh(self):
        """(vertices (n, 7) float32, indices (m,) uint32) copied to the host."""
        import torch
        from .api import _DeviceView
        if not self.ready:
            raise ValueError("leaf has no mesh yet")
        v = np.zeros((self.n_vertices, 7), np.float32)
        i = np.zeros(self.n_indices, np.uint32)
        if self.n_vertices:
            v = torch.as_tensor(_DeviceView(self._v, (self.n_vertices, 7), "<f4"),
                                device="cuda").cpu().numpy()
        if self.n_indices:
            i = torch.as_tensor(_DeviceView(self._i, (self.n_indices,), "<i4"),
                                device="cuda").cpu().numpy().view(np.uint32)
        return v, i


class ShapeMesh:
    """cg_shape_mesh: the octree, its meshes and the update rules."""

    def __init__(self, shape, bounds=None, resolution: int = 64, device: int = 0):
        self._lib = load()
        if bounds is None:
            bounds = shape.bounding_box()
        from .api import Span
        span = bounds if isinstance(bounds, Span) else Span(bounds[0], bounds[1])
        h = C.c_void_p()
        check(self._lib.cg_shape_mesh_create(device, C.byref(shape._cshape()),
                                             C.byref(span.to_c()), resolution, C.byref(h)))
        self.handle = h
        self.resolution = resolution

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cg_shape_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_options(self, normals: str = "fd", numerics: str = "exact"):
        """Normals ("fd" or "analytic") and numerics ("exact" or "fast") of
        the leaves meshed from the next update on."""
        nm = {"fd": _ffi.CG_NORMALS_FD, "analytic": _ffi.CG_NORMALS_ADJOINT}[normals]
        nu = {"exact": _ffi.CG_NUMERICS_EXACT, "fast": _ffi.CG_NUMERICS_FAST}[numerics]
        check(self._lib.cg_shape_mesh_set_options(self.handle, nm, nu))

    def update(self, camera: Camera, wait: bool = False) -> dict:
        st = _ffi.CgLodStats()
        check(self._lib.cg_shape_mesh_update(self.handle, C.byref(camera.to_c()), int(wait),
                                             C.byref(st)))
        return st.as_dict()

    def leaves(self):
        n = C.c_uint32()
        check(self._lib.cg_shape_mesh_leaves(self.handle, None, 0, C.byref(n)))
        arr = (_ffi.CgLeaf * max(n.value, 1))()
        check(self._lib.cg_shape_mesh_leaves(self.handle, arr, n.value, C.byref(n)))
        return [Leaf(arr[k]) for k in range(n.value)]

    def focii(self) -> np.ndarray:
        n = C.c_uint32()
        check(self._lib.cg_shape_mesh_focii(self.handle, None, 0, C.byref(n)))
        out = np.zeros((n.value, 3), np.float32)
        if n.value:
            check(self._lib.cg_shape_mesh_focii(self.handle, out.ctypes.data, n.value,
                                                C.byref(n)))
        return out
