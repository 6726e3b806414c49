"""CPU restatement of ShapeMesh's level-of-detail rules (src/mesh/mod.rs:24-243,
src/octree/mod.rs, src/octree/iter.rs, src/camera.rs).

Test infrastructure only: the tests run the GPU driver (cg_shape_mesh_*) and
this model side by side and compare the octrees they build.  Nothing in the
product imports it.

    tree = Octree(bounds)            # ShapeMesh::new: root and its children split
    rays = focus_rays(...)           # get_focii's rays (camera.rs + cgmath, f32)
    tree.split_near(cam, focii)      # the split loop of update (mod.rs:93-107)
    tree.leaves()                    # Octree::iter order (a stack)
"""
import numpy as np

from . import create_spans

f32 = np.float32
EMPTY, REQUESTED, READY = 0, 1, 2


def _normalize(v):
    """cgmath normalize: v * (1 / |v|), |v| = sqrt((x*x + y*y) + z*z)."""
    v = np.asarray(v, f32)
    m = np.sqrt(f32(f32(v[0] * v[0]) + f32(v[1] * v[1])) + f32(v[2] * v[2]))
    return (v * (f32(1.0) / f32(m))).astype(f32)


def _cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]], f32)


def focus_rays(position, direction, fov, aspect, near, focus_points=5):
    """get_focii's rays (mod.rs:205-229): grid centres on the near plane
    (Camera::near_plane_bb, camera.rs:117-134; near_plane_dimension,
    camera.rs:184-189), in iter::square order (x outer), moved to world space
    by the inverse of look_at_rh(pos, pos + dir, +z): pos + c.x s + c.y u -
    c.z f with f = normalize(dir), s = normalize(f x z), u = s x f."""
    F = int(focus_points)
    pos = np.asarray(position, f32)
    d = _normalize(direction)
    height = f32(f32(f32(2.0) * f32(near)) * f32(np.tan(f32(f32(fov) * f32(0.5)))))
    width = f32(height * f32(aspect))
    tl = np.array([-width / f32(2.0), -height / f32(2.0), -f32(near)], f32)
    br = np.array([width / f32(2.0), height / f32(2.0), -f32(near)], f32)
    sh, sv = f32(width / f32(F)), f32(height / f32(F))
    cdiff = ((br - tl) / f32(f32(2.0) * f32(F))).astype(f32)
    f = _normalize((pos + d).astype(f32) - pos)
    s = _normalize(_cross(f, np.array([0, 0, 1], f32)))
    u = _cross(s, f)
    org, dirs = [], []
    for x in range(F):
        for y in range(F):
            c = ((tl + np.array([f32(x) * sh, f32(y) * sv, 0], f32)).astype(f32) + cdiff).astype(f32)
            p = (((pos + s * c[0]).astype(f32) + u * c[1]).astype(f32) + f * (-c[2])).astype(f32)
            org.append(pos.copy())
            dirs.append(_normalize((p - pos).astype(f32)))
    return np.array(org, f32), np.array(dirs, f32)


class Octree:
    """Octree<MeshStatus, ()> of ShapeMesh (src/octree/mod.rs:36-98)."""

    def __init__(self, bounds, first_levels=2):
        b = np.asarray(bounds, f32).reshape(6)
        # node: [span (6 f32), first child index or -1, status, depth]
        self.span = [b.copy()]
        self.child = [-1]
        self.status = [EMPTY]
        self.depth = [0]
        self.split(0)
        if first_levels >= 2:
            for c in range(8):
                self.split(self.child[0] + c)

    def split(self, i):
        """NodeEntryMut::split (src/octree/mod.rs:280-296): the leaf's data
        is dropped and eight empty children take its place."""
        kids = create_spans(self.span[i])
        first = len(self.span)
        for k in range(8):
            self.span.append(kids[k].astype(f32))
            self.child.append(-1)
            self.status.append(EMPTY)
            self.depth.append(self.depth[i] + 1)
        self.child[i] = first
        self.status[i] = EMPTY

    @staticmethod
    def _contains(span, p):
        """SpanExt::contains (src/octree/mod.rs:25-31): half open."""
        return bool(np.all(span[:3] <= p) and np.all(p < span[3:]))

    def leaf_around(self, p):
        """Octree::leaf_around_mut (src/octree/mod.rs:71-85)."""
        p = np.asarray(p, f32)
        if not self._contains(self.span[0], p):
            return -1
        i = 0
        while self.child[i] >= 0:
            i = next(self.child[i] + c for c in range(8)
                     if self._contains(self.span[self.child[i] + c], p))
        return i

    def leaves(self):
        """Leaves in Octree::iter order (src/octree/iter.rs:24-33): pop a
        node, push its children 0..7."""
        out, stack = [], [0]
        while stack:
            i = stack.pop()
            if self.child[i] < 0:
                out.append(i)
            else:
                stack.extend(self.child[i] + c for c in range(8))
        return out

    def split_near(self, camera_position, focii):
        """The split loop of ShapeMesh::update (src/mesh/mod.rs:93-107):
        for each focus point, a READY leaf around it is split when the camera
        is closer to the point than twice the leaf's x extent."""
        cam = np.asarray(camera_position, f32)
        splits = 0
        for focus in np.asarray(focii, f32).reshape(-1, 3):
            i = self.leaf_around(focus)
            if i < 0 or self.status[i] != READY:
                continue
            dv = (cam - focus).astype(f32)
            dist = np.sqrt(f32(f32(dv[0] * dv[0]) + f32(dv[1] * dv[1])) + f32(dv[2] * dv[2]))
            sp = self.span[i]
            threshold = f32(f32(2.0) * abs(f32(sp[3] - sp[0])))
            if dist < threshold:
                self.split(i)
                splits += 1
        return splits

    def request_empty(self):
        """The job loop of update (mod.rs:125-161): every empty leaf gets a job."""
        started = 0
        for i in self.leaves():
            if self.status[i] == EMPTY:
                self.status[i] = REQUESTED
                started += 1
        return started

    def finish_requested(self):
        """All jobs in flight finish (their meshes go to the leaf around each
        span's centre, which is the requesting leaf)."""
        n = 0
        for i in self.leaves():
            if self.status[i] == REQUESTED:
                self.status[i] = READY
                n += 1
        return n
