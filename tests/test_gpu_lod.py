"""The level-of-detail driver (cg_shape_mesh_*) against the oracle's model of
ShapeMesh::update and against per-span meshing.

Bar: after every update the octree (leaf spans in traversal order, depths,
statuses) equals the model's, given the same focus points; the focus points
equal the oracle's march of the oracle's rays; every ready leaf's mesh is
bit-identical to generate_for_box of its span at the driver's resolution."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOUNDS = [-1.2, -1.2, -1.2, 1.2, 1.2, 1.2]


def tree_state(sm):
    return [(tuple(l.start.tolist()) + tuple(l.end.tolist()), l.depth, l.status)
            for l in sm.leaves()]


def model_state(t):
    return [(tuple(t.span[i].tolist()), t.depth[i], t.status[i]) for i in t.leaves()]


def check_meshes(cg, sm, res, limit=None):
    m = cg.Mesher(0)
    n = 0
    try:
        for leaf in sm.leaves():
            if not leaf.ready:
                continue
            v, i = leaf.mesh()
            rv, ri, nv, ni, _ = m.generate(cg.Span(leaf.start, leaf.end), sm_shape(sm), res,
                                           strict=False)
            assert len(v) == nv and len(i) == ni
            assert np.array_equal(i, ri[:ni])
            assert np.array_equal(v.view(np.uint32),
                                  rv[:nv].view(np.float32).reshape(-1, 7).view(np.uint32))
            n += 1
            if limit and n >= limit:
                break
    finally:
        m.close()
    return n


_SHAPES = {}


def sm_shape(sm):
    return _SHAPES[id(sm)]


def make(cg, shape, res=32):
    from cantucci_gb300.lod import ShapeMesh
    sm = ShapeMesh(shape, resolution=res)
    _SHAPES[id(sm)] = shape
    return sm


def test_first_updates_mesh_every_leaf(cg):
    from cantucci_gb300.lod import Camera, REQUESTED, READY
    from oracle import lod as olod
    shape = cg.Mandelbulb(8, 15, 2.5)
    sm = make(cg, shape, res=32)
    far = Camera(position=(0, -30, 0), direction=(0, 1, 0))
    s1 = sm.update(far, wait=True)
    assert s1["started"] == 64 and s1["leaves"] == 64 and s1["collected"] == 0
    assert all(l.status == REQUESTED for l in sm.leaves())
    t = olod.Octree(BOUNDS)
    t.request_empty()
    assert tree_state(sm) == model_state(t)
    s2 = sm.update(far, wait=True)
    assert s2["collected"] == 64 and s2["started"] == 0 and s2["active"] == 0
    assert all(l.status == READY for l in sm.leaves())
    assert check_meshes(cg, sm, 32) == 64
    sm.close()


def test_updates_follow_the_model(cg, orc):
    """A camera near the surface: focus points split leaves; the new leaves are
    meshed by the next update; the tree tracks the model step by step."""
    from cantucci_gb300.lod import Camera, focus_rays
    from oracle import lod as olod
    shape = cg.Mandelbulb(8, 15, 2.5)
    sm = make(cg, shape, res=32)
    t = olod.Octree(BOUNDS)
    cams = [Camera(position=(0, -30, 0), direction=(0, 1, 0)),
            Camera(position=(0, -30, 0), direction=(0, 1, 0)),
            Camera(position=(0.05, -1.45, 0.1), direction=(0, 1, 0.05)),
            Camera(position=(0.05, -1.45, 0.1), direction=(0, 1, 0.05)),
            Camera(position=(-0.3, -1.25, 0.2), direction=(0.2, 1, -0.1)),
            Camera(position=(-0.3, -1.25, 0.2), direction=(0.2, 1, -0.1))]
    total_splits = 0
    oshape = orc.mandelbulb(8, 15, 2.5)
    for cam in cams:
        st = sm.update(cam, wait=True)
        focii = sm.focii()
        # focus points: the oracle's march of the oracle's rays
        org, d = olod.focus_rays(cam.position, cam.direction, cam.fov, cam.aspect, cam.near)
        hits, hit = orc.march(oshape, org, d, max_steps=100, epsilon=1e-6)
        assert len(focii) == int(hit.sum()) == st["focii"]
        np.testing.assert_allclose(focii, hits[hit], rtol=0, atol=2e-5)
        # the same rules on the model, fed the driver's focus points
        assert t.split_near(cam.position, focii) == st["splits"]
        total_splits += st["splits"]
        assert t.finish_requested() == st["collected"]
        assert t.request_empty() == st["started"]
        assert tree_state(sm) == model_state(t)
    assert total_splits > 0, "the camera path should split some leaves"
    assert check_meshes(cg, sm, 32, limit=40) > 0
    # deeper leaves are meshed too
    assert any(l.depth > 2 and l.ready for l in sm.leaves())
    sm.close()


def test_update_without_wait_collects_later(cg):
    import torch
    from cantucci_gb300.lod import Camera
    sm = make(cg, cg.Mandelbulb(8, 15, 2.5), res=32)
    cam = Camera(position=(0, -30, 0), direction=(0, 1, 0))
    s1 = sm.update(cam, wait=False)
    assert s1["started"] == 64
    torch.cuda.synchronize()
    s2 = sm.update(cam, wait=False)
    # the run may still be in flight right after launch, but not after a
    # device synchronisation on the driver's stream's work
    assert s2["collected"] in (0, 64)
    if s2["collected"] == 0:
        s3 = sm.update(cam, wait=True)
        assert s3["collected"] == 64
    sm.close()


def test_update_takes_jobs_while_runs_are_in_flight(cg):
    """Like the reference's thread pool, which accepts jobs while older ones
    run: an update starts a run for newly empty leaves although an earlier
    run is still in flight (res-256 leaves, so the first run takes tens of
    milliseconds); later updates collect the runs in launch order, and every
    ready leaf ends with the mesh of its own span."""
    from cantucci_gb300.lod import Camera, EMPTY, REQUESTED
    sm = make(cg, cg.Mandelbulb(8, 15, 2.5), res=256)
    far = Camera(position=(0, -30, 0), direction=(0, 1, 0))
    sm.update(far, wait=True)
    sm.update(far, wait=True)
    near = [Camera(position=(0.05, -1.45, 0.1), direction=(0, 1, 0.05)),
            Camera(position=(-0.3, -1.25, 0.2), direction=(0.2, 1, -0.1)),
            Camera(position=(0.4, -1.3, -0.2), direction=(-0.2, 1, 0.1))]
    stats = [sm.update(cam, wait=False) for cam in near]
    started = [st["started"] for st in stats]
    assert started[0] > 0 and sum(started[1:]) > 0, started
    # a run started while the first one was still queued or running
    overlapped = [k for k in (1, 2) if started[k] > 0 and stats[k]["collected"] == 0
                  and stats[k]["active"] > started[k]]
    assert overlapped, stats
    assert all(l.status in (EMPTY, REQUESTED) or l.ready for l in sm.leaves())
    for _ in range(4):  # from far away nothing splits: collect, mesh the rest, collect
        st = sm.update(far, wait=True)
        if st["started"] == 0 and st["active"] == 0:
            break
    assert all(l.ready for l in sm.leaves())
    assert check_meshes(cg, sm, 256, limit=6) == 6
    sm.close()


def test_polar_shape_and_bad_arguments(cg):
    from cantucci_gb300 import CantucciError
    from cantucci_gb300.lod import Camera, ShapeMesh
    shape = cg.MandelbulbPolar(8.3, 15, 2.5, (0.2, 0.1, 0.0))
    sm = make(cg, shape, res=16)
    cam = Camera(position=(0, -30, 0), direction=(0, 1, 0))
    sm.update(cam, wait=True)
    sm.update(cam, wait=True)
    assert check_meshes(cg, sm, 16) == 64
    with pytest.raises(CantucciError):
        sm.update(Camera(direction=(0, 0, 0)))
    sm.close()
    with pytest.raises(CantucciError):
        ShapeMesh(shape, resolution=48)


def test_leaf_options(cg):
    """Analytic normals for the driver's leaves: every ready leaf equals the
    single-span mesher with analytic normals, bit for bit; fast numerics
    with analytic normals are refused."""
    from cantucci_gb300.lod import Camera
    shape = cg.Mandelbulb(8, 15, 2.5)
    sm = make(cg, shape, res=32)
    sm.set_options(normals="analytic")
    with pytest.raises(cg.CantucciError):
        sm.set_options(normals="analytic", numerics="fast")
    far = Camera(position=(0, -30, 0), direction=(0, 1, 0))
    sm.update(far, wait=True)
    sm.update(far, wait=True)
    m = cg.Mesher(0)
    m.set_normals("analytic")
    n = 0
    try:
        for leaf in sm.leaves():
            if not leaf.ready:
                continue
            v, i = leaf.mesh()
            rv, ri, nv, ni, _ = m.generate(cg.Span(leaf.start, leaf.end), shape, 32, strict=False)
            assert np.array_equal(i, ri[:ni])
            assert np.array_equal(v.view(np.uint32),
                                  rv[:nv].view(np.float32).reshape(-1, 7).view(np.uint32))
            n += 1
    finally:
        m.close()
    assert n == 64
    sm.close()
