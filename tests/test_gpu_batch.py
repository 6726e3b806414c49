"""Batched span meshing against per-span generate_for_box and the oracle.

Bar: every span's vertex and index lists are bit-identical to what
generate_for_box gives for that span alone (same kernels, same numerics),
whether the batch runs directly or replays from a CUDA graph; the index
lists equal the oracle's for P=8.
"""
import numpy as np
import pytest

from cantucci_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def per_span(cg, spans, res, shape):
    m = cg.Mesher(0)
    out = []
    try:
        for sp, r in zip(spans, res):
            v, i, nv, ni, _ = m.generate(cg.Span(sp[:3], sp[3:]), shape, int(r), strict=False)
            out.append((v[:nv].view(np.float32).reshape(-1, 7).copy(), i[:ni].copy()))
    finally:
        m.close()
    return out


@pytest.mark.parametrize("power,iters", [(8, 15), (6, 10), (10, 20)])
def test_batch_matches_per_span(cg, power, iters):
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(48, seed=power)
    shape = cg.Mandelbulb(power, iters, 2.5)
    b = BatchMesher(spans, res)
    out = b.run(shape)
    ref = per_span(cg, spans, res, shape)
    for j in range(len(res)):
        v, i = out.mesh(j)
        rv, ri = ref[j]
        assert np.array_equal(i, ri), j
        assert np.array_equal(v.view(np.uint32), rv.view(np.uint32)), j
    b.close()


def test_batch_graph_replay_matches_direct(cg):
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(64, seed=3)
    shape = cg.Mandelbulb(8, 15, 2.5)
    b = BatchMesher(spans, res)
    direct = b.run(shape)
    d = [direct.mesh(j) for j in range(len(res))]
    for _ in range(3):  # capture once, replay twice
        g = b.run(shape, graph=True)
        g._host = None
        for j in range(len(res)):
            v, i = g.mesh(j)
            assert np.array_equal(i, d[j][1])
            assert np.array_equal(v.view(np.uint32), d[j][0].view(np.uint32))
    b.close()


def test_batch_indices_match_oracle(cg, orc):
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(16, seed=7)
    b = BatchMesher(spans, res)
    out = b.run(cg.Mandelbulb(8, 15, 2.5))
    for j in range(len(res)):
        v, i = out.mesh(j)
        r = orc.generate_for_box(orc.mandelbulb(8, 15, 2.5), spans[j], int(res[j]))
        assert r["rc"] == 0
        assert np.array_equal(i, r["indices"])
        np.testing.assert_allclose(v[:, :3], r["vertices"]["position"], rtol=0, atol=1e-6)
    b.close()


def test_batch_mixed_small_and_large(cg):
    """Spans of res 2 and 128 next to each other (linear items and bricks)."""
    from cantucci_gb300.batch import BatchMesher
    spans = np.array([[-1.2, -1.2, -1.2, 1.2, 1.2, 1.2], [0.5, 0.5, -0.2, 0.8, 0.8, 0.1],
                      [-1.2, -1.2, -1.2, 1.2, 1.2, 1.2]], np.float32)
    res = [2, 128, 64]
    shape = cg.Mandelbulb(8, 15, 2.5)
    b = BatchMesher(spans, res)
    out = b.run(shape)
    ref = per_span(cg, spans, res, shape)
    for j in range(3):
        v, i = out.mesh(j)
        assert np.array_equal(i, ref[j][1])
        assert np.array_equal(v.view(np.uint32), ref[j][0].view(np.uint32))
    b.close()


def test_batch_capacity_reported(cg):
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(32, seed=9)
    shape = cg.Mandelbulb(8, 15, 2.5)
    full = BatchMesher(spans, res)
    f = full.run(shape)
    _, tot = f.host()
    small = BatchMesher(spans, res, vertex_cap=int(tot[0]) // 2, index_cap=int(tot[1]) * 3)
    s = small.run(shape)
    rec, stot = s.host()
    assert int(stot[0]) == int(tot[0]) and int(stot[1]) == int(tot[1])
    # spans whose vertices fit entirely are complete and identical
    frec, _ = f.host()
    for j in range(len(res)):
        r = rec[j]
        if int(r["vertex_offset"]) + int(r["vertices"]) <= small.vertex_cap:
            v, _ = s.mesh(j)
            fv, _ = f.mesh(j)
            assert np.array_equal(v.view(np.uint32), fv.view(np.uint32))
    full.close()
    small.close()


def test_batch_rejects_bad_job(cg):
    from cantucci_gb300.batch import BatchMesher
    spans = np.array([[0, 0, 0, 1, 1, 1], [0, 0, 0, -1, 1, 1]], np.float32)
    with pytest.raises(cg.CantucciError) as e:
        BatchMesher(spans, [8, 8])
    assert "job 1" in str(e.value)


def test_tuning_changes_no_output_bit(cg):
    """Every launch shape the autotuner can pick meshes the same bits."""
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(64, seed=5)
    shape = cg.Mandelbulb(8, 15, 2.5)
    b = BatchMesher(spans, res)
    base = b.run(shape)
    ref = [base.mesh(j) for j in range(len(res))]
    for knobs in [dict(brick_min_res=8), dict(brick_min_res=1 << 20), dict(de_block=512),
                  dict(de_block=128, de_chunk=1), dict(de_chunk=4096), dict(place_block=256),
                  dict(place_block=64)]:
        b.set_tuning(**knobs)
        for graph in (False, True):
            out = b.run(shape, graph=graph)
            out._host = None
            for j in range(len(res)):
                v, i = out.mesh(j)
                assert np.array_equal(i, ref[j][1]), (knobs, j)
                assert np.array_equal(v.view(np.uint32), ref[j][0].view(np.uint32)), (knobs, j)
    b.close()


def test_autotune_applies_and_caches(cg, tmp_path):
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(256, seed=6)
    shape = cg.Mandelbulb(8, 15, 2.5)
    b = BatchMesher(spans, res)
    ref = b.run(shape)
    ref = [ref.mesh(j) for j in range(len(res))]
    cache = str(tmp_path / "tune.json")
    r = b.autotune(shape, reps=2, cache_path=cache)
    assert not r["cached"] and r["ms"] > 0
    assert b.tuning == r["tuning"]
    out = b.run(shape, graph=True)
    for j in range(len(res)):
        v, i = out.mesh(j)
        assert np.array_equal(i, ref[j][1])
        assert np.array_equal(v.view(np.uint32), ref[j][0].view(np.uint32))
    b2 = BatchMesher(spans, res)
    r2 = b2.autotune(shape, cache_path=cache)
    assert r2["cached"] and b2.tuning == r["tuning"]
    b.close()
    b2.close()


def test_tuning_rejects_bad_values(cg):
    from cantucci_gb300 import CantucciError
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(4, seed=7)
    b = BatchMesher(spans, res)
    for knobs in [dict(de_block=96), dict(de_block=1024), dict(de_chunk=0),
                  dict(de_chunk=5000), dict(brick_min_res=1), dict(place_block=512)]:
        with pytest.raises(CantucciError):
            b.set_tuning(**knobs)
    b.close()


@pytest.mark.parametrize("normals,numerics", [("analytic", "exact"), ("fd", "fast")])
def test_batch_options_match_per_span(cg, normals, numerics):
    """Analytic normals and fast numerics in a batch: every span's mesh is
    bit-identical to the single-span mesher's under the same option, direct
    and replayed from a graph (the graph is captured again after the option
    changes); fast numerics with analytic normals are refused."""
    from cantucci_gb300.batch import BatchMesher
    spans, res, _, _ = W.batched_spans(40, seed=21)
    shape = cg.Mandelbulb(8, 15, 2.5)
    b = BatchMesher(spans, res)
    try:
        b.run(shape, graph=True)  # a graph with the default options first
        b.set_normals(normals)
        b.set_numerics(numerics)
        outs = [b.run(shape), b.run(shape, graph=True)]
        m = cg.Mesher(0)
        try:
            m.set_normals(normals)
            m.set_numerics(numerics)
            ref = []
            for sp, r in zip(spans, res):
                v, i, nv, ni, _ = m.generate(cg.Span(sp[:3], sp[3:]), shape, int(r), strict=False)
                ref.append((v[:nv].view(np.float32).reshape(-1, 7).copy(), i[:ni].copy()))
        finally:
            m.close()
        for out in outs:
            for j in range(len(res)):
                v, i = out.mesh(j)
                assert np.array_equal(i, ref[j][1]), j
                assert np.array_equal(v.view(np.uint32), ref[j][0].view(np.uint32)), j
        b.set_normals("analytic")
        b.set_numerics("fast")
        with pytest.raises(cg.CantucciError):
            b.run(shape)
    finally:
        b.close()
