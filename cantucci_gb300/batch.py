"""Batched span meshing: the GPU form of ShapeMesh::update's thread pool,
which runs one MeshBuffer::generate_for_box job per empty octree leaf
(src/mesh/mod.rs:129-161).

    b = BatchMesher(spans, resolutions)          # plan + workspace (once)
    out = b.run(Mandelbulb(6, 10, 2.5))          # one persistent launch chain
    vertices, indices = out.mesh(j)              # span j's MeshBuffer contents

`run(graph=True)` replays the whole batch from a CUDA graph.
`autotune(shape)` picks the batch's launch shapes by timing it
(cg_batch_autotune), remembering the winner in a small JSON cache keyed by
the GPU, the shape and the batch's resolution histogram.
"""
import ctypes as C
import hashlib
import json
import os

import numpy as np

from . import _ffi
from ._ffi import check, load


def _torch():
    import torch
    return torch


class BatchResult:
    """Device outputs of one batch run (torch CUDA tensors)."""

    def __init__(self, vertices, indices, results, totals):
        self.vertices = vertices          # (vertex_cap, 7) float32
        self.indices = indices            # (index_cap,) int32 (uint32 bits)
        self.results = results            # (n_jobs, 6) int32 view of cg_job_mesh
        self.totals = totals              # (3,) int32: vertices, quads, status
        self._host = None

    def host(self):
        if self._host is None:
            torch = _torch()
            torch.cuda.synchronize()
            raw = self.results.cpu().numpy().view(np.uint8).reshape(-1, C.sizeof(_ffi.CgJobMesh))
            rec = np.frombuffer(raw.tobytes(), dtype=np.dtype(
                [("vertex_offset", "<u8"), ("index_offset", "<u8"), ("vertices", "<u4"),
                 ("indices", "<u4")]))
            tot = self.totals.cpu().numpy().view(np.uint32)
            self._host = (rec, tot)
        return self._host

    @property
    def status(self):
        return int(self.host()[1][2])

    def mesh(self, j):
        """(vertices (nv, 7) float32, indices (ni,) uint32) of span j, on the host."""
        rec, _ = self.host()
        r = rec[j]
        v0, nv, i0, ni = int(r["vertex_offset"]), int(r["vertices"]), int(r["index_offset"]), int(
            r["indices"])
        v = self.vertices[v0:v0 + nv].cpu().numpy()
        i = self.indices[i0:i0 + ni].cpu().numpy().view(np.uint32)
        return v, i


class BatchMesher:
    """A planned batch of (span, resolution) jobs on one device."""

    def __init__(self, spans, resolutions, vertex_cap=None, index_cap=None, device=0):
        torch = _torch()
        spans = np.ascontiguousarray(spans, np.float32).reshape(-1, 6)
        res = np.asarray(resolutions, np.uint32).reshape(-1)
        assert len(spans) == len(res) and len(res) > 0
        self.n_jobs = len(res)
        self._resolutions = res.copy()
        jobs = (_ffi.CgSpanJob * self.n_jobs)()
        for j in range(self.n_jobs):
            for k in range(3):
                jobs[j].span.start[k] = float(spans[j, k])
                jobs[j].span.end[k] = float(spans[j, 3 + k])
            jobs[j].resolution = int(res[j])
        r3 = int(np.sum(res.astype(np.int64) ** 3))
        self.vertex_cap = int(vertex_cap if vertex_cap is not None else min(r3, 1 << 26))
        self.index_cap = int(index_cap if index_cap is not None else 6 * self.vertex_cap)
        self.device = device
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.cg_batch_create(device, jobs, self.n_jobs, self.vertex_cap, C.byref(h)))
        self.handle = h
        dev = "cuda:%d" % device
        self._verts = torch.empty((max(self.vertex_cap, 1), 7), dtype=torch.float32, device=dev)
        self._idx = torch.empty(max(self.index_cap, 1), dtype=torch.int32, device=dev)
        self._res = torch.empty((self.n_jobs, 6), dtype=torch.int32, device=dev)
        self._tot = torch.empty(3, dtype=torch.int32, device=dev)

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def tuning(self) -> dict:
        t = _ffi.CgBatchTuning()
        check(self._lib.cg_batch_get_tuning(self.handle, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **knobs):
        t = _ffi.CgBatchTuning(**{**self.tuning, **knobs})
        check(self._lib.cg_batch_set_tuning(self.handle, C.byref(t)))

    def set_normals(self, mode: str):
        """"fd" (the reference's six-sample difference, default) or
        "analytic" (one forward-mode pass per vertex)."""
        modes = {"fd": _ffi.CG_NORMALS_FD, "analytic": _ffi.CG_NORMALS_ADJOINT}
        check(self._lib.cg_batch_set_normals(self.handle, modes[mode]))

    def set_numerics(self, mode: str):
        """"exact" (the reference's bits, default) or "fast" (with "fd"
        normals only)."""
        modes = {"exact": _ffi.CG_NUMERICS_EXACT, "fast": _ffi.CG_NUMERICS_FAST}
        check(self._lib.cg_batch_set_numerics(self.handle, modes[mode]))

    def tuning_key(self, shape) -> str:
        """Cache key: GPU name and SM count, the shape, the resolutions."""
        torch = _torch()
        p = torch.cuda.get_device_properties(self.device)
        c = shape._cshape()
        h = hashlib.sha256(np.sort(self._resolutions).tobytes()).hexdigest()[:16]
        return "%s/%d/kind%d-p%d-%.4f-it%d/n%d-%s" % (p.name, p.multi_processor_count, c.kind,
                                                      c.power, c.power_f, c.max_iters,
                                                      self.n_jobs, h)

    def autotune(self, shape, reps=3, cache_path=None, stream=None) -> dict:
        """Picks and applies launch shapes for `shape` on this batch.

        With `cache_path` (default: $CANTUCCI_TUNING_CACHE when set) a
        previous winner for the same key is applied without timing, and a
        new winner is stored.  Returns {"tuning", "ms", "cached"}."""
        torch = _torch()
        cache_path = cache_path or os.environ.get("CANTUCCI_TUNING_CACHE")
        key = self.tuning_key(shape)
        cache = {}
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as f:
                cache = json.load(f)
            if key in cache:
                self.set_tuning(**cache[key]["tuning"])
                return {"tuning": self.tuning, "ms": cache[key]["ms"], "cached": True}
        stream = stream or torch.cuda.current_stream(self.device)
        best = _ffi.CgBatchTuning()
        ms = C.c_float()
        check(self._lib.cg_batch_autotune(
            self.handle, C.byref(shape._cshape()), C.c_void_p(self._verts.data_ptr()),
            self.vertex_cap, C.c_void_p(self._idx.data_ptr()), self.index_cap,
            C.c_void_p(self._res.data_ptr()), C.c_void_p(self._tot.data_ptr()),
            C.c_void_p(stream.cuda_stream), int(reps), C.byref(best), C.byref(ms)))
        out = {"tuning": best.as_dict(), "ms": float(ms.value), "cached": False}
        if cache_path:
            cache[key] = {"tuning": out["tuning"], "ms": out["ms"]}
            d = os.path.dirname(os.path.abspath(cache_path))
            os.makedirs(d, exist_ok=True)
            tmp = cache_path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(cache, f, indent=1, sort_keys=True)
            os.replace(tmp, cache_path)
        return out

    def run(self, shape, graph=False, stream=None) -> BatchResult:
        torch = _torch()
        stream = stream or torch.cuda.current_stream(self.device)
        fn = self._lib.cg_batch_mesh_graph if graph else self._lib.cg_batch_mesh
        check(fn(self.handle, C.byref(shape._cshape()), C.c_void_p(self._verts.data_ptr()),
                 self.vertex_cap, C.c_void_p(self._idx.data_ptr()), self.index_cap,
                 C.c_void_p(self._res.data_ptr()), C.c_void_p(self._tot.data_ptr()),
                 C.c_void_p(stream.cuda_stream)))
        return BatchResult(self._verts, self._idx, self._res, self._tot)
