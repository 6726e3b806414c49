"""Runs the mesh path's awkward cases through the library CANTUCCI_GPU_LIB
names (the bounds-checked build) and prints one JSON line: the number of
out-of-range array accesses the kernels skipped (cg_debug_oob) and the
source line of the first.  Used by tests/test_gpu_checked.py in a
subprocess, so that the checked library is the only one loaded."""
import ctypes as C
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

import cantucci_gb300 as cg  # noqa: E402
from cantucci_gb300 import workloads as W  # noqa: E402
from cantucci_gb300.batch import BatchMesher  # noqa: E402


def oob(lib, reset=1):
    n, line = C.c_uint64(), C.c_uint32()
    assert lib.cg_debug_oob(C.byref(n), C.byref(line), reset) == 0, "not the checked build"
    return n.value, line.value


def try_generate(m, span, shape, res, **kw):
    try:
        return m.generate(span, shape, res, strict=False, **kw)
    except cg.CantucciError:  # capacity too small: counts reported, prefix written
        return None


def main():
    lib = cg.load()
    oob(lib)
    spans = [cg.Span(*W.SPAN_C1), cg.Span((-0.3, 0.1, -1.1), (0.5, 0.9, -0.3)),
             cg.Span((1.5, 1.5, 1.5), (1.9, 1.9, 1.9))]  # the last one has no surface
    shapes = [cg.Mandelbulb(8, 15, 2.5), cg.Mandelbulb(6, 12, 2.5),
              cg.MandelbulbPolar(8.3, 15, 2.5, (0.2, 0.1, 0.0)),
              cg.Sphere((0.1, -0.05, 0.02), 0.9)]
    cases = 0
    m = cg.Mesher(0)
    for res in (2, 4, 8, 16, 32):
        for sp in spans:
            for sh in shapes:
                try_generate(m, sp, sh, res)
                cases += 1
    # every option, on a resolution with a ragged last sign word (n = 33)
    for opt in ("analytic", "root", "qef", "qef_root", "fast"):
        m2 = cg.Mesher(0)
        if opt == "analytic":
            m2.set_normals("analytic")
        if opt in ("root", "qef_root"):
            m2.set_crossings("root", 4)
        if opt in ("qef", "qef_root"):
            m2.set_placement("qef")
        if opt == "fast":
            m2.set_numerics("fast")
        for sh in shapes:
            try_generate(m2, spans[0], sh, 32)
            cases += 1
        m2.close()
    return lib, m, spans, shapes, cases


def rest(lib, m, spans, shapes, cases):
    p8 = shapes[0]
    # outputs smaller than the mesh (CG_ECAPACITY: only the prefix written)
    for vcap, icap in ((1, 1), (10, 30), (1000, 6)):
        v = np.empty(vcap, cg.VERTEX_DTYPE)
        i = np.empty(icap, np.uint32)
        try_generate(m, spans[0], p8, 64, vertices=v, indices=i)
        hv = torch.empty((vcap, 7), dtype=torch.float32).pin_memory()
        hi = torch.empty(icap, dtype=torch.int32).pin_memory()
        for res in (64, 256):  # staged through a graph / the overlapped pipeline
            try_generate(m, spans[0], p8, res, vertices=hv, indices=hi)
        cases += 3
    # device outputs, and pinned outputs with room, on both host paths
    dv = torch.empty((1 << 16, 7), dtype=torch.float32, device="cuda")
    di = torch.empty(6 << 16, dtype=torch.int32, device="cuda")
    m.generate_device(spans[1], p8, 32, dv, di, strict=False)
    hv = torch.empty((1 << 20, 7), dtype=torch.float32).pin_memory()
    hi = torch.empty(6 << 20, dtype=torch.int32).pin_memory()
    for res in (64, 256):
        try_generate(m, spans[0], p8, res, vertices=hv, indices=hi)
    cases += 3
    m.close()
    # a batch of mixed resolutions (the shared row functions)
    bs, br, _, _ = W.batched_spans(64, seed=4)
    b = BatchMesher(bs, br)
    b.run(p8)
    b.run(p8, graph=True)
    b.close()
    cases += 2
    n, line = oob(lib)
    print(json.dumps({"cases": cases, "out_of_range": n, "first_line": line}))


if __name__ == "__main__":
    rest(*main())
