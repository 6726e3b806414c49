"""The bounds-checked build (libcantucci_gpu_checked.so, -DCG_CHECKED), in
place of compute-sanitizer, which this GPU pool does not offer: every array
access of the mesh path names its array's size, and an access past it is
skipped and counted instead of performed.  tests/checked_cases.py drives
the awkward cases (resolutions 2 to 32, a span with no surface, every
option, outputs smaller than the mesh, both host-output paths, a batch)
through that library in a subprocess; the bar is zero skipped accesses."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_checked_build_sees_no_out_of_range_access(cg):
    from cantucci_gb300 import build
    lib = build.build(checked=True)
    env = dict(os.environ, CANTUCCI_GPU_LIB=lib)
    r = subprocess.run([sys.executable, os.path.join(HERE, "checked_cases.py")], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["cases"] > 90
    assert out["out_of_range"] == 0, out


def test_normal_build_has_no_checks(cg):
    import ctypes as C
    lib = cg.load()
    n, line = C.c_uint64(), C.c_uint32()
    assert lib.cg_debug_oob(C.byref(n), C.byref(line), 0) != 0
