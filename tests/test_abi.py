"""The C ABI library builds for sm_103a, loads, and exports every function
include/cantucci_gpu.h declares (no GPU needed; nothing is computed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cantucci_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    from cantucci_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("cg_min_distance_from", "cg_contains", "cg_de_span_grid", "cg_generate_for_box",
                 "cg_march", "cg_mesher_create"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    L = C.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_header(lib_path):
    from cantucci_gb300 import _ffi
    bound = {n for n, _, _ in _ffi.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_struct_layouts(lib_path):
    from cantucci_gb300 import _ffi
    L = _ffi.load()
    assert L.cg_sizeof_shape() == C.sizeof(_ffi.CgShape) == 48
    assert L.cg_sizeof_vertex() == 28
    assert L.cg_abi_version() == 1


def test_kernels_built_for_sm103a(lib_path):
    """Every kernel object carries sm_103a code (cuobjdump lists only the
    embedded ELF names, it does not disassemble)."""
    r = subprocess.run(["cuobjdump", "--list-elf", lib_path], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    elfs = [l for l in r.stdout.splitlines() if l.strip()]
    assert elfs and all("sm_103a" in l for l in elfs)


def test_no_device_does_not_crash(lib_path):
    """Without a GPU the stateless entry points fail with a status, not a crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    from cantucci_gb300 import _ffi
    L = _ffi.load()
    h = C.c_void_p()
    st = L.cg_mesher_create(0, C.byref(h))
    assert st in (_ffi.CG_ENODEV, _ffi.CG_ECUDA)


def test_ctypes_structs_match_header(tmp_path):
    """sizeof / offsetof of every struct in the header, compiled by the C
    compiler, equal the ctypes mirrors field by field."""
    from cantucci_gb300 import _ffi
    pairs = {"cg_shape": _ffi.CgShape, "cg_span": _ffi.CgSpan, "cg_timings": _ffi.CgTimings,
             "cg_span_job": _ffi.CgSpanJob, "cg_job_mesh": _ffi.CgJobMesh,
             "cg_camera": _ffi.CgCamera, "cg_batch_tuning": _ffi.CgBatchTuning}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "cantucci_gpu.h"',
             'int main(void) {']
    for cname, cls in pairs.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append('printf("cg_vertex %zu\\n", sizeof(cg_vertex)); return 0; }')
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    if r.returncode != 0 and "No such file" in r.stderr + r.stdout and "gcc" in r.stderr:
        pytest.skip("no C compiler")
    assert r.returncode == 0, r.stderr
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True,
                                                   text=True).stdout.splitlines())
    for cname, cls in pairs.items():
        assert int(got[cname]) == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(cls, f).offset, (cname, f)
    assert int(got["cg_vertex"]) == _ffi.VERTEX_DTYPE.itemsize == 28
