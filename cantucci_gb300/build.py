"""Builds libcantucci_gpu.so (the C ABI of include/cantucci_gpu.h) in-tree.

Every translation unit is compiled for sm_103a only, in parallel, and linked
into cantucci_gb300/_lib/libcantucci_gpu.so.  Host code is compiled with
-ffp-contract=off so the span set-up rounds like the reference.

build(checked=True) makes libcantucci_gpu_checked.so instead: the same
sources with -DCG_CHECKED, where the mesh path's array accesses are bounds
checked (an out-of-range access is skipped and counted, cg_debug_oob reads
the count).  It is a test tool, built on demand.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIB_DIR, "libcantucci_gpu.so")
CHECKED_LIB = os.path.join(LIB_DIR, "libcantucci_gpu_checked.so")

SOURCES = ["capi.cu", "de_kernels.cu", "mesh.cu", "mesh_batch.cu", "adjoint.cu", "trace.cu", "scan.cu",
           "noalloc.cu", "lod.cu"]
# Benchmark instrumentation, outside the C ABI library: the FP32 peak probe
# (a library of its own) and the native leaf-pool driver (an executable).
BENCH_SOURCE = os.path.join(CSRC, "bench", "fp32_peak.cu")
BENCH_LIB = os.path.join(LIB_DIR, "libcantucci_bench.so")
LEAF_POOL_SOURCE = os.path.join(CSRC, "bench", "leaf_pool.cpp")
LEAF_POOL_EXE = os.path.join(LIB_DIR, "cg_leaf_pool")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _inputs_digest(extra=()) -> str:
    h = hashlib.sha256()
    h.update(" ".join(extra).encode())
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            p = os.path.join(d, name)
            if os.path.isfile(p):
                h.update(name.encode())
                with open(p, "rb") as f:
                    h.update(f.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _compile(src: str, verbose: bool, obj_dir: str = OBJ_DIR, extra=()) -> str:
    obj = os.path.join(obj_dir, src.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-I", INCLUDE, "-I", CSRC, "-c",
           os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    """Compile (if sources changed) and return the path of the shared library
    (with checked=True, of the bounds-checked variant)."""
    extra = ("-DCG_CHECKED",) if checked else ()
    lib = CHECKED_LIB if checked else LIB
    obj_dir = os.path.join(OBJ_DIR, "checked") if checked else OBJ_DIR
    digest = _inputs_digest(extra)
    stamp = os.path.join(LIB_DIR, ".digest_checked" if checked else ".digest")
    if (not force and os.path.exists(lib) and os.path.exists(stamp)
            and open(stamp).read().strip() == digest):
        return lib
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, obj_dir, extra), SOURCES))
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    with open(stamp, "w") as f:
        f.write(digest)
    return lib


def build_bench(force: bool = False) -> str:
    """Compile the benchmark's FP32 peak probe into libcantucci_bench.so
    (not part of the C ABI) and return its path."""
    h = hashlib.sha256()
    with open(BENCH_SOURCE, "rb") as f:
        h.update(f.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    digest = h.hexdigest()
    stamp = os.path.join(LIB_DIR, ".digest_bench")
    if (not force and os.path.exists(BENCH_LIB) and os.path.exists(stamp)
            and open(stamp).read().strip() == digest):
        return BENCH_LIB
    os.makedirs(LIB_DIR, exist_ok=True)
    tmp = BENCH_LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-shared", BENCH_SOURCE, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (BENCH_SOURCE, r.stdout, r.stderr))
    os.replace(tmp, BENCH_LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return BENCH_LIB


def build_leaf_pool(force: bool = False) -> str:
    """Compile the native leaf-pool driver (T threads, one cg_mesher each,
    blocking cg_generate_for_box per octree leaf) against the C ABI library
    and return the executable's path."""
    lib = build()
    h = hashlib.sha256()
    for p in (LEAF_POOL_SOURCE, os.path.join(INCLUDE, "cantucci_gpu.h")):
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(os.uname().machine.encode())
    digest = h.hexdigest()
    stamp = os.path.join(LIB_DIR, ".digest_leaf_pool")
    if (not force and os.path.exists(LEAF_POOL_EXE) and os.path.exists(stamp)
            and open(stamp).read().strip() == digest):
        return LEAF_POOL_EXE
    tmp = LEAF_POOL_EXE + ".tmp%d" % os.getpid()
    cmd = [nvcc(), "-O2", "-std=c++17", LEAF_POOL_SOURCE, "-I", INCLUDE, "-L", LIB_DIR,
           "-lcantucci_gpu", "-Xlinker", "-rpath," + os.path.dirname(lib), "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (LEAF_POOL_SOURCE, r.stdout, r.stderr))
    os.replace(tmp, LEAF_POOL_EXE)
    with open(stamp, "w") as f:
        f.write(digest)
    return LEAF_POOL_EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                checked="--checked" in sys.argv))
