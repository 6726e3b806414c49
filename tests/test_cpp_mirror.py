"""The C++ mirror of the reference API (include/cantucci_gpu.hpp) compiles
against the C ABI (no GPU) and, on a GPU, meshes exactly like the goldens."""
import hashlib
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


@pytest.fixture(scope="module")
def mirror_bin(tmp_path_factory):
    from cantucci_gb300 import build
    lib = build.build()
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("mirror") / "mirror_main")
    cuda = cuda_home()
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "mirror_main.cpp"),
           "-o", out, "-L", os.path.dirname(lib), "-lcantucci_gpu",
           "-L", os.path.join(cuda, "lib64"), "-L", os.path.join(cuda, "lib"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_mirror_compiles(mirror_bin):
    assert os.path.exists(mirror_bin)


@pytest.mark.gpu
def test_cpp_mirror_meshes_like_reference(mirror_bin, golden, tmp_path):
    r = subprocess.run([mirror_bin, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    (nv, ni, tv, tf, panicked, child3_y, sphere_in, collected, splits, leaves,
     ready) = open(tmp_path / "summary.txt").read().split()
    assert int(collected) == 64 and int(splits) > 0
    assert int(leaves) == 64 + 7 * int(splits) and int(ready) == 64 - int(splits)
    assert [int(nv), int(ni)] == golden["c1_counts"].tolist()
    assert int(tf) * 6 == int(ni) and int(tv) == int(nv)
    idx = np.fromfile(tmp_path / "indices.u32", np.uint32)
    assert hashlib.sha256(idx.tobytes()).digest() == golden["c1_indices_sha"].tobytes()
    de = np.fromfile(tmp_path / "de.f32", np.float32)
    np.testing.assert_allclose(de[:2], golden["de_p8_i15_b2.5"][:2], rtol=1e-6)
    assert de.view(np.uint32)[2] == 0xFFC00000
    assert panicked == "1" and float(child3_y) == 0.0 and sphere_in == "1"
