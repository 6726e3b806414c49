"""Build recipe for oracle/_ref/libref_shader.so: cantucci's own estimator
shaders compiled as C++ (test infrastructure, like the rest of oracle/).

cantucci hands the GPU its distance estimator as GLSL text:
src/shape/mandelbulb.frag (the polar form, placeholders {POWER}, {MAX_ITERS},
{BAILOUT}) and src/shape/shape.frag (the sphere, {X}, {Y}, {Z}, {RADIUS}).
The shape fills the placeholders with Rust's Display of its parameters
(src/shape/mandelbulb.rs:82-85, src/shape/sphere.rs:42-46): the integer
power and iteration count as integers, f32 values as their shortest
round-trip decimal without an exponent ("2.5", "5", "-0.05").

This recipe reads those two files where they lie in the reference tree (the
directory named by the CANTUCCI_REFERENCE environment variable),
fills them the same way for each entry of CONFIGS, and writes the filled
text only under oracle/_ref/ (git-ignored), together with a generated
wrapper that puts each filled shader in its own namespace over the GLSL
shim oracle/ref_shader_shim.h.  It then compiles the wrapper with g++
(single-precision literals, no contraction) into a shared library:

    int ref_shader_count(void);
    void ref_shader_de(int config, const float* xyz, unsigned long long n, float* out);

The reference tree is only needed to build the library; the fixtures made
from it (tests/golden/make_shader_golden.py) travel without it.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_shader.so")
# The cantucci source tree; the recipe does nothing without it.
REFERENCE = os.environ.get("CANTUCCI_REFERENCE")
SHADERS = {"mandelbulb": "src/shape/mandelbulb.frag", "sphere": "src/shape/shape.frag"}

# (name, kind, parameters).  Mandelbulb: power (integer), max_iters, bailout.
# Sphere: centre x, y, z and radius.
CONFIGS = [
    ("p8_i15_b2.5", "mandelbulb", (8, 15, 2.5)),
    ("p8_i8_b5", "mandelbulb", (8, 8, 5.0)),
    ("p6_i10_b2.5", "mandelbulb", (6, 10, 2.5)),
    ("p3_i6_b2", "mandelbulb", (3, 6, 2.0)),
    ("p10_i20_b2.5", "mandelbulb", (10, 20, 2.5)),
    ("sphere_offset", "sphere", (0.1, -0.05, 0.02, 0.9)),
    ("sphere_unit", "sphere", (0.0, 0.0, 0.0, 1.0)),
]

# -fno-builtin keeps every libm call a call: with the power a literal, GCC
# would otherwise fold pow(r, 2.0) into r * r, which differs from glibc's
# powf in the last bit on some inputs (the P=3 shader).
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
            "-fsingle-precision-constant", "-fno-builtin", "-Wall"]


def rust_f32(x: float) -> str:
    """Display of an f32 in Rust: shortest round-trip digits, no exponent,
    no trailing ".0" ("2.5", "5", "-0.05")."""
    return np.format_float_positional(np.float32(x), unique=True, trim="-")


def fill(kind: str, params) -> str:
    with open(os.path.join(REFERENCE, SHADERS[kind])) as f:
        text = f.read()
    if kind == "mandelbulb":
        power, iters, bailout = params
        subs = {"{BAILOUT}": rust_f32(bailout), "{MAX_ITERS}": str(int(iters)),
                "{POWER}": str(int(power))}
    else:
        x, y, z, radius = params
        subs = {"{X}": rust_f32(x), "{Y}": rust_f32(y), "{Z}": rust_f32(z),
                "{RADIUS}": rust_f32(radius)}
    for k, v in subs.items():
        text = text.replace(k, v)
    return text


def available() -> bool:
    return bool(REFERENCE) and all(os.path.exists(os.path.join(REFERENCE, p))
                                   for p in SHADERS.values())


def _wrapper() -> str:
    lines = ['#include "ref_shader_shim.h"', ""]
    for i, (name, _, _) in enumerate(CONFIGS):
        lines += ["namespace cfg%d {  // %s" % (i, name), "using namespace glsl;",
                  '#include "cfg%d.frag"' % i, "}", ""]
    lines += ['extern "C" int ref_shader_count(void) { return %d; }' % len(CONFIGS), "",
              'extern "C" void ref_shader_de(int config, const float* xyz, '
              "unsigned long long n, float* out) {",
              "    for (unsigned long long i = 0; i < n; ++i) {",
              "        const glsl::vec3 p(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);",
              "        switch (config) {"]
    for i in range(len(CONFIGS)):
        lines.append("        case %d: out[i] = cfg%d::shape_de(p); break;" % (i, i))
    lines += ["        default: out[i] = 0.0f;", "        }", "    }", "}", ""]
    return "\n".join(lines)


def build(force: bool = False):
    """Fill, wrap and compile; returns the library path, or None when the
    reference tree is not present (then an earlier build is kept)."""
    if not available():
        return LIB if os.path.exists(LIB) else None
    os.makedirs(OUT_DIR, exist_ok=True)
    sources = {"cfg%d.frag" % i: fill(kind, params) for i, (_, kind, params) in enumerate(CONFIGS)}
    sources["shaders.cpp"] = _wrapper()
    changed = force or not os.path.exists(LIB)
    for name, text in sources.items():
        p = os.path.join(OUT_DIR, name)
        if not os.path.exists(p) or open(p).read() != text:
            with open(p, "w") as f:
                f.write(text)
            changed = True
    shim = os.path.join(HERE, "ref_shader_shim.h")
    if not changed and os.path.getmtime(LIB) >= max(os.path.getmtime(shim),
                                                    os.path.getmtime(__file__)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", *CXXFLAGS, "-I", HERE, "-I", OUT_DIR, os.path.join(OUT_DIR, "shaders.cpp"),
           "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
