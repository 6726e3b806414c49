/* ref_shader_shim.h -- the few GLSL types and built-ins that cantucci's
 * estimator shaders use (src/shape/mandelbulb.frag, src/shape/shape.frag),
 * as single-precision C++ on the host's libm, so that the shader source
 * itself compiles as C++.  Test infrastructure only: oracle/ref_build.py
 * fills the shader's placeholders as src/shape/mandelbulb.rs:82-85 and
 * src/shape/sphere.rs:42-46 do, wraps each filled shader in a namespace and
 * compiles it with this header into oracle/_ref/libref_shader.so.
 *
 * GLSL semantics kept here:
 *   - float literals are single precision (the recipe compiles with
 *     -fsingle-precision-constant);
 *   - length(v) = sqrt(dot(v, v)) with dot summed left to right,
 *     (x*x + y*y) + z*z, and no contraction (-ffp-contract=off);
 *   - atan(y, x) is the two-argument arctangent;
 *   - acos, pow, sin, cos, log are the single-precision libm functions.
 * No <math.h> or <cmath> is included, so the only overloads the shader
 * text sees are these float ones. */
#pragma once

extern "C" {
float sqrtf(float);
float acosf(float);
float atan2f(float, float);
float powf(float, float);
float sinf(float);
float cosf(float);
float logf(float);
}

namespace glsl {

struct vec3 {
    float x, y, z;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(float s, vec3 v) { return vec3(s * v.x, s * v.y, s * v.z); }

inline float length(vec3 v) { return sqrtf((v.x * v.x + v.y * v.y) + v.z * v.z); }
inline float acos(float x) { return acosf(x); }
inline float atan(float y, float x) { return atan2f(y, x); }
inline float pow(float x, float y) { return powf(x, y); }
inline float sin(float x) { return sinf(x); }
inline float cos(float x) { return cosf(x); }
inline float log(float x) { return logf(x); }

}  // namespace glsl
