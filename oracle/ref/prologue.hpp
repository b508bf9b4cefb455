// Prologue for compiling the reference compute shader (Assets/Tracer.comp)
// as C++ on the host, against the reference's own vendored glm 0.9.9.3.
//
// This is test infrastructure: it turns the reference's GLSL into a CPU
// program whose outputs pin the oracle (oracle/tracer_oracle.cpp).  Nothing
// in the product links it.  The shader source is never copied: ref/Makefile
// streams it from the reference tree through a few mechanical rewrites
// (listed there) straight into g++.
//
// GLSL -> C++ mapping used here:
//   * glm provides the GLSL built-ins (dot, normalize, reflect, refract, mix,
//     clamp, fract, sign, pow, sqrt, cos, sin) and the vector types.
//   * -fsingle-precision-constant makes unsuffixed literals float, as in GLSL.
//   * -ffp-contract=off: no fused multiply-add is formed behind our back.
//   * GLSL interface blocks (image, SSBO, push constants) become the globals
//     declared in interface.hpp, filled by driver.inc before each invocation.
#pragma once

#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>
#include <cmath>
#include <cstdint>
#include <cstring>

using namespace glm;

// GLSL converts ivec2 -> vec2 implicitly in `vec2 / ivec2` (Tracer.comp:563).
inline vec2 operator/(vec2 const& a, ivec2 const& b) { return a / vec2(b); }

// GLSL swizzles are plain vec3 values; glm's swizzle proxies need an
// explicit conversion before template deduction (cross(w.yzx, w),
// Tracer.comp:259).
template <int N, typename T, qualifier Q, int E0, int E1, int E2, int E3>
inline vec<3, T, Q> cross(detail::_swizzle<N, T, Q, E0, E1, E2, E3> const& a, vec<3, T, Q> const& b)
{
    return glm::cross(a(), b);
}

// GLSL converts the int literal to float in `max(vec3, 0)` (Tracer.comp:479).
inline vec3 max(vec3 const& a, int b) { return glm::max(a, float(b)); }

// GLSL pow(genType, genType): the int exponent literal becomes a float
// (Tracer.comp:444, :475).  Evaluated as float pow, like every other pow.
inline float pow(float b, int e) { return std::pow(b, float(e)); }

#if defined(REF_TRIG_RNG)
// Optional: route the shader's cos/sin through the oracle's portable
// project-written cos/sin, so the harness can be compared with the oracle
// in its portable-trig mode as well as in libm mode.
#include "../rng_trig.h"
#define cos(x) oracle_rng_cos(x)
#define sin(x) oracle_rng_sin(x)
#endif

// GLSL qualifiers with no C++ meaning.
#define in
#define rand shader_rand
#define main shader_main
