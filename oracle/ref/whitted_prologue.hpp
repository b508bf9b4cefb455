// Prologue for compiling the reference's legacy Whitted compute shader
// (Assets/Raytracer.comp) as C++ on the host, against the reference's
// vendored glm 0.9.9.3 -- the same approach as prologue.hpp for Tracer.comp
// (test infrastructure only; the shader is streamed from the reference tree
// by ref/Makefile, never copied).
#pragma once

#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>
#include <cmath>
#include <cstdint>
#include <cstring>

using namespace glm;

// GLSL converts ivec2 -> vec2 implicitly in `vec2 / ivec2` (Raytracer.comp:362).
inline vec2 operator/(vec2 const& a, ivec2 const& b) { return a / vec2(b); }

// GLSL converts the int bounds of clamp(float, -1, 1) to float (Raytracer.comp:197).
inline float clamp(float x, int lo, int hi) { return glm::clamp(x, float(lo), float(hi)); }

#define in
#define main shader_main
