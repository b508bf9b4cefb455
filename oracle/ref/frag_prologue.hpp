// Prologue for compiling the reference's present fragment shader
// (Assets/Fullscreen.frag) as C++: glm supplies the GLSL types and built-ins,
// and the GLSL resource interface becomes host globals of the same names.
//   uv_coords             the interpolated vertex output (Fullscreen.vert:4)
//   frag_color            the colour attachment output
//   raytraced_image,      combined image samplers at bindings 0 and 1
//   prev_raytraced_image  (Source/GraphicsDevice.cpp:955-983), sampled by
//                         present_sample (../present_sampler.h)
// texture() returns a value whose .rgb is the filtered texel; the shader reads
// nothing else of it.
#pragma once

#include <cstdint>
#include <glm/glm.hpp>

#include "../present_sampler.h"

using namespace glm;

struct HostSampler2D {
    PresentImage im;
};

struct HostTexel {
    vec3 rgb;
};

static inline HostTexel texture(const HostSampler2D& s, vec2 uv)
{
    float c[3];
    present_sample(s.im, uv.x, uv.y, c);
    return HostTexel{vec3(c[0], c[1], c[2])};
}

static vec2 uv_coords;
static vec4 frag_color;
static HostSampler2D raytraced_image;
static HostSampler2D prev_raytraced_image;
