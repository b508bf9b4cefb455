// Texture sampling as the reference's present pass configures it
// (Source/GraphicsDevice.cpp:770-790: linear min/mag filter, clamp-to-border
// with opaque black, normalised coordinates, one mip level), written from the
// texel-filtering equations of the Vulkan specification:
//   u = s * width - 0.5,  i0 = floor(u),  alpha = u - i0   (v, j0, beta alike)
//   tau = (1-alpha)(1-beta) T[i0,j0] + alpha(1-beta) T[i0+1,j0]
//       + (1-alpha) beta T[i0,j0+1] + alpha beta T[i0+1,j0+1]
// where a texel outside the image reads the border colour (0, 0, 0, 1).  The
// specification leaves the sub-texel precision of alpha and beta to the
// implementation; here they are exact floats.  An R8G8B8A8_UNORM texel c
// reads as c / 255.
//
// Test infrastructure: shared by the oracle and the harness that compiles
// the reference's fragment shader (Assets/Fullscreen.frag); the CUDA present
// kernel restates the same steps.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>

struct PresentImage {
    const void* data;  // w x h texels, row j = texel row j (t grows with j)
    uint32_t w, h;
    int is_float;      // 0: RGBA8 UNORM bytes; 1: RGBA float32
};

static inline void present_texel(const PresentImage& im, int i, int j, float out[3])
{
    if (i < 0 || j < 0 || i >= (int)im.w || j >= (int)im.h) {
        out[0] = out[1] = out[2] = 0.0f;
        return;
    }
    const size_t k = (size_t)j * im.w + (size_t)i;
    if (im.is_float) {
        const float* p = static_cast<const float*>(im.data) + 4 * k;
        out[0] = p[0];
        out[1] = p[1];
        out[2] = p[2];
    } else {
        const uint8_t* p = static_cast<const uint8_t*>(im.data) + 4 * k;
        out[0] = (float)p[0] / 255.0f;
        out[1] = (float)p[1] / 255.0f;
        out[2] = (float)p[2] / 255.0f;
    }
}

static inline void present_sample(const PresentImage& im, float s, float t, float out[3])
{
    const float u = s * (float)im.w - 0.5f;
    const float v = t * (float)im.h - 0.5f;
    const float fi = std::floor(u), fj = std::floor(v);
    const float al = u - fi, be = v - fj;
    const int i0 = (int)fi, j0 = (int)fj;
    const float w00 = (1.0f - al) * (1.0f - be);
    const float w10 = al * (1.0f - be);
    const float w01 = (1.0f - al) * be;
    const float w11 = al * be;
    float a[3], b[3], c[3], d[3];
    present_texel(im, i0, j0, a);
    present_texel(im, i0 + 1, j0, b);
    present_texel(im, i0, j0 + 1, c);
    present_texel(im, i0 + 1, j0 + 1, d);
    for (int k = 0; k < 3; ++k) out[k] = ((w00 * a[k] + w10 * b[k]) + w01 * c[k]) + w11 * d[k];
}
