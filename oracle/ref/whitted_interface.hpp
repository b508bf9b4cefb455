// Host stand-ins for the GLSL resource interface of Assets/Raytracer.comp:
// the rgba8 storage image at binding 0 (:19) and the FrameData push-constant
// block (:83-90: aspect_ratio @0, light_pos @16, camera @32 -- the same
// offsets as the host's FrameData, whose seed @4 this shader does not read).
// Included where the push-constant block stood, after the shader's Camera.
#pragma once

struct HostImage {
    int w = 0, h = 0;
    float* rgba32f = nullptr;
    uint8_t* rgba8 = nullptr;
};

struct HostInvocationId {
    uvec2 xy;
};

static HostImage result_image;
static HostInvocationId gl_GlobalInvocationID;

static float aspect_ratio;
static vec3 light_pos;
static Camera camera;

static inline ivec2 imageSize(HostImage const& img) { return ivec2(img.w, img.h); }

// UNORM8 conversion of an rgba8 storage image: clamp to [0,1], scale by 255,
// round to nearest; NaN stores 0.
static inline uint8_t unorm8(float x)
{
    if (!(x == x)) return 0;
    float c = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return (uint8_t)std::floor(c * 255.0f + 0.5f);
}

static inline void imageStore(HostImage& img, ivec2 p, vec4 c)
{
    size_t i = (size_t)p.y * (size_t)img.w + (size_t)p.x;
    if (img.rgba32f) {
        img.rgba32f[4 * i + 0] = c.x;
        img.rgba32f[4 * i + 1] = c.y;
        img.rgba32f[4 * i + 2] = c.z;
        img.rgba32f[4 * i + 3] = c.w;
    }
    if (img.rgba8) {
        img.rgba8[4 * i + 0] = unorm8(c.x);
        img.rgba8[4 * i + 1] = unorm8(c.y);
        img.rgba8[4 * i + 2] = unorm8(c.z);
        img.rgba8[4 * i + 3] = unorm8(c.w);
    }
}
