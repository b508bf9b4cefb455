// CPU restatement of the steps around the reference's compute dispatch:
//   - the present pass, Assets/Fullscreen.frag (with the fullscreen triangle
//     of Assets/Fullscreen.vert and the sampler of
//     Source/GraphicsDevice.cpp:770-790, present_sampler.h);
//   - the running mean that the progressive (accumulating) present mode
//     reads in place of the reference's two frame images;
//   - the camera controller, Source/Camera.cpp:5-64, driven by the input
//     handling of Source/Main.cpp:23-83 and :150-180.
//
// Test infrastructure only: tests, smoke() and the bench's CPU baseline call
// it as the checker.  Built with -ffp-contract=off: every float operation
// rounds once, in the order written.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "oracle_api.h"
#include "present_sampler.h"

namespace {

uint8_t unorm8(float x)
{
    if (!(x == x)) return 0;
    const float c = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return (uint8_t)std::floor(c * 255.0f + 0.5f);
}

// ---- camera (Camera.cpp with glm 0.9.9 float normalize / cross / dot) ----
struct V {
    float x, y, z;
};
V add(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V sub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V mul(V a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dot(V a, V b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
V normalize(V v)
{
    const float s = 1.0f / std::sqrt(dot(v, v));
    return mul(v, s);
}
V cross(V a, V b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
V ld(const float* p) { return {p[0], p[1], p[2]}; }
void st(float* p, V v)
{
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

// glm::radians(float): degrees times the float nearest to pi / 180.
constexpr float kDegToRad = 0.01745329251994329576923690768489f;

}  // namespace

extern "C" {

// One output pixel (x, y) of the present pass; (x, y) = (0, 0) is the top-left
// pixel of the framebuffer.  Fullscreen.vert:8-10 draws one triangle over the
// viewport with uv = (ndc + 1) / 2, so the fragment at pixel centre (x + 0.5,
// y + 0.5) of a W x H viewport has uv_coords = ((x + 0.5) / W, (y + 0.5) / H).
// Fullscreen.frag:16-30:
//   uv = (uv_coords.s, 1 - uv_coords.t)       (the traced image's row 0 is its bottom)
//   color_0 = image0(uv), color_1 = image1(uv)
//   N, S, E, W = image0(uv + (0, +-1/2048)), image0(uv + (+-1/2048, 0))
//   vT = dot(color_0 - color_1, color_0 - color_1)
//   out = vT > 0.0005 ? (N + S + E + W) / 4 : color_0, alpha 1
void oracle_present(const void* image0, const void* image1, int src_is_float, uint32_t src_w, uint32_t src_h,
                    uint32_t width, uint32_t height, float* out_rgba32f, uint8_t* out_rgba8)
{
    const PresentImage i0{image0, src_w, src_h, src_is_float};
    const PresentImage i1{image1, src_w, src_h, src_is_float};
    const float inv = 1.0f / 2048.0f;
#pragma omp parallel for schedule(static)
    for (int64_t y = 0; y < (int64_t)height; ++y) {
        for (uint32_t x = 0; x < width; ++x) {
            const float us = ((float)x + 0.5f) / (float)width;
            const float ut = ((float)y + 0.5f) / (float)height;
            const float s = us, t = 1.0f - ut;
            float c0[3], c1[3], n[3], so[3], e[3], w[3];
            present_sample(i0, s, t, c0);
            present_sample(i1, s, t, c1);
            present_sample(i0, s + 0.0f * inv, t + 1.0f * inv, n);
            present_sample(i0, s + 0.0f * inv, t + -1.0f * inv, so);
            present_sample(i0, s + 1.0f * inv, t + 0.0f * inv, e);
            present_sample(i0, s + -1.0f * inv, t + 0.0f * inv, w);
            const float d0 = c0[0] - c1[0], d1 = c0[1] - c1[1], d2 = c0[2] - c1[2];
            const float vT = (d0 * d0 + d1 * d1) + d2 * d2;
            float f[3];
            for (int k = 0; k < 3; ++k) f[k] = vT > 0.0005f ? (((n[k] + so[k]) + e[k]) + w[k]) / 4.0f : c0[k];
            const size_t o = (size_t)y * width + x;
            if (out_rgba32f) {
                out_rgba32f[4 * o + 0] = f[0];
                out_rgba32f[4 * o + 1] = f[1];
                out_rgba32f[4 * o + 2] = f[2];
                out_rgba32f[4 * o + 3] = 1.0f;
            }
            if (out_rgba8) {
                out_rgba8[4 * o + 0] = unorm8(f[0]);
                out_rgba8[4 * o + 1] = unorm8(f[1]);
                out_rgba8[4 * o + 2] = unorm8(f[2]);
                out_rgba8[4 * o + 3] = 255;
            }
        }
    }
}

// Progressive accumulation, one frame: sum += linear (float, per channel),
// then display = tonemap(sum / n) with the reference's tonemap
// (Tracer.comp:586-588: Reinhard x / (x + 1), then pow 1/2.2; no dither).
// n is the number of frames in the sum after this one.
void oracle_accumulate(const float* linear_rgba, float* sum_rgba, uint32_t n_pixels, uint32_t n, float* display_rgba)
{
    const float gam = 1.0f / 2.2f;
    for (uint32_t i = 0; i < n_pixels; ++i) {
        for (int c = 0; c < 3; ++c) {
            const float s = sum_rgba[4 * i + c] + linear_rgba[4 * i + c];
            sum_rgba[4 * i + c] = s;
            float m = s / (float)n;
            m = m / (m + 1.0f);
            display_rgba[4 * i + c] = std::pow(m, gam);
        }
        sum_rgba[4 * i + 3] = 1.0f;
        display_rgba[4 * i + 3] = 1.0f;
    }
}

// Camera::update, Camera.cpp:48-64.  cam: pos, dir, right, up (4 x float4),
// front (3), pitch, yaw.
void oracle_camera_update(oracle_camera_ctl* c)
{
    c->pitch = std::clamp(c->pitch, -89.0f, 89.0f);
    const float pr = c->pitch * kDegToRad;
    const float yr = c->yaw * kDegToRad;
    // cos/sin of a float argument: the C library's double functions (the
    // argument is promoted), products in double, rounded to float on store
    V front;
    front.x = (float)(std::cos((double)pr) * std::cos((double)yr));
    front.y = (float)std::sin((double)pr);
    front.z = (float)(std::cos((double)pr) * std::sin((double)yr));
    front = normalize(front);
    st(c->front, front);
    const V pos = ld(c->cam + 0);
    const V dir = normalize(sub(add(pos, front), pos));
    V up{0.0f, 1.0f, 0.0f};
    const V right = normalize(cross(up, dir));
    up = cross(dir, right);
    st(c->cam + 4, dir);
    st(c->cam + 8, right);
    st(c->cam + 12, up);
}

// Camera::Camera, Camera.cpp:5-10.
void oracle_camera_init(oracle_camera_ctl* c)
{
    std::memset(c, 0, sizeof *c);
    c->cam[0] = 0.0f;
    c->cam[1] = 64.0f;
    c->cam[2] = -48.0f;
    c->front[2] = -1.0f;
    c->pitch = 0.0f;
    c->yaw = 90.0f;
    oracle_camera_update(c);
}

// Camera::move_*, Camera.cpp:12-46.  dir: 0 forward, 1 backward, 2 left,
// 3 right, 4 up, 5 down.
void oracle_camera_move(oracle_camera_ctl* c, int dir, float speed)
{
    V pos = ld(c->cam);
    const V front = ld(c->front), right = ld(c->cam + 8), up = ld(c->cam + 12);
    switch (dir) {
    case 0: pos = add(pos, mul(front, speed)); break;
    case 1: pos = sub(pos, mul(front, speed)); break;
    case 2: pos = sub(pos, mul(right, speed)); break;
    case 3: pos = add(pos, mul(right, speed)); break;
    case 4: pos = add(pos, mul(up, speed)); break;
    case 5: pos = sub(pos, mul(up, speed)); break;
    default: return;
    }
    st(c->cam, pos);
    oracle_camera_update(c);
}

// mouse_callback, Main.cpp:66-83: the offset is taken in double against the
// float last position, stored to float, scaled by 0.21; yaw -= dx, pitch += dy.
void oracle_camera_mouse(oracle_camera_ctl* c, double x, double y)
{
    float ox = (float)(x - (double)c->last_mouse[0]);
    float oy = (float)((double)c->last_mouse[1] - y);
    c->last_mouse[0] = (float)x;
    c->last_mouse[1] = (float)y;
    const float sensitivity = 0.21f;
    ox *= sensitivity;
    oy *= sensitivity;
    c->yaw -= ox;
    c->pitch += oy;
    oracle_camera_update(c);
}

// poll_keyboard, Main.cpp:23-51: W else S, A else D, R else F, each moving by
// 111 * dt.  keys: bit 0 W, 1 S, 2 A, 3 D, 4 R, 5 F.
void oracle_camera_keyboard(oracle_camera_ctl* c, uint32_t keys, float dt)
{
    const float sensitivity = 111.0f;
    const float speed = sensitivity * dt;
    if (keys & 1u)
        oracle_camera_move(c, 0, speed);
    else if (keys & 2u)
        oracle_camera_move(c, 1, speed);
    if (keys & 4u)
        oracle_camera_move(c, 2, speed);
    else if (keys & 8u)
        oracle_camera_move(c, 3, speed);
    if (keys & 16u)
        oracle_camera_move(c, 4, speed);
    else if (keys & 32u)
        oracle_camera_move(c, 5, speed);
}

}  // extern "C"
