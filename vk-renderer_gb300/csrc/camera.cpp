// Camera controller of the C ABI: the reference's Camera (Source/Camera.cpp:
// 5-64) and the input handling of its main loop (Source/Main.cpp:23-83,
// :148-180), for scripted camera paths.  Host code, single precision, built
// with -ffp-contract=off so each operation rounds once as written; vector
// operations follow glm 0.9.9 (dot = (x*x' + y*y') + z*z', normalize = v *
// (1 / sqrt(dot(v, v))), cross componentwise as written).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "tracer_abi.h"

namespace {

struct Vec {
    float x, y, z;
};
Vec add(Vec a, Vec b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
Vec sub(Vec a, Vec b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
Vec scale(Vec a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dot(Vec a, Vec b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
Vec normalize(Vec v) { return scale(v, 1.0f / std::sqrt(dot(v, v))); }
Vec cross(Vec a, Vec b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
Vec get(const float* p) { return {p[0], p[1], p[2]}; }
void put(float* p, Vec v)
{
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

// glm::radians(float): degrees times the float nearest to pi / 180
constexpr float kRadPerDeg = 0.01745329251994329576923690768489f;

}  // namespace

extern "C" {

void tracer_camera_update(tracer_camera_controller* c)
{
    if (!c) return;
    c->pitch = std::clamp(c->pitch, -89.0f, 89.0f);
    const float pr = c->pitch * kRadPerDeg, yr = c->yaw * kRadPerDeg;
    // cos/sin of a float argument resolve to the C library's double
    // functions (the argument is promoted); the products are double and are
    // rounded to float when stored
    Vec front;
    front.x = (float)(std::cos((double)pr) * std::cos((double)yr));
    front.y = (float)std::sin((double)pr);
    front.z = (float)(std::cos((double)pr) * std::sin((double)yr));
    front = normalize(front);
    put(c->front, front);
    const Vec pos = get(c->data.pos);
    const Vec dir = normalize(sub(add(pos, front), pos));
    const Vec right = normalize(cross(Vec{0.0f, 1.0f, 0.0f}, dir));
    const Vec up = cross(dir, right);
    put(c->data.dir, dir);
    put(c->data.right, right);
    put(c->data.up, up);
}

void tracer_camera_init(tracer_camera_controller* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    put(c->data.pos, Vec{0.0f, 64.0f, -48.0f});
    put(c->front, Vec{0.0f, 0.0f, -1.0f});
    put(c->light_pos, Vec{0.0f, 64.0f, 0.0f});  // Main.cpp:141
    c->pitch = 0.0f;
    c->yaw = 90.0f;
    tracer_camera_update(c);
}

void tracer_camera_init_startup(tracer_camera_controller* c)
{
    if (!c) return;
    tracer_camera_init(c);
    put(c->data.pos, Vec{32.8509f, 30.6991f, -106.389f});
    c->pitch = 4.44998f;
    c->yaw = -602.79f;
    tracer_camera_update(c);
}

int tracer_camera_move(tracer_camera_controller* c, int direction, float speed)
{
    if (!c || direction < 0 || direction > 5) return TRACER_ERR_INVALID_ARG;
    Vec pos = get(c->data.pos);
    const Vec front = get(c->front), right = get(c->data.right), up = get(c->data.up);
    switch (direction) {
    case 0: pos = add(pos, scale(front, speed)); break;
    case 1: pos = sub(pos, scale(front, speed)); break;
    case 2: pos = sub(pos, scale(right, speed)); break;
    case 3: pos = add(pos, scale(right, speed)); break;
    case 4: pos = add(pos, scale(up, speed)); break;
    default: pos = sub(pos, scale(up, speed)); break;
    }
    put(c->data.pos, pos);
    tracer_camera_update(c);
    return TRACER_OK;
}

void tracer_camera_cursor(tracer_camera_controller* c, double x, double y)
{
    if (!c) return;
    // the offsets are taken in double against the float last position and
    // stored to float (Main.cpp:68-72)
    float ox = (float)(x - (double)c->last_mouse[0]);
    float oy = (float)((double)c->last_mouse[1] - y);
    c->last_mouse[0] = (float)x;
    c->last_mouse[1] = (float)y;
    const float sensitivity = 0.21f;
    ox *= sensitivity;
    oy *= sensitivity;
    c->yaw -= ox;
    c->pitch += oy;
    tracer_camera_update(c);
}

void tracer_camera_keys(tracer_camera_controller* c, uint32_t keys, float dt)
{
    if (!c) return;
    const float speed = 111.0f * dt;
    if (keys & TRACER_KEY_W)
        tracer_camera_move(c, 0, speed);
    else if (keys & TRACER_KEY_S)
        tracer_camera_move(c, 1, speed);
    if (keys & TRACER_KEY_A)
        tracer_camera_move(c, 2, speed);
    else if (keys & TRACER_KEY_D)
        tracer_camera_move(c, 3, speed);
    if (keys & TRACER_KEY_R)
        tracer_camera_move(c, 4, speed);
    else if (keys & TRACER_KEY_F)
        tracer_camera_move(c, 5, speed);
}

int tracer_camera_script(tracer_camera_controller* c, const tracer_input_frame* in, uint32_t n,
                         tracer_frame* frames_out)
{
    if (!c || (n && !in)) return TRACER_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i) {
        // events of this frame's poll (Main.cpp:170): cursor, then the E key
        if (in[i].has_cursor) tracer_camera_cursor(c, in[i].cursor_x, in[i].cursor_y);
        if (in[i].toggle_light) c->light_locked = !c->light_locked;
        tracer_camera_keys(c, in[i].keys, in[i].dt);  // Main.cpp:172
        // Main.cpp:176-178: while locked the light follows the camera; when
        // unlocked it stays where it was
        if (c->light_locked) put(c->light_pos, add(get(c->data.pos), Vec{0.0f, -1.0f, 0.0f}));
        if (frames_out) {
            frames_out[i].camera = c->data;
            std::memcpy(frames_out[i].light_pos, c->light_pos, sizeof c->light_pos);
        }
    }
    return TRACER_OK;
}

}  // extern "C"
