// Host driver for the reference's Source/Camera.cpp: computes CameraData
// (pos, dir, right, up; std430 16-byte lanes) from a position and the
// pitch/yaw pair, exactly as Camera::update does (Source/Camera.cpp:48-64).
#include <Camera.h>
#include <cstring>

extern "C" void ref_camera(float px, float py, float pz, float pitch, float yaw, float* out16)
{
    Camera cam;
    cam.data.pos = glm::vec3(px, py, pz);
    cam.aux.pitch = pitch;
    cam.aux.yaw = yaw;
    cam.update();
    const glm::vec3* v[4] = {&cam.data.pos, &cam.data.dir, &cam.data.right, &cam.data.up};
    for (int i = 0; i < 4; ++i) {
        out16[4 * i + 0] = v[i]->x;
        out16[4 * i + 1] = v[i]->y;
        out16[4 * i + 2] = v[i]->z;
        out16[4 * i + 3] = 0.0f;
    }
}
