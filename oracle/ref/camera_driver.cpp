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

// A sequence of Camera operations from the default-constructed camera
// (Camera.cpp:5-10): op 0..5 = move_forward, move_backward, move_left,
// move_right, move_up, move_down by arg[2i]; op 6 = yaw -= arg[2i], pitch +=
// arg[2i+1], update() (what Main.cpp:79-82 does with the scaled mouse
// offsets); op 7 = pos/pitch/yaw of the start-up camera (Main.cpp:134-139),
// update().  After each op: CameraData (16 floats), front (3), pitch, yaw.
extern "C" void ref_camera_ops(int n, const int* op, const float* arg, float* out21)
{
    Camera cam;
    for (int i = 0; i < n; ++i) {
        const float a = arg[2 * i], b = arg[2 * i + 1];
        switch (op[i]) {
        case 0: cam.move_forward(a); break;
        case 1: cam.move_backward(a); break;
        case 2: cam.move_left(a); break;
        case 3: cam.move_right(a); break;
        case 4: cam.move_up(a); break;
        case 5: cam.move_down(a); break;
        case 6:
            cam.aux.yaw -= a;
            cam.aux.pitch += b;
            cam.update();
            break;
        case 7:
            cam.data.pos = glm::vec3(32.8509f, 30.6991f, -106.389f);
            cam.aux.pitch = 4.44998f;
            cam.aux.yaw = -602.79f;
            cam.update();
            break;
        default: break;
        }
        float* o = out21 + 21 * (size_t)i;
        const glm::vec3* v[4] = {&cam.data.pos, &cam.data.dir, &cam.data.right, &cam.data.up};
        for (int k = 0; k < 4; ++k) {
            o[4 * k + 0] = v[k]->x;
            o[4 * k + 1] = v[k]->y;
            o[4 * k + 2] = v[k]->z;
            o[4 * k + 3] = 0.0f;
        }
        o[16] = cam.aux.front.x;
        o[17] = cam.aux.front.y;
        o[18] = cam.aux.front.z;
        o[19] = cam.aux.pitch;
        o[20] = cam.aux.yaw;
    }
}
