// CPU restatement of the reference's legacy Whitted compute shader,
// Assets/Raytracer.comp (its constant scene, one light, shadows, two mirror
// bounces blended by a decaying reflection strength).  The reference's
// program does not load this shader; it is the second shading model of its
// asset directory.
//
// Test infrastructure only (tests, smoke(), the bench's CPU baseline).
// Built with -ffp-contract=off; GLSL built-ins as glm 0.9.9.3 defines them:
// dot = (x*x' + y*y') + z*z', length = sqrt(dot), normalize = v * (1/sqrt(dot)),
// max(x, y) = x < y ? y : x, clamp = min(max()), mix(x, y, a) = x + a*(y - x).
#include <cmath>
#include <cstdint>

#include "oracle_api.h"

namespace {

struct V {
    float x, y, z;
};
V operator+(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V operator-(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V operator*(V a, V b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
V operator*(V a, float s) { return {a.x * s, a.y * s, a.z * s}; }
V operator*(float s, V a) { return {s * a.x, s * a.y, s * a.z}; }
V operator/(V a, float s) { return {a.x / s, a.y / s, a.z / s}; }
float dot(V a, V b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
float length(V v) { return std::sqrt(dot(v, v)); }
V normalize(V v) { return v * (1.0f / std::sqrt(dot(v, v))); }
V cross(V x, V y) { return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y}; }
float gmax(float x, float y) { return (x < y) ? y : x; }
float gmin(float x, float y) { return (y < x) ? y : x; }
float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }

struct Ray {
    V o, d;
};
struct Hit {
    uint32_t mat;
    float dist;
    V point, normal;
};

// Raytracer.comp:92-127: constants and the scene
constexpr float MAX_DISTANCE = 1000.0f, EPSILON = 0.01f;
constexpr uint32_t BOUNCES = 2;
struct Sph {
    uint32_t mat;
    V c;
    float r;
};
struct Pl {
    uint32_t mat;
    V n;
    float dist;
};
const Sph kSpheres[2] = {{5, {-14.0f, 12.0f, 32.0f}, 5.0f}, {4, {32.0f, 24.0f, 25.0f}, 12.0f}};
const Pl kPlanes[5] = {{0, {0.0f, 1.0f, 0.0f}, 0.0f},
                       {0, {0.0f, -1.0f, 0.0f}, 128.0f},
                       {2, {0.0f, 0.0f, -1.0f}, 64.0f},
                       {1, {1.0f, 0.0f, 0.0f}, 64.0f},
                       {3, {-1.0f, 0.0f, 0.0f}, 64.0f}};
const V kTri[3] = {{10.0f, 10.0f, 0.0f}, {0.0f, 20.0f, 0.0f}, {-10.0f, 10.0f, 0.0f}};
const uint32_t kTriMat = 1;
const bool kReflective[6] = {true, false, true, false, false, false};
const V kDiffuse[6] = {{1, 1, 1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}};

// :129-163
float tri_intersect(const Ray& r)
{
    const V v0v1 = kTri[1] - kTri[0];
    const V v0v2 = kTri[2] - kTri[0];
    const V pvec = cross(r.d, v0v2);
    const float det = dot(v0v1, pvec);
    if (det < EPSILON) return -1.0f;
    const float inv = 1.0f / det;
    const V tvec = r.o - kTri[0];
    const float u = dot(tvec, pvec) * inv;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    const V qvec = cross(tvec, v0v1);
    const float v = dot(r.d, qvec) * inv;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    return dot(v0v2, qvec) * inv;
}

// :165-180
float sphere_intersect(const Ray& r, const Sph& s)
{
    const V oc = r.o - s.c;
    const float b = 2.0f * dot(oc, r.d);
    const float c = dot(oc, oc) - s.r * s.r;
    const float h = b * b - 4.0f * c;
    if (h < 0.0f) return -1.0f;
    return (-b - std::sqrt(h)) / 2.0f;
}

// :182-194
float plane_intersect(const Ray& r, const Pl& p)
{
    const float d = dot(r.d, p.n);
    if (d == 0.0f) return 0.0f;
    const float dist = -(p.dist + dot(r.o, p.n)) / d;
    return gmax(dist, 0.0f);
}

// :218-270
bool trace(const Ray& r, Hit& h, oracle_stats* st, bool shadow)
{
    if (st) (shadow ? st->shadow_rays : st->closest_rays)++;
    bool found = false;
    const float td = tri_intersect(r);
    if (td > EPSILON && td < h.dist) {
        h.dist = td;
        h.mat = kTriMat;
        h.point = r.o + td * r.d;
        const V u = kTri[1] - kTri[0], v = kTri[2] - kTri[0];
        h.normal = {(u.y * v.z) - (u.z * v.y), (u.z * v.x) - (u.x * v.z), (u.x * v.y) - (u.y * v.x)};
        found = true;
    }
    for (const Sph& s : kSpheres) {
        const float sd = sphere_intersect(r, s);
        if (sd > EPSILON && sd < h.dist) {
            h.dist = sd;
            h.mat = s.mat;
            h.point = r.o + sd * r.d;
            h.normal = (h.point - s.c) / s.r;
            found = true;
        }
    }
    for (const Pl& p : kPlanes) {
        const float pd = plane_intersect(r, p);
        if (pd > EPSILON && pd < h.dist) {
            h.dist = pd;
            h.mat = p.mat;
            h.point = r.o + pd * r.d;
            h.normal = p.n;
            found = true;
        }
    }
    if (st && found && !shadow) st->hits++;
    return found;
}

struct C4 {
    float r, g, b, a;
};

// :272-340
C4 render_scene(Ray& ray, uint32_t& depth, V light_pos, V cam_pos, oracle_stats* st)
{
    V color{0.0f, 0.0f, 0.0f};
    Hit h;
    h.mat = 0;
    h.dist = MAX_DISTANCE;
    if (!trace(ray, h, st, false)) return {color.x, color.y, color.z, 1.0f};
    const V light_vec = normalize(light_pos - h.point);
    const float dist_to_light = length(light_pos - h.point);
    const V li = (540.0f * V{1.0f, 1.0f, 1.0f}) / (4.0f * 3.14159268f * dist_to_light);
    const V diffuse = li * kDiffuse[h.mat] * gmax(dot(h.normal, light_vec), 0.0f);
    const V half_vec = normalize(light_vec + normalize(cam_pos));
    const V specular = li * std::pow(gclamp(dot(h.normal, half_vec), 0.0f, 1.0f), 16.0f);
    color = diffuse + specular;
    Hit sh;
    sh.mat = 0;
    sh.dist = dist_to_light;
    const Ray shadow{h.point, light_vec};
    if (trace(shadow, sh, st, true)) {
        color = color * 0.5f;
        depth = BOUNCES + 1;
    }
    if (kReflective[h.mat]) {
        ray.d = ray.d - 2.0f * dot(h.normal, ray.d) * h.normal;
        ray.o = h.point;
    } else {
        depth = BOUNCES + 1;
    }
    return {color.x, color.y, color.z, 1.0f};
}

uint8_t unorm8(float x)
{
    if (!(x == x)) return 0;
    const float c = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return (uint8_t)std::floor(c * 255.0f + 0.5f);
}

}  // namespace

extern "C" void oracle_whitted(const float* f, uint32_t w, uint32_t h, float* rgba32f, uint8_t* rgba8,
                               oracle_stats* stats)
{
    const float aspect = f[0];
    const V light{f[4], f[5], f[6]};
    const V cpos{f[8], f[9], f[10]}, cdir{f[12], f[13], f[14]}, cright{f[16], f[17], f[18]}, cup{f[20], f[21], f[22]};
    oracle_stats total{};
#pragma omp parallel
    {
        oracle_stats st{};
#pragma omp for schedule(dynamic, 4)
        for (int64_t y = 0; y < (int64_t)h; ++y)
            for (uint32_t x = 0; x < w; ++x) {
                // :344-361
                const float uvx = (float)x / (float)w, uvy = (float)y / (float)h;
                const float tx = 2.0f * uvx - 1.0f, ty = 2.0f * uvy - 1.0f;
                V dir = (cdir + cright * tx) + cup * ty;
                dir = dir * V{aspect, 1.0f, aspect};
                uint32_t bounce = 0;
                Ray ray{cpos, normalize(dir)};
                C4 fc = render_scene(ray, bounce, light, cpos, &st);
                float rs = 0.4f;
                // :363-373
                while (++bounce <= BOUNCES) {
                    const C4 rc = render_scene(ray, bounce, light, cpos, &st);
                    const float k = 1.0f - rs;
                    const float ma[4] = {rc.r + k * (fc.r - rc.r), rc.g + k * (fc.g - rc.g), rc.b + k * (fc.b - rc.b),
                                         rc.a + k * (fc.a - rc.a)};
                    fc = {k * fc.r + rs * ma[0], k * fc.g + rs * ma[1], k * fc.b + rs * ma[2], k * fc.a + rs * ma[3]};
                    rs = rs * 0.5f;
                }
                const size_t i = (size_t)y * w + x;
                if (rgba32f) {
                    rgba32f[4 * i + 0] = fc.r;
                    rgba32f[4 * i + 1] = fc.g;
                    rgba32f[4 * i + 2] = fc.b;
                    rgba32f[4 * i + 3] = fc.a;
                }
                if (rgba8) {
                    rgba8[4 * i + 0] = unorm8(fc.r);
                    rgba8[4 * i + 1] = unorm8(fc.g);
                    rgba8[4 * i + 2] = unorm8(fc.b);
                    rgba8[4 * i + 3] = unorm8(fc.a);
                }
            }
#pragma omp critical
        {
            total.closest_rays += st.closest_rays;
            total.shadow_rays += st.shadow_rays;
            total.hits += st.hits;
        }
    }
    if (stats) *stats = total;
}
