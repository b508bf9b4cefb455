// The reference's legacy Whitted shader, Assets/Raytracer.comp, for sm_103a:
// one thread per pixel over the shader's constant scene (one triangle, two
// spheres, five planes; :92-127), Blinn-Phong shading from one point light
// with a shadow ray (:272-334), up to two mirror bounces blended with a
// reflection strength that halves per bounce (:363-373).  The reference's
// program never loads this shader (it dispatches Tracer.comp); it is built
// here as the second shading model of the reference's assets.
//
// Every operation is one IEEE single-precision operation in the shader's
// order (--fmad=false), so the output equals the oracle's bit for bit except
// where powf (the specular exponent 16, :305) differs in the last ulp between
// CUDA and the host C library.  The scene is tiny and constant: the kernel is
// compute-bound (~60 flops per primitive test, 8 tests per ray).

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_launch.h"

namespace vkt {

namespace whitted {

constexpr float MAX_DISTANCE = 1000.0f, EPS = 0.01f;  // Raytracer.comp:92-93
constexpr uint32_t BOUNCES = 2;                       // :94

struct Sph {
    uint32_t mat;
    float cx, cy, cz, r;
};
struct Pl {
    uint32_t mat;
    float nx, ny, nz, dist;
};
__constant__ Sph kSpheres[2] = {{5, -14.0f, 12.0f, 32.0f, 5.0f}, {4, 32.0f, 24.0f, 25.0f, 12.0f}};
__constant__ Pl kPlanes[5] = {{0, 0.0f, 1.0f, 0.0f, 0.0f},
                              {0, 0.0f, -1.0f, 0.0f, 128.0f},
                              {2, 0.0f, 0.0f, -1.0f, 64.0f},
                              {1, 1.0f, 0.0f, 0.0f, 64.0f},
                              {3, -1.0f, 0.0f, 0.0f, 64.0f}};
__constant__ float kTri[9] = {10.0f, 10.0f, 0.0f, 0.0f, 20.0f, 0.0f, -10.0f, 10.0f, 0.0f};
constexpr uint32_t kTriMat = 1;
__constant__ int kReflective[6] = {1, 0, 1, 0, 0, 0};
__constant__ float kDiffuse[18] = {1, 1, 1, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 1, 0, 1, 0, 1};

struct WHit {
    uint32_t mat;
    float dist;
    V3 point, normal;
};

__device__ __forceinline__ V3 tri_v(int k) { return v3(kTri[3 * k], kTri[3 * k + 1], kTri[3 * k + 2]); }

// :129-163 (one-sided, det < 0.01 misses)
__device__ __forceinline__ float tri_hit(const Ray& r)
{
    const V3 v0 = tri_v(0);
    const V3 v0v1 = tri_v(1) - v0, v0v2 = tri_v(2) - v0;
    const V3 pvec = cross(r.d, v0v2);
    const float det = dot(v0v1, pvec);
    if (det < EPS) return -1.0f;
    const float inv = 1.0f / det;
    const V3 tvec = r.o - v0;
    const float u = dot(tvec, pvec) * inv;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    const V3 qvec = cross(tvec, v0v1);
    const float v = dot(r.d, qvec) * inv;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    return dot(v0v2, qvec) * inv;
}

// :165-180 (the near root only)
__device__ __forceinline__ float sph_hit(const Ray& r, const Sph& s)
{
    const V3 oc = r.o - v3(s.cx, s.cy, s.cz);
    const float b = 2.0f * dot(oc, r.d);
    const float c = dot(oc, oc) - s.r * s.r;
    const float h = b * b - 4.0f * c;
    if (h < 0.0f) return -1.0f;
    return (-b - sqrtf(h)) / 2.0f;
}

// :182-194
__device__ __forceinline__ float pl_hit(const Ray& r, const Pl& p)
{
    const V3 n = v3(p.nx, p.ny, p.nz);
    const float d = dot(r.d, n);
    if (d == 0.0f) return 0.0f;
    const float dist = -(p.dist + dot(r.o, n)) / d;
    return gmax(dist, 0.0f);
}

// :218-270: triangle, spheres, planes; a later primitive wins only if strictly nearer
__device__ __forceinline__ bool trace(const Ray& r, WHit& h)
{
    bool found = false;
    const float td = tri_hit(r);
    if (td > EPS && td < h.dist) {
        h.dist = td;
        h.mat = kTriMat;
        h.point = r.o + td * r.d;
        const V3 u = tri_v(1) - tri_v(0), v = tri_v(2) - tri_v(0);
        h.normal = v3((u.y * v.z) - (u.z * v.y), (u.z * v.x) - (u.x * v.z), (u.x * v.y) - (u.y * v.x));
        found = true;
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const Sph s = kSpheres[i];
        const float sd = sph_hit(r, s);
        if (sd > EPS && sd < h.dist) {
            h.dist = sd;
            h.mat = s.mat;
            h.point = r.o + sd * r.d;
            h.normal = (h.point - v3(s.cx, s.cy, s.cz)) / s.r;
            found = true;
        }
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const Pl p = kPlanes[i];
        const float pd = pl_hit(r, p);
        if (pd > EPS && pd < h.dist) {
            h.dist = pd;
            h.mat = p.mat;
            h.point = r.o + pd * r.d;
            h.normal = v3(p.nx, p.ny, p.nz);
            found = true;
        }
    }
    return found;
}

// :272-340; returns the colour (alpha 1), updates the ray and the bounce depth
template <bool STATS>
__device__ __forceinline__ V3 render_scene(Ray& ray, uint32_t& depth, V3 light, V3 cpos, Counters& cnt)
{
    WHit h;
    h.mat = 0;
    h.dist = MAX_DISTANCE;
    if (STATS) cnt.c[C_CLOSEST]++;
    if (!trace(ray, h)) return splat(0.0f);
    if (STATS) cnt.c[C_HITS]++;
    const V3 light_vec = normalize(light - h.point);
    const float dist_to_light = length(light - h.point);
    const V3 li = (540.0f * splat(1.0f)) / (4.0f * 3.14159268f * dist_to_light);
    const V3 diffuse = li * v3(kDiffuse[3 * h.mat], kDiffuse[3 * h.mat + 1], kDiffuse[3 * h.mat + 2]) *
                       gmax(dot(h.normal, light_vec), 0.0f);
    const V3 half_vec = normalize(light_vec + normalize(cpos));
    const V3 specular = li * powf(gclamp(dot(h.normal, half_vec), 0.0f, 1.0f), 16.0f);
    V3 color = diffuse + specular;
    WHit sh;
    sh.mat = 0;
    sh.dist = dist_to_light;
    if (STATS) cnt.c[C_SHADOW]++;
    if (trace(Ray{h.point, light_vec}, sh)) {
        color = color * 0.5f;
        depth = BOUNCES + 1;
    }
    if (kReflective[h.mat]) {
        ray.d = ray.d - 2.0f * dot(h.normal, ray.d) * h.normal;
        ray.o = h.point;
    } else {
        depth = BOUNCES + 1;
    }
    return color;
}

}  // namespace whitted

template <bool STATS>
__global__ void __launch_bounds__(256) k_whitted(TraceArgs a)
{
    using namespace whitted;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    const uint32_t x = blockIdx.x * 16 + (threadIdx.x & 15);
    const uint32_t y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x < a.width && y < a.height) {
        // :344-361
        const float uvx = (float)x / (float)a.width, uvy = (float)y / (float)a.height;
        const float tx = 2.0f * uvx - 1.0f, ty = 2.0f * uvy - 1.0f;
        const V3 dir = ((a.fr.cdir + a.fr.cright * tx) + a.fr.cup * ty) * v3(a.fr.aspect, 1.0f, a.fr.aspect);
        uint32_t bounce = 0;
        Ray ray{a.fr.cpos, normalize(dir)};
        const V3 light = a.fr.light;
        V3 fc = render_scene<STATS>(ray, bounce, light, a.fr.cpos, cnt);
        float fa = 1.0f;
        float rs = 0.4f;
        // :363-373: final = (1 - s) final + s mix(reflection, final, 1 - s)
        while (++bounce <= BOUNCES) {
            const V3 rc = render_scene<STATS>(ray, bounce, light, a.fr.cpos, cnt);
            const float k = 1.0f - rs;
            const V3 m = rc + k * (fc - rc);
            const float ma = 1.0f + k * (fa - 1.0f);
            fc = k * fc + rs * m;
            fa = k * fa + rs * ma;
            rs = rs * 0.5f;
        }
        const size_t i = (size_t)y * a.width + x;
        if (a.rgba8) a.rgba8[i] = make_uchar4(unorm8(fc.x), unorm8(fc.y), unorm8(fc.z), unorm8(fa));
        if (a.rgba32f) a.rgba32f[i] = make_float4(fc.x, fc.y, fc.z, fa);
    }
    if (STATS) flush_counters(a, cnt);
}

cudaError_t launch_whitted(const TraceArgs& a, int stats, cudaStream_t s)
{
    const dim3 grid((a.width + 15) / 16, (a.height + 15) / 16);
    if (stats)
        k_whitted<true><<<grid, 256, 0, s>>>(a);
    else
        k_whitted<false><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace vkt
