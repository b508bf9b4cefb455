// Device-side math of the path tracer: vector helpers with GLSL semantics,
// the per-pixel RNG, the intersection routines, trace_ray and radiance.
//
// Restates Assets/Tracer.comp (stickyfingies/vk-renderer) for CUDA sm_103a.
// Compiled with --fmad=false: every + - * / rounds as written, in the order
// the shader writes it, so results agree bit for bit with any IEEE
// implementation of the same expressions.  The only fused operations are the
// explicit __fmaf_rn calls in the portable cos/sin and the BVH slab test,
// whose definitions use fma.  GLSL built-ins follow glm 0.9.9.3 (the
// reference's vendored GLSL library):
//   dot3 = (x*x' + y*y') + z*z'     normalize(v) = v * (1 / sqrt(dot(v, v)))
//   reflect(I, N) = I - N * dot(N, I) * 2      mix(x, y, a) = x + a * (y - x)
//   max(x, y) = x < y ? y : x       min(x, y) = y < x ? y : x
//   refract(I, N, eta): k = 1 - eta*eta*(1 - d*d); k >= 0 ? eta*I - (eta*d + sqrt k)*N : 0
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vkt {

// ------------------------------------------------------------ constants --
constexpr float PI = 3.14159265359f;       // Tracer.comp:176
constexpr float EPSILON = 1e-3f;           // Tracer.comp:177
constexpr uint32_t MAT_DIFFUSE = 0;        // Tracer.comp:51
constexpr uint32_t MAT_DIELECTRIC = 1;     // Tracer.comp:52
constexpr uint32_t NO_PRIM = 0xFFFFFFFFu;
constexpr float BOX_SLACK = 1.0f + 0x1.0p-20f;

enum : int { TIE_REFERENCE = 0, TIE_STRICT = 1 };
enum : int { ST_OK = 0, ST_TRAVERSAL_LIMIT = 1, ST_STACK_OVERFLOW = 2 };
enum : int { C_CLOSEST = 0, C_SHADOW, C_NODES, C_TRIS, C_SPHERES, C_PLANES, C_HITS, C_COUNT };

// ------------------------------------------------------------ vectors --
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 splat(float s) { return V3{s, s, s}; }
__device__ __forceinline__ V3 v3(float4 a) { return V3{a.x, a.y, a.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ V3 operator-(float s, V3 a) { return {s - a.x, s - a.y, s - a.z}; }
__device__ __forceinline__ V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
__device__ __forceinline__ V3 operator-(V3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
__device__ __forceinline__ bool operator==(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ __forceinline__ V3 vmax0(V3 a) { return {gmax(a.x, 0.0f), gmax(a.y, 0.0f), gmax(a.z, 0.0f)}; }
__device__ __forceinline__ V3 vclamp01(V3 a) { return {gclamp(a.x, 0.f, 1.f), gclamp(a.y, 0.f, 1.f), gclamp(a.z, 0.f, 1.f)}; }
__device__ __forceinline__ float gsign(float x) { return float(0.0f < x) - float(x < 0.0f); }

__device__ __forceinline__ float dot(V3 a, V3 b)
{
    V3 t = a * b;
    return t.x + t.y + t.z;
}
__device__ __forceinline__ float length(V3 v) { return sqrtf(dot(v, v)); }
__device__ __forceinline__ V3 normalize(V3 v) { return v * (1.0f / sqrtf(dot(v, v))); }
__device__ __forceinline__ V3 cross(V3 x, V3 y)
{
    return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
__device__ __forceinline__ V3 reflect(V3 I, V3 N) { return I - N * dot(N, I) * 2.0f; }
__device__ __forceinline__ V3 refract(V3 I, V3 N, float eta)
{
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    return (k >= 0.0f) ? (eta * I - (eta * d + sqrtf(k)) * N) : splat(0.0f);
}
__device__ __forceinline__ float gmix(float x, float y, float a) { return x + a * (y - x); }
__device__ __forceinline__ V3 vmix(V3 x, V3 y, float a) { return x + a * (y - x); }
__device__ __forceinline__ bool isnan3(V3 v) { return v.x != v.x || v.y != v.y || v.z != v.z; }
__device__ __forceinline__ float max3(V3 e) { return gmax(gmax(e.x, e.y), e.z); }  // Tracer.comp:236-239

// ------------------------------------------------- portable cos / sin --
// Cody-Waite reduction by pi/2 split in three floats (each the float nearest
// to what remains of pi/2, pi from Machin's formula), then Taylor series of
// cos to r^12 and sin to r^11 (coefficients 1/n! rounded to float), Horner
// with fma.  Every step is one IEEE single operation, so host and device give
// identical bits; this fixes the reference RNG's stream (its cos argument
// reaches ~1e6, where any ulp of cos error changes the stream).
constexpr float TRIG_TWO_OVER_PI = 0x1.45f306p-1f;
constexpr float TRIG_C1 = 0x1.921fb6p+0f;
constexpr float TRIG_C2 = -0x1.777a5cp-25f;
constexpr float TRIG_C3 = -0x1.ee59dap-50f;

__device__ __forceinline__ float trig_reduce(float x, int& q)
{
    float k = rintf(__fmul_rn(x, TRIG_TWO_OVER_PI));
    float r = __fmaf_rn(-k, TRIG_C1, x);
    r = __fmaf_rn(-k, TRIG_C2, r);
    r = __fmaf_rn(-k, TRIG_C3, r);
    float kq = k - 4.0f * floorf(k * 0.25f);
    q = (kq == kq) ? (int)kq : 0;
    return r;
}
__device__ __forceinline__ float cos_poly(float r)
{
    float z = __fmul_rn(r, r);
    float p = __fmaf_rn(z, 0x1.1eed8ep-29f, -0x1.27e4fcp-22f);
    p = __fmaf_rn(z, p, 0x1.a01a02p-16f);
    p = __fmaf_rn(z, p, -0x1.6c16c2p-10f);
    p = __fmaf_rn(z, p, 0x1.555556p-5f);
    p = __fmaf_rn(z, p, -0x1.0p-1f);
    return __fmaf_rn(z, p, 1.0f);
}
__device__ __forceinline__ float sin_poly(float r)
{
    float z = __fmul_rn(r, r);
    float p = __fmaf_rn(z, -0x1.ae6456p-26f, 0x1.71de3ap-19f);
    p = __fmaf_rn(z, p, -0x1.a01a02p-13f);
    p = __fmaf_rn(z, p, 0x1.111112p-7f);
    p = __fmaf_rn(z, p, -0x1.555556p-3f);
    return __fmaf_rn(__fmul_rn(r, z), p, r);
}
__device__ __forceinline__ float pcos(float x)
{
    int q;
    float r = trig_reduce(x, q);
    float c = cos_poly(r), s = sin_poly(r);
    return q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
}
__device__ __forceinline__ float psin(float x)
{
    int q;
    float r = trig_reduce(x, q);
    float c = cos_poly(r), s = sin_poly(r);
    return q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
}
// cos and sin of one angle with a single reduction (the quadrant logic is the
// same as pcos / psin, so the values are identical).
__device__ __forceinline__ void psincos(float x, float& s_out, float& c_out)
{
    int q;
    float r = trig_reduce(x, q);
    float c = cos_poly(r), s = sin_poly(r);
    c_out = q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
    s_out = q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
}

// ----------------------------------------------------------- 256-bit loads --
// One 32-byte record through the read-only path as a single 256-bit load
// (ld.global.nc.v8, sm_100 and later): a BVH node record (box min,
// reference) (box max, count), or two halves of a wider record.  p must be
// 32-byte aligned (every device array here starts on a 256-byte boundary and
// the records are 32 bytes or multiples of it).
__device__ __forceinline__ void ldg256(const float4* p, float4& a, float4& b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ void ldg256u(const void* p, uint32_t (&w)[8])
{
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
        : "l"(p));
}

// ------------------------------------------------------------------ RNG --
// Tracer.comp:221-234: rand() = fract(cos(dot((coords + ++rand_salt) * 5, K1)) * 12345.6789)
struct Rng {
    float salt, cx, cy;
};
__device__ __forceinline__ float rand01(Rng& g)
{
    g.salt = g.salt + 1.0f;
    float ax = (g.cx + g.salt) * 5.0f;
    float ay = (g.cy + g.salt) * 5.0f;
    float dp = ax * 23.14069263277926f + ay * 2.665144142690225f;
    float v = pcos(dp) * 12345.6789f;
    return v - floorf(v);
}

// ------------------------------------------------------------ scene data --
struct Material {
    V3 albedo;
    V3 emissive;
    float roughness, metalness;
    uint32_t type;
};
__device__ __forceinline__ Material load_material(const float4* m)  // 3 x float4 (48 B)
{
    float4 a = __ldg(m), b = __ldg(m + 1), c = __ldg(m + 2);
    Material r;
    r.albedo = v3(a.x, a.y, a.z);
    r.emissive = v3(b.x, b.y, b.z);
    r.roughness = b.w;
    r.metalness = c.x;
    r.type = __float_as_uint(c.y);
    return r;
}

// Device scene.  Triangles are stored in traversal order as
//   (v0, material id) (v1 - v0, original id) (v2 - v0, 0)
// v1 - v0 and v2 - v0 are the differences Tracer.comp:342-343 and :389-390
// compute per test; computing them once at upload gives the same floats.
struct DevScene {
    const float4* tri;
    const float4* mats;
    const float4* sph_geo;  // (centre, radius) in traversal order
    const uint32_t* sph_id; // original sphere index per traversal slot
    const float4* sph_rec;  // original 64 B sphere records
    const float4* planes;   // 64 B plane records
    const uint32_t* emit;   // original indices of spheres with nonzero emissive
    const float4* tri_nodes;
    const float4* sph_nodes;
    uint32_t nt, nm, ns, np, ne;
    uint32_t n_tri_nodes, n_sph_nodes;
    const float4* tri_wide;  // 4-wide nodes (8 float4 each) of the same BVHs, or NULL
    const float4* sph_wide;
    const float4* tri_enc;   // the binary nodes with each record's child reference pre-encoded in
    const float4* sph_enc;   // bmin's w lane (interior: children-pair index; leaf: leaf code)
    const float4* tri_cw8;        // compressed 8-wide nodes over the triangles (6 float4 each), or NULL
    const float4* tri_cw8_prims;  // the triangles in their 8-wide order, 64 B each
};

struct Counters {
    uint32_t c[C_COUNT];
};

// ------------------------------------------------------- intersections --
struct Ray {
    V3 o, d;
};

// Tracer.comp:314-329
__device__ __forceinline__ float sphere_intersect(const Ray& ray, V3 P, float r)
{
    const V3 oc = ray.o - P;
    const float b = 2.0f * dot(oc, ray.d);
    const float c = dot(oc, oc) - r * r;
    const float h = b * b - 4.0f * c;
    if (h < 0.0f) return -1.0f;
    return (-b - sqrtf(h)) / 2.0f;
}

// Tracer.comp:331-338 (when_neq(d, 0) = abs(sign(d)))
__device__ __forceinline__ float plane_intersect(const Ray& ray, V3 N, float len)
{
    float d = dot(ray.d, N);
    float dist = -(len + dot(ray.o, N)) / d;
    return fabsf(gsign(d - 0.0f)) * gmax(dist, 0.0f);
}

// Tracer.comp:340-372, with v0v1 = e1 and v0v2 = e2 precomputed.
__device__ __forceinline__ float tri_intersect(const Ray& ray, V3 v0, V3 e1, V3 e2)
{
    const V3 pvec = cross(ray.d, e2);
    const float det = dot(e1, pvec);
    if (det < EPSILON) return -1.0f;
    const float inv = 1.0f / det;
    const V3 tvec = ray.o - v0;
    const float u = dot(tvec, pvec) * inv;
    if (u < 0.0f || u > 1.0f) return -1.0f;
    const V3 qvec = cross(tvec, e1);
    const float v = dot(ray.d, qvec) * inv;
    if (v < 0.0f || u + v > 1.0f) return -1.0f;
    return dot(e2, qvec) * inv;
}

struct Hit {
    float t;
    uint32_t prim;  // global primitive id
    int kind;       // 0 none, 1 triangle, 2 sphere, 3 plane
    uint32_t slot;  // storage slot of the winning primitive
};

// Reference ties (Tracer.comp:382, :402, :418) or strict (t, id) order.
template <int TIE>
__device__ __forceinline__ bool accept(float t, uint32_t id, const Hit& h, float tmax, bool plane)
{
    if (!(t > EPSILON)) return false;
    if (TIE == TIE_REFERENCE) return plane ? (t < h.t - EPSILON) : (t < h.t + EPSILON);
    if (!(t < tmax)) return false;
    return (t < h.t) || (t == h.t && id < h.prim);
}

// ----------------------------------------------------------- slab test --
struct BoxRay {
    float ix, iy, iz, nx, ny, nz;
};
__device__ __forceinline__ float safe_inv(float d) { return 1.0f / ((fabsf(d) > 1e-30f) ? d : copysignf(1e-30f, d)); }
__device__ __forceinline__ BoxRay make_boxray(const Ray& r)
{
    BoxRay b;
    b.ix = safe_inv(r.d.x);
    b.iy = safe_inv(r.d.y);
    b.iz = safe_inv(r.d.z);
    b.nx = -(r.o.x * b.ix);
    b.ny = -(r.o.y * b.iy);
    b.nz = -(r.o.z * b.iz);
    return b;
}
// Three-input IEEE minNum / maxNum (one instruction on sm_100+).  Without NaN
// inputs they equal the pairwise fminf/fmaxf chains of the definition, up to
// the sign of a zero result, which no comparison below can see.
__device__ __forceinline__ float fmin3(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Node record = 2 x float4: (bmin, left_or_first) (bmax, count).  Definition
// (shared with the oracle): tmin = max(max(min(x0,x1), min(y0,y1)),
// max(min(z0,z1), 0)), tmax = min(min(max(x0,x1), max(y0,y1)),
// min(max(z0,z1), tbest)); hit iff tmin <= tmax * (1 + 2^-20).  Rays with a
// NaN direction never reach this test.
__device__ __forceinline__ bool box_hit_s(const BoxRay& r, float lx, float ly, float lz, float hx, float hy, float hz,
                                          float tbest, float& tnear)
{
    float x0 = __fmaf_rn(lx, r.ix, r.nx), x1 = __fmaf_rn(hx, r.ix, r.nx);
    float y0 = __fmaf_rn(ly, r.iy, r.ny), y1 = __fmaf_rn(hy, r.iy, r.ny);
    float z0 = __fmaf_rn(lz, r.iz, r.nz), z1 = __fmaf_rn(hz, r.iz, r.nz);
    float tmin = fmaxf(fmax3(fminf(x0, x1), fminf(y0, y1), fminf(z0, z1)), 0.0f);
    float tmax = fminf(fmin3(fmaxf(x0, x1), fmaxf(y0, y1), fmaxf(z0, z1)), tbest);
    tnear = tmin;
    return tmin <= tmax * BOX_SLACK;
}
__device__ __forceinline__ bool box_hit(const BoxRay& r, float4 lo, float4 hi, float tbest, float& tnear)
{
    return box_hit_s(r, lo.x, lo.y, lo.z, hi.x, hi.y, hi.z, tbest, tnear);
}

}  // namespace vkt
