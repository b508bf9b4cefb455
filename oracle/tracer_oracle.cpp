// CPU oracle for the path tracer: a line-by-line restatement of the
// reference compute shader Assets/Tracer.comp (stickyfingies/vk-renderer),
// plus the extensions the GPU path adds (scene buffers, BVH traversal, sky,
// Russian-roulette start depth, runtime spp/depth, strict closest-hit ties).
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py load this library, and only to check or time the
// CUDA path; the product never links or calls it.
//
// Parity pinning: in reference mode with libm trig (trig_mode = 1) this file
// reproduces, bit for bit, the reference shader compiled as C++ against its
// own glm 0.9.9.3 (oracle/ref/), which tests/test_oracle_pinning.py checks and
// tests/golden/ records.  GLSL built-ins follow glm's definitions:
//   dot3 = (x*x' + y*y') + z*z'          length = sqrt(dot(v,v))
//   normalize(v) = v * (1/sqrt(dot(v,v)))  reflect(I,N) = I - N*dot(N,I)*2
//   refract: k = 1 - eta*eta*(1 - d*d); k >= 0 ? eta*I - (eta*d + sqrt k)*N : 0
//   mix(x,y,a) = x + a*(y - x)   max(x,y) = x < y ? y : x   min(x,y) = y < x ? y : x
//   clamp = min(max(x,lo),hi)    sign(x) = (0 < x) - (x < 0)   fract = x - floor x
// Build with -ffp-contract=off: every operation rounds as written.
//
// Floating-point type T is float for parity; T = double gives the FP64 host
// evaluation used as the gradient reference (the RNG always runs in float so
// both follow the same paths).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "rng_trig.h"
#include "oracle_api.h"

namespace oracle {

// ---------------------------------------------------------------- vectors --
template <class T> struct V3 {
    T x, y, z;
};
template <class T> struct V2 {
    T x, y;
};

template <class T> static inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> static inline V3<T> splat(T s) { return V3<T>{s, s, s}; }
template <class T> static inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> static inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> static inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> static inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> static inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> static inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> static inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> static inline V3<T> operator-(T s, V3<T> a) { return {s - a.x, s - a.y, s - a.z}; }
template <class T> static inline V3<T> operator+(V3<T> a, T s) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> static inline V3<T> operator-(V3<T> a, T s) { return {a.x - s, a.y - s, a.z - s}; }
template <class T> static inline bool operator==(V3<T> a, V3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

template <class T> static inline T gmax(T x, T y) { return (x < y) ? y : x; }
template <class T> static inline T gmin(T x, T y) { return (y < x) ? y : x; }
template <class T> static inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> static inline V3<T> vmax(V3<T> a, V3<T> b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
template <class T> static inline V3<T> vclamp(V3<T> a, T lo, T hi)
{
    return {gclamp(a.x, lo, hi), gclamp(a.y, lo, hi), gclamp(a.z, lo, hi)};
}
template <class T> static inline T gsign(T x) { return T(T(0) < x) - T(x < T(0)); }

template <class T> static inline T dot(V3<T> a, V3<T> b)
{
    V3<T> t = a * b;
    return t.x + t.y + t.z;
}
template <class T> static inline T length(V3<T> v) { return std::sqrt(dot(v, v)); }
template <class T> static inline V3<T> normalize(V3<T> v) { return v * (T(1) / std::sqrt(dot(v, v))); }
template <class T> static inline V3<T> cross(V3<T> x, V3<T> y)
{
    return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
template <class T> static inline V3<T> reflect(V3<T> I, V3<T> N) { return I - N * dot(N, I) * T(2); }
template <class T> static inline V3<T> refract(V3<T> I, V3<T> N, T eta)
{
    T d = dot(N, I);
    T k = T(1) - eta * eta * (T(1) - d * d);
    return (k >= T(0)) ? (eta * I - (eta * d + std::sqrt(k)) * N) : splat(T(0));
}
template <class T> static inline T gmix(T x, T y, T a) { return x + a * (y - x); }
template <class T> static inline V3<T> vmix(V3<T> x, V3<T> y, T a) { return x + a * (y - x); }
template <class T> static inline T gpow(T b, T e) { return std::pow(b, e); }
template <class T> static inline V3<T> vpow(V3<T> b, T e) { return {gpow(b.x, e), gpow(b.y, e), gpow(b.z, e)}; }

template <class T> static inline bool isnan3(V3<T> v) { return v.x != v.x || v.y != v.y || v.z != v.z; }

// ------------------------------------------------------- constant set-up --
// Tracer.comp:176-180
static const float PI = 3.14159265359f;
static const float EPSILON = 1e-3f;
static const uint32_t MAT_TYPE_DIFFUSE = 0;     // Tracer.comp:51
static const uint32_t MAT_TYPE_DIELECTRIC = 1;  // Tracer.comp:52

template <class T> struct Material {  // Tracer.comp:59-74
    V3<T> albedo;
    V3<T> emissive;
    T roughness;
    T metalness;
    uint32_t type;
};

template <class T> struct Ray {  // Tracer.comp:42-49
    V3<T> origin;
    V3<T> dir;
};

template <class T> struct Isect {  // Tracer.comp:83-95, plus the primitive id
    Material<T> mat;
    T t;
    V3<T> P;
    V3<T> N;
    uint32_t prim;
};

struct Stats {
    uint64_t closest_rays = 0, shadow_rays = 0, node_fetches = 0;
    uint64_t tri_tests = 0, sphere_tests = 0, plane_tests = 0, hits = 0;
};

// std430 record readers -----------------------------------------------------
static inline float rdf(const float* p, int i) { return p[i]; }
static inline uint32_t rdu(const float* p, int i)
{
    uint32_t u;
    std::memcpy(&u, p + i, 4);
    return u;
}
static inline int32_t rdi(const void* p, int i)
{
    int32_t v;
    std::memcpy(&v, (const char*)p + 4 * i, 4);
    return v;
}

template <class T> static Material<T> load_material(const float* m)  // 48 B record
{
    Material<T> r;
    r.albedo = v3<T>(rdf(m, 0), rdf(m, 1), rdf(m, 2));
    r.emissive = v3<T>(rdf(m, 4), rdf(m, 5), rdf(m, 6));
    r.roughness = rdf(m, 7);
    r.metalness = rdf(m, 8);
    r.type = rdu(m, 9);
    return r;
}

template <class T> struct Scene {
    uint32_t nt = 0, nm = 0, ns = 0, np = 0;
    std::vector<V3<T>> tv0, tv1, tv2;   // triangle vertices
    std::vector<uint32_t> tmat;         // triangle material id (v0.w lane)
    std::vector<Material<T>> mats;      // material table
    std::vector<V3<T>> sP;              // sphere centres
    std::vector<T> sr;                  // sphere radii
    std::vector<Material<T>> smat;      // sphere materials
    std::vector<uint32_t> emitters;     // spheres whose emissive != 0 (Tracer.comp:462), in order
    std::vector<V3<T>> pN;              // plane normals
    std::vector<T> plen;                // plane offsets
    std::vector<Material<T>> pmat;
    const void* tri_nodes = nullptr;
    uint32_t n_tri_nodes = 0;
    const uint32_t* tri_idx = nullptr;
    const void* sph_nodes = nullptr;
    uint32_t n_sph_nodes = 0;
    const uint32_t* sph_idx = nullptr;
};

template <class T> static void load_scene(const oracle_scene* d, Scene<T>& s)
{
    s.nt = d->num_triangles;
    s.nm = d->num_materials;
    s.ns = d->num_spheres;
    s.np = d->num_planes;
    s.tv0.resize(s.nt);
    s.tv1.resize(s.nt);
    s.tv2.resize(s.nt);
    s.tmat.resize(s.nt);
    for (uint32_t i = 0; i < s.nt; ++i) {
        const float* t = d->triangles + 12 * (size_t)i;
        s.tv0[i] = v3<T>(t[0], t[1], t[2]);
        s.tv1[i] = v3<T>(t[4], t[5], t[6]);
        s.tv2[i] = v3<T>(t[8], t[9], t[10]);
        s.tmat[i] = rdu(t, 3);
    }
    for (uint32_t i = 0; i < s.nm; ++i) s.mats.push_back(load_material<T>(d->materials + 12 * (size_t)i));
    for (uint32_t i = 0; i < s.ns; ++i) {
        const float* q = d->spheres + 16 * (size_t)i;
        s.smat.push_back(load_material<T>(q));
        s.sP.push_back(v3<T>(q[12], q[13], q[14]));
        s.sr.push_back(q[15]);
        Material<float> mf = load_material<float>(q);
        if (!(mf.emissive == splat(0.0f))) s.emitters.push_back(i);
    }
    for (uint32_t i = 0; i < s.np; ++i) {
        const float* q = d->planes + 16 * (size_t)i;
        s.pmat.push_back(load_material<T>(q));
        s.pN.push_back(v3<T>(q[12], q[13], q[14]));
        s.plen.push_back(q[15]);
    }
    s.tri_nodes = d->tri_nodes;
    s.n_tri_nodes = d->num_tri_nodes;
    s.tri_idx = d->tri_prim_index;
    s.sph_nodes = d->sphere_nodes;
    s.n_sph_nodes = d->num_sphere_nodes;
    s.sph_idx = d->sphere_prim_index;
}

// -------------------------------------------------------------------- RNG --
// Per-invocation RNG state, Tracer.comp:221-234 (rand_salt, coords).
struct Rng {
    float salt;
    float cx, cy;
    int trig_mode;  // 0 = portable (rng_trig.h), 1 = libm
};

static inline float rng_cosf(float x, int mode) { return mode ? std::cos(x) : oracle_rng_cos(x); }
static inline float rng_sinf(float x, int mode) { return mode ? std::sin(x) : oracle_rng_sin(x); }

// Tracer.comp:225-234: fract(cos(dot((coords + ++rand_salt) * 5.0, K1)) * 12345.6789)
static inline float rand(Rng& g)
{
    const float K1x = 23.14069263277926f, K1y = 2.665144142690225f;
    g.salt = g.salt + 1.0f;
    float ax = (g.cx + g.salt) * 5.0f;
    float ay = (g.cy + g.salt) * 5.0f;
    float dp = ax * K1x + ay * K1y;
    float v = rng_cosf(dp, g.trig_mode) * 12345.6789f;
    return v - std::floor(v);
}

// Trig used by jitter (Tracer.comp:262).  float: the same cos/sin as the RNG;
// double: libm.
static inline float tcos(float x, int mode) { return rng_cosf(x, mode); }
static inline float tsin(float x, int mode) { return rng_sinf(x, mode); }
static inline double tcos(double x, int) { return std::cos(x); }
static inline double tsin(double x, int) { return std::sin(x); }

// --------------------------------------------------------------- helpers --
template <class T> static inline T max3(V3<T> e) { return gmax(gmax(e.x, e.y), e.z); }     // :236-239
template <class T> static inline T when_neq(T x, T y) { return std::fabs(gsign(x - y)); }  // :246-249
template <class T> static inline V3<T> when_gt(V3<T> x, V3<T> y)                            // :251-254
{
    V3<T> d = x - y;
    return vmax(v3<T>(gsign(d.x), gsign(d.y), gsign(d.z)), splat(T(0)));
}

// Tracer.comp:256-263
template <class T> static V3<T> jitter(V3<T> d, T phi, T sina, T cosa, int trig)
{
    const V3<T> w = normalize(d);
    const V3<T> u = normalize(cross(v3<T>(w.y, w.z, w.x), w));
    const V3<T> v = cross(w, u);
    return (u * tcos(phi, trig) + v * tsin(phi, trig)) * sina + w * cosa;
}

// Tracer.comp:265-272
template <class T> static T schlick(T cosine, T ior)
{
    T r0 = (T(1) - ior) / (T(1) + ior);
    r0 = r0 * r0;
    return r0 + (T(1) - r0) * gpow(T(1) - cosine, T(5));
}

// Tracer.comp:274-277
template <class T> static V3<T> fresnel_schlick(T cosTheta, V3<T> F0)
{
    return F0 + (T(1) - F0) * gpow(T(1) - cosTheta, T(5));
}

// Tracer.comp:279-292
template <class T> static T distribution_ggx(V3<T> N, V3<T> H, T roughness)
{
    const T a = roughness * roughness;
    const T a2 = a * a;
    const T NdotH = gmax(dot(N, H), T(0));
    const T NdotH2 = NdotH * NdotH;
    const T num = a2;
    T denom = (NdotH2 * (a2 - T(1)) + T(1));
    denom = T(PI) * denom * denom;
    return num / denom;
}

// Tracer.comp:294-303
template <class T> static T geometry_schlick_ggx(T NdotV, T roughness)
{
    const T r = (roughness + T(1));
    const T k = (r * r) / T(8);
    const T num = NdotV;
    const T denom = NdotV * (T(1) - k) + k;
    return num / denom;
}

// Tracer.comp:304-312
template <class T> static T geometry_smith(V3<T> N, V3<T> V, V3<T> L, T roughness)
{
    const T NdotV = gmax(dot(N, V), T(0));
    const T NdotL = gmax(dot(N, L), T(0));
    const T ggx2 = geometry_schlick_ggx(NdotV, roughness);
    const T ggx1 = geometry_schlick_ggx(NdotL, roughness);
    return ggx1 * ggx2;
}

// ----------------------------------------------------------- intersection --
// Tracer.comp:314-329
template <class T> static T sphere_intersect(const Ray<T>& ray, V3<T> P, T r)
{
    const V3<T> oc = ray.origin - P;
    const T b = T(2) * dot(oc, ray.dir);
    const T c = dot(oc, oc) - r * r;
    const T h = b * b - T(4) * c;
    if (h < T(0)) return T(-1);
    const T t = (-b - std::sqrt(h)) / T(2);
    return t;
}

// Tracer.comp:331-338
template <class T> static T plane_intersect(const Ray<T>& ray, V3<T> N, T len)
{
    T d = dot(ray.dir, N);
    T dist = -(len + dot(ray.origin, N)) / d;
    return when_neq(d, T(0)) * gmax(dist, T(0));
}

// Tracer.comp:340-372 (Moller-Trumbore, one-sided)
template <class T> static T tri_intersect(const Ray<T>& ray, V3<T> v0, V3<T> v1, V3<T> v2)
{
    const V3<T> v0v1 = v1 - v0;
    const V3<T> v0v2 = v2 - v0;
    const V3<T> pvec = cross(ray.dir, v0v2);
    const T determinant = dot(v0v1, pvec);
    if (determinant < T(EPSILON)) return T(-1);
    const T inverse_determinant = T(1) / determinant;
    const V3<T> tvec = ray.origin - v0;
    const T u = dot(tvec, pvec) * inverse_determinant;
    if (u < T(0) || u > T(1)) return T(-1);
    const V3<T> qvec = cross(tvec, v0v1);
    const T v = dot(ray.dir, qvec) * inverse_determinant;
    if (v < T(0) || u + v > T(1)) return T(-1);
    return dot(v0v2, qvec) * inverse_determinant;
}

// ------------------------------------------------------------- trace_ray --
enum { TIE_REFERENCE = 0, TIE_STRICT = 1 };

// Acceptance of a candidate hit.  Reference ties (Tracer.comp:382, :402, :418):
// triangles and spheres accept t < best + EPSILON, planes t < best - EPSILON,
// so the last primitive in scan order within EPSILON wins.  Strict ties: the
// hit with the smallest (t, primitive id) below the ray's tmax, independent
// of scan order (the only rule a BVH can honour).
template <class T> struct Hit {
    T t;
    uint32_t prim;
    int kind;   // 0 none, 1 triangle, 2 sphere, 3 plane
    uint32_t idx;
};

template <class T> static inline bool accept(int tie, T t, uint32_t id, const Hit<T>& h, T tmax, bool plane)
{
    if (!(t > T(EPSILON))) return false;
    if (tie == TIE_REFERENCE) return plane ? (t < h.t - T(EPSILON)) : (t < h.t + T(EPSILON));
    if (!(t < tmax)) return false;
    return (t < h.t) || (t == h.t && id < h.prim);
}

// BVH node (32 B): bmin[3], left_or_first, bmax[3], count (count > 0: leaf
// with primitives [first, first+count) of the index array; else interior with
// children at left and left + 1).
struct Node {
    float bmin[3];
    int32_t left;
    float bmax[3];
    int32_t count;
};
static inline Node load_node(const void* base, uint32_t i)
{
    Node n;
    std::memcpy(&n, (const char*)base + 32 * (size_t)i, 32);
    return n;
}

// Slab test, written to give the same bits on every IEEE machine: one fused
// multiply-add per slab plane, IEEE minNum/maxNum, and a relative slack of
// 2^-20 on the far distance so that rounding never culls a box a primitive
// hit lies in (boxes are also padded when the BVH is built).
struct BoxRay {
    float ix, iy, iz;   // 1/d with zero components replaced by +-1e-30
    float nx, ny, nz;   // -(o * 1/d)
};
static inline float safe_inv(float d) { return 1.0f / ((std::fabs(d) > 1e-30f) ? d : std::copysign(1e-30f, d)); }
static inline BoxRay make_boxray(const float o[3], const float d[3])
{
    BoxRay b;
    b.ix = safe_inv(d[0]);
    b.iy = safe_inv(d[1]);
    b.iz = safe_inv(d[2]);
    b.nx = -(o[0] * b.ix);
    b.ny = -(o[1] * b.iy);
    b.nz = -(o[2] * b.iz);
    return b;
}
static const float BOX_SLACK = 1.0f + 0x1.0p-20f;
static inline bool box_hit(const BoxRay& r, const Node& n, float tbest, float* tnear)
{
    float x0 = std::fma(n.bmin[0], r.ix, r.nx), x1 = std::fma(n.bmax[0], r.ix, r.nx);
    float y0 = std::fma(n.bmin[1], r.iy, r.ny), y1 = std::fma(n.bmax[1], r.iy, r.ny);
    float z0 = std::fma(n.bmin[2], r.iz, r.nz), z1 = std::fma(n.bmax[2], r.iz, r.nz);
    float tmin = std::fmax(std::fmax(std::fmin(x0, x1), std::fmin(y0, y1)), std::fmax(std::fmin(z0, z1), 0.0f));
    float tmax = std::fmin(std::fmin(std::fmax(x0, x1), std::fmax(y0, y1)), std::fmin(std::fmax(z0, z1), tbest));
    *tnear = tmin;
    return tmin <= tmax * BOX_SLACK;
}

template <class T> struct Tracer {
    const Scene<T>& s;
    int tie;
    Stats& st;

    // Tests the primitives a leaf (or a linear scan) covers.  Returns true when
    // an any-hit query may stop.
    bool test_tri(const Ray<T>& ray, uint32_t i, Hit<T>& h, T tmax, bool any)
    {
        st.tri_tests++;
        const T t = tri_intersect(ray, s.tv0[i], s.tv1[i], s.tv2[i]);
        if (accept(tie, t, i, h, tmax, false)) {
            h.t = t;
            h.prim = i;
            h.kind = 1;
            h.idx = i;
            return any;
        }
        return false;
    }
    bool test_sphere(const Ray<T>& ray, uint32_t i, Hit<T>& h, T tmax, bool any)
    {
        st.sphere_tests++;
        const T t = sphere_intersect(ray, s.sP[i], s.sr[i]);
        const uint32_t id = s.nt + i;
        if (accept(tie, t, id, h, tmax, false)) {
            h.t = t;
            h.prim = id;
            h.kind = 2;
            h.idx = i;
            return any;
        }
        return false;
    }

    // Stack traversal of a BVH whose children sit side by side.  The visiting
    // order is part of the definition (the node-fetch counters depend on it):
    // both children of an interior node are fetched and tested; hit leaves are
    // processed at once, nearer child first; of hit interior children the
    // nearer is entered and the farther pushed with its entry distance; a popped
    // entry whose distance exceeds the current best is dropped.
    template <class TestFn>
    bool traverse(const void* nodes, const uint32_t* idx, const BoxRay& br, Hit<T>& h, T tmax, bool any,
                  TestFn test)
    {
        auto best = [&]() -> float { return (float)h.t; };
        Node root = load_node(nodes, 0);
        st.node_fetches++;
        float tn;
        if (!box_hit(br, root, best(), &tn)) return false;
        if (root.count > 0) {
            for (int32_t k = 0; k < root.count; ++k)
                if (test(idx[root.left + k], h, tmax, any)) return true;
            return false;
        }
        struct Entry {
            int32_t ci;
            float tnear;
        };
        Entry stack[128];
        int sp = 0;
        int32_t ci = root.left;
        for (;;) {
            Node c[2] = {load_node(nodes, ci), load_node(nodes, ci + 1)};
            st.node_fetches += 2;
            float t0, t1;
            bool h0 = box_hit(br, c[0], best(), &t0);
            bool h1 = box_hit(br, c[1], best(), &t1);
            int first = (h1 && (!h0 || t1 < t0)) ? 1 : 0;
            bool hit[2] = {h0, h1};
            float tt[2] = {t0, t1};
            int32_t next = -1;
            for (int j = 0; j < 2; ++j) {
                int k = j == 0 ? first : 1 - first;
                if (!hit[k]) continue;
                if (c[k].count > 0) {
                    for (int32_t m = 0; m < c[k].count; ++m)
                        if (test(idx[c[k].left + m], h, tmax, any)) return true;
                } else if (next < 0) {
                    next = c[k].left;
                } else {
                    stack[sp++] = Entry{c[k].left, tt[k]};
                }
            }
            while (next < 0) {
                if (sp == 0) return false;
                Entry e = stack[--sp];
                if (e.tnear <= best() * BOX_SLACK) next = e.ci;
            }
            ci = next;
        }
    }

    // Tracer.comp:374-431.  Returns found; h carries the winning hit.
    bool trace(const Ray<T>& ray, Isect<T>& is, bool shadow)
    {
        if (shadow)
            st.shadow_rays++;
        else
            st.closest_rays++;
        Hit<T> h{is.t, 0xFFFFFFFFu, 0, 0};
        const T tmax = is.t;
        // A ray whose direction has a NaN component hits nothing (every
        // comparison in the intersection routines is false); it is not traversed.
        if (!isnan3(ray.dir)) {
            const bool any = shadow;
            bool done = false;
            if (s.tri_nodes && s.nt) {
                float o[3] = {(float)ray.origin.x, (float)ray.origin.y, (float)ray.origin.z};
                float d[3] = {(float)ray.dir.x, (float)ray.dir.y, (float)ray.dir.z};
                BoxRay br = make_boxray(o, d);
                done = traverse(s.tri_nodes, s.tri_idx, br, h, tmax, any,
                                [&](uint32_t i, Hit<T>& hh, T tm, bool a) { return test_tri(ray, i, hh, tm, a); });
            } else {
                for (uint32_t i = 0; i < s.nt && !done; ++i) done = test_tri(ray, i, h, tmax, any);
            }
            if (!done) {
                if (s.sph_nodes && s.ns) {
                    float o[3] = {(float)ray.origin.x, (float)ray.origin.y, (float)ray.origin.z};
                    float d[3] = {(float)ray.dir.x, (float)ray.dir.y, (float)ray.dir.z};
                    BoxRay br = make_boxray(o, d);
                    done = traverse(s.sph_nodes, s.sph_idx, br, h, tmax, any,
                                    [&](uint32_t i, Hit<T>& hh, T tm, bool a) { return test_sphere(ray, i, hh, tm, a); });
                } else {
                    for (uint32_t i = 0; i < s.ns && !done; ++i) done = test_sphere(ray, i, h, tmax, any);
                }
            }
            for (uint32_t i = 0; i < s.np && !done; ++i) {
                st.plane_tests++;
                const T t = plane_intersect(ray, s.pN[i], s.plen[i]);
                const uint32_t id = s.nt + s.ns + i;
                if (accept(tie, t, id, h, tmax, true)) {
                    h.t = t;
                    h.prim = id;
                    h.kind = 3;
                    h.idx = i;
                    done = any;
                }
            }
        }
        if (h.kind == 0) return false;
        if (!shadow) st.hits++;  // closest-hit rays that hit (each reads a material record)
        is.t = h.t;
        is.prim = h.prim;
        is.P = ray.origin + h.t * ray.dir;
        if (h.kind == 1) {
            // Tracer.comp:386-392: material from the table (the reference's
            // constant `mirror` is entry tri.material of the table), normal is
            // the unnormalised cross(v1 - v0, v2 - v0).
            is.mat = s.mats[s.tmat[h.idx]];
            const V3<T> u = s.tv1[h.idx] - s.tv0[h.idx];
            const V3<T> v = s.tv2[h.idx] - s.tv0[h.idx];
            is.N = v3<T>((u.y * v.z) - (u.z * v.y), (u.z * v.x) - (u.x * v.z), (u.x * v.y) - (u.y * v.x));
        } else if (h.kind == 2) {
            is.mat = s.smat[h.idx];
            is.N = (is.P - s.sP[h.idx]) / s.sr[h.idx];
        } else {
            is.mat = s.pmat[h.idx];
            is.N = s.pN[h.idx];
        }
        return true;
    }
};

struct Params {
    uint32_t width, height, spp, max_depth, rr_start;
    float sky[3];
    int tie, trig;
    bool sky_on;
};

template <class T> struct Frame {
    T aspect;
    float seed;
    V3<T> cpos, cdir, cright, cup;
};

// Tracer.comp:433-553, with the extensions: runtime max_depth, Russian
// roulette from depth rr_start on (the reference runs it at every depth,
// rr_start = 0), sky radiance on a miss (the reference adds nothing, sky = 0).
template <class T> static V3<T> radiance(Tracer<T>& tr, const Frame<T>& fr, const Params& p, Ray<T> ray, Rng& g,
                                         uint32_t* prim0, float* t0)
{
    V3<T> acc = splat(T(0));
    V3<T> mask = splat(T(1));
    const V3<T> sky = v3<T>(p.sky[0], p.sky[1], p.sky[2]);
    for (uint32_t depth = 0; depth < p.max_depth; ++depth) {
        acc = vclamp(acc, T(0), T(1));
        Isect<T> is;
        is.t = T(3000) / gpow(T(depth + 1), T(2));
        bool found = tr.trace(ray, is, false);
        if (depth == 0 && prim0) {
            *prim0 = found ? is.prim : 0xFFFFFFFFu;
            *t0 = found ? (float)is.t : -1.0f;
        }
        if (!found) {
            if (p.sky_on) acc = acc + mask * sky;
            break;
        }
        const Material<T> mat = is.mat;
        switch (mat.type) {
        case MAT_TYPE_DIFFUSE: {
            const T r2 = rand(g);
            const V3<T> d = jitter(is.N, T(2.0f * PI) * T(rand(g)), std::sqrt(r2), std::sqrt(T(1) - r2), g.trig_mode) *
                            (T(1) - mat.metalness);
            V3<T> e = splat(T(0));
            for (uint32_t si : tr.s.emitters) {
                const V3<T> sP = tr.s.sP[si];
                const T sr = tr.s.sr[si];
                const Material<T>& smat = tr.s.smat[si];
                const T t = length(sP - is.P) - sr;
                const V3<T> l0 = sP - is.P;
                const T cos_a_max = std::sqrt(T(1) - gclamp(sr * sr / dot(l0, l0), T(0), T(1)));
                const T cosa = gmix(cos_a_max, T(1), T(rand(g)));
                const V3<T> L = jitter(l0, T(2.0f * PI) * T(rand(g)), std::sqrt(T(1) - cosa * cosa), cosa, g.trig_mode);
                Isect<T> sh;
                sh.t = t;
                if (!tr.trace(Ray<T>{is.P, L}, sh, true)) {
                    V3<T> attenuation = smat.emissive * T(1) / gpow(t / sr + T(1), T(2));
                    attenuation = (attenuation - T(0.001f)) / (T(1) - T(0.001f));
                    attenuation = vmax(attenuation, splat(T(0)));
                    V3<T> F0 = splat(T(0.04f));
                    F0 = vmix(F0, mat.albedo, mat.metalness);
                    const V3<T> V = normalize(fr.cpos - is.P);
                    const V3<T> H = normalize(V + L);
                    const T NDF = distribution_ggx(is.N, H, mat.roughness);
                    const T G = geometry_smith(is.N, V, L, mat.roughness);
                    const V3<T> F = fresnel_schlick(gmax(dot(H, V), T(0)), F0);
                    const V3<T> kS = F;
                    V3<T> kD = T(1) - kS;
                    kD = kD * (T(1) - mat.metalness);
                    const V3<T> numerator = NDF * G * F;
                    const T denominator = T(4) * gmax(dot(is.N, V), T(0)) * gmax(dot(is.N, L), T(0));
                    const V3<T> specular = numerator / gmax(denominator, T(0.001f));
                    const T NdotL = gmax(dot(is.N, L), T(0));
                    e = e + (kD * mat.albedo / T(PI) + specular) * attenuation * NdotL;
                }
            }
            const V3<T> emissive =
                (when_gt(mat.emissive, splat(T(0))) == splat(T(1))) ? normalize(mat.emissive) : splat(T(0));
            acc = acc + mask * (emissive + e);
            mask = mask * mat.albedo;
            ray = Ray<T>{is.P, normalize(reflect(ray.dir, is.N) + d)};
            break;
        }
        case MAT_TYPE_DIELECTRIC: {
            acc = acc + mat.emissive * mask;
            mask = mask * mat.albedo;
            const V3<T> normal = is.N;
            const T nint = mat.roughness;
            const T cosine = -dot(ray.dir, is.N) / length(ray.dir);
            const V3<T> reflected = reflect(ray.dir, is.N);
            const V3<T> refracted = refract(ray.dir, normal, nint);
            const T prob = (refracted == splat(T(0))) ? T(1) : schlick(cosine, mat.roughness);
            ray = Ray<T>{is.P, normalize(T(rand(g)) < prob ? reflected : refracted)};
            break;
        }
        default:
            break;
        }
        if (depth >= p.rr_start) {
            const T prob_term = max3(mask);
            if (T(rand(g)) > prob_term) break;
            mask = mask * (T(1) / prob_term);
        }
    }
    return acc;
}

static inline uint8_t unorm8(float x)
{
    if (!(x == x)) return 0;
    float c = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return (uint8_t)std::floor(c * 255.0f + 0.5f);
}

template <class T> static Frame<T> load_frame(const float* f)
{
    Frame<T> fr;
    fr.aspect = f[0];
    fr.seed = f[1];
    fr.cpos = v3<T>(f[8], f[9], f[10]);
    fr.cdir = v3<T>(f[12], f[13], f[14]);
    fr.cright = v3<T>(f[16], f[17], f[18]);
    fr.cup = v3<T>(f[20], f[21], f[22]);
    return fr;
}

// Tracer.comp:557-593 for one pixel.  out: rgba32f (dithered colour, alpha 1).
template <class T> static void shade_pixel(Tracer<T>& tr, const Frame<T>& fr, const Params& p, uint32_t x, uint32_t y,
                                           float* rgba, uint32_t* prim0, float* t0, T* accum_out)
{
    const float uvx = (float)x / (float)p.width;
    const float uvy = (float)y / (float)p.height;
    Rng g;
    g.salt = uvy / uvx + fr.seed;
    g.cx = uvx;
    g.cy = uvy;
    g.trig_mode = p.trig;
    const T tx = T(2.0f * uvx - 1.0f);
    const T ty = T(2.0f * uvy - 1.0f);
    V3<T> dir = (fr.cdir + fr.cright * tx + fr.cup * ty) * v3<T>(fr.aspect, T(1), fr.aspect);
    Ray<T> primary{fr.cpos, normalize(dir)};
    V3<T> accum = splat(T(0));
    for (uint32_t i = 0; i < p.spp; ++i)
        accum = accum + radiance(tr, fr, p, primary, g, i == 0 ? prim0 : nullptr, t0);
    accum = accum / T(p.spp);
    if (accum_out) {
        accum_out[0] = accum.x;
        accum_out[1] = accum.y;
        accum_out[2] = accum.z;
    }
    accum = accum / (accum + splat(T(1)));
    accum = vpow(accum, T(1.0f / 2.2f));
    const T dither = T(rand(g)) / T(64);
    if (accum_out) accum_out[3] = dither;
    rgba[0] = (float)(accum.x + dither);
    rgba[1] = (float)(accum.y + dither);
    rgba[2] = (float)(accum.z + dither);
    rgba[3] = 1.0f;
}

static Params to_params(const oracle_params* pp)
{
    Params p;
    p.width = pp->width;
    p.height = pp->height;
    p.spp = pp->spp;
    p.max_depth = pp->max_depth;
    p.rr_start = pp->rr_start;
    p.sky[0] = pp->sky[0];
    p.sky[1] = pp->sky[1];
    p.sky[2] = pp->sky[2];
    p.sky_on = !(pp->sky[0] == 0.0f && pp->sky[1] == 0.0f && pp->sky[2] == 0.0f);
    p.tie = pp->tie_mode;
    p.trig = pp->trig_mode;
    return p;
}

template <class T>
static int render(const oracle_scene* sd, const float* frame, const oracle_params* pp, float* rgba32f, uint8_t* rgba8,
                  uint32_t* hit_id, float* hit_t, double* accum, oracle_stats* stats_out)
{
    Scene<T> sc;
    load_scene(sd, sc);
    const Params p = to_params(pp);
    const Frame<T> fr = load_frame<T>(frame);
    const uint32_t rb = pp->row_begin, re = pp->row_end ? pp->row_end : p.height;
    const uint32_t rs = pp->row_step ? pp->row_step : 1;
    std::vector<uint32_t> rows;
    for (uint32_t y = rb; y < re && y < p.height; y += rs) rows.push_back(y);
    Stats total;
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = pp->threads > 0 ? pp->threads : omp_get_max_threads();
#endif
    std::vector<Stats> per(nthreads);
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        Tracer<T> tr{sc, p.tie, per[tid]};
        // work items: runs of 64 pixels of one scanline (pixels are independent)
        const uint32_t run = 64, per_row = (p.width + run - 1) / run;
#pragma omp for schedule(dynamic, 1)
        for (long it = 0; it < (long)rows.size() * (long)per_row; ++it) {
            const uint32_t y = rows[it / per_row];
            const uint32_t x0 = (uint32_t)(it % per_row) * run;
            const uint32_t x1 = x0 + run < p.width ? x0 + run : p.width;
            for (uint32_t x = x0; x < x1; ++x) {
                const size_t i = (size_t)y * p.width + x;
                float rgba[4];
                uint32_t prim = 0xFFFFFFFFu;
                float t0 = -1.0f;
                T acc3[4];
                shade_pixel(tr, fr, p, x, y, rgba, &prim, &t0, acc3);
                if (rgba32f) std::memcpy(rgba32f + 4 * i, rgba, 16);
                if (rgba8)
                    for (int c = 0; c < 4; ++c) rgba8[4 * i + c] = unorm8(rgba[c]);
                if (hit_id) hit_id[i] = prim;
                if (hit_t) hit_t[i] = t0;
                if (accum)
                    for (int c = 0; c < 4; ++c) accum[4 * i + c] = (double)acc3[c];
            }
        }
    }
    for (auto& s : per) {
        total.closest_rays += s.closest_rays;
        total.shadow_rays += s.shadow_rays;
        total.node_fetches += s.node_fetches;
        total.tri_tests += s.tri_tests;
        total.sphere_tests += s.sphere_tests;
        total.plane_tests += s.plane_tests;
        total.hits += s.hits;
    }
    if (stats_out) {
        stats_out->closest_rays = total.closest_rays;
        stats_out->shadow_rays = total.shadow_rays;
        stats_out->node_fetches = total.node_fetches;
        stats_out->tri_tests = total.tri_tests;
        stats_out->sphere_tests = total.sphere_tests;
        stats_out->plane_tests = total.plane_tests;
        stats_out->hits = total.hits;
    }
    return 0;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

int oracle_render(const oracle_scene* scene, const float* frame, const oracle_params* params, float* rgba32f,
                  uint8_t* rgba8, uint32_t* hit_id, float* hit_t, oracle_stats* stats)
{
    return render<float>(scene, frame, params, rgba32f, rgba8, hit_id, hit_t, nullptr, stats);
}

int oracle_render_f64(const oracle_scene* scene, const float* frame, const oracle_params* params, float* rgba32f,
                      double* accum, oracle_stats* stats)
{
    return render<double>(scene, frame, params, rgba32f, nullptr, nullptr, nullptr, accum, stats);
}

void oracle_rand(float cx, float cy, float salt, int trig_mode, int n, float* out)
{
    Rng g{salt, cx, cy, trig_mode};
    for (int i = 0; i < n; ++i) out[i] = rand(g);
}

float oracle_cos(float x) { return oracle_rng_cos(x); }
float oracle_sin(float x) { return oracle_rng_sin(x); }

float oracle_tri_intersect(const float* o, const float* d, const float* tri48)
{
    Ray<float> r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2])};
    return tri_intersect(r, v3(tri48[0], tri48[1], tri48[2]), v3(tri48[4], tri48[5], tri48[6]),
                         v3(tri48[8], tri48[9], tri48[10]));
}

float oracle_sphere_intersect(const float* o, const float* d, const float* c, float radius)
{
    Ray<float> r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2])};
    return sphere_intersect(r, v3(c[0], c[1], c[2]), radius);
}

float oracle_plane_intersect(const float* o, const float* d, const float* n, float len)
{
    Ray<float> r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2])};
    return plane_intersect(r, v3(n[0], n[1], n[2]), len);
}

// trace_ray with isect.t = tmax on entry.  out: found, t, P[3], N[3],
// material (12 floats, std430), prim id (as float bits in out[20]).
int oracle_trace_ray(const oracle_scene* sd, int tie_mode, int shadow, const float* o, const float* d, float tmax,
                     float* out, oracle_stats* stats)
{
    Scene<float> sc;
    load_scene(sd, sc);
    Stats st;
    Tracer<float> tr{sc, tie_mode, st};
    Isect<float> is;
    std::memset(&is, 0, sizeof(is));
    is.t = tmax;
    Ray<float> r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2])};
    bool found = tr.trace(r, is, shadow != 0);
    std::memset(out, 0, 21 * 4);
    out[0] = found ? 1.0f : 0.0f;
    out[1] = is.t;
    out[2] = is.P.x;
    out[3] = is.P.y;
    out[4] = is.P.z;
    out[5] = is.N.x;
    out[6] = is.N.y;
    out[7] = is.N.z;
    out[8] = is.mat.albedo.x;
    out[9] = is.mat.albedo.y;
    out[10] = is.mat.albedo.z;
    out[12] = is.mat.emissive.x;
    out[13] = is.mat.emissive.y;
    out[14] = is.mat.emissive.z;
    out[15] = is.mat.roughness;
    out[16] = is.mat.metalness;
    std::memcpy(out + 17, &is.mat.type, 4);
    uint32_t prim = found ? is.prim : 0xFFFFFFFFu;
    std::memcpy(out + 20, &prim, 4);
    if (stats) {
        stats->closest_rays = st.closest_rays;
        stats->shadow_rays = st.shadow_rays;
        stats->node_fetches = st.node_fetches;
        stats->tri_tests = st.tri_tests;
        stats->sphere_tests = st.sphere_tests;
        stats->plane_tests = st.plane_tests;
        stats->hits = st.hits;
    }
    return found ? 1 : 0;
}

// radiance(ray) from a given RNG state; returns the salt after the call.
void oracle_radiance(const oracle_scene* sd, const float* frame, const oracle_params* pp, const float* o,
                     const float* d, float cx, float cy, float salt, float* out_rgb, float* out_salt)
{
    Scene<float> sc;
    load_scene(sd, sc);
    Stats st;
    const Params p = to_params(pp);
    Tracer<float> tr{sc, p.tie, st};
    Frame<float> fr = load_frame<float>(frame);
    Rng g{salt, cx, cy, p.trig};
    Ray<float> r{v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2])};
    V3<float> c = radiance(tr, fr, p, r, g, nullptr, nullptr);
    out_rgb[0] = c.x;
    out_rgb[1] = c.y;
    out_rgb[2] = c.z;
    *out_salt = g.salt;
}

}  // extern "C"
