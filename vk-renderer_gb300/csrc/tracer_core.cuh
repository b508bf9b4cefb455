// trace_ray, radiance and the per-pixel resolve of Assets/Tracer.comp,
// restated for CUDA, with the project's extensions (BVH traversal with a
// shared-memory stack, scene buffers instead of shader constants, sky on a
// miss, Russian roulette from a given depth, runtime spp and depth).
#pragma once

#include "tracer_device.cuh"

namespace vkt {

struct FrameArgs {
    float aspect, seed;
    V3 cpos, cdir, cright, cup;
    V3 light;  // FrameData::light_pos (read only by the legacy Whitted shader)
};

struct TraceArgs {
    DevScene sc;
    FrameArgs fr;
    uint32_t width, height, spp, max_depth, rr_start;
    V3 sky;
    int sky_on;
    uint32_t stack_depth;
    uint32_t trav_limit;
    // outputs (NULL = not written)
    uchar4* rgba8;
    float4* rgba32f;
    uint2* hit;
    float4* linear;  // accum / spp before tone mapping (input of the adjoint)
    unsigned long long* stats;  // C_COUNT counters
    int* status;
    // wavefront: first global path slot of this scene's pixels, and (in the
    // launch's own arguments) the number of slots of the launch
    uint32_t pixel_base;
    uint32_t num_slots;
};

// Traversal stack of one thread in shared memory: entry i of thread t at
// word i * stride + t (consecutive threads hit consecutive banks).
struct Stack {
    int* ci;
    float* tn;
    int stride;
    int cap;
};

template <int TIE, bool BVH, bool STATS>
struct Tracer {
    const DevScene& sc;
    Stack stk;
    Counters& cnt;
    int* status;
    uint32_t trav_limit;

    __device__ __forceinline__ void count(int k, uint32_t v = 1)
    {
        if (STATS) cnt.c[k] += v;
    }

    __device__ __forceinline__ bool test_tri(const Ray& ray, uint32_t slot, Hit& h, float tmax, bool any)
    {
        count(C_TRIS);
        const float4* t = sc.tri + 3 * (size_t)slot;
        const float4 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2);
        const float tt = tri_intersect(ray, v3(a), v3(b), v3(c));
        const uint32_t id = __float_as_uint(b.w);
        if (accept<TIE>(tt, id, h, tmax, false)) {
            h.t = tt;
            h.prim = id;
            h.kind = 1;
            h.slot = slot;
            return any;
        }
        return false;
    }

    __device__ __forceinline__ bool test_sphere(const Ray& ray, uint32_t slot, Hit& h, float tmax, bool any)
    {
        count(C_SPHERES);
        const float4 g = __ldg(sc.sph_geo + slot);
        const float tt = sphere_intersect(ray, v3(g), g.w);
        const uint32_t id = sc.nt + __ldg(sc.sph_id + slot);
        if (accept<TIE>(tt, id, h, tmax, false)) {
            h.t = tt;
            h.prim = id;
            h.kind = 2;
            h.slot = slot;
            return any;
        }
        return false;
    }

    // BVH traversal; the visiting order matches the oracle's definition:
    // fetch and test both children; hit leaves are processed at once, nearer
    // first; the nearer hit interior child is entered, the farther pushed with
    // its entry distance; popped entries beyond the current best are dropped.
    template <int PRIM>
    __device__ __forceinline__ bool traverse(const float4* nodes, uint32_t n_nodes, const Ray& ray, const BoxRay& br,
                                             Hit& h, float tmax, bool any)
    {
        float4 rlo, rhi;
        ldg256(nodes, rlo, rhi);
        count(C_NODES);
        float tn;
        if (!box_hit(br, rlo, rhi, h.t, tn)) return false;
        const int rcount = __float_as_int(rhi.w);
        const int rleft = __float_as_int(rlo.w);
        if (rcount > 0) {
            for (int k = 0; k < rcount; ++k) {
                bool stop = PRIM == 0 ? test_tri(ray, rleft + k, h, tmax, any) : test_sphere(ray, rleft + k, h, tmax, any);
                if (stop) return true;
            }
            return false;
        }
        int sp = 0;
        int ci = rleft;
        uint32_t steps = 0;
        for (;;) {
            if (++steps > trav_limit) {
                atomicCAS(status, ST_OK, ST_TRAVERSAL_LIMIT);
                return false;
            }
            const float4* c = nodes + 2 * (size_t)ci;
            float4 lo0, hi0, lo1, hi1;
            ldg256(c, lo0, hi0);
            ldg256(c + 2, lo1, hi1);
            count(C_NODES, 2);
            float t0, t1;
            const bool h0 = box_hit(br, lo0, hi0, h.t, t0);
            const bool h1 = box_hit(br, lo1, hi1, h.t, t1);
            const bool swap = h1 && (!h0 || t1 < t0);
            // child order: nearer first
            float4 flo = swap ? lo1 : lo0, fhi = swap ? hi1 : hi0;
            float4 slo = swap ? lo0 : lo1, shi = swap ? hi0 : hi1;
            bool fh = swap ? h1 : h0, shh = swap ? h0 : h1;
            float ft = swap ? t1 : t0, st = swap ? t0 : t1;
            int next = -1;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const bool hit = j == 0 ? fh : shh;
                if (!hit) continue;
                const float4 lo = j == 0 ? flo : slo;
                const float4 hi = j == 0 ? fhi : shi;
                const int cnt_ = __float_as_int(hi.w);
                const int left = __float_as_int(lo.w);
                if (cnt_ > 0) {
                    for (int k = 0; k < cnt_; ++k) {
                        bool stop = PRIM == 0 ? test_tri(ray, left + k, h, tmax, any)
                                              : test_sphere(ray, left + k, h, tmax, any);
                        if (stop) return true;
                    }
                } else if (next < 0) {
                    next = left;
                } else {
                    if (sp >= stk.cap) {
                        atomicCAS(status, ST_OK, ST_STACK_OVERFLOW);
                    } else {
                        stk.ci[sp * stk.stride] = left;
                        stk.tn[sp * stk.stride] = j == 0 ? ft : st;
                        ++sp;
                    }
                }
            }
            while (next < 0) {
                if (sp == 0) return false;
                --sp;
                const int e = stk.ci[sp * stk.stride];
                const float et = stk.tn[sp * stk.stride];
                if (et <= h.t * BOX_SLACK) next = e;
            }
            ci = next;
        }
    }

    // Tracer.comp:374-431.  h.t holds tmax on entry; on return h describes
    // the winning primitive (kind 0 = none).
    __device__ __forceinline__ bool trace(const Ray& ray, Hit& h, bool shadow)
    {
        count(shadow ? C_SHADOW : C_CLOSEST);
        const float tmax = h.t;
        h.prim = NO_PRIM;
        h.kind = 0;
        h.slot = 0;
        if (isnan3(ray.d)) return false;  // no intersection routine accepts a NaN direction
        const bool any = shadow;
        bool done = false;
        if (BVH && sc.n_tri_nodes && sc.nt) {
            BoxRay br = make_boxray(ray);
            done = traverse<0>(sc.tri_nodes, sc.n_tri_nodes, ray, br, h, tmax, any);
        } else {
            for (uint32_t i = 0; i < sc.nt && !done; ++i) done = test_tri(ray, i, h, tmax, any);
        }
        if (!done) {
            if (BVH && sc.n_sph_nodes && sc.ns) {
                BoxRay br = make_boxray(ray);
                done = traverse<1>(sc.sph_nodes, sc.n_sph_nodes, ray, br, h, tmax, any);
            } else {
                for (uint32_t i = 0; i < sc.ns && !done; ++i) done = test_sphere(ray, i, h, tmax, any);
            }
        }
        for (uint32_t i = 0; i < sc.np && !done; ++i) {
            count(C_PLANES);
            const float4* p = sc.planes + 4 * (size_t)i;
            const float4 q = __ldg(p + 3);
            const float tt = plane_intersect(ray, v3(q), q.w);
            const uint32_t id = sc.nt + sc.ns + i;
            if (accept<TIE>(tt, id, h, tmax, true)) {
                h.t = tt;
                h.prim = id;
                h.kind = 3;
                h.slot = i;
                done = any;
            }
        }
        if (h.kind == 0) return false;
        if (!shadow) count(C_HITS);  // closest-hit rays that hit (each reads a material record)
        return true;
    }

    // Surface data of a hit (Tracer.comp:384-392, :404-408, :420-424).
    __device__ __forceinline__ void surface(const Ray& ray, const Hit& h, V3& P, V3& N, Material& m)
    {
        P = ray.o + h.t * ray.d;
        if (h.kind == 1) {
            const float4* t = sc.tri + 3 * (size_t)h.slot;
            const float4 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2);
            const V3 u = v3(b), v = v3(c);
            N = v3((u.y * v.z) - (u.z * v.y), (u.z * v.x) - (u.x * v.z), (u.x * v.y) - (u.y * v.x));
            m = load_material(sc.mats + 3 * (size_t)__float_as_uint(a.w));
        } else if (h.kind == 2) {
            const float4 g = __ldg(sc.sph_geo + h.slot);
            N = (P - v3(g)) / g.w;
            m = load_material(sc.sph_rec + 4 * (size_t)__ldg(sc.sph_id + h.slot));
        } else {
            const float4* p = sc.planes + 4 * (size_t)h.slot;
            N = v3(__ldg(p + 3));
            m = load_material(p);
        }
    }
};

// Tracer.comp:256-263
__device__ __forceinline__ V3 jitter(V3 d, float phi, float sina, float cosa)
{
    const V3 w = normalize(d);
    const V3 u = normalize(cross(v3(w.y, w.z, w.x), w));
    const V3 v = cross(w, u);
    float s, c;
    psincos(phi, s, c);
    return (u * c + v * s) * sina + w * cosa;
}

// Tracer.comp:265-272
__device__ __forceinline__ float schlick(float cosine, float ior)
{
    float r0 = (1.0f - ior) / (1.0f + ior);
    r0 = r0 * r0;
    return r0 + (1.0f - r0) * powf(1.0f - cosine, 5.0f);
}

// Tracer.comp:279-312
__device__ __forceinline__ float distribution_ggx(V3 N, V3 H, float roughness)
{
    const float a = roughness * roughness;
    const float a2 = a * a;
    const float NdotH = gmax(dot(N, H), 0.0f);
    const float NdotH2 = NdotH * NdotH;
    float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
    denom = PI * denom * denom;
    return a2 / denom;
}
__device__ __forceinline__ float geometry_schlick_ggx(float NdotV, float roughness)
{
    const float r = (roughness + 1.0f);
    const float k = (r * r) / 8.0f;
    return NdotV / (NdotV * (1.0f - k) + k);
}
__device__ __forceinline__ float geometry_smith(V3 N, V3 V, V3 L, float roughness)
{
    const float NdotV = gmax(dot(N, V), 0.0f);
    const float NdotL = gmax(dot(N, L), 0.0f);
    return geometry_schlick_ggx(NdotL, roughness) * geometry_schlick_ggx(NdotV, roughness);
}

// One emitter's next-event contribution (Tracer.comp:458-504) for a diffuse
// hit; consumes two random numbers whether or not the light is visible.
template <class TR>
__device__ __forceinline__ V3 nee_one(TR& tr, const TraceArgs& a, uint32_t si, V3 P, V3 N, const Material& mat, Rng& g)
{
    const float4* rec = a.sc.sph_rec + 4 * (size_t)si;
    const float4 geo = __ldg(rec + 3);
    const V3 sP = v3(geo);
    const float sr = geo.w;
    const float t = length(sP - P) - sr;
    const V3 l0 = sP - P;
    const float cos_a_max = sqrtf(1.0f - gclamp(sr * sr / dot(l0, l0), 0.0f, 1.0f));
    const float cosa = gmix(cos_a_max, 1.0f, rand01(g));
    const V3 L = jitter(l0, (2.0f * PI) * rand01(g), sqrtf(1.0f - cosa * cosa), cosa);
    Hit sh;
    sh.t = t;
    if (tr.trace(Ray{P, L}, sh, true)) return splat(0.0f);
    const float4 em = __ldg(rec + 1);
    const float q = t / sr + 1.0f;
    V3 attenuation = v3(em) * 1.0f / (q * q);
    attenuation = (attenuation - 0.001f) / (1.0f - 0.001f);
    attenuation = vmax0(attenuation);
    V3 F0 = splat(0.04f);
    F0 = vmix(F0, mat.albedo, mat.metalness);
    const V3 V = normalize(a.fr.cpos - P);
    const V3 H = normalize(V + L);
    const float NDF = distribution_ggx(N, H, mat.roughness);
    const float G = geometry_smith(N, V, L, mat.roughness);
    const float cth = gmax(dot(H, V), 0.0f);
    const V3 F = F0 + (1.0f - F0) * powf(1.0f - cth, 5.0f);
    V3 kD = 1.0f - F;
    kD = kD * (1.0f - mat.metalness);
    const V3 numerator = NDF * G * F;
    const float denominator = 4.0f * gmax(dot(N, V), 0.0f) * gmax(dot(N, L), 0.0f);
    const V3 specular = numerator / gmax(denominator, 0.001f);
    const float NdotL = gmax(dot(N, L), 0.0f);
    return (kD * mat.albedo / PI + specular) * attenuation * NdotL;
}

// tmax of the closest-hit ray at a depth: 3000 / (depth + 1)^2 (Tracer.comp:444)
__device__ __forceinline__ float depth_tmax(uint32_t depth)
{
    const float dp1 = (float)(depth + 1);
    return 3000.0f / (dp1 * dp1);
}

// The part of one depth iteration of radiance (Tracer.comp:445-549) that
// follows trace_ray: sky on a miss, material scatter with next-event
// estimation, Russian roulette.  Updates acc, mask and ray; returns false
// when the path ends (miss or roulette).  acc must already be clamped
// (Tracer.comp:441; the clamp does not affect the trace, so it may run before
// or after it).  NEE = false leaves out the next-event code for scenes
// without emissive spheres (its loop would run no iteration there).
template <bool NEE = true, class TR>
__device__ __forceinline__ bool shade_bounce(TR& tr, const TraceArgs& a, uint32_t depth, bool found, const Hit& h,
                                             Ray& ray, V3& acc, V3& mask, Rng& g)
{
    if (!found) {
        if (a.sky_on) acc = acc + mask * a.sky;
        return false;
    }
    V3 P, N;
    Material mat;
    tr.surface(ray, h, P, N, mat);
    if (mat.type == MAT_DIFFUSE) {
        const float r2 = rand01(g);
        const V3 d = jitter(N, (2.0f * PI) * rand01(g), sqrtf(r2), sqrtf(1.0f - r2)) * (1.0f - mat.metalness);
        V3 e = splat(0.0f);
        if (NEE)
            for (uint32_t k = 0; k < a.sc.ne; ++k) e = e + nee_one(tr, a, __ldg(a.sc.emit + k), P, N, mat, g);
        const bool emits = mat.emissive.x > 0.0f && mat.emissive.y > 0.0f && mat.emissive.z > 0.0f;
        const V3 emissive = emits ? normalize(mat.emissive) : splat(0.0f);
        acc = acc + mask * (emissive + e);
        mask = mask * mat.albedo;
        ray = Ray{P, normalize(reflect(ray.d, N) + d)};
    } else if (mat.type == MAT_DIELECTRIC) {
        acc = acc + mat.emissive * mask;
        mask = mask * mat.albedo;
        const float cosine = -dot(ray.d, N) / length(ray.d);
        const V3 reflected = reflect(ray.d, N);
        const V3 refracted = refract(ray.d, N, mat.roughness);
        const float prob = (refracted == splat(0.0f)) ? 1.0f : schlick(cosine, mat.roughness);
        ray = Ray{P, normalize(rand01(g) < prob ? reflected : refracted)};
    }  // other types: the shader's switch has no default; the ray is left as it was
    if (depth >= a.rr_start) {
        const float p = max3(mask);
        if (rand01(g) > p) return false;
        mask = mask * (1.0f / p);
    }
    return true;
}

// Tracer.comp:433-553 (radiance), extensions: rr_start, sky, max_depth.
// prim0 / t0 receive the first ray's hit when non-null.
template <class TR>
__device__ __forceinline__ V3 radiance(TR& tr, const TraceArgs& a, Ray ray, Rng& g, uint32_t* prim0, float* t0)
{
    V3 acc = splat(0.0f);
    V3 mask = splat(1.0f);
    for (uint32_t depth = 0; depth < a.max_depth; ++depth) {
        acc = vclamp01(acc);
        Hit h;
        h.t = depth_tmax(depth);
        const bool found = tr.trace(ray, h, false);
        if (prim0 && depth == 0) {
            *prim0 = found ? h.prim : NO_PRIM;
            *t0 = found ? h.t : -1.0f;
        }
        if (!shade_bounce(tr, a, depth, found, h, ray, acc, mask, g)) break;
    }
    return acc;
}

__device__ __forceinline__ unsigned char unorm8(float x)
{
    if (!(x == x)) return 0;
    float c = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
    return (unsigned char)floorf(c * 255.0f + 0.5f);
}

// Tracer.comp:557-574: RNG seeding and the primary ray of pixel (x, y).
__device__ __forceinline__ void seed_rng(const TraceArgs& a, uint32_t x, uint32_t y, Rng& g)
{
    const float uvx = (float)x / (float)a.width;
    const float uvy = (float)y / (float)a.height;
    g.salt = uvy / uvx + a.fr.seed;
    g.cx = uvx;
    g.cy = uvy;
}
__device__ __forceinline__ Ray primary_ray(const TraceArgs& a, uint32_t x, uint32_t y)
{
    const float uvx = (float)x / (float)a.width;
    const float uvy = (float)y / (float)a.height;
    const float tx = 2.0f * uvx - 1.0f;
    const float ty = 2.0f * uvy - 1.0f;
    const V3 dir = (a.fr.cdir + a.fr.cright * tx + a.fr.cup * ty) * v3(a.fr.aspect, 1.0f, a.fr.aspect);
    return Ray{a.fr.cpos, normalize(dir)};
}

// Tracer.comp:585-592: average, Reinhard, gamma 1/2.2, dither, store.
__device__ __forceinline__ void resolve_pixel(const TraceArgs& a, uint32_t x, uint32_t y, V3 accum, Rng& g,
                                              uint32_t prim0, float t0)
{
    accum = accum / (float)a.spp;
    if (a.linear) a.linear[(size_t)y * a.width + x] = make_float4(accum.x, accum.y, accum.z, 1.0f);
    accum = accum / (accum + splat(1.0f));
    const float gam = 1.0f / 2.2f;
    accum = v3(powf(accum.x, gam), powf(accum.y, gam), powf(accum.z, gam));
    const float dither = rand01(g) / 64.0f;
    const float4 c = make_float4(accum.x + dither, accum.y + dither, accum.z + dither, 1.0f);
    const size_t i = (size_t)y * a.width + x;
    if (a.rgba32f) a.rgba32f[i] = c;
    if (a.rgba8) a.rgba8[i] = make_uchar4(unorm8(c.x), unorm8(c.y), unorm8(c.z), 255);
    if (a.hit) a.hit[i] = make_uint2(prim0, __float_as_uint(t0));
}

// Sums each counter over the warp and adds it to the global totals once.
__device__ __forceinline__ void flush_counters(const TraceArgs& a, Counters& cnt)
{
    const unsigned full = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) {
        unsigned long long v = cnt.c[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(full, v, off);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(a.stats + k, v);
        cnt.c[k] = 0;
    }
}

// Warp-level compaction: the lanes with want = true write value to
// consecutive entries of queue, reserved with one atomicAdd on count per warp.
// Every lane of the warp must call it.
__device__ __forceinline__ void warp_append(bool want, uint32_t value, uint32_t* queue, uint32_t* count)
{
    const unsigned full = 0xFFFFFFFFu;
    const unsigned m = __ballot_sync(full, want);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(full, base, leader);
    if (want) queue[base + __popc(m & ((1u << lane) - 1u))] = value;
}

}  // namespace vkt
