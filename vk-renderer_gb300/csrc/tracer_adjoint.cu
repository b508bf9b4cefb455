// Adjoint (reverse-mode) trace for sm_103a: gradients of an image loss with
// respect to the material table's albedo and emission and to the camera
// position, by path replay with O(1) state per path (the wavefront form
// keeps the current sample's pass-1 hits so that pass 2 need not trace).
//
// The image is I = tonemap(accum / spp) + dither (Tracer.comp:585-590), accum
// the sum of the samples' radiance (:578-581).  Given dL/dI per pixel:
//   delta = dL/dI * tonemap'(accum / spp) / spp               (per channel)
// and for every sample, replaying its path twice from the sample's RNG state:
//   pass 1 (primal): the radiance loop (:433-553) as in the forward kernels,
//     recording per channel the last depth at which the clamp of acc
//     (:441) was active -- contributions before it do not reach the output --
//     and the sum T of the contributions that do;
//   pass 2 (adjoint): the same path again.  At a bounce k on material m:
//     emission:  d/de_m of the contribution added at k (normalize(e) for
//                diffuse, :507; e * mask for dielectric, :516);
//     albedo:    every later contribution is proportional to a_m (mask *=
//                albedo, :510/:517), so d/da_m[c] += delta[c] * R[c] / a_m[c]
//                with R = T - (surviving contributions up to k) ("remaining
//                radiance", path replay backpropagation, Vicini et al. 2021);
//                plus the direct dependence of next-event estimation on the
//                albedo at k (kD * albedo / pi and F0 = mix(0.04, albedo,
//                metalness), :481-502);
//     camera:    forward-mode tangents of each ray's origin and direction with
//                respect to the camera position (the primary ray starts at
//                it, :574) carried through every hit, scatter and next-event
//                estimate; the camera enters radiance only through next-event
//                estimation (hit points, the light's cone, V = normalize(
//                camera.pos - P), :464-502).
// Discrete decisions (which primitive is hit, shadow visibility, dielectric
// reflect/refract choice, Russian-roulette survival) are those of the path;
// the Russian-roulette normalisation mask /= max3(mask) is treated as a
// constant (the gradient of the expected value; it has no effect on any
// contribution when roulette only runs at the last depth).  Gradients are
// reduced per block in shared memory and added to global memory once per block.

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_cw8.cuh"
#include "tracer_launch.h"
#include "tracer_wavefront.h"

namespace vkt {

// --------------------------------------------------------- JVP helpers --
__device__ __forceinline__ V3 dnorm(V3 x, V3 dx)
{
    const float il = 1.0f / sqrtf(dot(x, x));
    const V3 y = x * il;
    return (dx - y * dot(y, dx)) * il;
}
__device__ __forceinline__ V3 dcross(V3 a, V3 da, V3 b, V3 db) { return cross(da, b) + cross(a, db); }
__device__ __forceinline__ V3 dreflect(V3 I, V3 dI, V3 N, V3 dN)
{
    const float ni = dot(N, I);
    const float dni = dot(dN, I) + dot(N, dI);
    return dI - dN * (2.0f * ni) - N * (2.0f * dni);
}
__device__ __forceinline__ V3 drefract(V3 I, V3 dI, V3 N, V3 dN, float eta)
{
    const float d = dot(N, I);
    const float dd = dot(dN, I) + dot(N, dI);
    const float k = 1.0f - eta * eta * (1.0f - d * d);
    const float sk = sqrtf(k);
    const float dk = 2.0f * eta * eta * d * dd;
    return dI * eta - N * (eta * dd + dk / (2.0f * sk)) - dN * (eta * d + sk);
}
// d jitter(d, phi, sina, cosa) for varying d, sina, cosa (Tracer.comp:256-263)
__device__ __forceinline__ V3 djitter(V3 d, V3 dd, float cphi, float sphi, float sina, float dsina, float cosa,
                                      float dcosa)
{
    const V3 w = normalize(d);
    const V3 dw = dnorm(d, dd);
    const V3 t = cross(v3(w.y, w.z, w.x), w);
    const V3 dt = dcross(v3(w.y, w.z, w.x), v3(dw.y, dw.z, dw.x), w, dw);
    const V3 u = normalize(t);
    const V3 du = dnorm(t, dt);
    const V3 v = cross(w, u);
    const V3 dv = dcross(w, dw, u, du);
    return (du * cphi + dv * sphi) * sina + (u * cphi + v * sphi) * dsina + dw * cosa + w * dcosa;
}

struct AdjArgs {
    const float4* dldi;    // dL/dI per pixel (RGBA layout, alpha ignored)
    const float4* linear;  // accum / spp per pixel from the forward trace, or NULL (recomputed)
    double* grad;          // [nm x 3 albedo][nm x 3 emission][3 camera position], FP64 sums
    uint32_t nm;
    int smem_grad;         // reduce in shared memory first
};

__device__ __forceinline__ bool finite3(V3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }

// Gradient components are sums of many per-pixel terms of both signs (dL/dI
// changes sign across the image), so they are accumulated in FP64: float sums
// would lose relative precision to the cancellation.
__device__ __forceinline__ void gadd(double* g, int i, float v)
{
    if (v != 0.0f && isfinite(v)) atomicAdd(g + i, (double)v);
}

// One emitter's next-event estimate (same operations as nee_one) with its
// derivative with respect to the albedo at this bounce (componentwise, de_da)
// and, when CAM, with respect to the camera position (de_dc[j], j = x, y, z)
// given the tangents dP, dN of the hit point and normal.
template <bool CAM, class TR>
__device__ __forceinline__ V3 nee_one_grad(TR& tr, const TraceArgs& a, uint32_t si, V3 P, V3 N, const V3* dP,
                                           const V3* dN, const Material& mat, Rng& g, V3& de_da, V3* de_dc)
{
    const float4* rec = a.sc.sph_rec + 4 * (size_t)si;
    const float4 geo = __ldg(rec + 3);
    const V3 sP = v3(geo);
    const float sr = geo.w;
    const float t = length(sP - P) - sr;
    const V3 l0 = sP - P;
    const float ll = dot(l0, l0);
    const float q = sr * sr / ll;
    const float cos_a_max = sqrtf(1.0f - gclamp(q, 0.0f, 1.0f));
    const float rho = rand01(g);
    const float cosa = gmix(cos_a_max, 1.0f, rho);
    const float phi = (2.0f * PI) * rand01(g);
    const float sina = sqrtf(1.0f - cosa * cosa);
    const V3 L = jitter(l0, phi, sina, cosa);
    Hit sh;
    sh.t = t;
    if (tr.trace(Ray{P, L}, sh, true)) return splat(0.0f);
    const float4 em = __ldg(rec + 1);
    const float q2 = t / sr + 1.0f;
    const V3 att1 = (v3(em) * 1.0f / (q2 * q2) - 0.001f) / (1.0f - 0.001f);
    const V3 att = vmax0(att1);
    V3 F0 = splat(0.04f);
    F0 = vmix(F0, mat.albedo, mat.metalness);
    const V3 V = normalize(a.fr.cpos - P);
    const V3 H = normalize(V + L);
    const float rough = mat.roughness;
    const float ar = rough * rough, a2 = ar * ar;
    const float nh = dot(N, H);
    const float NdotH = gmax(nh, 0.0f);
    const float dden = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
    const float NDF = a2 / (PI * dden * dden);
    const float kg = (rough + 1.0f) * (rough + 1.0f) / 8.0f;
    const float nv = dot(N, V), nl = dot(N, L);
    const float NdotV = gmax(nv, 0.0f), NdotL = gmax(nl, 0.0f);
    const float gv = NdotV / (NdotV * (1.0f - kg) + kg), gl = NdotL / (NdotL * (1.0f - kg) + kg);
    const float G = gl * gv;
    const float hv = dot(H, V);
    const float cth = gmax(hv, 0.0f);
    const float s5 = powf(1.0f - cth, 5.0f);
    const V3 F = F0 + (1.0f - F0) * s5;
    const V3 kD = (1.0f - F) * (1.0f - mat.metalness);
    const float den4 = 4.0f * NdotV * NdotL;
    const float D = gmax(den4, 0.001f);
    const V3 spec = NDF * G * F / D;
    const V3 base = kD * mat.albedo / PI + spec;
    // d/d albedo (componentwise): dF/da = metal (1 - s5); dkD/da = -dF/da (1 - metal)
    {
        const float dFda = mat.metalness * (1.0f - s5);
        const float dkDda = -dFda * (1.0f - mat.metalness);
        const V3 dbase = (dkDda * mat.albedo + kD) / PI + splat(NDF * G * dFda / D);
        de_da = de_da + dbase * att * NdotL;
    }
    if (CAM) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const V3 dl0 = splat(0.0f) - dP[j];
            const float dt = dot(l0, dl0) / sqrtf(ll);
            const float dq = (q > 0.0f && q < 1.0f) ? -sr * sr * 2.0f * dot(l0, dl0) / (ll * ll) : 0.0f;
            const float dcm = cos_a_max > 0.0f ? -dq / (2.0f * cos_a_max) : 0.0f;
            const float dcosa = (1.0f - rho) * dcm;
            const float dsina = sina > 0.0f ? -cosa * dcosa / sina : 0.0f;
            float cphi, sphi;
            psincos(phi, sphi, cphi);
            const V3 dL = djitter(l0, dl0, cphi, sphi, sina, dsina, cosa, dcosa);
            const float dq2 = dt / sr;
            V3 datt = v3(em) * (-2.0f * dq2 / (q2 * q2 * q2)) / (1.0f - 0.001f);
            datt = v3(att1.x > 0.0f ? datt.x : 0.0f, att1.y > 0.0f ? datt.y : 0.0f, att1.z > 0.0f ? datt.z : 0.0f);
            const V3 ej = v3(j == 0 ? 1.0f : 0.0f, j == 1 ? 1.0f : 0.0f, j == 2 ? 1.0f : 0.0f);
            const V3 dV = dnorm(a.fr.cpos - P, ej - dP[j]);
            const V3 dH = dnorm(V + L, dV + dL);
            const float dNdotH = nh > 0.0f ? dot(dN[j], H) + dot(N, dH) : 0.0f;
            const float dNDF = -2.0f * a2 / (PI * dden * dden * dden) * (2.0f * NdotH * (a2 - 1.0f) * dNdotH);
            const float dNdotV = nv > 0.0f ? dot(dN[j], V) + dot(N, dV) : 0.0f;
            const float dNdotL = nl > 0.0f ? dot(dN[j], L) + dot(N, dL) : 0.0f;
            const float cv = NdotV * (1.0f - kg) + kg, cl = NdotL * (1.0f - kg) + kg;
            const float dG = kg / (cl * cl) * dNdotL * gv + gl * kg / (cv * cv) * dNdotV;
            const float dcth = hv > 0.0f ? dot(dH, V) + dot(H, dV) : 0.0f;
            const float om = 1.0f - cth;
            const float ds5 = -5.0f * om * om * om * om * dcth;
            const V3 dF = (1.0f - F0) * ds5;
            const V3 dkD = splat(0.0f) - dF * (1.0f - mat.metalness);
            const float dD = den4 > 0.001f ? 4.0f * (dNdotV * NdotL + NdotV * dNdotL) : 0.0f;
            const V3 dspec = (dNDF * G * F + NDF * dG * F + NDF * G * dF) / D - spec * (dD / D);
            const V3 dbase = dkD * mat.albedo / PI + dspec;
            de_dc[j] = de_dc[j] + (dbase * att + base * datt) * NdotL + base * att * dNdotL;
        }
    }
    return base * att * NdotL;
}

// tonemap(x) = (x / (x + 1))^(1/2.2) has slope g (x/(x+1))^(g-1) / (x+1)^2,
// infinite at 0: the slope is taken at x >= 1e-6.
__device__ __forceinline__ float tm_slope(float x)
{
    const float gam = 1.0f / 2.2f;
    x = gmax(x, 1e-6f);
    const float r = x / (x + 1.0f);
    return gam * powf(r, gam - 1.0f) / ((x + 1.0f) * (x + 1.0f));
}

// delta = dL/dI * tonemap'(accum / spp) / spp per channel: the weight of one
// sample's radiance in the loss.
__device__ __forceinline__ V3 pixel_delta(float4 dl, V3 lin, uint32_t spp)
{
    return v3(dl.x * tm_slope(lin.x), dl.y * tm_slope(lin.y), dl.z * tm_slope(lin.z)) / (float)spp;
}

// Pass 1: the radiance loop with clamp bookkeeping.  lc[c] = last depth whose
// clamp of acc[c] was active (-1: none); T = contributions that survive.
template <class TR>
__device__ __forceinline__ void primal_pass(TR& tr, const TraceArgs& a, Ray ray, Rng& g, int* lc, V3& T)
{
    V3 acc = splat(0.0f), mask = splat(1.0f);
    T = splat(0.0f);
    for (uint32_t depth = 0; depth < a.max_depth; ++depth) {
        if (acc.x < 0.0f || acc.x > 1.0f) { lc[0] = (int)depth; T.x = 0.0f; }
        if (acc.y < 0.0f || acc.y > 1.0f) { lc[1] = (int)depth; T.y = 0.0f; }
        if (acc.z < 0.0f || acc.z > 1.0f) { lc[2] = (int)depth; T.z = 0.0f; }
        acc = vclamp01(acc);
        Hit h;
        h.t = depth_tmax(depth);
        const bool found = tr.trace(ray, h, false);
        const V3 before = acc;
        const bool cont = shade_bounce(tr, a, depth, found, h, ray, acc, mask, g);
        T = T + (acc - before);
        if (!cont) break;
    }
}

template <int TIE, bool BVH, bool CAM>
__global__ void __launch_bounds__(128) k_adjoint(TraceArgs a, AdjArgs ga)
{
    extern __shared__ int smem[];
    const int tid = threadIdx.x, nthreads = blockDim.x;
    const Stack stk{smem + tid, reinterpret_cast<float*>(smem + (size_t)a.stack_depth * nthreads) + tid, nthreads,
                    (int)a.stack_depth};
    // gradient sums after the stack, 8-byte aligned
    double* sgrad = reinterpret_cast<double*>(smem + 2 * (size_t)a.stack_depth * nthreads);
    const uint32_t ngrad = 6 * ga.nm + 3;
    if (ga.smem_grad) {
        for (uint32_t k = tid; k < ngrad; k += nthreads) sgrad[k] = 0.0;
        __syncthreads();
    }
    double* grad = ga.smem_grad ? sgrad : ga.grad;
    double* gal = grad;
    double* gem = grad + 3 * ga.nm;
    double* gcam = grad + 6 * ga.nm;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    Tracer<TIE, BVH, true> tr{a.sc, stk, cnt, a.status, a.trav_limit};
    const uint32_t x = blockIdx.x * 16 + (tid & 15);
    const uint32_t y = blockIdx.y * (nthreads >> 4) + (tid >> 4);
    if (x < a.width && y < a.height) {
        const size_t i = (size_t)y * a.width + x;
        Rng g;
        seed_rng(a, x, y, g);
        const Ray pr = primary_ray(a, x, y);
        V3 lin;
        if (ga.linear) {
            lin = v3(ga.linear[i]);
        } else {
            Rng g0 = g;
            V3 acc = splat(0.0f);
            for (uint32_t s = 0; s < a.spp; ++s) acc = acc + radiance(tr, a, pr, g0, nullptr, nullptr);
            lin = acc / (float)a.spp;
        }
        const V3 delta = pixel_delta(ga.dldi[i], lin, a.spp);
        if (finite3(delta) && finite3(lin)) {
            for (uint32_t s = 0; s < a.spp; ++s) {
                const Rng gs = g;  // this sample's RNG state
                int lc[3] = {-1, -1, -1};
                V3 T;
                primal_pass(tr, a, pr, g, lc, T);  // advances g past the sample
                // pass 2: adjoint replay
                Rng g2 = gs;
                V3 mask = splat(1.0f), prefix = splat(0.0f);
                Ray ray = pr;
                V3 dO[3], dD[3];
                if (CAM) {
#pragma unroll
                    for (int j = 0; j < 3; ++j) {
                        dO[j] = v3(j == 0 ? 1.0f : 0.0f, j == 1 ? 1.0f : 0.0f, j == 2 ? 1.0f : 0.0f);
                        dD[j] = splat(0.0f);
                    }
                }
                for (uint32_t depth = 0; depth < a.max_depth; ++depth) {
                    Hit h;
                    h.t = depth_tmax(depth);
                    const bool found = tr.trace(ray, h, false);
                    const V3 surv = v3((int)depth >= lc[0] ? 1.0f : 0.0f, (int)depth >= lc[1] ? 1.0f : 0.0f,
                                       (int)depth >= lc[2] ? 1.0f : 0.0f);
                    const V3 w = delta * surv;
                    if (!found) {
                        if (a.sky_on) prefix = prefix + mask * a.sky * surv;
                        break;
                    }
                    V3 P, N;
                    Material mat;
                    tr.surface(ray, h, P, N, mat);
                    const int m = h.kind == 1 ? (int)__float_as_uint(__ldg(a.sc.tri + 3 * (size_t)h.slot).w) : -1;
                    V3 dP[3], dN[3];
                    if (CAM) {
                        const float nd = dot(N, ray.d);
#pragma unroll
                        for (int j = 0; j < 3; ++j) {
                            const V3 q = dO[j] + dD[j] * h.t;
                            const float dt = -dot(N, q) / nd;
                            dP[j] = q + ray.d * dt;
                            dN[j] = h.kind == 2 ? dP[j] / __ldg(a.sc.sph_geo + h.slot).w : splat(0.0f);
                        }
                    }
                    V3 C = splat(0.0f);
                    if (mat.type == MAT_DIFFUSE) {
                        const float r2 = rand01(g2);
                        const float phi = (2.0f * PI) * rand01(g2);
                        const float sa = sqrtf(r2), ca = sqrtf(1.0f - r2);
                        const V3 jd = jitter(N, phi, sa, ca);
                        const V3 d = jd * (1.0f - mat.metalness);
                        V3 e = splat(0.0f), de_da = splat(0.0f);
                        V3 de_dc[3] = {splat(0.0f), splat(0.0f), splat(0.0f)};
                        for (uint32_t k = 0; k < a.sc.ne; ++k)
                            e = e + nee_one_grad<CAM>(tr, a, __ldg(a.sc.emit + k), P, N, dP, dN, mat, g2, de_da, de_dc);
                        const bool emits = mat.emissive.x > 0.0f && mat.emissive.y > 0.0f && mat.emissive.z > 0.0f;
                        const V3 en = emits ? normalize(mat.emissive) : splat(0.0f);
                        C = mask * (en + e);
                        const V3 wm = w * mask;
                        if (m >= 0) {
                            if (emits) {  // d normalize(e) = (I - n n^T) / |e|
                                const float il = 1.0f / length(mat.emissive);
                                const V3 ge = (wm - en * dot(en, wm)) * il;
                                gadd(gem, 3 * m + 0, ge.x);
                                gadd(gem, 3 * m + 1, ge.y);
                                gadd(gem, 3 * m + 2, ge.z);
                            }
                            const V3 gd = wm * de_da;
                            gadd(gal, 3 * m + 0, gd.x);
                            gadd(gal, 3 * m + 1, gd.y);
                            gadd(gal, 3 * m + 2, gd.z);
                        }
                        if (CAM) {
#pragma unroll
                            for (int j = 0; j < 3; ++j) gadd(gcam, j, dot(wm, de_dc[j]));
                        }
                        prefix = prefix + C * surv;
                        if (m >= 0) {
                            const V3 R = T - prefix;
                            if (mat.albedo.x != 0.0f) gadd(gal, 3 * m + 0, delta.x * R.x / mat.albedo.x);
                            if (mat.albedo.y != 0.0f) gadd(gal, 3 * m + 1, delta.y * R.y / mat.albedo.y);
                            if (mat.albedo.z != 0.0f) gadd(gal, 3 * m + 2, delta.z * R.z / mat.albedo.z);
                        }
                        mask = mask * mat.albedo;
                        const V3 rf = reflect(ray.d, N);
                        if (CAM) {
                            float cphi, sphi;
                            psincos(phi, sphi, cphi);
#pragma unroll
                            for (int j = 0; j < 3; ++j) {
                                const V3 djd = djitter(N, dN[j], cphi, sphi, sa, 0.0f, ca, 0.0f);
                                const V3 drf = dreflect(ray.d, dD[j], N, dN[j]);
                                dD[j] = dnorm(rf + d, drf + djd * (1.0f - mat.metalness));
                                dO[j] = dP[j];
                            }
                        }
                        ray = Ray{P, normalize(rf + d)};
                    } else if (mat.type == MAT_DIELECTRIC) {
                        C = mat.emissive * mask;
                        if (m >= 0) {
                            const V3 ge = w * mask;
                            gadd(gem, 3 * m + 0, ge.x);
                            gadd(gem, 3 * m + 1, ge.y);
                            gadd(gem, 3 * m + 2, ge.z);
                        }
                        prefix = prefix + C * surv;
                        if (m >= 0) {
                            const V3 R = T - prefix;
                            if (mat.albedo.x != 0.0f) gadd(gal, 3 * m + 0, delta.x * R.x / mat.albedo.x);
                            if (mat.albedo.y != 0.0f) gadd(gal, 3 * m + 1, delta.y * R.y / mat.albedo.y);
                            if (mat.albedo.z != 0.0f) gadd(gal, 3 * m + 2, delta.z * R.z / mat.albedo.z);
                        }
                        mask = mask * mat.albedo;
                        const float cosine = -dot(ray.d, N) / length(ray.d);
                        const V3 reflected = reflect(ray.d, N);
                        const V3 refracted = refract(ray.d, N, mat.roughness);
                        const bool tir = refracted == splat(0.0f);
                        const float prob = tir ? 1.0f : schlick(cosine, mat.roughness);
                        const bool refl = rand01(g2) < prob;
                        const V3 nd = refl ? reflected : refracted;
                        if (CAM) {
#pragma unroll
                            for (int j = 0; j < 3; ++j) {
                                const V3 dr = refl ? dreflect(ray.d, dD[j], N, dN[j])
                                                   : drefract(ray.d, dD[j], N, dN[j], mat.roughness);
                                dD[j] = dnorm(nd, dr);
                                dO[j] = dP[j];
                            }
                        }
                        ray = Ray{P, normalize(nd)};
                    }
                    if (depth >= a.rr_start) {
                        const float p = max3(mask);
                        if (rand01(g2) > p) break;
                        mask = mask * (1.0f / p);
                    }
                }
            }
        }
    }
    flush_counters(a, cnt);
    if (ga.smem_grad) {
        __syncthreads();
        for (uint32_t k = tid; k < ngrad; k += nthreads)
            if (sgrad[k] != 0.0) atomicAdd(ga.grad + k, sgrad[k]);
    }
}

// ------------------------------------------------------ wavefront adjoint --
// The same two passes per sample for scenes without emissive spheres, as
// stages over the wavefront's path queue: the closest-hit rays of pass 1 (and
// of pass 2 when there is no hit log) go through the forward renderer's
// extend kernel, and wf_adj_shade runs one bounce of whichever pass a path is
// in; with the hit log, pass 2 runs whole where pass 1 ends (adj_advance).
// The camera gradient's interior part is zero here (below); its boundary part
// comes from the edge kernel.  A path's state between rounds:
//   ray_o/ray_d  the ray to trace next (tmax in ray_o.w)
//   acc          pass 1: acc; pass 2: the surviving prefix; .w the RNG salt
//   mask         mask; .w the three last-clamp depths (10 bits each, +1)
//   accum        T (pass 2 reads it); .w phase << 31 | sample << 16 | depth
//   pix          delta of the pixel; .w the RNG salt at the sample's start
//   prim0        the RNG salt at the sample's end (pass 2 restores it)
// Without emitters the camera position enters radiance only through which
// primitives are hit, so the interior part of its gradient is zero.

__device__ __forceinline__ uint32_t lc_pack(const int lc[3])
{
    return (uint32_t)(lc[0] + 1) | ((uint32_t)(lc[1] + 1) << 10) | ((uint32_t)(lc[2] + 1) << 20);
}
__device__ __forceinline__ void lc_unpack(uint32_t v, int lc[3])
{
    lc[0] = (int)(v & 0x3FFu) - 1;
    lc[1] = (int)((v >> 10) & 0x3FFu) - 1;
    lc[2] = (int)((v >> 20) & 0x3FFu) - 1;
}
constexpr uint32_t kPhaseReplay = 1u << 31;

__global__ void __launch_bounds__(256) wf_adj_generate(TraceArgs a, WfState s, AdjWf w)
{
    const uint32_t n = a.width * a.height;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool queued = false;
    if (i < n) {
        const uint32_t x = i % a.width, y = i / a.width;
        const V3 lin = v3(w.linear[i]);
        const V3 delta = pixel_delta(w.dldi[i], lin, a.spp);
        if (finite3(delta) && finite3(lin)) {  // as the per-pixel kernel: other pixels trace nothing
            Rng g;
            seed_rng(a, x, y, g);
            const Ray r = primary_ray(a, x, y);
            const int none[3] = {-1, -1, -1};
            s.ray_o[i] = make_float4(r.o.x, r.o.y, r.o.z, depth_tmax(0));
            s.ray_d[i] = make_float4(r.d.x, r.d.y, r.d.z, 0.0f);
            s.acc[i] = make_float4(0.0f, 0.0f, 0.0f, g.salt);
            s.mask[i] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(lc_pack(none)));
            s.accum[i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0u));
            w.pix[i] = make_float4(delta.x, delta.y, delta.z, g.salt);
            queued = true;
        }
    }
    warp_append(queued, i, s.queue[0], &s.count[0]);
}

// d/da_m[c] += delta[c] R[c] / a_m[c] for the material a path just scattered on.
__device__ __forceinline__ void albedo_grad(double* gal, int m, V3 delta, V3 R, V3 albedo)
{
    if (albedo.x != 0.0f) gadd(gal, 3 * m + 0, delta.x * R.x / albedo.x);
    if (albedo.y != 0.0f) gadd(gal, 3 * m + 1, delta.y * R.y / albedo.y);
    if (albedo.z != 0.0f) gadd(gal, 3 * m + 2, delta.z * R.z / albedo.z);
}

// One path of the wavefront adjoint between rounds, unpacked (the per-pixel
// delta and the two saved RNG states stay in memory: pix, prim0).
struct AdjPath {
    Ray ray;
    V3 acc, mask, T;
    int lc[3];
    uint32_t sample, depth;
    bool replay;
    Rng g;
};

__device__ __forceinline__ void adj_load(const WfState& s, const TraceArgs& a, uint32_t pid, uint32_t x, uint32_t y,
                                         AdjPath& p)
{
    const float4 ro = s.ray_o[pid], rd = s.ray_d[pid];
    const float4 acc4 = s.acc[pid], mask4 = s.mask[pid], accum4 = s.accum[pid];
    const uint32_t bits = __float_as_uint(accum4.w);
    p.replay = (bits & kPhaseReplay) != 0;
    p.sample = (bits >> 16) & 0x7FFFu;
    p.depth = bits & 0xFFFFu;
    lc_unpack(__float_as_uint(mask4.w), p.lc);
    p.g.salt = acc4.w;
    p.g.cx = (float)x / (float)a.width;
    p.g.cy = (float)y / (float)a.height;
    p.ray = Ray{v3(ro), v3(rd)};
    p.acc = v3(acc4);
    p.mask = v3(mask4);
    p.T = v3(accum4);
}

__device__ __forceinline__ void adj_store(const WfState& s, uint32_t pid, const AdjPath& p)
{
    s.ray_o[pid] = make_float4(p.ray.o.x, p.ray.o.y, p.ray.o.z, depth_tmax(p.depth));
    s.ray_d[pid] = make_float4(p.ray.d.x, p.ray.d.y, p.ray.d.z, 0.0f);
    s.acc[pid] = make_float4(p.acc.x, p.acc.y, p.acc.z, p.g.salt);
    s.mask[pid] = make_float4(p.mask.x, p.mask.y, p.mask.z, __uint_as_float(lc_pack(p.lc)));
    s.accum[pid] = make_float4(p.T.x, p.T.y, p.T.z,
                               __uint_as_float((p.replay ? kPhaseReplay : 0u) | (p.sample << 16) | p.depth));
}

// Pass 2's bounce at p.depth, given the closest hit h of its ray (the same
// ray and hit as pass 1's bounce at that depth): the gradient terms, then
// the same scatter and roulette as pass 1.  Returns true while the sample's
// path goes on.
template <class TR>
__device__ __forceinline__ bool adj_replay_bounce(TR& tr, const TraceArgs& a, const AdjWf& w, const Hit& h, V3 delta,
                                                  AdjPath& p)
{
    double* gal = w.grad;
    double* gem = w.grad + 3 * (size_t)w.nm;
    const bool found = h.kind != 0;
    const V3 surv = v3((int)p.depth >= p.lc[0] ? 1.0f : 0.0f, (int)p.depth >= p.lc[1] ? 1.0f : 0.0f,
                       (int)p.depth >= p.lc[2] ? 1.0f : 0.0f);
    const V3 wgt = delta * surv;
    bool cont = false;
    if (found) {
        V3 P, N;
        Material mat;
        tr.surface(p.ray, h, P, N, mat);
        const int m = h.kind == 1 ? (int)__float_as_uint(__ldg(a.sc.tri + 3 * (size_t)h.slot).w) : -1;
        if (mat.type == MAT_DIFFUSE) {
            const float r2 = rand01(p.g);
            const V3 d = jitter(N, (2.0f * PI) * rand01(p.g), sqrtf(r2), sqrtf(1.0f - r2)) * (1.0f - mat.metalness);
            const bool emits = mat.emissive.x > 0.0f && mat.emissive.y > 0.0f && mat.emissive.z > 0.0f;
            const V3 en = emits ? normalize(mat.emissive) : splat(0.0f);
            if (m >= 0 && emits) {  // d normalize(e) = (I - n n^T) / |e|
                const V3 wm = wgt * p.mask;
                const V3 ge = (wm - en * dot(en, wm)) * (1.0f / length(mat.emissive));
                gadd(gem, 3 * m + 0, ge.x);
                gadd(gem, 3 * m + 1, ge.y);
                gadd(gem, 3 * m + 2, ge.z);
            }
            p.acc = p.acc + p.mask * en * surv;
            if (m >= 0) albedo_grad(gal, m, delta, p.T - p.acc, mat.albedo);
            p.mask = p.mask * mat.albedo;
            p.ray = Ray{P, normalize(reflect(p.ray.d, N) + d)};
        } else if (mat.type == MAT_DIELECTRIC) {
            if (m >= 0) {
                const V3 ge = wgt * p.mask;
                gadd(gem, 3 * m + 0, ge.x);
                gadd(gem, 3 * m + 1, ge.y);
                gadd(gem, 3 * m + 2, ge.z);
            }
            p.acc = p.acc + mat.emissive * p.mask * surv;
            if (m >= 0) albedo_grad(gal, m, delta, p.T - p.acc, mat.albedo);
            p.mask = p.mask * mat.albedo;
            const float cosine = -dot(p.ray.d, N) / length(p.ray.d);
            const V3 reflected = reflect(p.ray.d, N);
            const V3 refracted = refract(p.ray.d, N, mat.roughness);
            const float prob = (refracted == splat(0.0f)) ? 1.0f : schlick(cosine, mat.roughness);
            p.ray = Ray{P, normalize(rand01(p.g) < prob ? reflected : refracted)};
        }
        cont = true;
        if (p.depth >= a.rr_start) {
            const float q = max3(p.mask);
            if (rand01(p.g) > q)
                cont = false;
            else
                p.mask = p.mask * (1.0f / q);
        }
    }
    p.depth++;
    return cont && p.depth < a.max_depth;
}

__device__ __forceinline__ uint4 hit_pack(const Hit& h)
{
    return make_uint4(__float_as_uint(h.t), h.prim, h.slot, (uint32_t)h.kind);
}
__device__ __forceinline__ Hit hit_unpack(uint4 v)
{
    Hit h;
    h.t = __uint_as_float(v.x);
    h.prim = v.y;
    h.slot = v.z;
    h.kind = (int)v.w;
    return h;
}

// One bounce of whichever pass the path is in, given the closest hit h of
// its ray, then the bookkeeping: pass 1 ends -> pass 2 of the same sample
// from the sample's first ray and RNG state; pass 2 ends -> the next sample
// (the RNG continues where pass 1 left it).  pix: the pixel's delta and the
// RNG salt at the sample's start; prim0: the salt at the end of pass 1.
// With a hit log (w.log), pass 1 records its hits and pass 2 runs right
// where pass 1 ends, from the log, without tracing: the same rays meet the
// same hits, so the gradients are those of tracing them again.
// Returns true while the pixel has a ray to trace.
template <class TR>
__device__ __forceinline__ bool adj_advance(TR& tr, const TraceArgs& a, const AdjWf& w, uint32_t pid, uint32_t x,
                                            uint32_t y, const Hit& h, AdjPath& p, float4* pix, uint32_t* prim0)
{
    uint4* log = w.log ? w.log + (size_t)pid * a.max_depth : nullptr;
    if (!p.replay) {
        // pass 1: clamp bookkeeping, then the forward bounce
        const bool found = h.kind != 0;
        if (p.acc.x < 0.0f || p.acc.x > 1.0f) { p.lc[0] = (int)p.depth; p.T.x = 0.0f; }
        if (p.acc.y < 0.0f || p.acc.y > 1.0f) { p.lc[1] = (int)p.depth; p.T.y = 0.0f; }
        if (p.acc.z < 0.0f || p.acc.z > 1.0f) { p.lc[2] = (int)p.depth; p.T.z = 0.0f; }
        p.acc = vclamp01(p.acc);
        const V3 before = p.acc;
        const bool cont = shade_bounce<false>(tr, a, p.depth, found, h, p.ray, p.acc, p.mask, p.g);  // no emitters
        p.T = p.T + (p.acc - before);
        if (log) log[p.depth] = hit_pack(h);
        p.depth++;
        if (cont && p.depth < a.max_depth) return true;
        // pass 2 of the same sample: its first ray and RNG state again
        const uint32_t bounces = p.depth;
        *prim0 = __float_as_uint(p.g.salt);
        p.g.salt = pix->w;
        p.ray = primary_ray(a, x, y);
        p.acc = splat(0.0f);
        p.mask = splat(1.0f);
        p.depth = 0;
        p.replay = true;
        if (!log) return true;
        const V3 delta = v3(*pix);
        while (adj_replay_bounce(tr, a, w, hit_unpack(log[p.depth]), delta, p) && p.depth < bounces) {
        }
    } else if (adj_replay_bounce(tr, a, w, h, v3(*pix), p)) {
        return true;
    }
    // sample finished: the RNG continues where pass 1 left it
    p.g.salt = __uint_as_float(*prim0);
    p.sample++;
    if (p.sample >= a.spp) return false;
    p.ray = primary_ray(a, x, y);
    p.acc = splat(0.0f);
    p.mask = splat(1.0f);
    p.T = splat(0.0f);
    p.lc[0] = p.lc[1] = p.lc[2] = -1;
    p.depth = 0;
    p.replay = false;
    pix->w = p.g.salt;  // the new sample's start
    return true;
}

template <int TIE, bool BVH>
__global__ void __launch_bounds__(256) wf_adj_shade(TraceArgs a, WfState s, AdjWf w, int qsel)
{
    const uint32_t n = s.count[qsel];
    const uint32_t* queue = qsel ? s.queue[1] : s.queue[0];
    uint32_t* next = qsel ? s.queue[0] : s.queue[1];
    if (blockIdx.x == 0 && threadIdx.x == 0) s.count[2] = 0;  // fetch cursor of the next round
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    // no emitters: shading traces no shadow rays and needs no stack
    Tracer<TIE, BVH, false> tr{a.sc, Stack{nullptr, nullptr, 0, 0}, cnt, a.status, a.trav_limit};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t qi = base + threadIdx.x;
        bool again = false;
        uint32_t pid = 0;
        if (qi < n) {
            pid = queue[qi];
            const uint32_t x = pid % a.width, y = pid / a.width;
            AdjPath p;
            adj_load(s, a, pid, x, y, p);
            const uint4 hr = s.hit[pid];
            Hit h;
            h.t = __uint_as_float(hr.x);
            h.prim = hr.y;
            h.slot = hr.z;
            h.kind = (int)hr.w;
            again = adj_advance(tr, a, w, pid, x, y, h, p, w.pix + pid, s.prim0 + pid);
            if (again) adj_store(s, pid, p);
        }
        warp_append(again, pid, next, &s.count[qsel ^ 1]);
    }
}

// The adjoint's finishing kernel (as wf_finish for the forward): each thread
// runs queued paths to the end of their pixels -- both passes of every
// remaining sample (pass 2 from the hit log when there is one) -- with the
// per-thread traversal for the closest hits.
template <int TIE, bool BVH, bool STATS>
__global__ void __launch_bounds__(128) wf_adj_finish(TraceArgs a, WfState s, AdjWf w, int qsel)
{
    extern __shared__ int smem[];
    const uint32_t n = s.count[qsel];
    const uint32_t* queue = qsel ? s.queue[1] : s.queue[0];
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    const Stack stk{smem + threadIdx.x, reinterpret_cast<float*>(smem + (size_t)a.stack_depth * blockDim.x) + threadIdx.x,
                    (int)blockDim.x, (int)a.stack_depth};
    // closest hits: the per-thread 8-wide traversal where the scene has one
    // (c3's 256^2 adjoint: 0.47 ms against 0.74 with the plain binary
    // traversal), else the plain traversal, which tests a hit leaf child as
    // soon as its parent is visited (on c3's short, latency-bound chains it
    // beat the pre-encoded binary traversal, 1.35 against 1.42 ms)
    Tracer<TIE, BVH, STATS> tr{a.sc, stk, cnt, a.status, a.trav_limit};
    // triangle-only scenes with an 8-wide BVH: the forward finishing kernel's
    // per-thread 8-wide traversal, its stack over the same shared memory
    // (stack_depth 8-byte entries per thread; nothing here traces shadow rays)
    const PairStack pstk{reinterpret_cast<int2*>(smem) + threadIdx.x, (int)blockDim.x, (int)a.stack_depth};
    const uint32_t threads = gridDim.x * blockDim.x;
    uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    while (qi < n) {
        const uint32_t pid = queue[qi];
        const uint32_t x = pid % a.width, y = pid / a.width;
        AdjPath p;
        adj_load(s, a, pid, x, y, p);
        for (;;) {
            Hit h;
            h.t = depth_tmax(p.depth);
            if (BVH && a.sc.tri_cw8 != nullptr)
                closest_cw8<STATS>(a.sc, p.ray, h, pstk, a.status, a.trav_limit, cnt);
            else
                tr.trace(p.ray, h, false);
            if (!adj_advance(tr, a, w, pid, x, y, h, p, w.pix + pid, s.prim0 + pid)) break;
        }
        qi = n > threads ? threads + atomicAdd(&s.count[2], 1u) : n;
    }
    if (STATS) flush_counters(a, cnt);
}

cudaError_t wf_launch_adj_generate(const TraceArgs& a, const WfState& s, const AdjWf& w, cudaStream_t st)
{
    const uint32_t n = a.width * a.height;
    wf_adj_generate<<<(n + 255) / 256, 256, 0, st>>>(a, s, w);
    return cudaGetLastError();
}

cudaError_t wf_launch_adj_shade(const TraceArgs& a, const WfState& s, const AdjWf& w, const WfConfig& c, int qsel,
                                cudaStream_t st)
{
    if (c.tie == TIE_REFERENCE)
        wf_adj_shade<TIE_REFERENCE, false><<<c.shade_grid, 256, 0, st>>>(a, s, w, qsel);
    else if (c.bvh)
        wf_adj_shade<TIE_STRICT, true><<<c.shade_grid, 256, 0, st>>>(a, s, w, qsel);
    else
        wf_adj_shade<TIE_STRICT, false><<<c.shade_grid, 256, 0, st>>>(a, s, w, qsel);
    return cudaGetLastError();
}

template <int TIE, bool BVH, bool STATS>
static size_t adj_finish_smem(const TraceArgs& a)
{
    const size_t smem = BVH ? (size_t)a.stack_depth * 128 * 8 : 0;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(wf_adj_finish<TIE, BVH, STATS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return smem;
}

template <int TIE, bool BVH, bool STATS>
static cudaError_t adj_finish_t(const TraceArgs& a, const WfState& s, const AdjWf& w, const WfConfig& c, int qsel,
                                cudaStream_t st)
{
    wf_adj_finish<TIE, BVH, STATS><<<c.finish_grid, 128, adj_finish_smem<TIE, BVH, STATS>(a), st>>>(a, s, w, qsel);
    return cudaGetLastError();
}

template <int TIE, bool BVH, bool STATS>
static int adj_finish_occ(const TraceArgs& a)
{
    int n = 0;
    const size_t smem = adj_finish_smem<TIE, BVH, STATS>(a);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wf_adj_finish<TIE, BVH, STATS>, 128, smem) == cudaSuccess
               ? n
               : 0;
}

template <bool STATS>
static cudaError_t adj_finish_s(const TraceArgs& a, const WfState& s, const AdjWf& w, const WfConfig& c, int qsel,
                                cudaStream_t st)
{
    if (c.tie == TIE_REFERENCE) return adj_finish_t<TIE_REFERENCE, false, STATS>(a, s, w, c, qsel, st);
    if (c.bvh) return adj_finish_t<TIE_STRICT, true, STATS>(a, s, w, c, qsel, st);
    return adj_finish_t<TIE_STRICT, false, STATS>(a, s, w, c, qsel, st);
}

template <bool STATS>
static int adj_finish_occ_s(const TraceArgs& a, const WfConfig& c)
{
    if (c.tie == TIE_REFERENCE) return adj_finish_occ<TIE_REFERENCE, false, STATS>(a);
    if (c.bvh) return adj_finish_occ<TIE_STRICT, true, STATS>(a);
    return adj_finish_occ<TIE_STRICT, false, STATS>(a);
}

cudaError_t wf_launch_adj_finish(const TraceArgs& a, const WfState& s, const AdjWf& w, const WfConfig& c, int qsel,
                                 cudaStream_t st)
{
    return c.stats ? adj_finish_s<true>(a, s, w, c, qsel, st) : adj_finish_s<false>(a, s, w, c, qsel, st);
}

int wf_adj_finish_blocks_per_sm(const TraceArgs& a, const WfConfig& c)
{
    return c.stats ? adj_finish_occ_s<true>(a, c) : adj_finish_occ_s<false>(a, c);
}

template <int TIE, bool BVH, bool CAM>
static cudaError_t adj_t(const TraceArgs& a, const AdjArgs& g, cudaStream_t s)
{
    const uint32_t block = 128;
    const size_t smem = (size_t)a.stack_depth * block * 8 + (g.smem_grad ? (6 * (size_t)g.nm + 3) * 8 : 0);
    auto k = k_adjoint<TIE, BVH, CAM>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((a.width + 15) / 16, (a.height + (block / 16) - 1) / (block / 16));
    k<<<grid, block, smem, s>>>(a, g);
    return cudaGetLastError();
}

__global__ void k_grad_to_float(const double* __restrict__ g, float* __restrict__ out, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = (float)g[i];
}

cudaError_t launch_grad_to_float(const double* g, float* out, uint32_t n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    k_grad_to_float<<<blocks, 256, 0, s>>>(g, out, n);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(const TraceArgs& a, const float4* dldi, const float4* linear, double* grad, uint32_t nm,
                           int tie, int bvh, cudaStream_t s)
{
    AdjArgs g{dldi, linear, grad, nm, (6 * (size_t)nm + 3) * 8 <= 96 * 1024 ? 1 : 0};
    const bool cam = a.sc.ne > 0;
    if (tie == TIE_REFERENCE) return cam ? adj_t<TIE_REFERENCE, false, true>(a, g, s) : adj_t<TIE_REFERENCE, false, false>(a, g, s);
    if (bvh) return cam ? adj_t<TIE_STRICT, true, true>(a, g, s) : adj_t<TIE_STRICT, true, false>(a, g, s);
    return cam ? adj_t<TIE_STRICT, false, true>(a, g, s) : adj_t<TIE_STRICT, false, false>(a, g, s);
}

}  // namespace vkt
