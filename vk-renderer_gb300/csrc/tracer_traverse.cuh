// Per-lane BVH traversal pieces shared by the wavefront kernels (the extend
// kernel's lanes, the forward and adjoint finishing kernels): the encoded
// child references, strict-tie acceptance, a lane's traversal state, the
// shared-memory stack, the plane scan, primitive tests, and one thread's
// closest hit over the pre-encoded BVHs.
#pragma once

#include "tracer_core.cuh"

namespace vkt {

// The traversal reads the binary BVH with each record's child reference
// encoded at upload (bmin.w): interior -> index of its children pair (>= 1),
// leaf -> -1 - ((first << 6) | (count - 1)).
__device__ __forceinline__ void leaf_dec(int enc, int& first, int& count)
{
    const int v = -1 - enc;
    first = v >> 6;
    count = (v & 63) + 1;
}

// Strict-tie acceptance without a separate tmax: the running best starts as
// (t = tmax, prim = 0), so a candidate at exactly tmax fails the id test and
// every candidate must satisfy t < tmax, as accept<TIE_STRICT> requires.
__device__ __forceinline__ bool accept_strict(float t, uint32_t id, const Hit& h)
{
    return (t > EPSILON) && ((t < h.t) || (t == h.t && id < h.prim));
}

struct Lane {
    V3 o, d;
    BoxRay br;
    Hit h;
    const float4* nodes;  // BVH of the current pass
    const float4* prims;  // its primitives (triangles or sphere centres/radii)
    int cur, sp, pass;  // cur: node pair to visit (> 0), leaf (< 0) or none (0)
    uint32_t pid, scene, steps;
    bool has;
};

// Planes after the BVHs (unbounded; scanned linearly, Tracer.comp:414-428).
template <bool STATS>
__device__ __forceinline__ void planes_pass(const DevScene& sc, const Ray& ray, Hit& h, Counters& cnt)
{
    for (uint32_t i = 0; i < sc.np; ++i) {
        if (STATS) cnt.c[C_PLANES]++;
        const float4 q = __ldg(sc.planes + 4 * (size_t)i + 3);
        const float tt = plane_intersect(ray, v3(q), q.w);
        const uint32_t id = sc.nt + sc.ns + i;
        if (accept_strict(tt, id, h)) {
            h.t = tt;
            h.prim = id;
            h.kind = 3;
            h.slot = i;
        }
    }
}

// The traversal stack in shared memory: one 8-byte entry (child reference,
// entry distance) per level, lanes interleaved (entry k of thread t at
// k * stride + t), so a push or a pop is one access.
struct PairStack {
    int2* e;
    int stride, cap;
};

__device__ __forceinline__ int pop(Lane& L, const PairStack& stk)
{
    const float limit = L.h.t * BOX_SLACK;
    while (L.sp > 0) {
        --L.sp;
        const int2 v = stk.e[L.sp * stk.stride];
        if (__int_as_float(v.y) <= limit) return v.x;
    }
    return 0;
}

__device__ __forceinline__ void push(Lane& L, const PairStack& stk, int e, float tn, int* status)
{
    if (L.sp >= stk.cap) {
        atomicCAS(status, ST_OK, ST_STACK_OVERFLOW);
        return;
    }
    stk.e[L.sp * stk.stride] = make_int2(e, __float_as_int(tn));
    ++L.sp;
}

// Tests primitive `slot` of the current pass (scene sc) for the lane's ray.
template <bool STATS>
__device__ __forceinline__ void test_prim_sc(const DevScene& sc, Lane& L, const Ray& ray, int slot, Counters& cnt)
{
    if (L.pass == 0) {
        if (STATS) cnt.c[C_TRIS]++;
        const float4* t = L.prims + 3 * (size_t)slot;
        const float4 ta = __ldg(t), tb = __ldg(t + 1), tc = __ldg(t + 2);
        const float tt = tri_intersect(ray, v3(ta), v3(tb), v3(tc));
        const uint32_t id = __float_as_uint(tb.w);
        if (accept_strict(tt, id, L.h)) {
            L.h.t = tt;
            L.h.prim = id;
            L.h.kind = 1;
            L.h.slot = slot;
        }
    } else {
        if (STATS) cnt.c[C_SPHERES]++;
        const float4 gg = __ldg(L.prims + slot);
        const float tt = sphere_intersect(ray, v3(gg), gg.w);
        const uint32_t id = sc.nt + __ldg(sc.sph_id + slot);
        if (accept_strict(tt, id, L.h)) {
            L.h.t = tt;
            L.h.prim = id;
            L.h.kind = 2;
            L.h.slot = slot;
        }
    }
}

// Closest hit of one ray by one thread over the pre-encoded BVHs, for the
// finishing kernels: the extend kernel's node step, leaf test and acceptance
// (strict ties) without the warp's phases -- a leaf is tested as soon as it is
// reached -- so the same hit as extend and as the plain traversal.  h.t holds
// tmax on entry; on a miss h.kind = 0 and h.prim = NO_PRIM, as Tracer::trace.
template <bool STATS>
__device__ __forceinline__ bool closest_enc(const DevScene& sc, const Ray& ray, Hit& h, const PairStack& stk,
                                            int* status, uint32_t trav_limit, Counters& cnt)
{
    if (STATS) cnt.c[C_CLOSEST]++;
    Lane L;
    L.h.t = h.t;
    L.h.prim = 0;  // see accept_strict
    L.h.kind = 0;
    L.h.slot = 0;
    if (!isnan3(ray.d)) {
        L.br = make_boxray(ray);
        for (int pass = 0; pass < 2; ++pass) {
            const bool any = pass == 0 ? (sc.n_tri_nodes > 0 && sc.nt > 0) : (sc.n_sph_nodes > 0 && sc.ns > 0);
            if (!any) continue;
            L.pass = pass;
            L.prims = pass == 0 ? sc.tri : sc.sph_geo;
            L.nodes = pass == 0 ? sc.tri_enc : sc.sph_enc;
            L.sp = 0;
            uint32_t steps = 0;
            float4 rlo, rhi;
            ldg256(L.nodes, rlo, rhi);
            if (STATS) cnt.c[C_NODES]++;
            float tn;
            int cur = box_hit(L.br, rlo, rhi, L.h.t, tn) ? __float_as_int(rlo.w) : 0;
            while (cur != 0) {
                if (cur < 0) {
                    int first, count;
                    leaf_dec(cur, first, count);
                    for (int k = 0; k < count; ++k) test_prim_sc<STATS>(sc, L, ray, first + k, cnt);
                    cur = pop(L, stk);
                    continue;
                }
                if (++steps > trav_limit) {
                    atomicCAS(status, ST_OK, ST_TRAVERSAL_LIMIT);
                    break;
                }
                const float4* c = L.nodes + 2 * (size_t)cur;
                float4 lo0, hi0, lo1, hi1;
                ldg256(c, lo0, hi0);
                ldg256(c + 2, lo1, hi1);
                if (STATS) cnt.c[C_NODES] += 2;
                float t0, t1;
                const bool h0 = box_hit(L.br, lo0, hi0, L.h.t, t0);
                const bool h1 = box_hit(L.br, lo1, hi1, L.h.t, t1);
                if (!h0 && !h1) {
                    cur = pop(L, stk);
                } else {
                    const bool swap = h1 && (!h0 || t1 < t0);
                    const int e0 = __float_as_int(lo0.w), e1 = __float_as_int(lo1.w);
                    cur = swap ? e1 : e0;
                    if (h0 && h1) push(L, stk, swap ? e0 : e1, swap ? t0 : t1, status);
                }
            }
        }
        planes_pass<STATS>(sc, ray, L.h, cnt);
    }
    h = L.h;
    if (h.kind == 0) {
        h.prim = NO_PRIM;
        return false;
    }
    if (STATS) cnt.c[C_HITS]++;
    return true;
}

}  // namespace vkt
