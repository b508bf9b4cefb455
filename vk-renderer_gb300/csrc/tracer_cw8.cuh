// Device side of the compressed 8-wide BVH (layout: bvh_cw8.h): one node's
// eight quantised slab tests and the node groups a traversal keeps.
//
// A node group is (child_base, remaining hit interior children << 24 | imask):
// bit 24 + (k ^ s ^ 7) stands for slot k (s = the ray's direction octant), so
// the highest set bit is the next child to visit and slot k's node index is
// child_base + popc(imask & ((1 << k) - 1)).  A primitive group is
// (prim_base, bit i = primitive prim_base + i still to test).
#pragma once

#include "tracer_traverse.cuh"

namespace vkt {

// The ray's quantities for the 8-wide slab test: the direction octant and,
// per axis, the slab planes' order (near plane = low bound for a
// non-negative inverse direction).
struct Cw8Ray {
    BoxRay br;
    uint32_t oct7;  // (octant s) ^ 7
};

__device__ __forceinline__ Cw8Ray make_cw8ray(const Ray& r)
{
    Cw8Ray c;
    c.br = make_boxray(r);
    const uint32_t s = (c.br.ix < 0.0f ? 1u : 0u) | (c.br.iy < 0.0f ? 2u : 0u) | (c.br.iz < 0.0f ? 4u : 0u);
    c.oct7 = s ^ 7u;
    return c;
}

// Byte k of w as a float (exact).  An integer-to-float conversion: the
// kernel's busiest pipe is the integer ALU (58 % in ncu), and the
// conversion's pipe is another one; a byte permute into 2^23 + b minus 2^23
// (ALU + FMA) measured slower on c1 (71.8 against 69.1 ms per frame), and so
// did a conversion of the low byte of the shifted word (cvt.rn.f32.u8: 61.8
// against 60.4).
__device__ __forceinline__ float ubyte_f(uint32_t w, int k)
{
    return __uint2float_rn((w >> (8 * k)) & 0xFFu);
}

// Visits node `idx`: tests its children's boxes against the ray with the
// current best distance tbest and returns the node group of the interior
// children hit (G) and the primitive group of the leaf children hit (P).
// Each box is [p + q_lo * step, p + q_hi * step] per axis, which contains
// the binary child's padded box; the slab distances are
// fma(q, step * ix, fma(p, ix, -o * ix)), and a child is hit iff
// max(near distances, 0) <= min(far distances, tbest) * (1 + 2^-20): the
// binary test's acceptance, on a box that contains the binary box, so every
// box the binary traversal enters is entered here too.
__device__ __forceinline__ void cw8_visit(const float4* nodes, uint32_t idx, const Cw8Ray& r, float tbest, uint2& G,
                                          uint2& P)
{
    uint32_t a[8], b[8], c[8];
    const float4* n = nodes + 6 * (size_t)idx;
    ldg256u(n, a);
    ldg256u(n + 2, b);
    ldg256u(n + 4, c);
    const float px = __uint_as_float(a[0]), py = __uint_as_float(a[1]), pz = __uint_as_float(a[2]);
    const float sx = __uint_as_float((a[3] & 0xFFu) << 23);
    const float sy = __uint_as_float(((a[3] >> 8) & 0xFFu) << 23);
    const float sz = __uint_as_float(((a[3] >> 16) & 0xFFu) << 23);
    const float ax = sx * r.br.ix, ay = sy * r.br.iy, az = sz * r.br.iz;
    const float bx = __fmaf_rn(px, r.br.ix, r.br.nx);
    const float by = __fmaf_rn(py, r.br.iy, r.br.ny);
    const float bz = __fmaf_rn(pz, r.br.iz, r.br.nz);
    // near / far plane words per axis (two words = eight slots)
    const bool fx = r.br.ix < 0.0f, fy = r.br.iy < 0.0f, fz = r.br.iz < 0.0f;
    // b = w8..w15: lo x (b0, b1), lo y (b2, b3), lo z (b4, b5), hi x (b6, b7)
    // c = w16..w23: hi y (c0, c1), hi z (c2, c3), bits (c4, c5), positions (c6, c7)
    const uint32_t lox[2] = {b[0], b[1]}, loy[2] = {b[2], b[3]}, loz[2] = {b[4], b[5]};
    const uint32_t hix[2] = {b[6], b[7]}, hiy[2] = {c[0], c[1]}, hiz[2] = {c[2], c[3]};
    const uint32_t oct4 = r.oct7 * 0x01010101u;
    uint32_t mask = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t qnx = fx ? hix[h] : lox[h], qfx = fx ? lox[h] : hix[h];
        const uint32_t qny = fy ? hiy[h] : loy[h], qfy = fy ? loy[h] : hiy[h];
        const uint32_t qnz = fz ? hiz[h] : loz[h], qfz = fz ? loz[h] : hiz[h];
        const uint32_t bits4 = c[4 + h];
        const uint32_t pos4 = c[6 + h] ^ (oct4 & a[6 + h]);  // interior children: slot ^ s ^ 7
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float tnx = __fmaf_rn(ubyte_f(qnx, k), ax, bx);
            const float tny = __fmaf_rn(ubyte_f(qny, k), ay, by);
            const float tnz = __fmaf_rn(ubyte_f(qnz, k), az, bz);
            const float tfx = __fmaf_rn(ubyte_f(qfx, k), ax, bx);
            const float tfy = __fmaf_rn(ubyte_f(qfy, k), ay, by);
            const float tfz = __fmaf_rn(ubyte_f(qfz, k), az, bz);
            const float tmin = fmaxf(fmax3(tnx, tny, tnz), 0.0f);
            const float tmax = fminf(fmin3(tfx, tfy, tfz), tbest);
            if (tmin <= tmax * BOX_SLACK)
                mask |= __byte_perm(bits4, 0u, 0x4440u | (uint32_t)k) << __byte_perm(pos4, 0u, 0x4440u | (uint32_t)k);
        }
    }
    G = make_uint2(a[4], (mask & 0xFF000000u) | (a[3] >> 24));
    P = make_uint2(a[5], mask & 0x00FFFFFFu);
}

// Takes the next child of a node group (which has one): its node index; the
// group keeps the others.
__device__ __forceinline__ uint32_t cw8_next(uint2& G, uint32_t oct7)
{
    const int bit = 31 - __clz(G.y);
    const uint32_t slot = (uint32_t)(bit - 24) ^ oct7;
    G.y &= ~(1u << bit);
    return G.x + __popc(G.y & ((1u << slot) - 1u) & 0xFFu);
}

// Tests primitive k of the 8-wide order: a 64-byte record
// (v0, original id) (v1 - v0, leaf-ordered slot) (v2 - v0, 0) (0), read as a
// 256-bit and a 128-bit load (the last 16 bytes are padding); on acceptance
// the hit records the leaf-ordered slot (the storage slot every other kernel
// indexes).
__device__ __forceinline__ float cw8_tri(const float4* tris, uint32_t k, const Ray& ray, uint32_t& id, uint32_t& slot)
{
    float4 ta, tb;
    ldg256(tris + 4 * (size_t)k, ta, tb);
    const float4 tc = __ldg(tris + 4 * (size_t)k + 2);
    id = __float_as_uint(ta.w);
    slot = __float_as_uint(tb.w);
    return tri_intersect(ray, v3(ta), v3(tb), v3(tc));
}

template <bool STATS>
__device__ __forceinline__ void cw8_test_tri(const float4* tris, uint32_t k, const Ray& ray, Hit& h, Counters& cnt)
{
    if (STATS) cnt.c[C_TRIS]++;
    uint32_t id, slot;
    const float tt = cw8_tri(tris, k, ray, id, slot);
    if (accept_strict(tt, id, h)) {
        h.t = tt;
        h.prim = id;
        h.kind = 1;
        h.slot = slot;
    }
}

// Tests primitives k0 and, if two, k1: both records are fetched before
// either test, so the two L2 round trips overlap.
template <bool STATS>
__device__ __forceinline__ void cw8_test_tri2(const float4* tris, uint32_t k0, uint32_t k1, bool two, const Ray& ray,
                                              Hit& h, Counters& cnt)
{
    if (STATS) cnt.c[C_TRIS] += two ? 2 : 1;
    float4 a0, b0, a1, b1;
    ldg256(tris + 4 * (size_t)k0, a0, b0);
    const float4 c0 = __ldg(tris + 4 * (size_t)k0 + 2);
    const uint32_t k = two ? k1 : k0;
    ldg256(tris + 4 * (size_t)k, a1, b1);
    const float4 c1 = __ldg(tris + 4 * (size_t)k + 2);
    const float t0 = tri_intersect(ray, v3(a0), v3(b0), v3(c0));
    const float t1 = tri_intersect(ray, v3(a1), v3(b1), v3(c1));
    if (accept_strict(t0, __float_as_uint(a0.w), h)) {
        h.t = t0;
        h.prim = __float_as_uint(a0.w);
        h.kind = 1;
        h.slot = __float_as_uint(b0.w);
    }
    if (two && accept_strict(t1, __float_as_uint(a1.w), h)) {
        h.t = t1;
        h.prim = __float_as_uint(a1.w);
        h.kind = 1;
        h.slot = __float_as_uint(b1.w);
    }
}

// Position of the n-th (from 0) set bit of m, which has more than n.
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t n)
{
    for (; n != 0u; --n) m &= m - 1u;
    return (uint32_t)(__ffs(m) - 1);
}

// Per-lane record of the shared primitive phase, in shared memory: what the
// other lanes of the warp need to test this lane's primitives for it.
struct alignas(16) Cw8Share {
    float4 o, d;               // the ray
    unsigned long long best;   // (distance bits << 32) | id of the best hit so far
    const float4* tris;        // the lane's scene's primitives (8-wide order)
    uint32_t excl, first;      // the lane's first item in the warp's order, its first group entry
    uint32_t slot, pad;        // storage slot of the hit that set `best`
};
static_assert(sizeof(Cw8Share) == 64, "shared record is 64 bytes");

// (distance, id) as one integer that orders like the strict (t, id) order
// for non-negative distances (their bit patterns order like their values).
__device__ __forceinline__ unsigned long long hit_key(float t, uint32_t id)
{
    return ((unsigned long long)__float_as_uint(t) << 32) | id;
}

// Position of the n-th (from 0) set bit of m, which has more than n: popc
// bisection, a fixed number of steps.
__device__ __forceinline__ uint32_t nth_bit32(uint32_t m, uint32_t n)
{
    uint32_t pos = 0;
#pragma unroll
    for (int w = 16; w >= 2; w >>= 1) {
        const uint32_t c = (uint32_t)__popc(m & ((1u << w) - 1u));
        if (n >= c) {
            n -= c;
            pos += (uint32_t)w;
            m >>= w;
        }
    }
    return pos + ((n >= (m & 1u)) ? 1u : 0u);
}

// The warp's remaining held primitives, shared out over all 32 lanes: item i
// of the warp (lanes' items in lane order, each lane's in group and bit
// order) is tested by lane i % 32 in step i / 32.  Each lane with items
// publishes its ray, primitive array, best hit and item offset in its
// Cw8Share record; a step's lanes find their owners from a ballot of the
// owners with items in the step and the step's segment starts, fetch the
// owner's ray from its record, and lower the owner's best (distance, id) key
// with a shared-memory atomic minimum (a candidate counts when distance >
// EPSILON; min over the keys is the strict-ties order, so the owner ends with
// the hit it would get testing every item itself, in any order); the lane
// whose candidate is the minimum after the step records its slot.  Every
// lane of the warp calls this (warp-synchronous).
//   held: the calling lane's group entries (entry g at held[g * stride]),
//   readable by the other lanes of the warp; sh: the calling lane's record
//   (the warp's lanes' records adjacent); rest: the lane has items left:
//   `cur` (its group in progress, taken from entry j - 1) and entries
//   j .. nh - 1.
template <bool STATS>
__device__ __forceinline__ void cw8_warp_prims(const float4* tris, uint2* held, Cw8Share* sh, int stride, int lane,
                                               bool rest, uint2 cur, int j, int nh, const Ray& ray, Hit& h,
                                               Counters& cnt)
{
    const unsigned full = 0xFFFFFFFFu;
    int first = j;
    uint32_t r = 0;
    if (rest) {
        if (cur.y != 0u) {
            --first;  // j >= 1: cur came from entry j - 1
            held[first * stride] = cur;
        }
        for (int g = first; g < nh; ++g) r += (uint32_t)__popc(held[g * stride].y);
    }
    uint32_t incl = r;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(full, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t excl = incl - r;
    const uint32_t total = __shfl_sync(full, incl, 31);
    const unsigned long long key0 = hit_key(h.t, h.prim);
    if (rest) {
        sh->o = make_float4(ray.o.x, ray.o.y, ray.o.z, 0.0f);
        sh->d = make_float4(ray.d.x, ray.d.y, ray.d.z, 0.0f);
        sh->best = key0;
        sh->tris = tris;
        sh->excl = excl;
        sh->first = (uint32_t)first;
    }
    __syncwarp();
    Cw8Share* const wsh = sh - lane;
    for (uint32_t base = 0; base < total; base += 32u) {
        const uint32_t idx = base + (uint32_t)lane;
        // owners with items in this step, in lane order = the step's segments
        const unsigned in = __ballot_sync(full, r != 0u && excl < base + 32u && incl > base);
        const unsigned starts =
            __reduce_or_sync(full, (r != 0u && excl >= base && excl < base + 32u) ? 1u << (excl - base) : 0u);
        unsigned long long key = ~0ull;
        Cw8Share* osh = wsh;
        uint32_t slot = 0;
        if (idx < total) {
            // segment of this lane: starts at or before it, plus one if the
            // step opens inside an earlier owner's items
            const unsigned upto = lane == 31 ? starts : (starts & ((2u << lane) - 1u));
            const uint32_t n = (uint32_t)__popc(upto) - 1u + ((starts & 1u) ? 0u : 1u);
            const int o = (int)nth_bit32(in, n);
            osh = wsh + o;
            uint32_t rank = idx - osh->excl;
            const uint2* hg = held + (o - lane);
            int g = (int)osh->first;
            uint2 grp = hg[g * stride];
            uint32_t c = (uint32_t)__popc(grp.y);
            while (rank >= c) {
                rank -= c;
                ++g;
                grp = hg[g * stride];
                c = (uint32_t)__popc(grp.y);
            }
            if (STATS) cnt.c[C_TRIS]++;
            const Ray ro{v3(osh->o), v3(osh->d)};
            uint32_t tid;
            const float tt = cw8_tri(osh->tris, grp.x + nth_set_bit(grp.y, rank), ro, tid, slot);
            if (tt > EPSILON) {
                key = hit_key(tt, tid);
                atomicMin(&osh->best, key);
            }
        }
        __syncwarp();
        if (key != ~0ull && key == *reinterpret_cast<volatile unsigned long long*>(&osh->best)) osh->slot = slot;
        __syncwarp();
    }
    if (rest) {
        const unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&sh->best);
        if (k != key0) {
            h.t = __uint_as_float((uint32_t)(k >> 32));
            h.prim = (uint32_t)k;
            h.kind = 1;
            h.slot = *reinterpret_cast<volatile uint32_t*>(&sh->slot);
        }
    }
    __syncwarp();
}

// Closest hit of one ray by one thread over the 8-wide BVH of a
// triangle-only scene, for the finishing kernel: the extend kernel's node
// visit and triangle test (strict ties), without the warp's phases -- a
// node's leaves are tested right after the visit -- so the same hit.  h.t
// holds tmax on entry; on a miss h.kind = 0 and h.prim = NO_PRIM.  stk: the
// thread's stack of node groups (8-byte entries, interleaved by thread).
template <bool STATS>
__device__ __forceinline__ bool closest_cw8(const DevScene& sc, const Ray& ray, Hit& h, const PairStack& stk,
                                            int* status, uint32_t trav_limit, Counters& cnt)
{
    if (STATS) cnt.c[C_CLOSEST]++;
    Hit b;
    b.t = h.t;
    b.prim = 0;  // see accept_strict
    b.kind = 0;
    b.slot = 0;
    if (!isnan3(ray.d)) {
        if (sc.n_tri_nodes > 0 && sc.nt > 0) {
            const Cw8Ray cr = make_cw8ray(ray);
            uint2 G = make_uint2(0u, (1u << (24 + (0u ^ cr.oct7))) | 1u);
            int sp = 0;
            uint32_t steps = 0;
            for (;;) {
                if ((G.y & 0xFF000000u) == 0u) {
                    if (sp == 0) break;
                    --sp;
                    const int2 e = stk.e[sp * stk.stride];
                    G = make_uint2((uint32_t)e.x, (uint32_t)e.y);
                }
                if (++steps > trav_limit) {
                    atomicCAS(status, ST_OK, ST_TRAVERSAL_LIMIT);
                    break;
                }
                const uint32_t idx = cw8_next(G, cr.oct7);
                if (G.y & 0xFF000000u) {
                    if (sp >= stk.cap) {
                        atomicCAS(status, ST_OK, ST_STACK_OVERFLOW);
                    } else {
                        stk.e[sp * stk.stride] = make_int2((int)G.x, (int)G.y);
                        ++sp;
                    }
                }
                uint2 P;
                cw8_visit(sc.tri_cw8, idx, cr, b.t, G, P);
                if (STATS) cnt.c[C_NODES] += 3;
                for (uint32_t m = P.y; m != 0u; m &= m - 1u)
                    cw8_test_tri<STATS>(sc.tri_cw8_prims, P.x + (uint32_t)(__ffs(m) - 1), ray, b, cnt);
            }
        }
        planes_pass<STATS>(sc, ray, b, cnt);
    }
    h = b;
    if (h.kind == 0) {
        h.prim = NO_PRIM;
        return false;
    }
    if (STATS) cnt.c[C_HITS]++;
    return true;
}

}  // namespace vkt
