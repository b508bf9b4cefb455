// Wavefront path tracing for sm_103a: the radiance loop of Assets/Tracer.comp
// split into stages that each run as their own kernel over a queue of live
// paths, one path per pixel.
//
//   wf_generate  seeds every pixel's RNG (Tracer.comp:563-566), writes its
//                primary ray (:568-574) and queues all pixels.
//   wf_extend    persistent warps trace the queued rays (trace_ray,
//                :374-431).  Each lane owns one ray at a time and takes the
//                next ray from the queue as soon as its ray is finished
//                (warp-aggregated fetch: ballot + popc + one atomicAdd).
//                BVH traversal is the speculative while-while scheme: all
//                lanes step through interior nodes together, each holding
//                back up to four leaves it finds, then all test their held
//                leaves together, one primitive per lane and step; stacks
//                and held leaves live in shared memory.  Small register
//                footprint, so many warps per SM hide the L1/L2 latency of
//                node fetches.
//   wf_shade     one thread per queued path: the rest of the depth iteration
//                (:441-549: clamp, sky, scatter, next-event estimation, Russian
//                roulette).  A surviving path appends itself to the next queue
//                (warp-aggregated atomics = warp-level ray compaction); a
//                finished sample starts the pixel's next sample, whose RNG
//                continues where the last one stopped (the shader's rand_salt
//                runs across samples, :578-581); a finished pixel is resolved
//                (:585-592).
//   wf_finish    for the last rounds, when few paths are live: each thread
//                runs queued paths to the end of their pixels (all remaining
//                bounces and samples), without per-round launches.
//
// MULTI = true runs many scenes of different size and resolution in the same
// queues (the batched form): every path slot belongs to one scene, whose
// TraceArgs (scene pointers into one device arena, camera, image size,
// parameters, output pointers) live in a device table.
//
// Per pixel the operations are exactly those of the plain kernel, in the same
// order, so images and hits are identical to it and to the oracle.  Only the
// order of node visits inside one ray's traversal differs (it depends on the
// warp), which changes no result under strict ties but does change the node
// counters.

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_cw8.cuh"
#include "tracer_traverse.cuh"
#include "tracer_wavefront.h"

namespace vkt {

// The TraceArgs a path belongs to: the launch's own (single scene) or its
// scene's entry in the table (batched).
#define SCENE_ARGS(MULTI, a, slots, sid) ((MULTI) ? (slots)[(sid)] : (a))

// ---------------------------------------------------------------- generate --
template <bool MULTI>
__global__ void __launch_bounds__(256) wf_generate(TraceArgs a, WfState s, const TraceArgs* slots, uint32_t nslots)
{
    const uint32_t n = a.num_slots;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        s.count[0] = n;
        s.count[1] = 0;
        s.count[2] = 0;
    }
    if (i >= n) return;
    uint32_t sid = 0;
    if (MULTI) {  // the scene whose slot range holds i: last pixel_base <= i
        uint32_t lo = 0, hi = nslots;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (slots[mid].pixel_base <= i)
                lo = mid;
            else
                hi = mid;
        }
        sid = lo;
        s.scene_of[i] = sid;
    }
    const TraceArgs& A = SCENE_ARGS(MULTI, a, slots, sid);
    const uint32_t p = i - A.pixel_base;
    const uint32_t x = p % A.width, y = p / A.width;
    Rng g;
    seed_rng(A, x, y, g);
    const Ray r = primary_ray(A, x, y);
    s.ray_o[i] = make_float4(r.o.x, r.o.y, r.o.z, depth_tmax(0));
    s.ray_d[i] = make_float4(r.d.x, r.d.y, r.d.z, 0.0f);
    s.acc[i] = make_float4(0.0f, 0.0f, 0.0f, g.salt);
    s.mask[i] = make_float4(1.0f, 1.0f, 1.0f, -1.0f);
    s.accum[i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0u));
    s.prim0[i] = NO_PRIM;
    s.queue[0][i] = i;
}

// ------------------------------------------------------------------ extend --
__device__ __forceinline__ void order2(float& ta, int& ra, float& tb, int& rb)
{
    if (tb < ta) {
        const float t = ta;
        ta = tb;
        tb = t;
        const int r = ra;
        ra = rb;
        rb = r;
    }
}

// One 4-wide node: the slab test of each child's box (the binary node's box,
// the same test as box_hit), the nearest child hit becomes the next
// reference, the others are pushed farthest first.  Which boxes are tested
// differs from the binary traversal only in order and in skipping interior
// boxes, so the closest hit under strict ties is the same.
template <bool STATS>
__device__ __forceinline__ void visit_wide(Lane& L, int w, const PairStack& stk, int* status, Counters& cnt)
{
    // node = four (box min, reference) (box max, 0) records
    const float4* n = L.nodes + 8 * (size_t)w;
    const float INF = __int_as_float(0x7f800000);
    float t0, t1, t2, t3;
    int r0, r1, r2, r3;
    auto child = [&](int k, float& t, int& r) {
        const float4 lo = __ldg(n + 2 * k), hi = __ldg(n + 2 * k + 1);
        r = __float_as_int(lo.w);
        if (STATS) cnt.c[C_NODES] += r != 0;
        if (!(r != 0 && box_hit(L.br, lo, hi, L.h.t, t))) {
            t = INF;
            r = 0;
        }
    };
    child(0, t0, r0);
    child(1, t1, r1);
    child(2, t2, r2);
    child(3, t3, r3);
    // sorting network: ascending distance (misses last)
    order2(t0, r0, t1, r1);
    order2(t2, r2, t3, r3);
    order2(t0, r0, t2, r2);
    order2(t1, r1, t3, r3);
    order2(t1, r1, t2, r2);
    if (r3) push(L, stk, r3, t3, status);
    if (r2) push(L, stk, r2, t2, status);
    if (r1) push(L, stk, r1, t1, status);
    L.cur = r0 ? r0 : pop(L, stk);
}

// Leaves a lane may hold back while the warp's slowest lane is still looking
// for its first (measured on c1: 2 -> 95.8 ms, 4 -> 91.0, 6 -> 91.0, 8 -> 91.2).
constexpr int kPostpone = 4;

// Moves leaf references from L.cur into the lane's buffer of postponed leaves
// (entry j at lbuf[j * stride]), taking the next stack entry after each,
// until L.cur is an interior node or empty or the buffer is full.
__device__ __forceinline__ void postpone_leaves(Lane& L, const PairStack& stk, int* lbuf, int stride, int& nl)
{
    while (L.cur < 0 && nl < kPostpone) {
        lbuf[nl * stride] = L.cur;
        ++nl;
        L.cur = pop(L, stk);
    }
}

template <bool STATS, bool WIDE>
__device__ __forceinline__ void start_pass(const DevScene& sc, Lane& L, Counters& cnt, const PairStack& stk,
                                           int* lbuf, int stride, int& nl, int* status)
{
    L.prims = L.pass == 0 ? sc.tri : sc.sph_geo;
    L.sp = 0;
    if (WIDE) {
        L.nodes = L.pass == 0 ? sc.tri_wide : sc.sph_wide;
        visit_wide<STATS>(L, 0, stk, status, cnt);
    } else {
        L.nodes = L.pass == 0 ? sc.tri_enc : sc.sph_enc;  // references pre-encoded in bmin.w
        float4 lo, hi;
        ldg256(L.nodes, lo, hi);
        if (STATS) cnt.c[C_NODES]++;
        float tn;
        L.cur = box_hit(L.br, lo, hi, L.h.t, tn) ? __float_as_int(lo.w) : 0;  // the root may be a leaf
    }
    postpone_leaves(L, stk, lbuf, stride, nl);
}

// Tests primitive `slot` of the current pass for the lane's ray.
template <bool STATS, bool MULTI>
__device__ __forceinline__ void test_prim(const TraceArgs& a, const TraceArgs* slots, Lane& L, const Ray& ray,
                                          int slot, Counters& cnt)
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
        const DevScene& sc = SCENE_ARGS(MULTI, a, slots, L.scene).sc;
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

// 1024 resident threads per SM (63 registers).  Each outer iteration: idle
// lanes fetch rays; all lanes step through interior nodes until every lane
// still tracing holds a leaf, lanes that already hold some keep going (up to
// kPostpone leaves, speculatively: their best hit is not yet updated by
// them); then all lanes test their held leaves' primitives, one primitive per
// lane and iteration.
template <int TIE, bool STATS, bool MULTI, int BLOCK, bool WIDE>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK)
    wf_extend_bvh(TraceArgs a, WfState s, int qsel, const TraceArgs* slots)
{
    extern __shared__ int smem[];
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const PairStack stk{reinterpret_cast<int2*>(smem) + threadIdx.x, BLOCK, (int)a.stack_depth};
    int* lbuf = smem + 2 * (size_t)a.stack_depth * BLOCK + threadIdx.x;  // postponed leaves, stride BLOCK
    const uint32_t total = s.count[qsel];
    const uint32_t* queue = qsel ? s.queue[1] : s.queue[0];
    if (blockIdx.x == 0 && threadIdx.x == 0) s.count[qsel ^ 1] = 0;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    Lane L;
    L.has = false;
    int nl = 0;  // postponed leaves held
    bool exhausted = false;
    for (;;) {
        // 1) idle lanes take the next rays of the queue
        const unsigned need = __ballot_sync(full, !L.has && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&s.count[2], (uint32_t)__popc(need));
            base = __shfl_sync(full, base, leader);
            if (!L.has && !exhausted) {
                const uint32_t qi = base + __popc(need & ((1u << lane) - 1u));
                if (qi >= total) {
                    exhausted = true;
                } else {
                    L.pid = queue[qi];
                    L.scene = MULTI ? s.scene_of[L.pid] : 0;
                    const DevScene& sc = SCENE_ARGS(MULTI, a, slots, L.scene).sc;
                    const float4 ro = s.ray_o[L.pid];
                    const float4 rd = s.ray_d[L.pid];
                    L.o = v3(ro);
                    L.d = v3(rd);
                    L.h.t = ro.w;
                    L.h.prim = 0;  // see accept_strict
                    L.h.kind = 0;
                    L.h.slot = 0;
                    L.steps = 0;
                    if (STATS) cnt.c[C_CLOSEST]++;
                    L.has = true;
                    const bool has_tri = sc.n_tri_nodes > 0 && sc.nt > 0;
                    const bool has_sph = sc.n_sph_nodes > 0 && sc.ns > 0;
                    if (isnan3(L.d) || (!has_tri && !has_sph)) {
                        // no BVH work: NaN directions hit nothing; planes only
                        if (!isnan3(L.d)) planes_pass<STATS>(sc, Ray{L.o, L.d}, L.h, cnt);
                        if (STATS && L.h.kind) cnt.c[C_HITS]++;
                        s.hit[L.pid] = make_uint4(__float_as_uint(L.h.t), L.h.prim, L.h.slot, (uint32_t)L.h.kind);
                        L.has = false;
                    } else {
                        L.br = make_boxray(Ray{L.o, L.d});
                        L.pass = has_tri ? 0 : 1;
                        start_pass<STATS, WIDE>(sc, L, cnt, stk, lbuf, BLOCK, nl, a.status);
                    }
                }
            }
        }
        if (!__any_sync(full, L.has)) {
            if (__all_sync(full, exhausted)) break;
            continue;
        }
        // 2) interior nodes, until every lane still tracing holds a leaf
        for (;;) {
            const bool can = L.has && L.cur > 0 && nl < kPostpone;
            if (!__any_sync(full, can && nl == 0)) break;
            if (can) {
                if (++L.steps > a.trav_limit) {
                    atomicCAS(a.status, ST_OK, ST_TRAVERSAL_LIMIT);
                    L.cur = 0;
                    L.sp = 0;
                } else if (WIDE) {
                    visit_wide<STATS>(L, L.cur, stk, a.status, cnt);
                } else {
                    const float4* c = L.nodes + 2 * (size_t)L.cur;
                    float4 lo0, hi0, lo1, hi1;
                    ldg256(c, lo0, hi0);
                    ldg256(c + 2, lo1, hi1);
                    if (STATS) cnt.c[C_NODES] += 2;
                    float t0, t1;
                    const bool h0 = box_hit(L.br, lo0, hi0, L.h.t, t0);
                    const bool h1 = box_hit(L.br, lo1, hi1, L.h.t, t1);
                    const int e0 = __float_as_int(lo0.w), e1 = __float_as_int(lo1.w);
                    if (!h0 && !h1) {
                        L.cur = pop(L, stk);
                    } else {
                        const bool swap = h1 && (!h0 || t1 < t0);
                        L.cur = swap ? e1 : e0;
                        if (h0 && h1) push(L, stk, swap ? e0 : e1, swap ? t0 : t1, a.status);
                    }
                }
                postpone_leaves(L, stk, lbuf, BLOCK, nl);
            }
        }
        // 3) the held leaves, one primitive per lane and iteration
        {
            int lj = 0, lfirst = 0, lcount = 0;
            const Ray ray{L.o, L.d};
            for (;;) {
                const bool lf = L.has && (lcount > 0 || lj < nl);
                if (!__any_sync(full, lf)) break;
                if (lf) {
                    if (lcount == 0) {
                        leaf_dec(lbuf[lj * BLOCK], lfirst, lcount);
                        ++lj;
                    }
                    test_prim<STATS, MULTI>(a, slots, L, ray, lfirst, cnt);
                    ++lfirst;
                    --lcount;
                }
            }
        }
        nl = 0;
        if (L.has) postpone_leaves(L, stk, lbuf, BLOCK, nl);  // a leaf met with the buffer full
        // 4) finished passes: next primitive kind, or planes and the result
        if (L.has && L.cur == 0 && nl == 0) {
            const DevScene& sc = SCENE_ARGS(MULTI, a, slots, L.scene).sc;
            if (L.pass == 0 && sc.n_sph_nodes > 0 && sc.ns > 0) {
                L.pass = 1;
                start_pass<STATS, WIDE>(sc, L, cnt, stk, lbuf, BLOCK, nl, a.status);
            } else {
                planes_pass<STATS>(sc, Ray{L.o, L.d}, L.h, cnt);
                if (STATS && L.h.kind) cnt.c[C_HITS]++;
                s.hit[L.pid] = make_uint4(__float_as_uint(L.h.t), L.h.prim, L.h.slot, (uint32_t)L.h.kind);
                L.has = false;
            }
        }
    }
    if (STATS) flush_counters(a, cnt);
}

// Primitive groups a lane of the 8-wide traversal may hold back while the
// warp's slowest lane is still looking for its first (c1 frame, ms: 1 ->
// 100.8, 2 -> 69.1, 4 -> 61.1, 6 -> 60.9, 8 -> 61.1, 12 -> 63.1; with the
// shared primitive phase below: 4 -> 61.4, 5 -> 60.6, 6 -> 60.4).  Capping
// the primitives held instead (12, 16, 20) measured 61.3-63.1.
constexpr int kCw8Postpone = 6;

// Held primitives are tested two per lane and step while at least this many
// lanes of the warp have some left; the rest are shared out over all 32
// lanes (cw8_warp_prims).  1 = never shared, 33 = always.  c1 frame, ms:
// 1 -> 60.4, 8 -> 58.1, 12 -> 58.0, 16 -> 58.4, 24 -> 61.3, 33 -> 67.8: a
// shared step (owner look-up, the owner's ray from shared memory, an atomic
// minimum) takes longer than a sequential one, so only the tail is shared.
// (One primitive per sequential step and the owner found by shuffles
// instead: 61.4 unshared, 60.1-60.4 at 8.)
constexpr int kCw8SharedBelow = 12;
// (Lanes whose ray is done and who hold no primitives taking their next ray
// inside the node phase, rather than idling until the primitive phase ends:
// 62.6 against 57.9 ms -- the fetch in every node step costs more than the
// idle lanes.)

// The extend kernel over the compressed 8-wide BVH (triangle scenes; strict
// ties).  Same phases as wf_extend_bvh: idle lanes fetch rays; all lanes visit
// 8-wide nodes (one per lane and step: eight quantised slab tests, the hit
// interior children become a node group on the stack, the hit leaves a
// primitive group held back) until every lane still tracing holds some
// primitives, lanes that hold fewer than kCw8Postpone groups going on; then
// all lanes test their held primitives, two per lane and step (both records
// fetched before either test), the warp sharing out the last ones.  Node
// groups are visited nearest-octant first; which boxes are entered depends
// on the order, the closest hit under strict ties does not.
// 64 registers, eight 128-thread blocks per SM; bounds for 10 or 12 blocks
// (48 or 40 registers) spill 190 / 298 bytes and measured 65.7 / 75.0 ms on
// the c1 frame against 60.4.
template <bool STATS, bool MULTI, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK)
    wf_extend_cw8(TraceArgs a, WfState s, int qsel, const TraceArgs* slots)
{
    extern __shared__ int smem[];
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    // stack of node groups, then held primitive groups (entry j of a thread
    // at j * BLOCK + threadIdx.x), then the threads' shared-phase records
    uint2* stk = reinterpret_cast<uint2*>(smem) + threadIdx.x;
    uint2* held = reinterpret_cast<uint2*>(smem) + (size_t)a.stack_depth * BLOCK + threadIdx.x;
    Cw8Share* shr =
        reinterpret_cast<Cw8Share*>(reinterpret_cast<uint2*>(smem) + ((size_t)a.stack_depth + kCw8Postpone) * BLOCK) +
        threadIdx.x;
    const int cap = (int)a.stack_depth;
    const uint32_t total = s.count[qsel];
    const uint32_t* queue = qsel ? s.queue[1] : s.queue[0];
    if (blockIdx.x == 0 && threadIdx.x == 0) s.count[qsel ^ 1] = 0;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    bool has = false, exhausted = false;
    uint32_t pid = 0, scene = 0, steps = 0;
    Ray ray{};
    Cw8Ray cr{};
    Hit h{};
    uint2 G = make_uint2(0u, 0u);
    int sp = 0, nh = 0;
    const float4* nodes = nullptr;
    const float4* tris = nullptr;
    // idle lanes take the next rays of the queue (warp-aggregated: one
    // atomic per warp and call)
    auto fetch = [&]() {
        const unsigned need = __ballot_sync(full, !has && !exhausted);
        if (!need) return;
        const int leader = __ffs(need) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&s.count[2], (uint32_t)__popc(need));
        base = __shfl_sync(full, base, leader);
        if (has || exhausted) return;
        const uint32_t qi = base + __popc(need & ((1u << lane) - 1u));
        if (qi >= total) {
            exhausted = true;
            return;
        }
        pid = queue[qi];
        scene = MULTI ? s.scene_of[pid] : 0;
        const DevScene& sc = SCENE_ARGS(MULTI, a, slots, scene).sc;
        const float4 ro = s.ray_o[pid];
        const float4 rd = s.ray_d[pid];
        ray = Ray{v3(ro), v3(rd)};
        h.t = ro.w;
        h.prim = 0;  // see accept_strict
        h.kind = 0;
        h.slot = 0;
        steps = 0;
        if (STATS) cnt.c[C_CLOSEST]++;
        has = true;
        if (isnan3(ray.d) || !(sc.n_tri_nodes > 0 && sc.nt > 0)) {
            // no BVH work: NaN directions hit nothing; planes only
            if (!isnan3(ray.d)) planes_pass<STATS>(sc, ray, h, cnt);
            if (STATS && h.kind) cnt.c[C_HITS]++;
            s.hit[pid] = make_uint4(__float_as_uint(h.t), h.prim, h.slot, (uint32_t)h.kind);
            has = false;
        } else {
            cr = make_cw8ray(ray);
            nodes = sc.tri_cw8;
            tris = sc.tri_cw8_prims;
            // the root: the one interior child (slot 0) of a group of its own
            G = make_uint2(0u, (1u << (24 + (0u ^ cr.oct7))) | 1u);
            sp = 0;
        }
    };
    // a ray whose traversal is over and whose primitives are all tested:
    // planes, then its result
    auto finish_ray = [&]() {
        const DevScene& sc = SCENE_ARGS(MULTI, a, slots, scene).sc;
        planes_pass<STATS>(sc, ray, h, cnt);
        if (STATS && h.kind) cnt.c[C_HITS]++;
        s.hit[pid] = make_uint4(__float_as_uint(h.t), h.prim, h.slot, (uint32_t)h.kind);
        has = false;
    };
    for (;;) {
        // 1) idle lanes take the next rays of the queue
        fetch();
        if (!__any_sync(full, has)) {
            if (__all_sync(full, exhausted)) break;
            continue;
        }
        // 2) nodes, until every lane still tracing holds primitives
        for (;;) {
            const bool search = has && nh < kCw8Postpone && ((G.y & 0xFF000000u) != 0u || sp > 0);
            if (!__any_sync(full, search && nh == 0)) break;
            if (search) {
                if ((G.y & 0xFF000000u) == 0u) {
                    --sp;
                    G = stk[sp * BLOCK];
                }
                if (++steps > a.trav_limit) {
                    atomicCAS(a.status, ST_OK, ST_TRAVERSAL_LIMIT);
                    G = make_uint2(0u, 0u);
                    sp = 0;
                } else {
                    const uint32_t idx = cw8_next(G, cr.oct7);
                    if (G.y & 0xFF000000u) {
                        if (sp >= cap) {
                            atomicCAS(a.status, ST_OK, ST_STACK_OVERFLOW);
                        } else {
                            stk[sp * BLOCK] = G;
                            ++sp;
                        }
                    }
                    uint2 P;
                    cw8_visit(nodes, idx, cr, h.t, G, P);
                    if (STATS) cnt.c[C_NODES] += 3;
                    if (P.y) {
                        held[nh * BLOCK] = P;
                        ++nh;
                    }
                }
            }
        }
        // 3) the held primitives: two per lane and step while at least
        // kCw8SharedBelow lanes have some left, then the rest shared out
        // over the warp
        {
            int j = 0;
            uint2 cur = make_uint2(0u, 0u);
            for (;;) {
                const bool lf = has && (cur.y != 0u || j < nh);
                if (__popc(__ballot_sync(full, lf)) < kCw8SharedBelow) break;
                if (lf) {
                    if (cur.y == 0u) {
                        cur = held[j * BLOCK];
                        ++j;
                    }
                    const uint32_t k0 = cur.x + (uint32_t)(__ffs(cur.y) - 1);
                    cur.y &= cur.y - 1u;
                    if (cur.y == 0u && j < nh) {
                        cur = held[j * BLOCK];
                        ++j;
                    }
                    const bool two = cur.y != 0u;
                    const uint32_t k1 = two ? cur.x + (uint32_t)(__ffs(cur.y) - 1) : k0;
                    if (two) cur.y &= cur.y - 1u;
                    cw8_test_tri2<STATS>(tris, k0, k1, two, ray, h, cnt);
                }
            }
            const bool rest = has && (cur.y != 0u || j < nh);
            if (__any_sync(full, rest)) cw8_warp_prims<STATS>(tris, held, shr, BLOCK, lane, rest, cur, j, nh, ray, h, cnt);
        }
        nh = 0;
        // 4) finished rays: planes and the result
        if (has && (G.y & 0xFF000000u) == 0u && sp == 0) finish_ray();
    }
    if (STATS) flush_counters(a, cnt);
}

// Linear-scan scenes (the reference's own trace_ray, reference or strict ties):
// persistent lanes with a per-warp fetch.  Single scene only.
template <int TIE, bool STATS>
__global__ void __launch_bounds__(128) wf_extend_linear(TraceArgs a, WfState s, int qsel)
{
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const uint32_t total = s.count[qsel];
    const uint32_t* queue = qsel ? s.queue[1] : s.queue[0];
    if (blockIdx.x == 0 && threadIdx.x == 0) s.count[qsel ^ 1] = 0;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    Tracer<TIE, false, STATS> tr{a.sc, Stack{nullptr, nullptr, 0, 0}, cnt, a.status, a.trav_limit};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&s.count[2], 32u);
        base = __shfl_sync(full, base, 0);
        if (base >= total) break;
        const uint32_t qi = base + lane;
        if (qi < total) {
            const uint32_t pid = queue[qi];
            const float4 ro = s.ray_o[pid];
            const float4 rd = s.ray_d[pid];
            Hit h;
            h.t = ro.w;
            tr.trace(Ray{v3(ro), v3(rd)}, h, false);
            s.hit[pid] = make_uint4(__float_as_uint(h.t), h.prim, h.slot, (uint32_t)h.kind);
        }
    }
    if (STATS) flush_counters(a, cnt);
}

// ------------------------------------------------------------- path state --
// One path slot between rounds, unpacked from the WfState arrays.
struct PathRegs {
    Ray ray;
    V3 acc, mask, accum;
    float t0;  // t of the pixel's primary hit (-1: none)
    uint32_t prim0, sample, depth;
    Rng g;
};

__device__ __forceinline__ void load_path(const WfState& s, const TraceArgs& A, uint32_t pid, uint32_t x, uint32_t y,
                                          PathRegs& p)
{
    const float4 ro = s.ray_o[pid], rd = s.ray_d[pid];
    const float4 acc4 = s.acc[pid], mask4 = s.mask[pid], accum4 = s.accum[pid];
    p.ray = Ray{v3(ro), v3(rd)};
    p.acc = v3(acc4);
    p.mask = v3(mask4);
    p.accum = v3(accum4);
    p.t0 = mask4.w;
    p.prim0 = s.prim0[pid];
    const uint32_t sd = __float_as_uint(accum4.w);
    p.sample = sd >> 16;
    p.depth = sd & 0xFFFFu;
    p.g.salt = acc4.w;
    p.g.cx = (float)x / (float)A.width;
    p.g.cy = (float)y / (float)A.height;
}

__device__ __forceinline__ void store_path(const WfState& s, uint32_t pid, const PathRegs& p)
{
    s.ray_o[pid] = make_float4(p.ray.o.x, p.ray.o.y, p.ray.o.z, depth_tmax(p.depth));
    s.ray_d[pid] = make_float4(p.ray.d.x, p.ray.d.y, p.ray.d.z, 0.0f);
    s.acc[pid] = make_float4(p.acc.x, p.acc.y, p.acc.z, p.g.salt);
    s.mask[pid] = make_float4(p.mask.x, p.mask.y, p.mask.z, p.t0);
    s.accum[pid] = make_float4(p.accum.x, p.accum.y, p.accum.z, __uint_as_float((p.sample << 16) | p.depth));
    s.prim0[pid] = p.prim0;
}

// The rest of one depth iteration after its closest hit h (Tracer.comp:441-549:
// clamp, sky, scatter, next-event estimation, Russian roulette), then the
// sample and pixel bookkeeping (:578-592): the next depth, else the pixel's
// next sample (its RNG continues where the last sample stopped), else the
// resolve.  Returns true while the pixel has another ray to trace: p.ray, with
// tmax depth_tmax(p.depth).  NEE: as shade_bounce.
template <bool NEE, class TR>
__device__ __forceinline__ bool advance_path(TR& tr, const TraceArgs& A, uint32_t x, uint32_t y, const Hit& h,
                                             PathRegs& p)
{
    const bool found = h.kind != 0;
    if (p.sample == 0 && p.depth == 0) {
        p.prim0 = found ? h.prim : NO_PRIM;
        p.t0 = found ? h.t : -1.0f;
    }
    p.acc = vclamp01(p.acc);
    const bool cont = shade_bounce<NEE>(tr, A, p.depth, found, h, p.ray, p.acc, p.mask, p.g);
    p.depth++;
    if (cont && p.depth < A.max_depth) return true;
    p.accum = p.accum + p.acc;
    p.sample++;
    p.depth = 0;
    if (p.sample < A.spp) {
        p.ray = primary_ray(A, x, y);
        p.acc = splat(0.0f);
        p.mask = splat(1.0f);
        return true;
    }
    resolve_pixel(A, x, y, p.accum, p.g, p.prim0, p.t0);
    return false;
}

// ------------------------------------------------------------------- shade --
template <int TIE, bool BVH, bool STATS, bool MULTI, bool NEE>
__global__ void __launch_bounds__(256) wf_shade(TraceArgs a, WfState s, int qsel, const TraceArgs* slots)
{
    extern __shared__ int smem[];
    const uint32_t n = s.count[qsel];
    const uint32_t* queue = qsel ? s.queue[1] : s.queue[0];
    uint32_t* next = qsel ? s.queue[0] : s.queue[1];
    if (blockIdx.x == 0 && threadIdx.x == 0) s.count[2] = 0;  // fetch cursor of the next round
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    const Stack stk{smem + threadIdx.x, reinterpret_cast<float*>(smem + (size_t)a.stack_depth * blockDim.x) + threadIdx.x,
                    (int)blockDim.x, (int)a.stack_depth};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t qi = base + threadIdx.x;
        bool again = false;
        uint32_t pid = 0;
        if (qi < n) {
            pid = queue[qi];
            const TraceArgs& A = SCENE_ARGS(MULTI, a, slots, MULTI ? s.scene_of[pid] : 0);
            Tracer<TIE, BVH, STATS> tr{A.sc, stk, cnt, a.status, A.trav_limit};
            const uint32_t p = pid - A.pixel_base;
            const uint32_t x = p % A.width, y = p / A.width;
            PathRegs ps;
            load_path(s, A, pid, x, y, ps);
            const uint4 hr = s.hit[pid];
            Hit h;
            h.t = __uint_as_float(hr.x);
            h.prim = hr.y;
            h.slot = hr.z;
            h.kind = (int)hr.w;
            again = advance_path<NEE>(tr, A, x, y, h, ps);
            if (again) store_path(s, pid, ps);
        }
        warp_append(again, pid, next, &s.count[qsel ^ 1]);
    }
    if (STATS) flush_counters(a, cnt);
}

// ------------------------------------------------------------------ finish --
// Runs every queued path to the end of its pixel in one launch: a thread takes
// a path and traces and shades it bounce after bounce, sample after sample,
// with the per-thread traversal, until the pixel is resolved; then it takes
// the next.  For the last rounds of a wavefront, when few paths are live, and
// for whole frames with fewer pixels than that: the paths then need no
// launches per round and do not wait each round for that round's slowest ray.
// The operations per pixel are those of extend + shade, in the same order, so
// the results are identical.
// First path of a thread: queue entry = its global index; later ones from the
// cursor count[2] (zeroed by the generate or shade that wrote the queue),
// offset by the number of threads.
template <int TIE, bool BVH, bool STATS, bool MULTI, bool NEE>
__global__ void __launch_bounds__(128) wf_finish(TraceArgs a, WfState s, int qsel, const TraceArgs* slots)
{
    extern __shared__ int smem[];
    const uint32_t n = s.count[qsel];
    const uint32_t* queue = qsel ? s.queue[1] : s.queue[0];
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    const Stack stk{smem + threadIdx.x, reinterpret_cast<float*>(smem + (size_t)a.stack_depth * blockDim.x) + threadIdx.x,
                    (int)blockDim.x, (int)a.stack_depth};
    // the closest-hit traversal's stack (8-byte entries interleaved by thread)
    // after the shadow rays' (stk: 4-byte entries interleaved by thread, used
    // only with NEE), so no thread's entries overlap another's
    const size_t pbase = NEE ? 2 * (size_t)a.stack_depth * blockDim.x : 0;  // in ints
    const PairStack pstk{reinterpret_cast<int2*>(smem + pbase) + threadIdx.x, (int)blockDim.x, (int)a.stack_depth};
    const uint32_t threads = gridDim.x * blockDim.x;
    uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    while (qi < n) {
        const uint32_t pid = queue[qi];
        const TraceArgs& A = SCENE_ARGS(MULTI, a, slots, MULTI ? s.scene_of[pid] : 0);
        Tracer<TIE, BVH, STATS> tr{A.sc, stk, cnt, a.status, A.trav_limit};
        const uint32_t p = pid - A.pixel_base;
        const uint32_t x = p % A.width, y = p / A.width;
        PathRegs ps;
        load_path(s, A, pid, x, y, ps);
        for (;;) {
            Hit h;
            h.t = depth_tmax(ps.depth);
            if (BVH && A.sc.tri_cw8 != nullptr)  // triangle-only scenes with an 8-wide BVH
                closest_cw8<STATS>(A.sc, ps.ray, h, pstk, a.status, A.trav_limit, cnt);
            else if (BVH)
                closest_enc<STATS>(A.sc, ps.ray, h, pstk, a.status, A.trav_limit, cnt);
            else
                tr.trace(ps.ray, h, false);
            if (!advance_path<NEE>(tr, A, x, y, h, ps)) break;
        }
        qi = n > threads ? threads + atomicAdd(&s.count[2], 1u) : n;
    }
    if (STATS) flush_counters(a, cnt);
}

// ---------------------------------------------------------------- dispatch --
template <class K>
static void smem_attr(K k, size_t smem)
{
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// Dynamic shared memory of the extend kernel: every thread's traversal stack
// (8 B per entry) and its held leaves (binary and 4-wide: 4 B per leaf
// reference) or held primitive groups (8-wide: 8 B per group).
static size_t wf_extend_smem(size_t stack_depth, uint32_t block, int wide)
{
    return (stack_depth * 8 + (wide == WF_WIDTH_8 ? kCw8Postpone * 8 + sizeof(Cw8Share) : kPostpone * 4)) * block;
}

template <int TIE, bool STATS, bool MULTI, int BLOCK>
static cudaError_t extend_bvh_b(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st)
{
    auto k = c.wide == WF_WIDTH_8   ? wf_extend_cw8<STATS, MULTI, BLOCK>
             : c.wide == WF_WIDTH_4 ? wf_extend_bvh<TIE, STATS, MULTI, BLOCK, true>
                                    : wf_extend_bvh<TIE, STATS, MULTI, BLOCK, false>;
    if (c.wide == WF_WIDTH_8 && c.cw8_stack != 0) {
        TraceArgs a8 = a;
        a8.stack_depth = c.cw8_stack;
        const size_t smem = wf_extend_smem(a8.stack_depth, BLOCK, c.wide);
        smem_attr(k, smem);
        k<<<c.extend_grid, BLOCK, smem, st>>>(a8, s, qsel, c.slots);
        return cudaGetLastError();
    }
    const size_t smem = wf_extend_smem(a.stack_depth, BLOCK, c.wide);
    smem_attr(k, smem);
    k<<<c.extend_grid, BLOCK, smem, st>>>(a, s, qsel, c.slots);
    return cudaGetLastError();
}

template <int TIE, bool BVH, bool STATS, bool MULTI>
static cudaError_t extend_t(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st)
{
    if (BVH) {
        if (c.block == 64) return extend_bvh_b<TIE, STATS, MULTI, 64>(a, s, c, qsel, st);
        if (c.block == 256) return extend_bvh_b<TIE, STATS, MULTI, 256>(a, s, c, qsel, st);
        return extend_bvh_b<TIE, STATS, MULTI, 128>(a, s, c, qsel, st);
    }
    wf_extend_linear<TIE, STATS><<<c.extend_grid, 128, 0, st>>>(a, s, qsel);
    return cudaGetLastError();
}

template <int TIE, bool BVH, bool STATS, bool MULTI>
static cudaError_t shade_t(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st)
{
    auto k = c.has_emitters ? wf_shade<TIE, BVH, STATS, MULTI, true> : wf_shade<TIE, BVH, STATS, MULTI, false>;
    const size_t smem = (BVH && c.has_emitters) ? (size_t)a.stack_depth * 256 * 8 : 0;
    smem_attr(k, smem);
    k<<<c.shade_grid, 256, smem, st>>>(a, s, qsel, c.slots);
    return cudaGetLastError();
}

// Dynamic shared memory of the finishing kernel (128 threads): the closest-hit
// stack and, with next-event estimation, the shadow rays' stack before it.
static size_t wf_finish_smem(bool bvh, bool nee, size_t stack_depth)
{
    return bvh ? stack_depth * 128 * 8 * (nee ? 2 : 1) : 0;
}

template <int TIE, bool BVH, bool STATS, bool MULTI>
static cudaError_t finish_t(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st)
{
    auto k = c.has_emitters ? wf_finish<TIE, BVH, STATS, MULTI, true> : wf_finish<TIE, BVH, STATS, MULTI, false>;
    const size_t smem = wf_finish_smem(BVH, c.has_emitters != 0, a.stack_depth);
    smem_attr(k, smem);
    k<<<c.finish_grid, 128, smem, st>>>(a, s, qsel, c.slots);
    return cudaGetLastError();
}

template <int TIE, bool BVH, bool STATS, bool MULTI>
static int finish_occ(size_t smem, bool nee)
{
    auto k = nee ? wf_finish<TIE, BVH, STATS, MULTI, true> : wf_finish<TIE, BVH, STATS, MULTI, false>;
    smem_attr(k, smem);
    int n = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 128, smem) == cudaSuccess ? n : 0;
}

// Template selection: ties, BVH (strict only), statistics, multi-scene (BVH only).
#define WF_DISPATCH(fn)                                                                                    \
    if (c.multi) {                                                                                         \
        return c.stats ? fn<TIE_STRICT, true, true, true>(a, s, c, qsel, st)                              \
                       : fn<TIE_STRICT, true, false, true>(a, s, c, qsel, st);                            \
    }                                                                                                      \
    if (c.tie == TIE_REFERENCE)                                                                            \
        return c.stats ? fn<TIE_REFERENCE, false, true, false>(a, s, c, qsel, st)                         \
                       : fn<TIE_REFERENCE, false, false, false>(a, s, c, qsel, st);                       \
    if (c.bvh)                                                                                             \
        return c.stats ? fn<TIE_STRICT, true, true, false>(a, s, c, qsel, st)                             \
                       : fn<TIE_STRICT, true, false, false>(a, s, c, qsel, st);                           \
    return c.stats ? fn<TIE_STRICT, false, true, false>(a, s, c, qsel, st)                                \
                   : fn<TIE_STRICT, false, false, false>(a, s, c, qsel, st);

cudaError_t wf_launch_generate(const TraceArgs& a, const WfState& s, const WfConfig& c, cudaStream_t st)
{
    const uint32_t n = a.num_slots;
    if (c.multi)
        wf_generate<true><<<(n + 255) / 256, 256, 0, st>>>(a, s, c.slots, c.nslots);
    else
        wf_generate<false><<<(n + 255) / 256, 256, 0, st>>>(a, s, nullptr, 0);
    return cudaGetLastError();
}

cudaError_t wf_launch_extend(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st)
{
    WF_DISPATCH(extend_t)
}

cudaError_t wf_launch_shade(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st)
{
    WF_DISPATCH(shade_t)
}

cudaError_t wf_launch_finish(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st)
{
    WF_DISPATCH(finish_t)
}

int wf_finish_blocks_per_sm(const WfConfig& c, uint32_t stack_depth)
{
    const bool nee = c.has_emitters != 0;
    const size_t smem = wf_finish_smem(c.bvh != 0, nee, stack_depth);
    if (c.multi) return c.stats ? finish_occ<TIE_STRICT, true, true, true>(smem, nee)
                                : finish_occ<TIE_STRICT, true, false, true>(smem, nee);
    if (c.tie == TIE_REFERENCE) return c.stats ? finish_occ<TIE_REFERENCE, false, true, false>(smem, nee)
                                               : finish_occ<TIE_REFERENCE, false, false, false>(smem, nee);
    if (c.bvh) return c.stats ? finish_occ<TIE_STRICT, true, true, false>(smem, nee)
                              : finish_occ<TIE_STRICT, true, false, false>(smem, nee);
    return c.stats ? finish_occ<TIE_STRICT, false, true, false>(smem, nee)
                   : finish_occ<TIE_STRICT, false, false, false>(smem, nee);
}

template <int TIE, bool STATS, bool MULTI, int BLOCK>
static cudaError_t occ_bvh_b(int& n, int wide, size_t smem)
{
    auto k = wide == WF_WIDTH_8   ? wf_extend_cw8<STATS, MULTI, BLOCK>
             : wide == WF_WIDTH_4 ? wf_extend_bvh<TIE, STATS, MULTI, BLOCK, true>
                                  : wf_extend_bvh<TIE, STATS, MULTI, BLOCK, false>;
    smem_attr(k, smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, BLOCK, smem);
}

template <int TIE, bool STATS, bool MULTI>
static int occ_bvh(uint32_t block, size_t stack_depth, int wide)
{
    int n = 0;
    const size_t smem = wf_extend_smem(stack_depth, block, wide);
    cudaError_t e;
    if (block == 64)
        e = occ_bvh_b<TIE, STATS, MULTI, 64>(n, wide, smem);
    else if (block == 256)
        e = occ_bvh_b<TIE, STATS, MULTI, 256>(n, wide, smem);
    else
        e = occ_bvh_b<TIE, STATS, MULTI, 128>(n, wide, smem);
    return e == cudaSuccess ? n : 0;
}

int wf_extend_blocks_per_sm(const WfConfig& c, uint32_t stack_depth)
{
    const int w = c.wide;
    if (w == WF_WIDTH_8 && c.cw8_stack != 0) stack_depth = c.cw8_stack;
    if (c.multi) return c.stats ? occ_bvh<TIE_STRICT, true, true>(c.block, stack_depth, w)
                                : occ_bvh<TIE_STRICT, false, true>(c.block, stack_depth, w);
    if (c.bvh) return c.stats ? occ_bvh<TIE_STRICT, true, false>(c.block, stack_depth, w)
                              : occ_bvh<TIE_STRICT, false, false>(c.block, stack_depth, w);
    int n = 0;
    cudaError_t e;
    if (c.tie == TIE_REFERENCE)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, c.stats ? wf_extend_linear<TIE_REFERENCE, true> : wf_extend_linear<TIE_REFERENCE, false>, 128, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &n, c.stats ? wf_extend_linear<TIE_STRICT, true> : wf_extend_linear<TIE_STRICT, false>, 128, 0);
    return e == cudaSuccess ? n : 0;
}

}  // namespace vkt
