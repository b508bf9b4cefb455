// Boundary term of the camera-position gradient (no counterpart in the
// reference): how the image changes because triangle outlines move across
// pixels when the camera moves.
//
// The forward pass shoots every sample of pixel (x, y) through one point of
// the image plane (uv = (x, y) / size, Tracer.comp:562-574), so as the camera
// translates, a pixel's value is constant until an outline crosses that
// point, then jumps.  Averaged over where outlines fall relative to the
// pixel grid (the pixel as a box of one pixel around its sample point), the
// rate of change is the edge integral of Li et al., "Differentiable Monte
// Carlo Ray Tracing through Edge Sampling" (SIGGRAPH Asia 2018), restricted
// to primary visibility:
//   dL/dc_j = sum over triangle edges of the integral along the edge's image
//             of (dL/dI_p . (I_inside - I_outside)) * (n . du/dc_j) dl,
// with I_inside / I_outside the pixel's forward value (all samples, the
// pixel's own random numbers, tone mapping and dither) for a primary ray just
// inside / outside the outline, n the image-space normal pointing out of the
// triangle, and du/dc_j the image-space velocity of the edge point when the
// camera moves along axis j.  Where the triangle faces away from the ray or
// something is in front of it, both sides see the same and the piece is
// skipped (no primary-visibility change there).  Each edge's image is split into
// `samples` pieces (one thread each), and each piece into the parts inside
// single pixel boxes, integrated by their midpoints (perspective-correct 3D
// points for the velocity): inside one box the pixel's loss weight is
// constant, so the estimate does not alias the pixel grid.  Secondary
// visibility (outlines seen by bounce rays) and sphere outlines are not
// included.
//
// Image coordinates are in pixels, with pixel (x, y)'s sample point at (x, y)
// (uv = (x, y) / size: no half-pixel offset) and row 0 at the bottom.

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_cw8.cuh"
#include "tracer_edges.h"

namespace vkt {

// The primary ray through image point (ux, uy) (pixel units, as
// primary_ray, Tracer.comp:568-574).
__device__ __forceinline__ Ray primary_ray_at(const TraceArgs& a, float ux, float uy)
{
    const float tx = 2.0f * (ux / (float)a.width) - 1.0f;
    const float ty = 2.0f * (uy / (float)a.height) - 1.0f;
    const V3 dir = (a.fr.cdir + a.fr.cright * tx + a.fr.cup * ty) * v3(a.fr.aspect, 1.0f, a.fr.aspect);
    return Ray{a.fr.cpos, normalize(dir)};
}

// Closest hit of a path ray: over the compressed 8-wide BVH where the scene
// has one (the same hit, fewer dependent fetches), else the plain traversal.
template <class TR>
__device__ __forceinline__ bool closest(TR& tr, const TraceArgs& a, const PairStack& pstk, const Ray& ray, Hit& h,
                                        Counters& cnt)
{
    if (a.sc.tri_cw8 != nullptr) return closest_cw8<false>(a.sc, ray, h, pstk, a.status, a.trav_limit, cnt);
    return tr.trace(ray, h, false);
}

// The forward value of pixel (x, y) for the primary ray r (through another
// image point than the pixel's own sample point) whose closest hit h0 is
// given (found0: it hit): every sample (the pixel's random numbers) through
// the radiance loop (Tracer.comp:433-553), Reinhard, gamma 1/2.2 and the
// dither, as resolve_pixel (:578-590).  Every sample starts with the same
// primary ray, so its hit is traced once, by the caller.
template <class TR>
__device__ __forceinline__ V3 pixel_value_from(TR& tr, const TraceArgs& a, const PairStack& pstk, uint32_t x,
                                               uint32_t y, const Ray& r, bool found0, const Hit& h0, Counters& cnt)
{
    Rng g;
    seed_rng(a, x, y, g);
    V3 accum = splat(0.0f);
    for (uint32_t s = 0; s < a.spp; ++s) {
        V3 acc = splat(0.0f), mask = splat(1.0f);
        Ray ray = r;
        for (uint32_t depth = 0; depth < a.max_depth; ++depth) {
            acc = vclamp01(acc);
            Hit h = h0;
            bool found = found0;
            if (depth > 0) {
                h.t = depth_tmax(depth);
                found = closest(tr, a, pstk, ray, h, cnt);
            }
            if (!shade_bounce(tr, a, depth, found, h, ray, acc, mask, g)) break;
        }
        accum = accum + acc;
    }
    accum = accum / (float)a.spp;
    accum = accum / (accum + splat(1.0f));
    const float gam = 1.0f / 2.2f;
    accum = v3(powf(accum.x, gam), powf(accum.y, gam), powf(accum.z, gam));
    const float dither = rand01(g) / 64.0f;
    return accum + splat(dither);
}

// The camera-space coefficients q = (lambda, mu, nu) of X:
// X - cpos = lambda * (cdir + right * tx + up * ty) * (aspect, 1, aspect),
// tx = mu / lambda, ty = nu / lambda (the primary ray's construction,
// Tracer.comp:568-574, solved for the image point).
__device__ __forceinline__ V3 cam_coeffs(const EdgeArgs& e, const TraceArgs& a, V3 X)
{
    const V3 d = X - a.fr.cpos;
    const V3 Y = v3(d.x / a.fr.aspect, d.y, d.z / a.fr.aspect);
    return v3(e.binv[0] * Y.x + e.binv[1] * Y.y + e.binv[2] * Y.z, e.binv[3] * Y.x + e.binv[4] * Y.y + e.binv[5] * Y.z,
              e.binv[6] * Y.x + e.binv[7] * Y.y + e.binv[8] * Y.z);
}

// The loss weight of one visible outline part of pixel (px, py): dL/dI .
// (I_inside - I_outside), the pixel evaluated for primary rays through the
// inside point (ix, iy), whose closest hit hin is known, and the outside
// point (ox, oy).
template <class TR>
__device__ __forceinline__ float part_weight(TR& tr, const TraceArgs& a, const PairStack& pstk, const EdgeArgs& e,
                                             uint32_t px, uint32_t py, float ix, float iy, float ox, float oy,
                                             const Hit& hin, Counters& cnt)
{
    const float4 dl = __ldg(e.dldi + (size_t)py * a.width + px);
    const Ray rin = primary_ray_at(a, ix, iy);
    const Ray rout = primary_ray_at(a, ox, oy);
    Hit hout;
    hout.t = depth_tmax(0);
    const bool fout = closest(tr, a, pstk, rout, hout, cnt);
    const V3 vin = pixel_value_from(tr, a, pstk, px, py, rin, true, hin, cnt);
    const V3 vout = pixel_value_from(tr, a, pstk, px, py, rout, fout, hout, cnt);
    return dl.x * (vin.x - vout.x) + dl.y * (vin.y - vout.y) + dl.z * (vin.z - vout.z);
}

// Block sum of the three camera-axis contributions in FP64, added to e.gcam.
__device__ __forceinline__ void add_contrib(const EdgeArgs& e, const float (&contrib)[3], double (&red)[3][4])
{
    const int tid = threadIdx.x;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        double v = (double)(isfinite(contrib[j]) ? contrib[j] : 0.0f);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
        if ((tid & 31) == 0) red[j][tid >> 5] = v;
    }
    __syncthreads();
    if (tid < 3) {
        const double v = red[tid][0] + red[tid][1] + red[tid][2] + red[tid][3];
        if (v != 0.0) atomicAdd(e.gcam + tid, v);
    }
}

// A visible outline part handed from the walk to k_edge_values: 3 float4 =
// (inside point, outside point) (inside hit t, prim, slot, px | py << 16)
// (the part's velocity factors n . du/dc_j times its length, j = x, y, z).
constexpr uint32_t kEdgeSegFloat4 = 3;

// The walk: one thread per (triangle edge, piece of it); the visible parts
// it finds go to e.segs (or, without room there, are evaluated here);
// block sums in FP64.
template <int TIE, bool BVH>
__global__ void __launch_bounds__(128) k_edge_campos(TraceArgs a, EdgeArgs e)
{
    extern __shared__ int smem[];
    __shared__ double red[3][4];
    const int tid = threadIdx.x;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    Tracer<TIE, BVH, false> tr{a.sc,
                               Stack{smem + tid, reinterpret_cast<float*>(smem + (size_t)a.stack_depth * blockDim.x) + tid,
                                     (int)blockDim.x, (int)a.stack_depth},
                               cnt, a.status, a.trav_limit};
    // the 8-wide traversal's stack of node groups, after the plain traversal's
    const PairStack pstk{reinterpret_cast<int2*>(smem + 2 * (size_t)a.stack_depth * blockDim.x) + tid,
                         (int)blockDim.x, (int)a.stack_depth};
    float contrib[3] = {0.0f, 0.0f, 0.0f};
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + tid;
    const uint64_t total = (uint64_t)a.sc.nt * 3u * e.samples;
    if (i < total) {
        const uint32_t slot = (uint32_t)(i / (3u * e.samples));
        const uint32_t edge = (uint32_t)((i / e.samples) % 3u);
        const uint32_t k = (uint32_t)(i % e.samples);
        const float4* t = a.sc.tri + 3 * (size_t)slot;
        const float4 t1 = __ldg(t + 1);
        const V3 v0 = v3(__ldg(t)), e1 = v3(t1), e2 = v3(__ldg(t + 2));
        const uint32_t tri_id = __float_as_uint(t1.w);
        // the triangle the Moller-Trumbore test sees: v0, v0 + e1, v0 + e2
        const V3 P[3] = {v0, v0 + e1, v0 + e2};
        const V3 A = P[edge], B = P[(edge + 1) % 3], C = P[(edge + 2) % 3];
        const V3 qa = cam_coeffs(e, a, A), qb = cam_coeffs(e, a, B), qc = cam_coeffs(e, a, C);
        if (qa.x > 0.0f && qb.x > 0.0f && qc.x > 0.0f) {  // the whole triangle in front of the camera
            const float hw = 0.5f * (float)a.width, hh = 0.5f * (float)a.height;
            const float uax = (qa.y / qa.x + 1.0f) * hw, uay = (qa.z / qa.x + 1.0f) * hh;
            const float ubx = (qb.y / qb.x + 1.0f) * hw, uby = (qb.z / qb.x + 1.0f) * hh;
            const float ucx = (qc.y / qc.x + 1.0f) * hw, ucy = (qc.z / qc.x + 1.0f) * hh;
            const float ex = ubx - uax, ey = uby - uay;
            const float len = sqrtf(ex * ex + ey * ey);
            if (len > 0.0f) {
                // outward normal (away from the third vertex's image)
                float nx = ey / len, ny = -ex / len;
                if (nx * (ucx - uax) + ny * (ucy - uay) > 0.0f) {
                    nx = -nx;
                    ny = -ny;
                }
                // this thread's piece [s0, s1] of the edge's image, cut where it
                // crosses pixel boxes (box of pixel p: [p - 1/2, p + 1/2) per
                // axis): within a box the integrand's pixel weight and values are
                // those of one pixel, so each cut piece is integrated by its
                // midpoint times its length
                const float s0 = (float)k / (float)e.samples, s1 = (float)(k + 1) / (float)e.samples;
                const float vx = uax + s0 * ex + 0.5f, vy = uay + s0 * ey + 0.5f;  // box coordinates
                const float dx = (s1 - s0) * ex, dy = (s1 - s0) * ey;
                // the part of the piece inside the image, [0, W] x [0, H] in box coordinates
                float tlo = 0.0f, thi = 1.0f;
                if (dx != 0.0f) {
                    const float ta = (0.0f - vx) / dx, tb = ((float)a.width - vx) / dx;
                    tlo = fmaxf(tlo, fminf(ta, tb));
                    thi = fminf(thi, fmaxf(ta, tb));
                } else if (!(vx >= 0.0f && vx < (float)a.width)) {
                    thi = -1.0f;
                }
                if (dy != 0.0f) {
                    const float ta = (0.0f - vy) / dy, tb = ((float)a.height - vy) / dy;
                    tlo = fmaxf(tlo, fminf(ta, tb));
                    thi = fminf(thi, fmaxf(ta, tb));
                } else if (!(vy >= 0.0f && vy < (float)a.height)) {
                    thi = -1.0f;
                }
                const float px0 = vx + tlo * dx, py0 = vy + tlo * dy;
                int cx = (int)floorf(px0), cy = (int)floorf(py0);
                const int stx = dx > 0.0f ? 1 : -1, sty = dy > 0.0f ? 1 : -1;
                const float INF = __int_as_float(0x7f800000);
                float tmx = dx != 0.0f ? tlo + (dx > 0.0f ? ((float)cx + 1.0f - px0) : (px0 - (float)cx)) / fabsf(dx) : INF;
                float tmy = dy != 0.0f ? tlo + (dy > 0.0f ? ((float)cy + 1.0f - py0) : (py0 - (float)cy)) / fabsf(dy) : INF;
                const float tdx = dx != 0.0f ? 1.0f / fabsf(dx) : INF, tdy = dy != 0.0f ? 1.0f / fabsf(dy) : INF;
                // boxes the clipped piece can cross (at most W + H + 2 inside the image)
                const int cells = thi > tlo ? (int)fminf((thi - tlo) * (fabsf(dx) + fabsf(dy)) + 3.0f, 65536.0f) : 0;
                float t0 = tlo;
                for (int it = 0; it < cells && t0 < thi; ++it) {
                    const float t1 = fminf(fminf(tmx, tmy), thi);
                    if (t1 > t0) {
                        const float tm = 0.5f * (t0 + t1);
                        const float ux = vx - 0.5f + tm * dx, uy = vy - 0.5f + tm * dy;
                        if (ux >= -0.5f && ux < (float)a.width - 0.5f && uy >= -0.5f && uy < (float)a.height - 0.5f) {
                            const uint32_t px = (uint32_t)floorf(ux + 0.5f), py = (uint32_t)floorf(uy + 0.5f);
                            const float eps = e.offset_px;
                            const float ix = ux - eps * nx, iy = uy - eps * ny, ox = ux + eps * nx, oy = uy + eps * ny;
                            // the outline is visible here only if the inside ray sees this
                            // triangle: it faces the ray (the one-sided test's det, no
                            // trace needed) and nothing is in front of it; otherwise
                            // both sides see the same and there is nothing to trace
                            const Ray rin = primary_ray_at(a, ix, iy);
                            if (dot(e1, cross(rin.d, e2)) >= EPSILON) {
                                Hit hin;
                                hin.t = depth_tmax(0);
                                if (closest(tr, a, pstk, rin, hin, cnt) && hin.prim == tri_id) {
                                    // velocity factors of the part: (n . du/dc_j) * its length,
                                    // at the 3D point (1 / lambda is linear along the image)
                                    float vel[3];
                                    const float sm = s0 + tm * (s1 - s0);
                                    const float tt = sm * qa.x / ((1.0f - sm) * qb.x + sm * qa.x);
                                    const V3 X = A + tt * (B - A);
                                    const V3 q = cam_coeffs(e, a, X);
                                    const float il = 1.0f / q.x;
                                    const float seg = (t1 - t0) * (s1 - s0) * len;
#pragma unroll
                                    for (int j = 0; j < 3; ++j) {
                                        // dY/dc_j = -e_j / (aspect, 1, aspect)_j; dq = binv dY
                                        const float m = (j == 1) ? 1.0f : a.fr.aspect;
                                        const float dlam = -e.binv[0 + j] / m, dmu = -e.binv[3 + j] / m,
                                                    dnu = -e.binv[6 + j] / m;
                                        const float dux = (dmu * q.x - q.y * dlam) * il * il * hw;
                                        const float duy = (dnu * q.x - q.z * dlam) * il * il * hh;
                                        vel[j] = (nx * dux + ny * duy) * seg;
                                    }
                                    const uint32_t at = e.segs ? atomicAdd(e.nsegs, 1u) : 0xFFFFFFFFu;
                                    if (at < e.seg_cap) {
                                        float4* r = e.segs + (size_t)kEdgeSegFloat4 * at;
                                        r[0] = make_float4(ix, iy, ox, oy);
                                        r[1] = make_float4(hin.t, __uint_as_float(hin.prim), __uint_as_float(hin.slot),
                                                           __uint_as_float(px | py << 16));
                                        r[2] = make_float4(vel[0], vel[1], vel[2], 0.0f);
                                    } else {
                                        const float w = part_weight(tr, a, pstk, e, px, py, ix, iy, ox, oy, hin, cnt);
                                        if (w != 0.0f && isfinite(w)) {
#pragma unroll
                                            for (int j = 0; j < 3; ++j) contrib[j] += w * vel[j];
                                        }
                                    }
                                }
                            }
                        }
                    }
                    t0 = t1;
                    if (tmx < tmy) {
                        cx += stx;
                        tmx += tdx;
                    } else {
                        cy += sty;
                        tmy += tdy;
                    }
                }
            }
        }
    }
    add_contrib(e, contrib, red);
}

// The visible parts the walk handed over: one per thread (grid-stride), the
// pixel on both sides of each; block sums in FP64.
template <int TIE, bool BVH>
__global__ void __launch_bounds__(128) k_edge_values(TraceArgs a, EdgeArgs e)
{
    extern __shared__ int smem[];
    __shared__ double red[3][4];
    const int tid = threadIdx.x;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    Tracer<TIE, BVH, false> tr{a.sc,
                               Stack{smem + tid, reinterpret_cast<float*>(smem + (size_t)a.stack_depth * blockDim.x) + tid,
                                     (int)blockDim.x, (int)a.stack_depth},
                               cnt, a.status, a.trav_limit};
    const PairStack pstk{reinterpret_cast<int2*>(smem + 2 * (size_t)a.stack_depth * blockDim.x) + tid,
                         (int)blockDim.x, (int)a.stack_depth};
    float contrib[3] = {0.0f, 0.0f, 0.0f};
    const uint32_t found = *e.nsegs;
    const uint32_t n = found < e.seg_cap ? found : e.seg_cap;
    for (uint32_t r = blockIdx.x * blockDim.x + tid; r < n; r += gridDim.x * blockDim.x) {
        const float4* rec = e.segs + (size_t)kEdgeSegFloat4 * r;
        const float4 pts = rec[0], hr = rec[1], vel = rec[2];
        Hit hin;
        hin.t = hr.x;
        hin.prim = __float_as_uint(hr.y);
        hin.slot = __float_as_uint(hr.z);
        hin.kind = 1;
        const uint32_t pp = __float_as_uint(hr.w);
        const float w = part_weight(tr, a, pstk, e, pp & 0xFFFFu, pp >> 16, pts.x, pts.y, pts.z, pts.w, hin, cnt);
        if (w != 0.0f && isfinite(w)) {
            contrib[0] += w * vel.x;
            contrib[1] += w * vel.y;
            contrib[2] += w * vel.z;
        }
    }
    add_contrib(e, contrib, red);
}

template <int TIE, bool BVH>
static cudaError_t edge_t(const TraceArgs& a, const EdgeArgs& e, cudaStream_t st)
{
    const uint32_t block = 128;
    const size_t smem = 2 * (size_t)a.stack_depth * block * 8;  // plain and 8-wide traversal stacks
    auto k = k_edge_campos<TIE, BVH>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const uint64_t n = (uint64_t)a.sc.nt * 3u * e.samples;
    const uint64_t blocks = (n + block - 1) / block;
    if (blocks == 0) return cudaSuccess;
    if (blocks > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    k<<<(uint32_t)blocks, block, smem, st>>>(a, e);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess || !e.segs) return err;
    auto kv = k_edge_values<TIE, BVH>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const uint64_t vb = ((uint64_t)e.seg_cap + block - 1) / block;
    kv<<<(uint32_t)(vb < 65535 ? vb : 65535), block, smem, st>>>(a, e);
    return cudaGetLastError();
}

cudaError_t launch_edge_campos(const TraceArgs& a, const EdgeArgs& e, int tie, int bvh, cudaStream_t st)
{
    if (tie == TIE_REFERENCE) return edge_t<TIE_REFERENCE, false>(a, e, st);
    if (bvh) return edge_t<TIE_STRICT, true>(a, e, st);
    return edge_t<TIE_STRICT, false>(a, e, st);
}

}  // namespace vkt
