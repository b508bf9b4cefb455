// Forward path-tracing kernels for sm_103a.
//
//  k_plain       one thread per pixel, 16-wide pixel tiles, the shader's
//                nested sample / bounce loops.  The straightforward form of
//                the reference dispatch (GraphicsDevice.cpp:1266), kept as the
//                1x bar.
//  k_persistent  persistent warps sized to the machine (SM count x resident
//                CTAs).  The sample and bounce loops are flattened into one
//                loop whose every iteration advances each lane's path by one
//                bounce; a lane whose pixel is finished takes the next pixel
//                from a global counter, fetched once per warp for all idle
//                lanes (ballot + popc + one atomicAdd).  Lanes stay busy until
//                the image runs out instead of idling while the slowest path
//                of their warp finishes.
//
// Both compute exactly the same per-pixel sequence of operations as the
// oracle (oracle/tracer_oracle.cpp).

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_launch.h"

namespace vkt {

// Pixel tile of a warp in the persistent kernel: 8 x 4.
constexpr uint32_t TILE_W = 8, TILE_H = 4;

__device__ __forceinline__ Stack make_stack(int* smem, uint32_t depth, int nthreads, int tid)
{
    return Stack{smem + tid, reinterpret_cast<float*>(smem + (size_t)depth * nthreads) + tid, nthreads, (int)depth};
}

template <int TIE, bool BVH, bool STATS>
__global__ void __launch_bounds__(256) k_plain(TraceArgs a)
{
    extern __shared__ int smem[];
    const int tid = threadIdx.x;
    const int nthreads = blockDim.x;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    Tracer<TIE, BVH, STATS> tr{a.sc, make_stack(smem, a.stack_depth, nthreads, tid), cnt, a.status, a.trav_limit};
    // 16-pixel-wide tiles, blockDim / 16 rows
    const uint32_t x = blockIdx.x * 16 + (tid & 15);
    const uint32_t y = blockIdx.y * (nthreads >> 4) + (tid >> 4);
    if (x < a.width && y < a.height) {
        Rng g;
        const Ray pr = primary_ray(a, x, y, g);
        V3 accum = splat(0.0f);
        uint32_t prim0 = NO_PRIM;
        float t0 = -1.0f;
        for (uint32_t s = 0; s < a.spp; ++s) accum = accum + radiance(tr, a, pr, g, s == 0 ? &prim0 : nullptr, &t0);
        resolve_pixel(a, x, y, accum, g, prim0, t0);
    }
    if (STATS) flush_counters(a, cnt);
}

// Path state of one lane in the persistent kernel.
struct Lane {
    uint32_t px, py;
    uint32_t sample, depth;
    Ray primary, ray;
    V3 acc, mask, accum;
    Rng g;
    uint32_t prim0;
    float t0;
    bool busy;
};

template <int TIE, bool BVH, bool STATS>
__global__ void __launch_bounds__(256) k_persistent(TraceArgs a)
{
    extern __shared__ int smem[];
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const unsigned full = 0xFFFFFFFFu;
    Counters cnt;
#pragma unroll
    for (int k = 0; k < C_COUNT; ++k) cnt.c[k] = 0;
    Tracer<TIE, BVH, STATS> tr{a.sc, make_stack(smem, a.stack_depth, blockDim.x, tid), cnt, a.status, a.trav_limit};
    const uint32_t tiles_x = (a.width + TILE_W - 1) / TILE_W;
    const uint32_t total = a.num_pixels;  // tiles_x * tiles_y * 32 ids
    Lane L;
    L.busy = false;
    bool exhausted = false;
    for (;;) {
        // Hand out pixels to every idle lane of the warp at once.
        const unsigned need = __ballot_sync(full, !L.busy && !exhausted);
        if (need) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(a.work, (uint32_t)__popc(need));
            base = __shfl_sync(full, base, leader);
            if (!L.busy && !exhausted) {
                const uint32_t id = base + __popc(need & ((1u << lane) - 1u));
                if (id >= total) {
                    exhausted = true;
                } else {
                    const uint32_t tile = id >> 5, w = id & 31;
                    L.px = (tile % tiles_x) * TILE_W + (w % TILE_W);
                    L.py = (tile / tiles_x) * TILE_H + (w / TILE_W);
                    if (L.px < a.width && L.py < a.height) {
                        L.busy = true;
                        L.primary = primary_ray(a, L.px, L.py, L.g);
                        L.sample = 0;
                        L.depth = 0;
                        L.accum = splat(0.0f);
                        L.prim0 = NO_PRIM;
                        L.t0 = -1.0f;
                    }
                }
            }
        }
        if (!__any_sync(full, L.busy || !exhausted)) break;
        if (!L.busy) continue;

        // One iteration of radiance's depth loop (Tracer.comp:438-550).
        if (L.depth == 0) {
            L.ray = L.primary;
            L.acc = splat(0.0f);
            L.mask = splat(1.0f);
        }
        bool end = false;
        L.acc = vclamp01(L.acc);
        Hit h;
        const float dp1 = (float)(L.depth + 1);
        h.t = 3000.0f / (dp1 * dp1);
        const bool found = tr.trace(L.ray, h, false);
        if (L.sample == 0 && L.depth == 0) {
            L.prim0 = found ? h.prim : NO_PRIM;
            L.t0 = found ? h.t : -1.0f;
        }
        if (!found) {
            if (a.sky_on) L.acc = L.acc + L.mask * a.sky;
            end = true;
        } else {
            V3 P, N;
            Material mat;
            tr.surface(L.ray, h, P, N, mat);
            if (mat.type == MAT_DIFFUSE) {
                const float r2 = rand01(L.g);
                const V3 d =
                    jitter(N, (2.0f * PI) * rand01(L.g), sqrtf(r2), sqrtf(1.0f - r2)) * (1.0f - mat.metalness);
                V3 e = splat(0.0f);
                for (uint32_t k = 0; k < a.sc.ne; ++k) e = e + nee_one(tr, a, __ldg(a.sc.emit + k), P, N, mat, L.g);
                const bool emits = mat.emissive.x > 0.0f && mat.emissive.y > 0.0f && mat.emissive.z > 0.0f;
                const V3 emissive = emits ? normalize(mat.emissive) : splat(0.0f);
                L.acc = L.acc + L.mask * (emissive + e);
                L.mask = L.mask * mat.albedo;
                L.ray = Ray{P, normalize(reflect(L.ray.d, N) + d)};
            } else if (mat.type == MAT_DIELECTRIC) {
                L.acc = L.acc + mat.emissive * L.mask;
                L.mask = L.mask * mat.albedo;
                const float cosine = -dot(L.ray.d, N) / length(L.ray.d);
                const V3 reflected = reflect(L.ray.d, N);
                const V3 refracted = refract(L.ray.d, N, mat.roughness);
                const float prob = (refracted == splat(0.0f)) ? 1.0f : schlick(cosine, mat.roughness);
                L.ray = Ray{P, normalize(rand01(L.g) < prob ? reflected : refracted)};
            }
            if (L.depth >= a.rr_start) {
                const float p = max3(L.mask);
                if (rand01(L.g) > p)
                    end = true;
                else
                    L.mask = L.mask * (1.0f / p);
            }
        }
        L.depth++;
        if (end || L.depth >= a.max_depth) {
            L.accum = L.accum + L.acc;
            L.depth = 0;
            if (++L.sample == a.spp) {
                resolve_pixel(a, L.px, L.py, L.accum, L.g, L.prim0, L.t0);
                L.busy = false;
            }
        }
    }
    if (STATS) flush_counters(a, cnt);
}

// ------------------------------------------------------------- dispatch --
template <int TIE, bool BVH, bool STATS>
static cudaError_t launch_t(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s)
{
    const size_t smem = (size_t)a.stack_depth * lc.block * 8;
    if (lc.kernel == TRACER_KERNEL_PERSISTENT) {
        auto k = k_persistent<TIE, BVH, STATS>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k<<<lc.grid, lc.block, smem, s>>>(a);
    } else {
        auto k = k_plain<TIE, BVH, STATS>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dim3 grid((a.width + 15) / 16, (a.height + (lc.block / 16) - 1) / (lc.block / 16));
        k<<<grid, lc.block, smem, s>>>(a);
    }
    return cudaGetLastError();
}

template <int TIE, bool BVH>
static cudaError_t launch_s(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s)
{
    return lc.stats ? launch_t<TIE, BVH, true>(a, lc, s) : launch_t<TIE, BVH, false>(a, lc, s);
}

cudaError_t launch_trace(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s)
{
    if (lc.tie == TIE_REFERENCE) return launch_s<TIE_REFERENCE, false>(a, lc, s);
    if (lc.bvh) return launch_s<TIE_STRICT, true>(a, lc, s);
    return launch_s<TIE_STRICT, false>(a, lc, s);
}

int persistent_blocks_per_sm(const LaunchConfig& lc, uint32_t stack_depth, int stats, int bvh, int tie)
{
    const size_t smem = (size_t)stack_depth * lc.block * 8;
    int n = 0;
    cudaError_t e;
    if (tie == TIE_REFERENCE)
        e = stats ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<TIE_REFERENCE, false, true>, lc.block, smem)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<TIE_REFERENCE, false, false>, lc.block, smem);
    else if (bvh)
        e = stats ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<TIE_STRICT, true, true>, lc.block, smem)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<TIE_STRICT, true, false>, lc.block, smem);
    else
        e = stats ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<TIE_STRICT, false, true>, lc.block, smem)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<TIE_STRICT, false, false>, lc.block, smem);
    if (e != cudaSuccess) return 0;
    return n;
}

uint32_t persistent_ids(uint32_t width, uint32_t height)
{
    return ((width + TILE_W - 1) / TILE_W) * ((height + TILE_H - 1) / TILE_H) * 32u;
}

}  // namespace vkt
