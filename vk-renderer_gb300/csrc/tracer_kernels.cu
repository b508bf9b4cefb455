// Plain forward kernel for sm_103a: one thread per pixel, 16-pixel-wide
// tiles, the shader's nested sample / bounce loops -- the straightforward form
// of the reference dispatch (vkCmdDispatch(res/16, res/16, 1),
// GraphicsDevice.cpp:1266).  Kept as the 1x bar for the wavefront and batched
// paths and as the canonical definition of the traversal counters (its node
// visiting order is the oracle's).

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_launch.h"

namespace vkt {

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
    const uint32_t x = blockIdx.x * 16 + (tid & 15);
    const uint32_t y = blockIdx.y * (nthreads >> 4) + (tid >> 4);
    if (x < a.width && y < a.height) {
        Rng g;
        seed_rng(a, x, y, g);
        const Ray pr = primary_ray(a, x, y);
        V3 accum = splat(0.0f);
        uint32_t prim0 = NO_PRIM;
        float t0 = -1.0f;
        for (uint32_t s = 0; s < a.spp; ++s) accum = accum + radiance(tr, a, pr, g, s == 0 ? &prim0 : nullptr, &t0);
        resolve_pixel(a, x, y, accum, g, prim0, t0);
    }
    if (STATS) flush_counters(a, cnt);
}

template <int TIE, bool BVH, bool STATS>
static cudaError_t launch_t(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s)
{
    const size_t smem = (size_t)a.stack_depth * lc.block * 8;
    auto k = k_plain<TIE, BVH, STATS>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((a.width + 15) / 16, (a.height + (lc.block / 16) - 1) / (lc.block / 16));
    k<<<grid, lc.block, smem, s>>>(a);
    return cudaGetLastError();
}

template <int TIE, bool BVH>
static cudaError_t launch_s(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s)
{
    return lc.stats ? launch_t<TIE, BVH, true>(a, lc, s) : launch_t<TIE, BVH, false>(a, lc, s);
}

// Reads n 16-byte words `passes` times with loads that are cached in L2 only
// (ld.global.cg), so a buffer smaller than L2 is served by L2 after the first
// pass; one word per thread is written so the loads are not optimised away.
__global__ void __launch_bounds__(256) k_l2_read(const uint4* __restrict__ buf, size_t n, uint32_t passes,
                                                 uint32_t* __restrict__ sink)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t acc = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        for (size_t i = tid; i < n; i += stride) {
            const uint4 v = __ldcg(buf + i);
            acc ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    }
    sink[tid] = acc;
}

cudaError_t launch_l2_read(const void* buf, size_t bytes, uint32_t passes, uint32_t* sink, uint32_t blocks,
                           cudaStream_t s)
{
    k_l2_read<<<blocks, 256, 0, s>>>(static_cast<const uint4*>(buf), bytes / 16, passes, sink);
    return cudaGetLastError();
}

cudaError_t launch_plain(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s)
{
    if (lc.tie == TIE_REFERENCE) return launch_s<TIE_REFERENCE, false>(a, lc, s);
    if (lc.bvh) return launch_s<TIE_STRICT, true>(a, lc, s);
    return launch_s<TIE_STRICT, false>(a, lc, s);
}

}  // namespace vkt
