// Internal interface between the host C ABI and the kernel launchers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tracer_abi.h"
#include "tracer_wavefront.h"

namespace vkt {

struct TraceArgs;

struct LaunchConfig {
    uint32_t block;  // threads per block
    int stats;
    int tie;
    int bvh;
};

cudaError_t launch_plain(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s);
// The legacy Whitted shader over its constant scene (uses a.fr, a.width,
// a.height, a.rgba8 / a.rgba32f, a.stats).
cudaError_t launch_whitted(const TraceArgs& a, int stats, cudaStream_t s);
cudaError_t launch_adjoint(const TraceArgs& a, const float4* dldi, const float4* linear, double* grad, uint32_t nm,
                           int tie, int bvh, cudaStream_t s);
// out[i] = (float)g[i], i < n
cudaError_t launch_grad_to_float(const double* g, float* out, uint32_t n, cudaStream_t s);

// Wavefront adjoint (scenes without emissive spheres): per-pixel inputs and
// outputs beside the wavefront state.
struct AdjWf {
    const float4* dldi;    // dL/dI per pixel
    const float4* linear;  // accum / spp per pixel from the forward trace
    double* grad;          // [nm x 3 albedo][nm x 3 emission][3 camera position]
    uint32_t nm;
    float4* pix;           // per pixel: delta, RNG salt at the current sample's start
    uint4* log;            // pass 1's closest hits of the current sample, max_depth per pixel
                           // (pixel-major); nullptr = pass 2 traces its rays again
};
// Seeds every pixel with a finite delta and queues it in queue 0 (counts must be zero).
cudaError_t wf_launch_adj_generate(const TraceArgs& a, const WfState& s, const AdjWf& w, cudaStream_t st);
cudaError_t wf_launch_adj_shade(const TraceArgs& a, const WfState& s, const AdjWf& w, const WfConfig& c, int qsel,
                                cudaStream_t st);
// The adjoint's finishing kernel: every path of queue qsel to the end of its
// pixel (c.finish_grid blocks of 128 threads; the cursor count[2] starts at 0).
cudaError_t wf_launch_adj_finish(const TraceArgs& a, const WfState& s, const AdjWf& w, const WfConfig& c, int qsel,
                                 cudaStream_t st);
int wf_adj_finish_blocks_per_sm(const TraceArgs& a, const WfConfig& c);
// L2 read-bandwidth probe: reads bytes (a multiple of 16) passes times;
// sink holds blocks * 256 words.
cudaError_t launch_l2_read(const void* buf, size_t bytes, uint32_t passes, uint32_t* sink, uint32_t blocks,
                           cudaStream_t s);

}  // namespace vkt
