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
cudaError_t launch_adjoint(const TraceArgs& a, const float4* dldi, const float4* linear, double* grad, uint32_t nm,
                           int tie, int bvh, cudaStream_t s);
// out[i] = (float)g[i], i < n
cudaError_t launch_grad_to_float(const double* g, float* out, uint32_t n, cudaStream_t s);

}  // namespace vkt
