// Internal interface between the host C ABI and the kernel launchers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tracer_abi.h"

namespace vkt {

struct TraceArgs;

struct LaunchConfig {
    int kernel;      // TRACER_KERNEL_PLAIN or TRACER_KERNEL_PERSISTENT
    uint32_t block;  // threads per block
    uint32_t grid;   // persistent kernel: number of CTAs
    int stats;
    int tie;
    int bvh;
};

cudaError_t launch_trace(const TraceArgs& a, const LaunchConfig& lc, cudaStream_t s);
int persistent_blocks_per_sm(const LaunchConfig& lc, uint32_t stack_depth, int stats, int bvh, int tie);
uint32_t persistent_ids(uint32_t width, uint32_t height);

}  // namespace vkt
