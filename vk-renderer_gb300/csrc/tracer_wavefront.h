// Wavefront path state and launchers (see tracer_wavefront.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vkt {

struct TraceArgs;

// One slot per pixel (index y * width + x), structure of arrays.
struct WfState {
    float4* ray_o;     // origin, tmax
    float4* ray_d;     // direction
    uint4* hit;        // t bits, primitive id, storage slot, kind (0 = miss)
    float4* acc;       // acc, rand_salt
    float4* mask;      // mask, t of the pixel's primary hit
    float4* accum;     // sum of finished samples, (sample << 16 | depth) bits
    uint32_t* prim0;   // primary-hit primitive id
    uint32_t* queue[2];
    uint32_t* count;   // [0], [1]: queue lengths; [2]: extend's fetch cursor
};

struct WfConfig {
    int tie, bvh, stats;
    uint32_t extend_grid, shade_grid;
};

cudaError_t wf_launch_generate(const TraceArgs& a, const WfState& s, cudaStream_t st);
cudaError_t wf_launch_extend(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st);
cudaError_t wf_launch_shade(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st);
int wf_extend_blocks_per_sm(uint32_t stack_depth, int bvh, int tie, int stats);

}  // namespace vkt
