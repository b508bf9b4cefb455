// Wavefront path state and launchers (see tracer_wavefront.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vkt {

struct TraceArgs;

// BVH the extend kernel traverses: the binary BVH, its 4-wide collapse, or
// its compressed 8-wide collapse (bvh_wide.h, bvh_cw8.h).
enum : int { WF_WIDTH_2 = 0, WF_WIDTH_4 = 1, WF_WIDTH_8 = 2 };

// One slot per pixel (index = scene's pixel_base + y * width + x), structure
// of arrays.
struct WfState {
    float4* ray_o;       // origin, tmax
    float4* ray_d;       // direction
    uint4* hit;          // t bits, primitive id, storage slot, kind (0 = miss)
    float4* acc;         // acc, rand_salt
    float4* mask;        // mask, t of the pixel's primary hit
    float4* accum;       // sum of finished samples, (sample << 16 | depth) bits
    uint32_t* prim0;     // primary-hit primitive id
    uint32_t* queue[2];
    uint32_t* count;     // [0], [1]: queue lengths; [2]: extend's fetch cursor
    uint32_t* scene_of;  // batched: scene index of each slot (written by generate)
};

struct WfConfig {
    int tie, bvh, stats;
    int multi;                // batched: per-slot scene table
    int has_emitters;         // some scene has emissive spheres (shade needs a traversal stack)
    int wide;                 // extend's BVH: WF_WIDTH_2 (binary), WF_WIDTH_4 or WF_WIDTH_8 (every scene has it)
    uint32_t cw8_stack;       // WF_WIDTH_8: the extend kernel's stack entries (the 8-wide depth; 0 = the
                              // launch's stack_depth, which the shade and finishing kernels use)
    uint32_t block;           // extend kernel threads per block: 64, 128 or 256
    uint32_t extend_grid, shade_grid;
    uint32_t finish_grid;     // blocks of 128 threads of the finishing kernel
    const TraceArgs* slots;   // batched: device table of per-scene arguments
    uint32_t nslots;
};

cudaError_t wf_launch_generate(const TraceArgs& a, const WfState& s, const WfConfig& c, cudaStream_t st);
cudaError_t wf_launch_extend(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st);
cudaError_t wf_launch_shade(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st);
cudaError_t wf_launch_finish(const TraceArgs& a, const WfState& s, const WfConfig& c, int qsel, cudaStream_t st);
int wf_extend_blocks_per_sm(const WfConfig& c, uint32_t stack_depth);
int wf_finish_blocks_per_sm(const WfConfig& c, uint32_t stack_depth);

}  // namespace vkt
