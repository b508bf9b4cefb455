// Boundary term of the camera-position gradient (tracer_edges.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vkt {

struct TraceArgs;

struct EdgeArgs {
    const float4* dldi;  // dL/dI per pixel (alpha ignored)
    double* gcam;        // the three camera-position sums (FP64), added to
    float binv[9];       // inverse of the 3x3 matrix whose columns are the camera's dir, right and up (row-major)
    uint32_t samples;    // stratified samples per edge
    float offset_px;     // distance of the inside / outside rays from the outline, in pixels
    float4* segs;        // visible outline parts found by the walk, 3 float4 each (EdgeSeg), for the
                         // second kernel to evaluate; nullptr = the walking thread evaluates them
    uint32_t* nsegs;     // their count (zeroed before the walk); parts beyond seg_cap are evaluated in place
    uint32_t seg_cap;
};

// Adds the primary-visibility boundary term of dL/d(camera position) over
// every triangle edge of a.sc to e.gcam: a walk along every edge's image
// that finds the visible outline parts, then (with e.segs) a second kernel
// that evaluates the pixel on both sides of each part, one part per thread.
cudaError_t launch_edge_campos(const TraceArgs& a, const EdgeArgs& e, int tie, int bvh, cudaStream_t st);

}  // namespace vkt
