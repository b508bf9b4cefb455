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
};

// Adds the primary-visibility boundary term of dL/d(camera position) over
// every triangle edge of a.sc to e.gcam.
cudaError_t launch_edge_campos(const TraceArgs& a, const EdgeArgs& e, int tie, int bvh, cudaStream_t st);

}  // namespace vkt
