// Present pass and progressive accumulation launchers (tracer_present.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vkt {

struct PresentArgs {
    uint32_t src_w, src_h;  // source images (row 0 = bottom, as the trace writes them)
    uint32_t width, height; // framebuffer (row 0 = top)
    uchar4* out8;           // RGBA8 UNORM output, or NULL
    float4* out32;          // float output, or NULL
};

// img0 = the image bound as raytraced_image, img1 = prev_raytraced_image;
// both uchar4 (RGBA8 UNORM) or both float4.
cudaError_t launch_present(const PresentArgs& p, const void* img0, const void* img1, int src_float, cudaStream_t st);
cudaError_t launch_accumulate(const float4* lin, float4* sum, float4* disp, uint32_t npx, uint32_t n, int sm_count,
                              cudaStream_t st);

}  // namespace vkt
