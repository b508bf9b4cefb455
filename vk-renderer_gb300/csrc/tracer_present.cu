// The steps after the compute dispatch, for sm_103a:
//
//   k_present     the reference's present pass, Assets/Fullscreen.frag, over
//                 a headless framebuffer: per output pixel, the fragment's
//                 uv (Fullscreen.vert:8-10 draws one triangle over the
//                 viewport), flipped vertically (:16), five bilinear taps of
//                 the current image and one of the previous image (:18-24),
//                 the temporal variance vT (:26) and either the four-tap
//                 average or the centre tap (:28).
//   k_accumulate  progressive accumulation: the running sum of the frames'
//                 linear radiance and its tonemapped mean, which the present
//                 pass then reads in place of the two frame images.
//
// Sampling restates the reference's sampler (Source/GraphicsDevice.cpp:
// 770-790: linear filter, clamp-to-border with opaque black) from the texel
// filtering equations of the Vulkan specification, with exact float weights:
//   u = s * width - 0.5, i0 = floor(u), alpha = u - i0 (likewise v, j0, beta)
//   tau = (1-a)(1-b) T[i0,j0] + a(1-b) T[i0+1,j0] + (1-a) b T[i0,j0+1] + a b T[i0+1,j0+1]
// An RGBA8 UNORM texel c reads as c / 255.  Every operation is one IEEE
// single-precision operation in the order written (--fmad=false), so the
// output is bit-identical to the oracle's.
//
// Both kernels stream their images once; taps of neighbouring threads share
// texels through L1, so the DRAM traffic is the two source images plus the
// output (HBM-bound; a few microseconds at 1024 x 1024).

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_present.h"

namespace vkt {

// c / 255 for the 256 UNORM8 codes (IEEE division, computed once per block
// into shared memory: the same values as dividing per texel)
struct Unorm {
    const float* lut;
};

__device__ __forceinline__ V3 texel(const uchar4* im, uint32_t w, uint32_t h, int i, int j, Unorm u)
{
    if (i < 0 || j < 0 || i >= (int)w || j >= (int)h) return splat(0.0f);
    const uchar4 c = __ldg(im + (size_t)j * w + i);
    return v3(u.lut[c.x], u.lut[c.y], u.lut[c.z]);
}

__device__ __forceinline__ V3 texel(const float4* im, uint32_t w, uint32_t h, int i, int j, Unorm)
{
    if (i < 0 || j < 0 || i >= (int)w || j >= (int)h) return splat(0.0f);
    return v3(__ldg(im + (size_t)j * w + i));
}

template <class T>
__device__ __forceinline__ V3 bilinear(const T* im, uint32_t w, uint32_t h, float s, float t, Unorm un)
{
    const float u = s * (float)w - 0.5f;
    const float v = t * (float)h - 0.5f;
    const float fi = floorf(u), fj = floorf(v);
    const float al = u - fi, be = v - fj;
    const int i0 = (int)fi, j0 = (int)fj;
    const float w00 = (1.0f - al) * (1.0f - be);
    const float w10 = al * (1.0f - be);
    const float w01 = (1.0f - al) * be;
    const float w11 = al * be;
    const V3 a = texel(im, w, h, i0, j0, un), b = texel(im, w, h, i0 + 1, j0, un);
    const V3 c = texel(im, w, h, i0, j0 + 1, un), d = texel(im, w, h, i0 + 1, j0 + 1, un);
    return ((a * w00 + b * w10) + c * w01) + d * w11;
}

template <class T>
__global__ void __launch_bounds__(256) k_present(PresentArgs p, const T* __restrict__ img0, const T* __restrict__ img1)
{
    __shared__ float lut[256];
    for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = (float)i / 255.0f;
    __syncthreads();
    const Unorm un{lut};
    const uint32_t x = blockIdx.x * 32 + (threadIdx.x & 31);
    const uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= p.width || y >= p.height) return;
    const float s = ((float)x + 0.5f) / (float)p.width;
    const float t = 1.0f - ((float)y + 0.5f) / (float)p.height;
    const float inv = 1.0f / 2048.0f;  // Fullscreen.frag:12, half a texel of the reference's 1024^2 image
    const V3 c0 = bilinear(img0, p.src_w, p.src_h, s, t, un);
    const V3 c1 = bilinear(img1, p.src_w, p.src_h, s, t, un);
    const V3 d = c0 - c1;
    const float vT = dot(d, d);
    V3 f = c0;
    if (vT > 0.0005f) {  // the four taps are only read where the variance test fires
        const V3 n = bilinear(img0, p.src_w, p.src_h, s + 0.0f * inv, t + 1.0f * inv, un);
        const V3 so = bilinear(img0, p.src_w, p.src_h, s + 0.0f * inv, t + -1.0f * inv, un);
        const V3 e = bilinear(img0, p.src_w, p.src_h, s + 1.0f * inv, t + 0.0f * inv, un);
        const V3 w = bilinear(img0, p.src_w, p.src_h, s + -1.0f * inv, t + 0.0f * inv, un);
        f = (((n + so) + e) + w) / 4.0f;
    }
    const size_t o = (size_t)y * p.width + x;
    if (p.out8) p.out8[o] = make_uchar4(unorm8(f.x), unorm8(f.y), unorm8(f.z), 255);
    if (p.out32) p.out32[o] = make_float4(f.x, f.y, f.z, 1.0f);
}

// sum += linear; display = tonemap(sum / n) (Tracer.comp:586-588 without the
// dither).  Grid-stride over pixels.
__global__ void __launch_bounds__(256) k_accumulate(const float4* __restrict__ lin, float4* __restrict__ sum,
                                                    float4* __restrict__ disp, uint32_t npx, uint32_t n)
{
    const float gam = 1.0f / 2.2f;
    const float fn = (float)n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x) {
        const float4 l = lin[i];
        float4 s = sum[i];
        s.x = s.x + l.x;
        s.y = s.y + l.y;
        s.z = s.z + l.z;
        s.w = 1.0f;
        sum[i] = s;
        V3 m = v3(s.x / fn, s.y / fn, s.z / fn);
        m = m / (m + splat(1.0f));
        disp[i] = make_float4(powf(m.x, gam), powf(m.y, gam), powf(m.z, gam), 1.0f);
    }
}

cudaError_t launch_present(const PresentArgs& p, const void* img0, const void* img1, int src_float, cudaStream_t st)
{
    const dim3 grid((p.width + 31) / 32, (p.height + 7) / 8);
    if (src_float)
        k_present<float4><<<grid, 256, 0, st>>>(p, static_cast<const float4*>(img0), static_cast<const float4*>(img1));
    else
        k_present<uchar4><<<grid, 256, 0, st>>>(p, static_cast<const uchar4*>(img0), static_cast<const uchar4*>(img1));
    return cudaGetLastError();
}

cudaError_t launch_accumulate(const float4* lin, float4* sum, float4* disp, uint32_t npx, uint32_t n, int sm_count,
                              cudaStream_t st)
{
    const uint32_t need = (npx + 255) / 256;
    const uint32_t cap = 8u * (uint32_t)sm_count;
    k_accumulate<<<need < cap ? need : cap, 256, 0, st>>>(lin, sum, disp, npx, n);
    return cudaGetLastError();
}

}  // namespace vkt
