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
// k_present reads each source texel from DRAM once (taps of neighbouring
// threads share texels through L1) and is bound by instruction issue: six
// bilinear taps of twelve texel channels each.  Hence the UNORM conversion
// and the floor / float-to-int steps below avoid the conversion unit (its
// throughput is an eighth of the FMA pipe's), and the four neighbour taps are
// only evaluated where the variance test needs them.

#include <cuda_runtime.h>

#include "tracer_core.cuh"
#include "tracer_present.h"

namespace vkt {

// c / 255, correctly rounded, for the UNORM8 codes c = 0..255: q = c * (1/255)
// and one residual correction (Markstein's method: r = c - 255 q exactly by
// fma, q + r / 255 ~ q + r * (1/255)).  Equal to the IEEE quotient for all 256
// codes (checked exhaustively with exact rational arithmetic), three
// instructions instead of a division.  The byte becomes a float without the
// conversion unit: one byte permute builds the float 2^23 + c, and
// subtracting 2^23 leaves c exactly.
template <int K>
__device__ __forceinline__ float unorm_to_float(uint32_t word)
{
    const float fc = __uint_as_float(__byte_perm(word, 0x4B000000u, K | (4 << 4) | (4 << 8) | (7 << 12))) - 8388608.0f;
    const float inv = 1.0f / 255.0f;
    const float q = fc * inv;
    const float r = __fmaf_rn(-q, 255.0f, fc);
    return __fmaf_rn(r, inv, q);
}

__device__ __forceinline__ V3 texel_at(const uchar4* im, size_t k)
{
    const uint32_t c = __ldg(reinterpret_cast<const uint32_t*>(im) + k);  // R in the low byte
    return v3(unorm_to_float<0>(c), unorm_to_float<1>(c), unorm_to_float<2>(c));
}
__device__ __forceinline__ V3 texel_at(const float4* im, size_t k) { return v3(__ldg(im + k)); }

// floor(x) and (int)x of an integer-valued x, for |x| < 2^22, on the FMA and
// integer pipes (adding 1.5 x 2^23 rounds x to an integer in the low mantissa
// bits): the same values as floorf and the float-to-int conversion.
__device__ __forceinline__ float floor_small(float x)
{
    const float r = (x + 12582912.0f) - 12582912.0f;  // x rounded to the nearest integer
    return r > x ? r - 1.0f : r;
}
__device__ __forceinline__ int int_of_small(float x) { return __float_as_int(x + 12582912.0f) - 0x4B400000; }

template <class T>
__device__ __forceinline__ V3 texel(const T* im, uint32_t w, uint32_t h, int i, int j)
{
    if (i < 0 || j < 0 || i >= (int)w || j >= (int)h) return splat(0.0f);  // border: black
    return texel_at(im, (size_t)j * w + i);
}

// fw, fh: the image size as floats (exact below 2^24)
template <class T>
__device__ __forceinline__ V3 bilinear(const T* im, uint32_t w, uint32_t h, float fw, float fh, float s, float t)
{
    const float u = s * fw - 0.5f;
    const float v = t * fh - 0.5f;
    const float fi = floor_small(u), fj = floor_small(v);
    const float al = u - fi, be = v - fj;
    const int i0 = int_of_small(fi), j0 = int_of_small(fj);
    const float w00 = (1.0f - al) * (1.0f - be);
    const float w10 = al * (1.0f - be);
    const float w01 = (1.0f - al) * be;
    const float w11 = al * be;
    V3 a, b, c, d;
    if (i0 >= 0 && j0 >= 0 && i0 + 1 < (int)w && j0 + 1 < (int)h) {  // all four inside
        const size_t k = (size_t)j0 * w + i0;
        a = texel_at(im, k);
        b = texel_at(im, k + 1);
        c = texel_at(im, k + w);
        d = texel_at(im, k + w + 1);
    } else {
        a = texel(im, w, h, i0, j0);
        b = texel(im, w, h, i0 + 1, j0);
        c = texel(im, w, h, i0, j0 + 1);
        d = texel(im, w, h, i0 + 1, j0 + 1);
    }
    return ((a * w00 + b * w10) + c * w01) + d * w11;
}

template <class T>
__global__ void __launch_bounds__(256) k_present(PresentArgs p, const T* __restrict__ img0, const T* __restrict__ img1)
{
    const uint32_t x = blockIdx.x * 32 + (threadIdx.x & 31);
    const uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= p.width || y >= p.height) return;
    const float s = ((float)x + 0.5f) / (float)p.width;
    const float t = 1.0f - ((float)y + 0.5f) / (float)p.height;
    const float inv = 1.0f / 2048.0f;  // Fullscreen.frag:12, half a texel of the reference's 1024^2 image
    const float fw = (float)p.src_w, fh = (float)p.src_h;
    const V3 c0 = bilinear(img0, p.src_w, p.src_h, fw, fh, s, t);
    const V3 c1 = bilinear(img1, p.src_w, p.src_h, fw, fh, s, t);
    const V3 d = c0 - c1;
    const float vT = dot(d, d);
    V3 f = c0;
    if (vT > 0.0005f) {  // the four taps are only read where the variance test fires
        const V3 n = bilinear(img0, p.src_w, p.src_h, fw, fh, s + 0.0f * inv, t + 1.0f * inv);
        const V3 so = bilinear(img0, p.src_w, p.src_h, fw, fh, s + 0.0f * inv, t + -1.0f * inv);
        const V3 e = bilinear(img0, p.src_w, p.src_h, fw, fh, s + 1.0f * inv, t + 0.0f * inv);
        const V3 w = bilinear(img0, p.src_w, p.src_h, fw, fh, s + -1.0f * inv, t + 0.0f * inv);
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
