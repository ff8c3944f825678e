// Device arithmetic shared by the kernels.
//
// All translation units are compiled with -fmad=false: a product followed by
// a sum is rounded twice, exactly as the reference's expressions read, so the
// kernels reproduce the CPU restatement bit for bit.  Where a fused
// multiply-add is intended it is written explicitly (fmaf).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vsc {

// exp(x) in single precision: Cody & Waite range reduction x = k*ln2 + r with
// ln2 split into a 16-bit head and its tail, the degree-7 Taylor polynomial
// of exp(r) on |r| <= ln2/2 in Horner form (truncation < 1e-8 relative,
// result within 0.6 ulp of exp), and scaling by 2^k through the exponent
// field.  Results below 2^-126 flush to zero — every caller clamps values
// below 1e-3 to zero, so the flush never reaches an output.
__device__ __forceinline__ float expf_cw(float x)
{
    if (x != x)
        return x;
    if (x > 88.72283f)
        return __int_as_float(0x7f800000);
    if (x < -87.33654f)
        return 0.0f;
    const float kf = rintf(__fmul_rn(x, 1.44269502f));
    float r = fmaf(kf, -0.693145751953125f, x);
    r = fmaf(kf, -1.42860682e-6f, r);
    float p = 1.98412701e-4f;
    p = fmaf(p, r, 1.38888892e-3f);
    p = fmaf(p, r, 8.33333377e-3f);
    p = fmaf(p, r, 4.16666679e-2f);
    p = fmaf(p, r, 1.66666672e-1f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int k = static_cast<int>(kf);
    if (k > 127) {
        p = p * 2.0f;
        k -= 1;
    }
    return p * __int_as_float((k + 127) << 23);
}

// expf_cw for an argument known to be <= 0 and not NaN: the same value for
// x >= -87.33654 (the NaN, overflow and k > 127 branches cannot apply);
// below, expf_cw gives 0 and this expf_cw(-87.33654) = 2^-126, which every
// caller's cut at 0.001 (also after a factor of magnitude <= 1e30) turns
// into the same 0.
__device__ __forceinline__ float expf_cw_nonpos(float x)
{
    x = fmaxf(x, -87.33654f);
    const float kf = rintf(__fmul_rn(x, 1.44269502f));
    float r = fmaf(kf, -0.693145751953125f, x);
    r = fmaf(kf, -1.42860682e-6f, r);
    float p = 1.98412701e-4f;
    p = fmaf(p, r, 1.38888892e-3f);
    p = fmaf(p, r, 8.33333377e-3f);
    p = fmaf(p, r, 4.16666679e-2f);
    p = fmaf(p, r, 1.66666672e-1f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return p * __int_as_float((static_cast<int>(kf) + 127) << 23);
}

// Programmatic dependent launch: wait until the preceding kernel of the stream
// has completed (its writes visible), then let the following kernel be
// scheduled, so that its launch overlaps this kernel.  The following kernel
// can start only once every block of this one has started, so a waiting grid
// never holds resources this one still needs.  Without the launch attribute
// both instructions do nothing.
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" :::);
}

// Asks L2 for the line holding *p (a hint: no result, nothing waits for it).
// A gather kernel issues it for its own pixel's position in each source
// before the flow read, so the source lines come from DRAM while the flow
// is in flight and the taps, near that position, find them in L2.
__device__ __forceinline__ void prefetch_l2(const void* p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ int64_t pix_index(int x, int y, int w) { return static_cast<int64_t>(y) * w + x; }

// The flow estimator's coarse-to-fine step: channel ch of the 2-channel
// planar sw x sh flow `in` upsampled 2x at pixel (x, y) (half-pixel centres,
// clamped taps) and doubled -- the value the estimator's upsampled flow holds
// there, computed where it is used.
__device__ __forceinline__ float up2_sample(const float* __restrict__ in, int sw, int sh, int x, int y, int ch)
{
    float sx = (static_cast<float>(x) + 0.5f) * 0.5f - 0.5f;
    float sy = (static_cast<float>(y) + 0.5f) * 0.5f - 0.5f;
    if (sx < 0.0f)
        sx = 0.0f;
    if (sy < 0.0f)
        sy = 0.0f;
    int x0 = static_cast<int>(floorf(sx)), y0 = static_cast<int>(floorf(sy));
    if (x0 > sw - 1)
        x0 = sw - 1;
    if (y0 > sh - 1)
        y0 = sh - 1;
    const int x1 = x0 + 1 < sw ? x0 + 1 : sw - 1;
    const int y1 = y0 + 1 < sh ? y0 + 1 : sh - 1;
    const float lx = sx - static_cast<float>(x0), ly = sy - static_cast<float>(y0);
    const float* s = in + static_cast<int64_t>(ch) * sw * sh;
    const float top = (1.0f - lx) * s[static_cast<int64_t>(y0) * sw + x0] + lx * s[static_cast<int64_t>(y0) * sw + x1];
    const float bot = (1.0f - lx) * s[static_cast<int64_t>(y1) * sw + x0] + lx * s[static_cast<int64_t>(y1) * sw + x1];
    return ((1.0f - ly) * top + ly * bot) * 2.0f;
}

// One output pixel of kernel_bilinear (flowconsistency.cu:50-75): the c
// channels of the iw x ih image `in` sampled at (ox * iw / ow, oy * ih / oh),
// taps clamped to the last row and column, in the reference's expression.
__device__ __forceinline__ void bilinear_px(const float* __restrict__ in, int iw, int ih, int ow, int oh, int c,
    int ox, int oy, float* __restrict__ dst)
{
    const float xx = static_cast<float>(ox) * static_cast<float>(iw) / static_cast<float>(ow);
    const float yy = static_cast<float>(oy) * static_cast<float>(ih) / static_cast<float>(oh);
    // xx < iw for every size the API accepts; the clamp only guards the index
    const int ix = min(static_cast<int>(floorf(xx)), iw - 1);
    const int iy = min(static_cast<int>(floorf(yy)), ih - 1);
    const float fx = xx - static_cast<float>(ix);
    const float fy = yy - static_cast<float>(iy);
    const int ix1 = min(ix + 1, iw - 1);
    const int iy1 = min(iy + 1, ih - 1);
    for (int k = 0; k < c; ++k) {
        const float v00 = in[pix_index(ix, iy, iw) * c + k];
        const float v10 = in[pix_index(ix1, iy, iw) * c + k];
        const float v01 = in[pix_index(ix, iy1, iw) * c + k];
        const float v11 = in[pix_index(ix1, iy1, iw) * c + k];
        dst[k] = v00 * (1 - fx) * (1 - fy) + v10 * fx * (1 - fy) + v01 * (1 - fx) * fy + v11 * fx * fy;
    }
}

// RGBA8 quantisation of gpuimage.cu:64: (uint8)__float2uint_rd(|v| * 255),
// alpha = 1.
__device__ __forceinline__ uint8_t quantize(float v)
{
    return static_cast<uint8_t>(__float2uint_rd(fabsf(v) * 255.0f));
}

__device__ __forceinline__ uint32_t pack_rgba(float r, float g, float b)
{
    return static_cast<uint32_t>(quantize(r)) | (static_cast<uint32_t>(quantize(g)) << 8) |
           (static_cast<uint32_t>(quantize(b)) << 16) | (1u << 24);
}

}  // namespace vsc
