// Learned 2x flow upsampler for the FLOWDOWNSCALE fast mode (no counterpart
// in the reference, whose fast mode upsamples the flow bilinearly,
// flowmodel.cpp:158-161).
//
// Input at the full resolution: the bilinear upsampling of the coarse flow
// with its vectors scaled to the full-resolution grid (the "base" flow) and
// the luma of the full-resolution frame.  Four 3x3 convolutions (3 -> 32 ->
// 32 -> 32 -> 2, zero padding, ReLU between) predict a residual r; the
// output flow is base + r where max(|r_u|, |r_v|) <= max_residual, else the
// base flow (the bilinear fallback).  19,970 parameters, kept in FP32 for
// training and rounded to FP16 for inference.
//
// The training kernels are written here, in FP32: direct convolutions on the
// CUDA cores over NHWC activations (one thread per pixel, the layer's weights
// in shared memory, fused multiply-adds), a backward pass for the data and
// the weights, an L1 loss against the full-resolution flow and Adam.  The
// input preparation is shared with the inference, which runs on the tensor
// cores (vsc_upsampler_tc.cu).  Nothing here has a bit-exact contract
// (contraction is spelled out with __fmaf_rn, the library being built
// without automatic contraction).
#include "vsc_internal.h"
#include "vsc_math.cuh"

#include <cuda_fp16.h>

#include <cmath>
#include <vector>

namespace vsc {
namespace {

constexpr int kParams = 19970;
static_assert(kUpLayers[3].b_off + 2 == kParams, "parameter layout");
constexpr int kThreads = 128;

__device__ __forceinline__ float luma(const float* p) { return 0.299f * p[0] + 0.587f * p[1] + 0.114f * p[2]; }

// ---- input: base flow and luma ------------------------------------------------------
// base = bilinear(coarse) at the frame's size (kernel_bilinear's sampling,
// flowconsistency.cu:50-75) times the size ratio per axis.
__global__ void prepare_kernel(const float* __restrict__ coarse, int cw, int ch, int cfc, const float* __restrict__ img,
    float* __restrict__ input, int w, int h, int64_t s_coarse, int64_t s_img, int64_t s_in)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int n = blockIdx.z;
    if (x >= w || y >= h)
        return;
    const float* cf = coarse + n * s_coarse;
    const float xx = static_cast<float>(x) * static_cast<float>(cw) / static_cast<float>(w);
    const float yy = static_cast<float>(y) * static_cast<float>(ch) / static_cast<float>(h);
    const int ix = min(static_cast<int>(floorf(xx)), cw - 1), iy = min(static_cast<int>(floorf(yy)), ch - 1);
    const float fx = xx - static_cast<float>(ix), fy = yy - static_cast<float>(iy);
    const int ix1 = min(ix + 1, cw - 1), iy1 = min(iy + 1, ch - 1);
    const float sx = static_cast<float>(w) / static_cast<float>(cw), sy = static_cast<float>(h) / static_cast<float>(ch);
    float v[2];
    for (int k = 0; k < 2; ++k) {
        const float v00 = cf[pix_index(ix, iy, cw) * cfc + k], v10 = cf[pix_index(ix1, iy, cw) * cfc + k];
        const float v01 = cf[pix_index(ix, iy1, cw) * cfc + k], v11 = cf[pix_index(ix1, iy1, cw) * cfc + k];
        v[k] = v00 * (1 - fx) * (1 - fy) + v10 * fx * (1 - fy) + v01 * (1 - fx) * fy + v11 * fx * fy;
    }
    float* o = input + n * s_in + pix_index(x, y, w) * 3;
    o[0] = v[0] * sx;
    o[1] = v[1] * sy;
    o[2] = luma(img + n * s_img + pix_index(x, y, w) * 3);
}

// ---- forward: one 3x3 convolution, NHWC, batch n along blockIdx.y ---------------------
template <int CI, int CO, bool kRelu, typename WT>
__global__ void __launch_bounds__(kThreads) conv_fwd_kernel(const float* __restrict__ x, const WT* __restrict__ wts,
    const float* __restrict__ bias, float* __restrict__ y, int H, int W)
{
    __shared__ float sw[CO * 9 * CI];
    __shared__ float sb[CO];
    for (int i = threadIdx.x; i < CO * 9 * CI; i += blockDim.x)
        sw[i] = static_cast<float>(wts[i]);
    for (int i = threadIdx.x; i < CO; i += blockDim.x)
        sb[i] = bias[i];
    __syncthreads();
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= HW)
        return;
    const int n = blockIdx.y;
    const int py = static_cast<int>(p / W), px = static_cast<int>(p % W);
    const float* xb = x + n * HW * CI;
    float acc[CO];
#pragma unroll
    for (int o = 0; o < CO; ++o)
        acc[o] = sb[o];
    for (int t = 0; t < 9; ++t) {
        const int yy = py + t / 3 - 1, xx = px + t % 3 - 1;
        if (yy < 0 || yy >= H || xx < 0 || xx >= W)
            continue;
        const float* xs = xb + (static_cast<int64_t>(yy) * W + xx) * CI;
#pragma unroll 4
        for (int c = 0; c < CI; ++c) {
            const float xv = xs[c];
#pragma unroll
            for (int o = 0; o < CO; ++o)
                acc[o] = __fmaf_rn(sw[(o * 9 + t) * CI + c], xv, acc[o]);
        }
    }
    float* yo = y + (n * HW + p) * CO;
#pragma unroll
    for (int o = 0; o < CO; ++o)
        yo[o] = kRelu ? fmaxf(acc[o], 0.0f) : acc[o];
}

// ---- backward ---------------------------------------------------------------------------
// dz_prev = (sum over taps and output channels of w * dz) * (a_prev > 0)
template <int CI, int CO, bool kMask>
__global__ void __launch_bounds__(kThreads) conv_bwd_data_kernel(const float* __restrict__ dz,
    const float* __restrict__ wts, const float* __restrict__ a_prev, float* __restrict__ dz_prev, int H, int W)
{
    __shared__ float sw[CO * 9 * CI];
    for (int i = threadIdx.x; i < CO * 9 * CI; i += blockDim.x)
        sw[i] = wts[i];
    __syncthreads();
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= HW)
        return;
    const int n = blockIdx.y;
    const int py = static_cast<int>(p / W), px = static_cast<int>(p % W);
    float acc[CI];
#pragma unroll
    for (int c = 0; c < CI; ++c)
        acc[c] = 0.0f;
    for (int t = 0; t < 9; ++t) {
        // the output pixel whose tap t read this pixel
        const int yy = py - (t / 3 - 1), xx = px - (t % 3 - 1);
        if (yy < 0 || yy >= H || xx < 0 || xx >= W)
            continue;
        const float* g = dz + (n * HW + static_cast<int64_t>(yy) * W + xx) * CO;
        for (int o = 0; o < CO; ++o) {
            const float gv = g[o];
#pragma unroll
            for (int c = 0; c < CI; ++c)
                acc[c] = __fmaf_rn(sw[(o * 9 + t) * CI + c], gv, acc[c]);
        }
    }
    const float* ap = a_prev + (n * HW + p) * CI;
    float* out = dz_prev + (n * HW + p) * CI;
#pragma unroll
    for (int c = 0; c < CI; ++c)
        out[c] = (!kMask || ap[c] > 0.0f) ? acc[c] : 0.0f;
}

// dw[o][t][c] += sum over pixels of dz[o] * x[tap t][c]; db[o] += sum dz[o].
// Block (o, t) over a slice of the pixels (blockIdx.z), reduced in shared
// memory, one atomic add per weight and block.
template <int CI, int CO>
__global__ void __launch_bounds__(kThreads) conv_wgrad_kernel(const float* __restrict__ x, const float* __restrict__ dz,
    float* __restrict__ dw, float* __restrict__ db, int N, int H, int W)
{
    __shared__ float red[kThreads][CI + 1];
    const int o = blockIdx.x, t = blockIdx.y;
    const int dy = t / 3 - 1, dx = t % 3 - 1;
    const int64_t HW = static_cast<int64_t>(H) * W, total = N * HW;
    const int64_t chunk = (total + gridDim.z - 1) / gridDim.z;
    const int64_t p0 = blockIdx.z * chunk, p1 = min(total, p0 + chunk);
    float acc[CI + 1];
#pragma unroll
    for (int c = 0; c <= CI; ++c)
        acc[c] = 0.0f;
    for (int64_t q = p0 + threadIdx.x; q < p1; q += blockDim.x) {
        const int64_t n = q / HW, p = q % HW;
        const int py = static_cast<int>(p / W), px = static_cast<int>(p % W);
        const float g = dz[q * CO + o];
        acc[CI] += g;
        const int yy = py + dy, xx = px + dx;
        if (g == 0.0f || yy < 0 || yy >= H || xx < 0 || xx >= W)
            continue;
        const float* xs = x + (n * HW + static_cast<int64_t>(yy) * W + xx) * CI;
#pragma unroll
        for (int c = 0; c < CI; ++c)
            acc[c] = __fmaf_rn(g, xs[c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c <= CI; ++c)
        red[threadIdx.x][c] = acc[c];
    __syncthreads();
    for (int c = threadIdx.x; c <= CI; c += blockDim.x) {
        float s = 0.0f;
        for (int i = 0; i < kThreads; ++i)
            s += red[i][c];
        if (c < CI)
            atomicAdd(&dw[(o * 9 + t) * CI + c], s);
        else if (t == 0)
            atomicAdd(&db[o], s);
    }
}

// L1 loss of base + r against the target flow; dr = sign / (pixels); loss summed.
__global__ void loss_kernel(const float* __restrict__ input, const float* __restrict__ r,
    const float* __restrict__ target, float* __restrict__ dr, float* __restrict__ loss, int64_t npx, float inv)
{
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    float l = 0.0f;
    if (p < npx) {
        for (int k = 0; k < 2; ++k) {
            const float d = input[p * 3 + k] + r[p * 2 + k] - target[p * 2 + k];
            l += fabsf(d);
            dr[p * 2 + k] = d > 0.0f ? inv : (d < 0.0f ? -inv : 0.0f);
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(loss, l * inv);
}

__global__ void adam_kernel(float* __restrict__ prm, const float* __restrict__ g, float* __restrict__ m,
    float* __restrict__ v, int n, float lr, float b1, float b2, float c1, float c2, float eps)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float gi = g[i];
    m[i] = b1 * m[i] + (1.0f - b1) * gi;
    v[i] = b2 * v[i] + (1.0f - b2) * gi * gi;
    prm[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}

uint64_t splitmix(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// weights: the layers' weight arrays (parameter layout offsets) in type WT
template <typename WT>
cudaError_t forward(const WT* wts, const float* prm, const float* input, float* a1, float* a2, float* a3, float* r,
    int N, int H, int W, cudaStream_t st)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    const dim3 g(static_cast<unsigned>((HW + kThreads - 1) / kThreads), N);
    const WT* w0 = wts + kUpLayers[0].w_off;
    const WT* w1 = wts + kUpLayers[1].w_off;
    const WT* w2 = wts + kUpLayers[2].w_off;
    const WT* w3 = wts + kUpLayers[3].w_off;
    conv_fwd_kernel<3, 32, true, WT><<<g, kThreads, 0, st>>>(input, w0, prm + kUpLayers[0].b_off, a1, H, W);
    conv_fwd_kernel<32, 32, true, WT><<<g, kThreads, 0, st>>>(a1, w1, prm + kUpLayers[1].b_off, a2, H, W);
    conv_fwd_kernel<32, 32, true, WT><<<g, kThreads, 0, st>>>(a2, w2, prm + kUpLayers[2].b_off, a3, H, W);
    conv_fwd_kernel<32, 2, false, WT><<<g, kThreads, 0, st>>>(a3, w3, prm + kUpLayers[3].b_off, r, H, W);
    return cudaGetLastError();
}

}  // namespace

int upsampler_param_count() { return kParams; }

void upsampler_init_params(float* host, uint64_t seed)
{
    uint64_t s = seed;
    for (const UpLayer& l : kUpLayers) {
        const float bound = std::sqrt(6.0f / static_cast<float>(9 * l.ci));  // He-uniform
        for (int i = 0; i < l.co * 9 * l.ci; ++i)
            host[l.w_off + i] = (static_cast<float>(splitmix(&s) >> 40) * (1.0f / 16777216.0f) * 2.0f - 1.0f) * bound;
        for (int i = 0; i < l.co; ++i)
            host[l.b_off + i] = 0.0f;
    }
    // the last layer starts near zero: the initial prediction is the base flow
    for (int i = 0; i < kUpLayers[3].co * 9 * kUpLayers[3].ci; ++i)
        host[kUpLayers[3].w_off + i] *= 0.01f;
}

cudaError_t launch_upsampler_prepare(const float* coarse, int cw, int ch, int cfc, const float* img, float* input, int w,
    int h, int N, int64_t s_coarse, int64_t s_img, int64_t s_in, cudaStream_t st)
{
    const dim3 b(32, 8);
    const dim3 g((w + 31) / 32, (h + 7) / 8, N);
    prepare_kernel<<<g, b, 0, st>>>(coarse, cw, ch, cfc, img, input, w, h, s_coarse, s_img, s_in);
    return cudaGetLastError();
}

// One Adam step on a batch: forward, L1 loss, backward, update.
// work: upsampler_act_floats(N,H,W) * 2 + kParams * 2 (+ slack) floats.
cudaError_t upsampler_train_step(float* prm, float* grad, float* m, float* v, int step, const float* input,
    const float* target, int N, int H, int W, float lr, float* work, float* loss_dev, cudaStream_t st)
{
    const int64_t px = static_cast<int64_t>(N) * H * W;
    float* a1 = work;
    float* a2 = a1 + px * 32;
    float* a3 = a2 + px * 32;
    float* r = a3 + px * 32;
    float* dr = r + px * 2;
    float* dz3 = dr + px * 2;
    float* dz2 = dz3 + px * 32;
    float* dz1 = dz2 + px * 32;
    cudaError_t e = forward<float>(prm, prm, input, a1, a2, a3, r, N, H, W, st);
    if (e != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(grad, 0, kParams * sizeof(float), st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(loss_dev, 0, sizeof(float), st)) != cudaSuccess)
        return e;
    loss_kernel<<<static_cast<unsigned>((px + 255) / 256), 256, 0, st>>>(input, r, target, dr, loss_dev, px,
        1.0f / static_cast<float>(px));
    const int64_t HW = static_cast<int64_t>(H) * W;
    const dim3 g(static_cast<unsigned>((HW + kThreads - 1) / kThreads), N);
    const unsigned slices = static_cast<unsigned>(std::min<int64_t>(64, (px + 4095) / 4096));
    // layer 4 (32 -> 2)
    conv_wgrad_kernel<32, 2><<<dim3(2, 9, slices), kThreads, 0, st>>>(a3, dr, grad + kUpLayers[3].w_off,
        grad + kUpLayers[3].b_off, N, H, W);
    conv_bwd_data_kernel<32, 2, true><<<g, kThreads, 0, st>>>(dr, prm + kUpLayers[3].w_off, a3, dz3, H, W);
    // layer 3
    conv_wgrad_kernel<32, 32><<<dim3(32, 9, slices), kThreads, 0, st>>>(a2, dz3, grad + kUpLayers[2].w_off,
        grad + kUpLayers[2].b_off, N, H, W);
    conv_bwd_data_kernel<32, 32, true><<<g, kThreads, 0, st>>>(dz3, prm + kUpLayers[2].w_off, a2, dz2, H, W);
    // layer 2
    conv_wgrad_kernel<32, 32><<<dim3(32, 9, slices), kThreads, 0, st>>>(a1, dz2, grad + kUpLayers[1].w_off,
        grad + kUpLayers[1].b_off, N, H, W);
    conv_bwd_data_kernel<32, 32, true><<<g, kThreads, 0, st>>>(dz2, prm + kUpLayers[1].w_off, a1, dz1, H, W);
    // layer 1 (3 -> 32): weights only
    conv_wgrad_kernel<3, 32><<<dim3(32, 9, slices), kThreads, 0, st>>>(input, dz1, grad + kUpLayers[0].w_off,
        grad + kUpLayers[0].b_off, N, H, W);
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, static_cast<float>(step)), c2 = 1.0f - std::pow(b2, static_cast<float>(step));
    adam_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(prm, grad, m, v, kParams, lr, b1, b2, c1, c2, 1e-8f);
    return cudaGetLastError();
}

size_t upsampler_train_work_floats(int N, int H, int W)
{
    const size_t px = static_cast<size_t>(N) * H * W;
    return px * (32 * 3 + 2 + 2 + 32 * 3);
}

}  // namespace vsc
