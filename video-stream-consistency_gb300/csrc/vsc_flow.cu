// Weight-free optical-flow estimator built from the two operators.
//
// The reference computes flow with a PWC-Net ONNX graph that calls
// custom::Warp and custom::Correlation (model-conversion/pwc_pytorch/
// pwcnet.py:418-430, :950-967; src/stabilization/flowmodel.cpp:121-168).
// Its trained weights are not part of the reference tree, so this module
// keeps the graph's operator skeleton and replaces the learned parts:
//   pyramid   : 1/4 .. 1/64 of the frame resized to a multiple of 64
//               (convert_onnx.py:15-20), channels {32, 64, 96, 128, 196};
//   features  : L2-normalised random projections of 3x3 RGB patches made
//               zero-mean per colour (weights from a splitmix64 stream
//               seeded per level): correlations are patch NCCs;
//   per level : upsample the coarser flow (x2), Warp the second frame's
//               features by it, Correlation (max displacement 4) against the
//               first frame's features, arg-max over the 81 displacements
//               minus a small-displacement prior, soft 3x3 centroid, and a
//               confidence-weighted 3x3 mean of the refinement;
//   output    : bilinear upsampling of the 1/4-level flow to the frame size,
//               3-channel (u, v, 0) like the reference's computed flows.
// All arithmetic follows the CPU restatement operation for operation
// (-fmad=false), so the estimated flow matches it bit for bit.
#include "vsc_internal.h"
#include "vsc_math.cuh"

#include <algorithm>
#include <mutex>

namespace vsc {
namespace {

constexpr int kLevelC[kFlowLevels] = {32, 64, 96, 128, 196};
constexpr int kWeightOff[kFlowLevels] = {0, 32 * 27, 96 * 27, 192 * 27, 320 * 27};
constexpr int kWeightTotal = 516 * 27;
// decoder constants: soft-centroid sharpness, confidence floor of the
// smoothing, small-displacement prior per level (x4 per coarser level)
constexpr float kTemp = 20.0f;
constexpr float kEps = 0.1f;
constexpr float kLevelPrior[kFlowLevels] = {0.01f, 0.01f * 4.0f, 0.01f * 16.0f, 0.01f * 64.0f, 0.01f * 256.0f};

// the feature weights, in global memory: each features_kernel block stages its
// level's weights in shared memory (the small levels' 196 x 27 weights exceed
// what the constant cache keeps, and every warp would stream them from it)
__device__ float g_flow_w[kWeightTotal];

uint64_t splitmix64(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// the column (row) of the FW-wide (FH-high) frame that the nearest-neighbour
// resize to w (h) samples at x (y)
__device__ __forceinline__ int nearest_src(int x, int w, int FW)
{
    const int64_t num = (2 * static_cast<int64_t>(x) + 1) * FW;
    const int v = num < (int64_t{1} << 31) ? static_cast<int>(static_cast<int>(num) / (2 * w))
                                           : static_cast<int>(num / (2 * static_cast<int64_t>(w)));
    return min(FW - 1, v);
}

struct PyrOut {
    float* lev[kFlowLevels];
    int lw0, lh0;
};

// The estimator's image pyramid in one launch.  Level 0 (a quarter of the
// frame padded to a multiple of 64) averages 4 x 4 half-pixel bilinear
// samples of the image per pixel; level l + 1 is the 2 x 2 mean of level l.
// A block of 16 x 16 threads computes a 16 x 16 tile of level 0 and pools it
// in shared memory to the tile's pixels of levels 1-4: level 0 is a
// multiple of 16 in both directions, so each level-4 pixel comes from one
// block.  kNearest: the w x h image is the nearest-neighbour resize of the
// FW x FH frame `full` (FLOWDOWNSCALE: the reference scales the frame with
// Qt::FastTransformation, flowmodel.cpp:126-133; pixel x samples column
// min(FW - 1, (2x + 1) FW / (2w)), rows alike) and is read through that
// mapping, not from a resized copy.  Same values, same operation order as
// the restatement.
template <bool kNearest>
__global__ void __launch_bounds__(256) pyramid_kernel(const float* __restrict__ img, int w, int h,
    const float* __restrict__ full, int FW, int FH, PyrOut po)
{
    pdl_enter();
    __shared__ float t[2][16 * 16 * 3];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int x = blockIdx.x * 16 + tx, y = blockIdx.y * 16 + ty;  // inside level 0 (a multiple of 16)
    const int lw = po.lw0, lh = po.lh0;
    {
        const int pw = lw * 4, ph = lh * 4;
        const float scx = static_cast<float>(w) / static_cast<float>(pw);
        const float scy = static_cast<float>(h) / static_cast<float>(ph);
        // the 4 sample columns and rows of this pixel (half-pixel centres,
        // clamped taps), their element offsets in the source and fractions
        const float* src = kNearest ? full : img;
        const int sw = kNearest ? FW : w;
        int64_t cx0[4], cx1[4], ry0[4], ry1[4];
        float lxs[4], lys[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float sx = (static_cast<float>(x * 4 + i) + 0.5f) * scx - 0.5f;
            if (sx < 0.0f)
                sx = 0.0f;
            int x0 = static_cast<int>(floorf(sx));
            if (x0 > w - 1)
                x0 = w - 1;
            const int x1 = x0 + 1 < w ? x0 + 1 : w - 1;
            lxs[i] = sx - static_cast<float>(x0);
            cx0[i] = 3 * static_cast<int64_t>(kNearest ? nearest_src(x0, w, FW) : x0);
            cx1[i] = 3 * static_cast<int64_t>(kNearest ? nearest_src(x1, w, FW) : x1);
            float sy = (static_cast<float>(y * 4 + i) + 0.5f) * scy - 0.5f;
            if (sy < 0.0f)
                sy = 0.0f;
            int y0 = static_cast<int>(floorf(sy));
            if (y0 > h - 1)
                y0 = h - 1;
            const int y1 = y0 + 1 < h ? y0 + 1 : h - 1;
            lys[i] = sy - static_cast<float>(y0);
            ry0[i] = static_cast<int64_t>(kNearest ? nearest_src(y0, h, FH) : y0) * sw * 3;
            ry1[i] = static_cast<int64_t>(kNearest ? nearest_src(y1, h, FH) : y1) * sw * 3;
        }
        float acc[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float ly = lys[j];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float lx = lxs[i];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float v00 = src[ry0[j] + cx0[i] + k];
                    const float v01 = src[ry0[j] + cx1[i] + k];
                    const float v10 = src[ry1[j] + cx0[i] + k];
                    const float v11 = src[ry1[j] + cx1[i] + k];
                    const float top = (1.0f - lx) * v00 + lx * v01;
                    const float bot = (1.0f - lx) * v10 + lx * v11;
                    acc[k] += (1.0f - ly) * top + ly * bot;
                }
            }
        }
        float* o = po.lev[0] + (static_cast<int64_t>(y) * lw + x) * 3;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float v = acc[k] * 0.0625f;
            o[k] = v;
            t[0][(ty * 16 + tx) * 3 + k] = v;
        }
    }
    // levels 1..4: tile side 8, 4, 2, 1; source tile in t[(l - 1) & 1], side s
#pragma unroll
    for (int l = 1; l < kFlowLevels; ++l) {
        __syncthreads();
        const int s = 16 >> (l - 1), n = s >> 1;
        const float* src = t[(l - 1) & 1];
        float* dst = t[l & 1];
        if (tx < n && ty < n) {
            const int cw = lw >> l;
            const int gx = blockIdx.x * n + tx, gy = blockIdx.y * n + ty;
            float* o = po.lev[l] + (static_cast<int64_t>(gy) * cw + gx) * 3;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float a = src[((2 * ty) * s + 2 * tx) * 3 + k];
                const float b = src[((2 * ty) * s + 2 * tx + 1) * 3 + k];
                const float c = src[((2 * ty + 1) * s + 2 * tx) * 3 + k];
                const float e = src[((2 * ty + 1) * s + 2 * tx + 1) * 3 + k];
                const float v = ((a + b) + (c + e)) * 0.25f;
                o[k] = v;
                dst[(ty * n + tx) * 3 + k] = v;
            }
        }
    }
}

// Block (32 pixels of one row) x (8 channel groups).  Every thread builds
// its pixel's zero-mean patch; the warp of group g computes channels
// g, g+8, g+16, ... (uniform constant-bank reads); the squared norm is then
// summed by one thread per pixel in channel order, as the restatement does.
constexpr int kFeatGroups = 8;
constexpr int kFeatMaxC = 196;

// The five levels' features in one launch: a flat list of blocks, each
// level's blocks (ceil(lw / 32) x lh) after the previous level's, coarsest
// (fewest pixels, most channels) first.
struct FeatLevels {
    const float* im[kFlowLevels];
    float* out[kFlowLevels];
    int lw[kFlowLevels], lh[kFlowLevels], lc[kFlowLevels], woff[kFlowLevels];
    int block0[kFlowLevels + 1];
};

__global__ void __launch_bounds__(32 * kFeatGroups) features_kernel(const __grid_constant__ FeatLevels fl)
{
    pdl_enter();
    __shared__ float sf[kFeatMaxC][32];
    __shared__ float snrm[32];
    __shared__ float sw[kFeatMaxC * 27];
    int l = 0;
    while (l + 1 < kFlowLevels && static_cast<int>(blockIdx.x) >= fl.block0[l + 1])
        ++l;
    const float* __restrict__ im = fl.im[l];
    float* __restrict__ out = fl.out[l];
    const int lw = fl.lw[l], lh = fl.lh[l], lc = fl.lc[l], woff = fl.woff[l];
    const int nbx = (lw + 31) / 32, b = blockIdx.x - fl.block0[l];
    const int tx = threadIdx.x, g = threadIdx.y;
    for (int i = g * 32 + tx; i < lc * 27; i += 32 * kFeatGroups)
        sw[i] = g_flow_w[woff + i];
    __syncthreads();
    const int x = (b % nbx) * 32 + tx;
    const int y = b / nbx;
    const bool ok = x < lw;
    const int xc = ok ? x : lw - 1;
    const int64_t plane = static_cast<int64_t>(lw) * lh;
    float p[27];
#pragma unroll
    for (int ky = -1; ky <= 1; ++ky) {
        const int yy = clampi(y + ky, 0, lh - 1);
#pragma unroll
        for (int kx = -1; kx <= 1; ++kx) {
            const int xx = clampi(xc + kx, 0, lw - 1);
#pragma unroll
            for (int ch = 0; ch < 3; ++ch)
                p[((ky + 1) * 3 + (kx + 1)) * 3 + ch] = im[(static_cast<int64_t>(yy) * lw + xx) * 3 + ch] - 0.5f;
        }
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        float m = 0.0f;
#pragma unroll
        for (int k = ch; k < 27; k += 3)
            m += p[k];
        m = __fdiv_rn(m, 9.0f);
#pragma unroll
        for (int k = ch; k < 27; k += 3)
            p[k] = p[k] - m;
    }
    for (int c = g; c < lc; c += kFeatGroups) {
        float f = 0.0f;
#pragma unroll
        for (int k = 0; k < 27; ++k)
            f += sw[c * 27 + k] * p[k];
        sf[c][tx] = f;
    }
    __syncthreads();
    if (g == 0) {
        float ss = 0.0f;
        for (int c = 0; c < lc; ++c) {
            const float f = sf[c][tx];
            ss += f * f;
        }
        snrm[tx] = __fsqrt_rn(ss + 1e-12f);
    }
    __syncthreads();
    if (!ok)
        return;
    const float nrm = snrm[tx];
    float* o = out + static_cast<int64_t>(y) * lw + x;
    for (int c = g; c < lc; c += kFeatGroups)
        o[c * plane] = __fdiv_rn(sf[c][tx], nrm);
}

__global__ void up2_kernel(const float* __restrict__ in, int sw, int sh, float* __restrict__ out, int dw, int dh,
    int64_t bs)
{
    pdl_enter();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh)
        return;
    in += blockIdx.z * bs;
    out += blockIdx.z * bs;
    const int64_t dp = static_cast<int64_t>(dw) * dh;
#pragma unroll
    for (int ch = 0; ch < 2; ++ch)
        out[ch * dp + static_cast<int64_t>(y) * dw + x] = up2_sample(in, sw, sh, x, y, ch);
}

// One thread per pixel, 64 per block: the pixel's 81 cost values are first
// copied to its own column of shared memory (81 independent loads, all in
// flight before the first store: one round trip, which the coarse levels'
// few blocks cannot hide nine times over), then the arg-max, the soft
// centroid and the confidence read them from there -- the same operations
// in the same order as a direct walk over the cost volume.
constexpr int kDecodeThreads = 64;

__global__ void __launch_bounds__(kDecodeThreads) decode_kernel(const float* __restrict__ cv, float* __restrict__ res,
    float* __restrict__ conf, int64_t plane, float prior, int64_t bs)
{
    pdl_enter();
    __shared__ float sv[81][kDecodeThreads];
    const int t = threadIdx.x;
    const int64_t p = blockIdx.x * static_cast<int64_t>(kDecodeThreads) + t;
    if (p >= plane)
        return;
    cv += blockIdx.z * bs;
    res += blockIdx.z * bs;
    conf += blockIdx.z * bs;
    {
        float v[81];
#pragma unroll
        for (int d = 0; d < 81; ++d)
            v[d] = __ldg(cv + d * plane + p);
#pragma unroll
        for (int d = 0; d < 81; ++d)
            sv[d][t] = v[d];
    }
    int best = 0;
    float cmax = sv[0][t] - prior * 32.0f;
    float csum = sv[0][t];
    for (int d = 1; d < 81; ++d) {
        const int ddx = d % 9 - 4, ddy = d / 9 - 4;
        const float raw = sv[d][t];
        csum += raw;
        const float v = raw - prior * static_cast<float>(ddx * ddx + ddy * ddy);
        if (v > cmax) {
            cmax = v;
            best = d;
        }
    }
    const int by = best / 9, bx = best % 9;
    float sw = 0.0f, sx = 0.0f, sy = 0.0f;
    for (int ny = by - 1; ny <= by + 1; ++ny) {
        if (ny < 0 || ny > 8)
            continue;
        for (int nx = bx - 1; nx <= bx + 1; ++nx) {
            if (nx < 0 || nx > 8)
                continue;
            const float sc =
                sv[ny * 9 + nx][t] - prior * static_cast<float>((nx - 4) * (nx - 4) + (ny - 4) * (ny - 4));
            const float e = expf_cw((sc - cmax) * kTemp);
            sw += e;
            sx += e * static_cast<float>(nx - 4);
            sy += e * static_cast<float>(ny - 4);
        }
    }
    res[p] = __fdiv_rn(sx, sw);
    res[plane + p] = __fdiv_rn(sy, sw);
    const float k = sv[best][t] - __fdiv_rn(csum, 81.0f);
    conf[p] = k > 0.0f ? k : 0.0f;
}

// confidence-weighted 3x3 mean (edge clamp) of the refinement, added to the
// upsampled coarser flow (zero at the coarsest level): read from `up`, or
// with `coarse` non-null upsampled here from the cw x chh coarser flow
__global__ void smooth_kernel(const float* __restrict__ res, const float* __restrict__ conf,
    const float* __restrict__ up, float* __restrict__ out, int lw, int lh, int64_t bs,
    const float* __restrict__ coarse, int cw, int chh)
{
    pdl_enter();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= lw || y >= lh)
        return;
    res += blockIdx.z * bs;
    conf += blockIdx.z * bs;
    out += blockIdx.z * bs;
    if (up)
        up += blockIdx.z * bs;
    const int64_t plane = static_cast<int64_t>(lw) * lh;
    float sx = 0.0f, sy = 0.0f, sw = 0.0f;
#pragma unroll
    for (int ky = -1; ky <= 1; ++ky) {
        const int yy = clampi(y + ky, 0, lh - 1);
#pragma unroll
        for (int kx = -1; kx <= 1; ++kx) {
            const int xx = clampi(x + kx, 0, lw - 1);
            const int64_t q = static_cast<int64_t>(yy) * lw + xx;
            const float c = conf[q];
            sx += c * res[q];
            sy += c * res[plane + q];
            sw += c;
        }
    }
    const int64_t p = static_cast<int64_t>(y) * lw + x;
    const float den = sw + kEps;
    float ux = 0.0f, uy = 0.0f;
    if (coarse) {
        coarse += blockIdx.z * bs;
        ux = up2_sample(coarse, cw, chh, x, y, 0);
        uy = up2_sample(coarse, cw, chh, x, y, 1);
    } else if (up) {
        ux = up[p];
        uy = up[plane + p];
    }
    out[p] = ux + __fdiv_rn(sx, den);
    out[plane + p] = uy + __fdiv_rn(sy, den);
}

__global__ void final_flow_kernel(const float* __restrict__ S, int lw, int lh, float* __restrict__ out, int w, int h,
    int64_t bs, int64_t so)
{
    pdl_enter();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h)
        return;
    S += blockIdx.z * bs;
    out += blockIdx.z * so;
    const int64_t plane = static_cast<int64_t>(lw) * lh;
    const float rx = static_cast<float>(lw) / static_cast<float>(w);
    const float ry = static_cast<float>(lh) / static_cast<float>(h);
    const float gx = static_cast<float>(w) / static_cast<float>(lw);
    const float gy = static_cast<float>(h) / static_cast<float>(lh);
    float sx = (static_cast<float>(x) + 0.5f) * rx - 0.5f;
    float sy = (static_cast<float>(y) + 0.5f) * ry - 0.5f;
    if (sx < 0.0f)
        sx = 0.0f;
    if (sy < 0.0f)
        sy = 0.0f;
    int x0 = static_cast<int>(floorf(sx)), y0 = static_cast<int>(floorf(sy));
    if (x0 > lw - 1)
        x0 = lw - 1;
    if (y0 > lh - 1)
        y0 = lh - 1;
    const int x1 = x0 + 1 < lw ? x0 + 1 : lw - 1;
    const int y1 = y0 + 1 < lh ? y0 + 1 : lh - 1;
    const float lx = sx - static_cast<float>(x0), ly = sy - static_cast<float>(y0);
    float r[2];
#pragma unroll
    for (int ch = 0; ch < 2; ++ch) {
        const float* s = S + ch * plane;
        const float top = (1.0f - lx) * s[static_cast<int64_t>(y0) * lw + x0] + lx * s[static_cast<int64_t>(y0) * lw + x1];
        const float bot = (1.0f - lx) * s[static_cast<int64_t>(y1) * lw + x0] + lx * s[static_cast<int64_t>(y1) * lw + x1];
        r[ch] = (1.0f - ly) * top + ly * bot;
    }
    float* o = out + (static_cast<int64_t>(y) * w + x) * 3;
    o[0] = r[0] * gx;
    o[1] = r[1] * gy;
    o[2] = 0.0f;
}

inline dim3 g2(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

}  // namespace

FlowDims flow_dims(int w, int h)
{
    FlowDims d;
    const int pw = ((w + 63) / 64) * 64, ph = ((h + 63) / 64) * 64;
    size_t off = 0;
    d.max_plane = 0;
    d.max_c = 0;
    for (int l = 0; l < kFlowLevels; ++l) {
        d.lw[l] = pw >> (l + 2);
        d.lh[l] = ph >> (l + 2);
        d.lc[l] = kLevelC[l];
        d.off[l] = off;
        off += static_cast<size_t>(d.lw[l]) * d.lh[l] * d.lc[l];
        const size_t plane = static_cast<size_t>(d.lw[l]) * d.lh[l];
        if (plane > d.max_plane)
            d.max_plane = plane;
        if (d.lc[l] > d.max_c)
            d.max_c = d.lc[l];
    }
    d.feat_floats = off;
    return d;
}

cudaError_t flow_upload_weights()
{
    // Once per device: the constant bank is per device (and per context).
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 64 && done[dev])
        return cudaSuccess;
    static float host_w[kWeightTotal];
    for (int l = 0; l < kFlowLevels; ++l) {
        uint64_t s = 0x5653432D464C4F57ULL ^ (static_cast<uint64_t>(l + 1) * 0x9E3779B97F4A7C15ULL);
        for (int i = 0; i < kLevelC[l] * 27; ++i) {
            const uint64_t z = splitmix64(&s);
            host_w[kWeightOff[l] + i] = static_cast<float>(static_cast<uint32_t>(z >> 40)) * (1.0f / 8388608.0f) - 1.0f;
        }
    }
    e = cudaMemcpyToSymbol(g_flow_w, host_w, sizeof(host_w));
    if (e == cudaSuccess && dev >= 0 && dev < 64)
        done[dev] = true;
    return e;
}

size_t flow_feature_scratch_floats(const FlowDims& d)
{
    size_t n = 0;
    for (int l = 0; l < kFlowLevels; ++l)
        n += static_cast<size_t>(d.lw[l]) * d.lh[l] * 3;
    return n;
}

cudaError_t launch_flow_features(const float* img, int w, int h, const FlowDims& d, float* feats, float* scratch,
    cudaStream_t st, int* launches, const float* full, int FW, int FH)
{
    float* lev[kFlowLevels];
    size_t off = 0;
    PyrOut po{};
    for (int l = 0; l < kFlowLevels; ++l) {
        lev[l] = scratch + off;
        po.lev[l] = lev[l];
        off += static_cast<size_t>(d.lw[l]) * d.lh[l] * 3;
    }
    po.lw0 = d.lw[0];
    po.lh0 = d.lh[0];
    if (d.lw[0] % 16 != 0 || d.lh[0] % 16 != 0 || (d.lw[0] >> (kFlowLevels - 1)) * 16 != d.lw[0])
        return cudaErrorInvalidValue;  // flow_dims pads the frame to a multiple of 64: never
    const dim3 g(static_cast<unsigned>(d.lw[0] / 16), static_cast<unsigned>(d.lh[0] / 16));
    cudaError_t e = full ? launch_pdl(pyramid_kernel<true>, g, dim3(256), 0, st, img, w, h, full, FW, FH, po)
                         : launch_pdl(pyramid_kernel<false>, g, dim3(256), 0, st, img, w, h, full, FW, FH, po);
    int nl = 1;
    FeatLevels fl{};
    fl.block0[0] = 0;
    for (int k = 0; k < kFlowLevels; ++k) {
        const int l = kFlowLevels - 1 - k;  // coarsest first
        fl.im[k] = lev[l];
        fl.out[k] = feats + d.off[l];
        fl.lw[k] = d.lw[l];
        fl.lh[k] = d.lh[l];
        fl.lc[k] = d.lc[l];
        fl.woff[k] = kWeightOff[l];
        fl.block0[k + 1] = fl.block0[k] + ((d.lw[l] + 31) / 32) * d.lh[l];
    }
    if (e == cudaSuccess)
        e = launch_pdl(features_kernel, dim3(fl.block0[kFlowLevels]), dim3(32, kFeatGroups), 0, st, fl);
    ++nl;
    if (launches)
        *launches += nl;
    return e != cudaSuccess ? e : cudaGetLastError();
}

size_t flow_estimate_scratch_floats(const FlowDims& d)
{
    size_t maxcl = 0;
    for (int l = 0; l < kFlowLevels; ++l) {
        const size_t v = static_cast<size_t>(d.lw[l]) * d.lh[l] * d.lc[l];
        if (v > maxcl)
            maxcl = v;
    }
    // up (2 ch) + refinement and confidence (3) + two smoothed flows (2 + 2),
    // warped features, cost volume
    return 9 * d.max_plane + maxcl + 81 * d.max_plane;
}

size_t tc_level_offset(const FlowDims& d, int level)
{
    size_t off = 0;
    for (int l = 0; l < level; ++l)
        off += (static_cast<size_t>(d.lw[l]) * d.lh[l] * tc_padded_channels(d.lc[l]) * 2 + 255) / 256 * 256;
    return off;
}

size_t tc_frame_bytes(const FlowDims& d) { return tc_level_offset(d, kFlowLevels); }

size_t tc_warped_bytes(const FlowDims& d)
{
    size_t m = 0;
    for (int l = 0; l < kFlowLevels; ++l)
        m = std::max(m, (static_cast<size_t>(d.lw[l]) * d.lh[l] * tc_padded_channels(d.lc[l]) * 2 + 255) / 256 * 256);
    return m;
}

cudaError_t launch_flow_features_chunked(const float* feats, const FlowDims& d, void* chunked, const float* scale,
    bool bf16, cudaStream_t st, int* launches)
{
    const float* in[kFlowLevels];
    void* out[kFlowLevels];
    int C[kFlowLevels], H[kFlowLevels], W[kFlowLevels];
    for (int l = 0; l < kFlowLevels; ++l) {
        in[l] = feats + d.off[l];
        out[l] = static_cast<unsigned char*>(chunked) + tc_level_offset(d, l);
        C[l] = d.lc[l];
        H[l] = d.lh[l];
        W[l] = d.lw[l];
    }
    const cudaError_t e = launch_to_chunked_levels(in, out, C, H, W, kFlowLevels, scale, bf16, st);
    if (launches)
        *launches += 1;
    return e;
}

cudaError_t launch_flow_pair(const float* featA, int64_t sA, const float* featB, int64_t sB, int w, int h,
    const FlowDims& d, float* flow_out, int64_t s_out, float* scratch, cudaStream_t st, int* launches,
    const FlowTc* tc)
{
    const dim3 b(32, 8);
    const int64_t bs = static_cast<int64_t>(flow_estimate_scratch_floats(d));  // per-direction scratch
    float* up = scratch;
    float* raw = up + 2 * d.max_plane;
    float* sm[2] = {raw + 3 * d.max_plane, raw + 5 * d.max_plane};
    float* warped = raw + 7 * d.max_plane;
    size_t maxcl = 0;
    for (int l = 0; l < kFlowLevels; ++l)
        maxcl = std::max(maxcl, static_cast<size_t>(d.lw[l]) * d.lh[l] * d.lc[l]);
    float* cv = warped + maxcl;
    int nl = 0;
    int cur = 0;
    cudaError_t e;
    for (int l = kFlowLevels - 1; l >= 0; --l) {
        const int lw = d.lw[l], lh = d.lh[l], lc = d.lc[l];
        const int64_t plane = static_cast<int64_t>(lw) * lh;
        const float* fa = featA + d.off[l];
        const float* fb = featB + d.off[l];
        const float* upp = nullptr;
        const float* coarse = nullptr;  // the tensor-core form upsamples the coarser flow where it reads it
        const float* fb_use = fb;
        int64_t sb_use = sB;
        if (l < kFlowLevels - 1) {
            if (tc) {
                coarse = sm[cur];
                e = launch_warp_to_chunked(fb, coarse, tc->warped, tc->scales, 2, lc, lh, lw, sB, bs,
                    static_cast<int64_t>(tc_warped_bytes(d)), tc->bf16, st, d.lw[l + 1], d.lh[l + 1]);
            } else {
                dim3 g = g2(lw, lh, b);
                g.z = 2;
                if ((e = launch_pdl(up2_kernel, g, b, 0, st, sm[cur], d.lw[l + 1], d.lh[l + 1], up, lw, lh, bs)) !=
                    cudaSuccess)
                    return e;
                ++nl;
                upp = up;
                e = launch_warp_op(fb, up, warped, 2, lc, lh, lw, st, sB, bs, bs);
                fb_use = warped;
                sb_use = bs;
            }
            if (e != cudaSuccess)
                return e;
            ++nl;
        }
        if (tc) {
            // the tensor-core correlations of both directions in one launch
            // (each direction's operands are separate tensors)
            const size_t lo = tc_level_offset(d, l);
            const void* ac[2];
            const void* bc[2];
            for (int dir = 0; dir < 2; ++dir) {
                ac[dir] = static_cast<const unsigned char*>(tc->a[dir]) + lo;
                bc[dir] = l < kFlowLevels - 1
                              ? static_cast<const void*>(static_cast<const unsigned char*>(tc->warped) +
                                                         dir * tc_warped_bytes(d))
                              : static_cast<const void*>(static_cast<const unsigned char*>(tc->b[dir]) + lo);
            }
            e = launch_corr_tc_chunked2(ac[0], bc[0], cv, ac[1], bc[1], cv + bs, tc->scales, 1,
                tc_padded_channels(lc), lh, lw, 4, tc->bf16, st);
            if (e != cudaSuccess)
                return e;
            ++nl;
        } else {
            e = launch_correlation(fa, fb_use, cv, 2, lc, lh, lw, 4, 0, st, sA, sb_use, bs);
            if (e != cudaSuccess)
                return e;
            ++nl;
        }
        if ((e = launch_pdl(decode_kernel, dim3(static_cast<unsigned>((plane + kDecodeThreads - 1) / kDecodeThreads), 1, 2),
                 dim3(kDecodeThreads), 0, st, cv, raw, raw + 2 * plane, plane, kLevelPrior[l], bs)) != cudaSuccess)
            return e;
        ++nl;
        cur ^= 1;
        dim3 g = g2(lw, lh, b);
        g.z = 2;
        const int cw = coarse ? d.lw[l + 1] : 0, chh = coarse ? d.lh[l + 1] : 0;
        if ((e = launch_pdl(smooth_kernel, g, b, 0, st, raw, raw + 2 * plane, upp, sm[cur], lw, lh, bs, coarse, cw,
                 chh)) != cudaSuccess)
            return e;
        ++nl;
    }
    dim3 g = g2(w, h, b);
    g.z = 2;
    if ((e = launch_pdl(final_flow_kernel, g, b, 0, st, sm[cur], d.lw[0], d.lh[0], flow_out, w, h, bs, s_out)) !=
        cudaSuccess)
        return e;
    ++nl;
    if (launches)
        *launches += nl;
    return cudaGetLastError();
}

}  // namespace vsc
