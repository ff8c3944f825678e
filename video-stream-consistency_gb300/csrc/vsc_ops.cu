// Correlation (cost volume) and Warp operators for sm_103a.
//
// Correlation, legacy = 0 (reference semantics: correlation.cc:147-275,
// correlation_cuda.cu:97-175):
//   out[n][i][j][h][w] = sum_c f1[n][c][h][w] * f2[n][c][h+i-md][w+j-md]
// The reference CUDA path transposes both maps to NHWC in cudaMalloc'd
// temporaries and gives each output pixel one 32-thread block with a serial
// 81-step shared-memory reduction.  Here a CTA owns a TH x 32 pixel tile and
// all (2md+1)^2 displacements: channel chunks of f1 (tile) and f2 (tile plus
// an md-pixel halo) are staged in shared memory straight from the NCHW
// inputs (no temporaries), and every thread keeps 4 adjacent pixels x
// (2md+1) horizontal displacements of one vertical displacement in
// registers.  Per channel a thread reads 1 + ceil((4+2md)/4) 128-bit words
// of shared memory for 4*(2md+1) multiply-adds.  Sums run in channel order
// with separately rounded products and sums (-fmad=false), which is the
// reference CPU op's arithmetic, so results match it bit for bit.  (The
// packed f32x2 instructions would halve the issue count, but ptxas fuses a
// packed multiply followed by a packed add into an FMA even under
// -fmad=false, which changes the rounding; they are not used.)
//
// Warp (warp.cc:71-133, warp_cuda.cu:28-98): one thread per pixel and group
// of 8 channels; the flow, the four bilinear weights and the 0.999 edge mask
// are computed once per pixel instead of once per (pixel, channel).
#include "vsc_internal.h"
#include "vsc_math.cuh"

namespace vsc {
namespace {

constexpr int kCorrTW = 32;  // tile width (pixels)
constexpr int kCorrTH = 4;   // tile height (rows)
constexpr int kCorrCC = 16;  // channels per shared-memory stage

template <int MD>
struct CorrGeom {
    static constexpr int P = 2 * MD + 1;
    static constexpr int RH = kCorrTH + 2 * MD;                    // f2 tile rows
    static constexpr int S2W = ((kCorrTW + 2 * MD) + 3) / 4 * 4;   // f2 tile row pitch (floats)
    static constexpr int NB = (4 + 2 * MD + 3) / 4;                // float4 words of f2 per thread row
    static constexpr int S1 = kCorrCC * kCorrTH * kCorrTW;
    static constexpr int S2 = kCorrCC * RH * S2W;
};

template <int MD>
__global__ void __launch_bounds__(8 * kCorrTH * (2 * MD + 1))
    corr_tile_kernel(const float* __restrict__ in1, const float* __restrict__ in2, float* __restrict__ out, int C,
        int H, int W, int legacy, int vec_store, int64_t sa, int64_t sb, int64_t so)
{
    using G = CorrGeom<MD>;
    constexpr int P = G::P;
    __shared__ __align__(16) float s1[G::S1];
    __shared__ __align__(16) float s2[G::S2];

    const int tx = threadIdx.x;  // x quad
    const int ty = threadIdx.y;  // row in tile
    const int tz = threadIdx.z;  // vertical displacement index
    const int tid = (tz * kCorrTH + ty) * 8 + tx;
    const int nthreads = 8 * kCorrTH * P;
    const int lane = tid & 31, warp = tid >> 5, nwarps = (nthreads + 31) >> 5;

    const int n = blockIdx.z;
    const int X0 = blockIdx.x * kCorrTW;
    const int Y0 = blockIdx.y * kCorrTH;
    const int64_t HW = static_cast<int64_t>(H) * W;
    const float* a_n = in1 + n * sa;  // batch strides in elements (may be negative)
    const float* b_n = in2 + n * sb;

    float acc[P][4];
#pragma unroll
    for (int j = 0; j < P; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            acc[j][i] = 0.0f;

    for (int c0 = 0; c0 < C; c0 += kCorrCC) {
        const int cc = min(kCorrCC, C - c0);
        // stage f1 tile: cc x TH x TW
        for (int r = warp; r < kCorrCC * kCorrTH; r += nwarps) {
            const int c = r / kCorrTH, row = r % kCorrTH;
            const int gy = Y0 + row, gx = X0 + lane;
            float v = 0.0f;
            if (c < cc && gy < H && gx < W)
                v = __ldg(a_n + static_cast<int64_t>(c0 + c) * HW + static_cast<int64_t>(gy) * W + gx);
            s1[(c * kCorrTH + row) * kCorrTW + lane] = v;
        }
        // stage f2 tile with halo: cc x (TH + 2md) x (TW + 2md), zero outside the map
        for (int r = warp; r < kCorrCC * G::RH; r += nwarps) {
            const int c = r / G::RH, row = r % G::RH;
            const int gy = Y0 - MD + row;
            const bool rowok = (c < cc) && gy >= 0 && gy < H;
            const float* src = b_n + static_cast<int64_t>(c0 + c) * HW + static_cast<int64_t>(gy) * W;
            for (int col = lane; col < G::S2W; col += 32) {
                const int gx = X0 - MD + col;
                float v = 0.0f;
                if (rowok && col < kCorrTW + 2 * MD && gx >= 0 && gx < W)
                    v = __ldg(src + gx);
                s2[(c * G::RH + row) * G::S2W + col] = v;
            }
        }
        __syncthreads();
        for (int c = 0; c < cc; ++c) {
            const float4 av = *reinterpret_cast<const float4*>(&s1[(c * kCorrTH + ty) * kCorrTW + 4 * tx]);
            const float a[4] = {av.x, av.y, av.z, av.w};
            float b[4 * G::NB];
            const float* brow = &s2[(c * G::RH + ty + tz) * G::S2W + 4 * tx];
#pragma unroll
            for (int q = 0; q < G::NB; ++q) {
                const float4 bv = *reinterpret_cast<const float4*>(brow + 4 * q);
                b[4 * q + 0] = bv.x;
                b[4 * q + 1] = bv.y;
                b[4 * q + 2] = bv.z;
                b[4 * q + 3] = bv.w;
            }
#pragma unroll
            for (int j = 0; j < P; ++j)
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    acc[j][i] = acc[j][i] + a[i] * b[i + j];
        }
        __syncthreads();
    }

    const int y = Y0 + ty;
    if (y >= H)
        return;
    const int dy = tz - MD;
    const bool yok = (y + dy >= 0) && (y + dy < H);
    const int x0 = X0 + 4 * tx;
    const float fc = static_cast<float>(C);
#pragma unroll
    for (int j = 0; j < P; ++j) {
        const int dx = j - MD;
        float r[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int xs = x0 + i + dx;
            float v = (yok && xs >= 0 && xs < W) ? acc[j][i] : 0.0f;
            if (legacy)
                v = __fdiv_rn(v, fc);
            r[i] = v;
        }
        float* dst = out + n * so + static_cast<int64_t>(tz * P + j) * HW + static_cast<int64_t>(y) * W + x0;
        if (vec_store && x0 + 3 < W) {
            *reinterpret_cast<float4*>(dst) = make_float4(r[0], r[1], r[2], r[3]);
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (x0 + i < W)
                    dst[i] = r[i];
        }
    }
}

// Any max_displacement: one thread per output element, channel-order sum.
__global__ void corr_generic_kernel(const float* __restrict__ in1, const float* __restrict__ in2,
    float* __restrict__ out, int N, int C, int H, int W, int md, int legacy)
{
    const int P = 2 * md + 1;
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t total = static_cast<int64_t>(N) * P * P * HW;
    for (int64_t idx = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; idx < total;
         idx += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t pix = idx % HW;
        const int64_t nd = idx / HW;
        const int d = static_cast<int>(nd % (P * P));
        const int n = static_cast<int>(nd / (P * P));
        const int y = static_cast<int>(pix / W), x = static_cast<int>(pix % W);
        const int y2 = y + d / P - md, x2 = x + d % P - md;
        float acc = 0.0f;
        if (y2 >= 0 && y2 < H && x2 >= 0 && x2 < W) {
            const float* a = in1 + static_cast<int64_t>(n) * C * HW + pix;
            const float* b = in2 + static_cast<int64_t>(n) * C * HW + static_cast<int64_t>(y2) * W + x2;
            for (int c = 0; c < C; ++c)
                acc = acc + __ldg(a + c * HW) * __ldg(b + c * HW);
        }
        if (legacy)
            acc = __fdiv_rn(acc, static_cast<float>(C));
        out[idx] = acc;
    }
}

template <int MD>
cudaError_t launch_corr_tile(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int legacy,
    int64_t s1, int64_t s2, int64_t so, cudaStream_t st)
{
    dim3 block(8, kCorrTH, 2 * MD + 1);
    dim3 grid((W + kCorrTW - 1) / kCorrTW, (H + kCorrTH - 1) / kCorrTH, N);
    // 128-bit stores need rows that start on 16 bytes: W % 4 == 0 and aligned outputs
    const int vec = ((W & 3) == 0) && ((reinterpret_cast<uintptr_t>(out) & 15) == 0) && ((so & 3) == 0);
    corr_tile_kernel<MD><<<grid, block, 0, st>>>(f1, f2, out, C, H, W, legacy, vec, s1, s2, so);
    return cudaGetLastError();
}

constexpr int kWarpCG = 8;  // channels per thread

__global__ void warp_op_kernel(const float* __restrict__ in, const float* __restrict__ flow, float* __restrict__ out,
    int C, int H, int W, int64_t sin, int64_t sfl, int64_t sout)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= HW)
        return;
    const int n = blockIdx.z;
    const int c0 = blockIdx.y * kWarpCG;
    const int y = static_cast<int>(p / W), x = static_cast<int>(p % W);
    const float* fl = flow + n * sfl;
    const float xf = static_cast<float>(x) + __ldg(fl + p);
    const float yf = static_cast<float>(y) + __ldg(fl + HW + p);
    const float fxl = floorf(xf), fyt = floorf(yf);
    const float a = xf - fxl, b = yf - fyt;
    const float xR = fxl + 1.0f, yB = fyt + 1.0f;
    const bool mL = (0.0f <= fxl && fxl <= static_cast<float>(W - 1));
    const bool mR = (0.0f <= xR && xR <= static_cast<float>(W - 1));
    const bool mT = (0.0f <= fyt && fyt <= static_cast<float>(H - 1));
    const bool mB = (0.0f <= yB && yB <= static_cast<float>(H - 1));
    const float ia = 1.0f - a, ib = 1.0f - b;
    const float wTL = ia * ib, wTR = a * ib, wBL = ia * b, wBR = a * b;
    const bool tl = mT && mL, tr = mT && mR, bl = mB && mL, br = mB && mR;
    float mask = 0.0f;
    mask += tl ? wTL : 0.0f;
    mask += tr ? wTR : 0.0f;
    mask += bl ? wBL : 0.0f;
    mask += br ? wBR : 0.0f;
    const bool take = mask > 0.999f;
    const int xl = take ? static_cast<int>(fxl) : 0;
    const int yt = take ? static_cast<int>(fyt) : 0;
    const int64_t oTL = static_cast<int64_t>(yt) * W + xl;
    const int cend = min(C, c0 + kWarpCG);
    for (int c = c0; c < cend; ++c) {
        const float* src = in + n * sin + static_cast<int64_t>(c) * HW;
        float val = 0.0f;
        if (take) {
            val += tl ? wTL * __ldg(src + oTL) : 0.0f;
            val += tr ? wTR * __ldg(src + oTL + 1) : 0.0f;
            val += bl ? wBL * __ldg(src + oTL + W) : 0.0f;
            val += br ? wBR * __ldg(src + oTL + W + 1) : 0.0f;
        }
        out[n * sout + static_cast<int64_t>(c) * HW + p] = val;
    }
}

}  // namespace

cudaError_t launch_correlation(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md,
    int legacy, cudaStream_t st, int64_t s1, int64_t s2, int64_t so)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t P = 2 * md + 1;
    if (s1 < 0 && s2 < 0 && so < 0) {  // contiguous N x C x H x W batches
        s1 = s2 = C * HW;
        so = P * P * HW;
    }
    switch (md) {
        case 1:
            return launch_corr_tile<1>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        case 2:
            return launch_corr_tile<2>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        case 3:
            return launch_corr_tile<3>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        case 4:
            return launch_corr_tile<4>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        default: {
            if (s1 != C * HW || s2 != C * HW || so != P * P * HW)
                return cudaErrorInvalidValue;  // the generic kernel takes contiguous batches only
            const int64_t total = static_cast<int64_t>(N) * P * P * HW;
            const int64_t blocks = (total + 255) / 256;
            corr_generic_kernel<<<static_cast<unsigned>(blocks < 152 * 64 ? blocks : 152 * 64), 256, 0, st>>>(
                f1, f2, out, N, C, H, W, md, legacy);
            return cudaGetLastError();
        }
    }
}

cudaError_t launch_warp_op(const float* in, const float* flow, float* out, int N, int C, int H, int W,
    cudaStream_t st, int64_t sin, int64_t sfl, int64_t sout)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    if (sin < 0 && sfl < 0 && sout < 0) {
        sin = sout = C * HW;
        sfl = 2 * HW;
    }
    dim3 grid(static_cast<unsigned>((HW + 255) / 256), (C + kWarpCG - 1) / kWarpCG, N);
    warp_op_kernel<<<grid, 256, 0, st>>>(in, flow, out, C, H, W, sin, sfl, sout);
    return cudaGetLastError();
}

}  // namespace vsc
