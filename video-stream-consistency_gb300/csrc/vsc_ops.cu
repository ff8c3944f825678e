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
// inputs (no temporaries) by cp.async, double-buffered so the next channel
// chunk streams in while the current one is consumed, and every thread keeps
// 4 adjacent pixels x
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

#include <mutex>

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

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Asynchronous global -> shared copies; when `valid` is false nothing is read
// and the destination is zero-filled (src-size 0).
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(float* dst, const float* src, bool valid)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Stages one chunk of kCorrCC channels: the f1 tile and the f2 tile with its
// md halo, zero outside the map.  vec: 16-byte copies (rows and tile origins
// on the 16-byte grid, so a 4-float vector is entirely inside or outside).
template <int MD>
__device__ __forceinline__ void corr_stage(float* s1, float* s2, const float* a_n, const float* b_n, int c0, int cc,
    int X0, int Y0, int H, int W, int64_t HW, int tid, int nthreads, bool vec)
{
    using G = CorrGeom<MD>;
    if (vec) {
        constexpr int V1 = kCorrCC * kCorrTH * (kCorrTW / 4);
        for (int v = tid; v < V1; v += nthreads) {
            const int c = v / (kCorrTH * (kCorrTW / 4)), rem = v % (kCorrTH * (kCorrTW / 4));
            const int row = rem / (kCorrTW / 4), q = rem % (kCorrTW / 4);
            const int gy = Y0 + row, gx = X0 + 4 * q;
            const bool ok = c < cc && gy < H && gx < W;
            const float* src = ok ? a_n + static_cast<int64_t>(c0 + c) * HW + static_cast<int64_t>(gy) * W + gx : a_n;
            cp_async16(s1 + (c * kCorrTH + row) * kCorrTW + 4 * q, src, ok);
        }
        constexpr int Q2 = G::S2W / 4;
        constexpr int V2 = kCorrCC * G::RH * Q2;
        for (int v = tid; v < V2; v += nthreads) {
            const int c = v / (G::RH * Q2), rem = v % (G::RH * Q2);
            const int row = rem / Q2, q = rem % Q2;
            const int gy = Y0 - MD + row, gx = X0 - MD + 4 * q;
            const bool ok = c < cc && gy >= 0 && gy < H && gx >= 0 && gx < W && 4 * q < kCorrTW + 2 * MD;
            const float* src = ok ? b_n + static_cast<int64_t>(c0 + c) * HW + static_cast<int64_t>(gy) * W + gx : b_n;
            cp_async16(s2 + (c * G::RH + row) * G::S2W + 4 * q, src, ok);
        }
    } else {
        constexpr int E1 = kCorrCC * kCorrTH * kCorrTW;
        for (int v = tid; v < E1; v += nthreads) {
            const int c = v / (kCorrTH * kCorrTW), rem = v % (kCorrTH * kCorrTW);
            const int row = rem / kCorrTW, col = rem % kCorrTW;
            const int gy = Y0 + row, gx = X0 + col;
            const bool ok = c < cc && gy < H && gx < W;
            const float* src = ok ? a_n + static_cast<int64_t>(c0 + c) * HW + static_cast<int64_t>(gy) * W + gx : a_n;
            cp_async4(s1 + v, src, ok);
        }
        constexpr int E2 = kCorrCC * G::RH * G::S2W;
        for (int v = tid; v < E2; v += nthreads) {
            const int c = v / (G::RH * G::S2W), rem = v % (G::RH * G::S2W);
            const int row = rem / G::S2W, col = rem % G::S2W;
            const int gy = Y0 - MD + row, gx = X0 - MD + col;
            const bool ok = c < cc && gy >= 0 && gy < H && gx >= 0 && gx < W && col < kCorrTW + 2 * MD;
            const float* src = ok ? b_n + static_cast<int64_t>(c0 + c) * HW + static_cast<int64_t>(gy) * W + gx : b_n;
            cp_async4(s2 + v, src, ok);
        }
    }
}

template <int MD>
__global__ void __launch_bounds__(8 * kCorrTH * (2 * MD + 1))
    corr_tile_kernel(const float* __restrict__ in1, const float* __restrict__ in2, float* __restrict__ out, int C,
        int H, int W, int legacy, int vec_store, int vec_load, int64_t sa, int64_t sb, int64_t so)
{
    pdl_enter();
    using G = CorrGeom<MD>;
    constexpr int P = G::P;
    // two stages of (f1 tile, f2 tile): the next channel chunk streams in
    // while the current one is consumed
    extern __shared__ __align__(16) float corr_smem[];

    const int tx = threadIdx.x;  // x quad
    const int ty = threadIdx.y;  // row in tile
    const int tz = threadIdx.z;  // vertical displacement index
    const int tid = (tz * kCorrTH + ty) * 8 + tx;
    const int nthreads = 8 * kCorrTH * P;

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

    int cur = 0;
    corr_stage<MD>(corr_smem, corr_smem + G::S1, a_n, b_n, 0, min(kCorrCC, C), X0, Y0, H, W, HW, tid, nthreads,
        vec_load != 0);
    cp_async_commit();
    for (int c0 = 0; c0 < C; c0 += kCorrCC) {
        const int cc = min(kCorrCC, C - c0);
        if (c0 + kCorrCC < C) {
            float* nb = corr_smem + (cur ^ 1) * (G::S1 + G::S2);
            corr_stage<MD>(nb, nb + G::S1, a_n, b_n, c0 + kCorrCC, min(kCorrCC, C - c0 - kCorrCC), X0, Y0, H, W, HW,
                tid, nthreads, vec_load != 0);
        }
        cp_async_commit();
        cp_async_wait_prev();  // the chunk of this iteration has landed
        __syncthreads();
        const float* s1 = corr_smem + cur * (G::S1 + G::S2);
        const float* s2 = s1 + G::S1;
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
        __syncthreads();  // the next iteration refills this stage
        cur ^= 1;
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

// Any max_displacement, and the small pyramid levels (where the tile kernel
// would run on a handful of CTAs): one thread per output element, the
// channel sum in channel order; batch n at base + n * stride.
__global__ void corr_generic_kernel(const float* __restrict__ in1, const float* __restrict__ in2,
    float* __restrict__ out, int N, int C, int H, int W, int md, int legacy, int64_t s1, int64_t s2, int64_t so)
{
    pdl_enter();
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
            const float* a = in1 + n * s1 + pix;
            const float* b = in2 + n * s2 + static_cast<int64_t>(y2) * W + x2;
            for (int c = 0; c < C; ++c)
                acc = acc + __ldg(a + c * HW) * __ldg(b + c * HW);
        }
        if (legacy)
            acc = __fdiv_rn(acc, static_cast<float>(C));
        out[n * so + static_cast<int64_t>(d) * HW + pix] = acc;
    }
}

cudaError_t launch_corr_generic(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md,
    int legacy, int64_t s1, int64_t s2, int64_t so, cudaStream_t st)
{
    const int64_t P = 2 * md + 1;
    const int64_t total = static_cast<int64_t>(N) * P * P * H * W;
    const int64_t blocks = (total + 255) / 256;
    const cudaError_t e = launch_pdl(corr_generic_kernel, dim3(static_cast<unsigned>(blocks < 152 * 64 ? blocks : 152 * 64)),
        dim3(256), 0, st, f1, f2, out, N, C, H, W, md, legacy, s1, s2, so);
    return e != cudaSuccess ? e : cudaGetLastError();
}

template <int MD>
cudaError_t launch_corr_tile(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int legacy,
    int64_t s1, int64_t s2, int64_t so, cudaStream_t st)
{
    using G = CorrGeom<MD>;
    constexpr int smem = 2 * (G::S1 + G::S2) * static_cast<int>(sizeof(float));
    // > 48 KB of dynamic shared memory: opt in once per device
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (dev < 0 || dev >= 64)
            return cudaErrorInvalidDevice;
        if (!done[dev]) {
            if ((e = cudaFuncSetAttribute(corr_tile_kernel<MD>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) !=
                cudaSuccess)
                return e;
            done[dev] = true;
        }
    }
    auto a16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    dim3 block(8, kCorrTH, 2 * MD + 1);
    dim3 grid((W + kCorrTW - 1) / kCorrTW, (H + kCorrTH - 1) / kCorrTH, N);
    // 128-bit stores need rows that start on 16 bytes: W % 4 == 0 and aligned outputs
    const int vec = ((W & 3) == 0) && a16(out) && ((so & 3) == 0);
    // 128-bit loads additionally need the f2 halo origin X0 - md on the grid
    const int vec_load = ((W & 3) == 0) && (MD % 4 == 0) && a16(f1) && a16(f2) && ((s1 & 3) == 0) && ((s2 & 3) == 0);
    const cudaError_t el = launch_pdl(corr_tile_kernel<MD>, grid, block, smem, st, f1, f2, out, C, H, W, legacy, vec,
        vec_load, s1, s2, so);
    if (el != cudaSuccess)
        return el;
    return cudaGetLastError();
}

constexpr int kWarpCG = 8;  // channels per thread

// The Warp op's per-pixel taps (warp.cc:71-133): bilinear weights, the
// in-range mask and whether the sample is taken (mask > 0.999).
struct OpTap {
    float wTL, wTR, wBL, wBR;
    bool tl, tr, bl, br, take;
    int xl, yt;
};

__device__ __forceinline__ OpTap op_tap(float flx, float fly, int x, int y, int H, int W)
{
    const float xf = static_cast<float>(x) + flx;
    const float yf = static_cast<float>(y) + fly;
    const float fxl = floorf(xf), fyt = floorf(yf);
    const float a = xf - fxl, b = yf - fyt;
    const float xR = fxl + 1.0f, yB = fyt + 1.0f;
    const bool mL = (0.0f <= fxl && fxl <= static_cast<float>(W - 1));
    const bool mR = (0.0f <= xR && xR <= static_cast<float>(W - 1));
    const bool mT = (0.0f <= fyt && fyt <= static_cast<float>(H - 1));
    const bool mB = (0.0f <= yB && yB <= static_cast<float>(H - 1));
    const float ia = 1.0f - a, ib = 1.0f - b;
    OpTap t;
    t.wTL = ia * ib;
    t.wTR = a * ib;
    t.wBL = ia * b;
    t.wBR = a * b;
    t.tl = mT && mL;
    t.tr = mT && mR;
    t.bl = mB && mL;
    t.br = mB && mR;
    float mask = 0.0f;
    mask += t.tl ? t.wTL : 0.0f;
    mask += t.tr ? t.wTR : 0.0f;
    mask += t.bl ? t.wBL : 0.0f;
    mask += t.br ? t.wBR : 0.0f;
    t.take = mask > 0.999f;
    t.xl = t.take ? static_cast<int>(fxl) : 0;
    t.yt = t.take ? static_cast<int>(fyt) : 0;
    return t;
}

// The Warp op for planes of fewer than 2^31 pixels: 64 x (4 PX) pixels per
// block (a warp on 32 consecutive pixels of a row: coalesced flow reads and
// output writes), PX pixels per thread (rows y, y + 4, ...), CG channels
// each, every tap of the thread loaded before the first blend (one branch on
// `take` per pixel, the in-range predicate per tap); blockIdx.z = batch *
// groups + channel group.  kFull: C is a multiple of CG.  Where the sample
// is taken every weight is finite and >= 0, so a tap that is not loaded
// (held as 0) adds w * 0 = +0, the same +0 the reference's guarded sum adds
// (warp.cc:116-126); where it is not taken the output is 0 (the weights may
// then be NaN, from a NaN or infinite flow).
template <int CG, bool kFull, int PX>
__global__ void __launch_bounds__(256) warp_op2d_kernel(const float* __restrict__ in, const float* __restrict__ flow,
    float* __restrict__ out, int C, int H, int W, int64_t sin, int64_t sfl, int64_t sout, int groups)
{
    pdl_enter();
    const int x = blockIdx.x * 64 + (threadIdx.x & 63);
    const int yb = blockIdx.y * (4 * PX) + (threadIdx.x >> 6);
    if (x >= W || yb >= H)
        return;
    const int n = blockIdx.z / groups;
    const int c0 = (blockIdx.z - n * groups) * CG;
    const int HW = H * W;
    const float* fl = flow + n * sfl;
    const float* src = in + n * sin + static_cast<int64_t>(c0) * HW;
    OpTap t[PX];
    int oTL[PX];
#pragma unroll
    for (int k = 0; k < PX; ++k) {
        const int y = min(yb + 4 * k, H - 1);  // a row past the end repeats the last (not stored)
        const int p = y * W + x;
        t[k] = op_tap(__ldg(fl + p), __ldg(fl + HW + p), x, y, H, W);
        oTL[k] = t[k].yt * W + t[k].xl;
    }
    float q[PX][CG][4];
#pragma unroll
    for (int k = 0; k < PX; ++k) {
#pragma unroll
        for (int c = 0; c < CG; ++c)
#pragma unroll
            for (int j = 0; j < 4; ++j)
                q[k][c][j] = 0.0f;
        if (t[k].take) {
#pragma unroll
            for (int c = 0; c < CG; ++c) {
                const float* sc = src + static_cast<int64_t>(c) * HW + oTL[k];
                const bool ok = kFull || c0 + c < C;
                if (ok && t[k].tl)
                    q[k][c][0] = __ldg(sc);
                if (ok && t[k].tr)
                    q[k][c][1] = __ldg(sc + 1);
                if (ok && t[k].bl)
                    q[k][c][2] = __ldg(sc + W);
                if (ok && t[k].br)
                    q[k][c][3] = __ldg(sc + W + 1);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < PX; ++k) {
        const int y = yb + 4 * k;
        if (y >= H)
            continue;
        float* dst = out + n * sout + static_cast<int64_t>(c0) * HW + (y * W + x);
#pragma unroll
        for (int c = 0; c < CG; ++c) {
            if (!(kFull || c0 + c < C))
                continue;
            float val = 0.0f;
            val += t[k].wTL * q[k][c][0];
            val += t[k].wTR * q[k][c][1];
            val += t[k].wBL * q[k][c][2];
            val += t[k].wBR * q[k][c][3];
            dst[static_cast<int64_t>(c) * HW] = t[k].take ? val : 0.0f;
        }
    }
}

__global__ void warp_op_kernel(const float* __restrict__ in, const float* __restrict__ flow, float* __restrict__ out,
    int C, int H, int W, int64_t sin, int64_t sfl, int64_t sout)
{
    pdl_enter();
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

// ---- double-precision ops (correlation.cc:115-139, warp.cc:48-58) ----------
// The reference's CPU kernels also accept DOUBLE tensors.  These are the
// same loops on the device: one thread per output element, the channel sum
// in channel order, every product and sum rounded separately (the library is
// built without contraction), so they equal correlation.cc / warp.cc's
// double instantiations bit for bit.  Correctness paths, not hot paths.
__global__ void corr_f64_kernel(const double* __restrict__ f1, const double* __restrict__ f2, double* __restrict__ out,
    int C, int H, int W, int md)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= HW)
        return;
    const int P = 2 * md + 1;
    const int pp = blockIdx.y;
    const int n = blockIdx.z;
    const int h = static_cast<int>(i / W), w = static_cast<int>(i % W);
    const int h2 = h + pp / P - md, w2 = w + pp % P - md;
    const double* a = f1 + static_cast<int64_t>(n) * C * HW + i;
    double acc = 0.0;
    if (h2 >= 0 && h2 < H && w2 >= 0 && w2 < W) {
        const double* b = f2 + static_cast<int64_t>(n) * C * HW + static_cast<int64_t>(h2) * W + w2;
        for (int c = 0; c < C; ++c)
            acc += a[c * HW] * b[c * HW];
    }
    out[(static_cast<int64_t>(n) * P * P + pp) * HW + i] = acc;
}

__global__ void warp_f64_kernel(const double* __restrict__ in, const double* __restrict__ flow,
    double* __restrict__ out, int C, int H, int W)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= HW)
        return;
    const int n = blockIdx.z;
    const int y = static_cast<int>(i / W), x = static_cast<int>(i % W);
    const double xf = static_cast<double>(x) + flow[static_cast<int64_t>(n) * 2 * HW + i];
    const double yf = static_cast<double>(y) + flow[(static_cast<int64_t>(n) * 2 + 1) * HW + i];
    const double alpha = xf - floor(xf);
    const double beta = yf - floor(yf);
    const double xL = floor(xf), xR = floor(xf) + 1.0;
    const double yT = floor(yf), yB = floor(yf) + 1.0;
    const bool mL = 0 <= xL && xL <= static_cast<double>(W - 1);
    const bool mR = 0 <= xR && xR <= static_cast<double>(W - 1);
    const bool mT = 0 <= yT && yT <= static_cast<double>(H - 1);
    const bool mB = 0 <= yB && yB <= static_cast<double>(H - 1);
    const bool tl = mT && mL, tr = mT && mR, bl = mB && mL, br = mB && mR;
    double mask = 0.0;
    mask += (1.0 - alpha) * (1.0 - beta) * (tl ? 1.0 : 0.0);
    mask += (alpha) * (1.0 - beta) * (tr ? 1.0 : 0.0);
    mask += (1.0 - alpha) * (beta) * (bl ? 1.0 : 0.0);
    mask += (alpha) * (beta) * (br ? 1.0 : 0.0);
    const bool keep = mask > 0.999;
    // tap offsets only where the tap is inside the map
    const int64_t oTL = tl ? static_cast<int64_t>(yT) * W + static_cast<int64_t>(xL) : 0;
    const int64_t oTR = tr ? static_cast<int64_t>(yT) * W + static_cast<int64_t>(xR) : 0;
    const int64_t oBL = bl ? static_cast<int64_t>(yB) * W + static_cast<int64_t>(xL) : 0;
    const int64_t oBR = br ? static_cast<int64_t>(yB) * W + static_cast<int64_t>(xR) : 0;
    for (int c = 0; c < C; ++c) {
        const double* src = in + (static_cast<int64_t>(n) * C + c) * HW;
        double val = 0.0;
        if (keep) {
            val += (1.0 - alpha) * (1.0 - beta) * (tl ? src[oTL] : 0.0);
            val += (alpha) * (1.0 - beta) * (tr ? src[oTR] : 0.0);
            val += (1.0 - alpha) * (beta) * (bl ? src[oBL] : 0.0);
            val += (alpha) * (beta) * (br ? src[oBR] : 0.0);
        }
        out[(static_cast<int64_t>(n) * C + c) * HW + i] = val;
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
    // the tile kernel's CTAs: 32 x 4 pixels each; below 64 of them the
    // per-output kernel has far more parallelism (same sums, same bits)
    const int64_t tile_ctas = static_cast<int64_t>((W + 31) / 32) * ((H + 3) / 4) * N;
    if (md >= 1 && md <= 4 && tile_ctas < 64)
        return launch_corr_generic(f1, f2, out, N, C, H, W, md, legacy, s1, s2, so, st);
    switch (md) {
        case 1:
            return launch_corr_tile<1>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        case 2:
            return launch_corr_tile<2>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        case 3:
            return launch_corr_tile<3>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        case 4:
            return launch_corr_tile<4>(f1, f2, out, N, C, H, W, legacy, s1, s2, so, st);
        default:
            return launch_corr_generic(f1, f2, out, N, C, H, W, md, legacy, s1, s2, so, st);
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
    if (HW < (int64_t(1) << 31)) {
        // image-shaped inputs (C = 3) take one group of three; feature maps groups of eight
        const int cg = C == 3 ? 3 : kWarpCG;
        const int groups = (C + cg - 1) / cg;
        const int px = C == 3 ? 2 : 1;  // pixels per thread
        const int rows = 4 * px;
        if (static_cast<int64_t>(N) * groups <= 65535 && (H + rows - 1) / rows <= 65535) {
            dim3 grid(static_cast<unsigned>((W + 63) / 64), static_cast<unsigned>((H + rows - 1) / rows), N * groups);
            auto k = C == 3 ? warp_op2d_kernel<3, true, 2>
                   : (C % kWarpCG == 0 ? warp_op2d_kernel<kWarpCG, true, 1> : warp_op2d_kernel<kWarpCG, false, 1>);
            const cudaError_t e = launch_pdl(k, grid, dim3(256), 0, st, in, flow, out, C, H, W, sin, sfl, sout, groups);
            return e != cudaSuccess ? e : cudaGetLastError();
        }
    }
    dim3 grid(static_cast<unsigned>((HW + 255) / 256), (C + kWarpCG - 1) / kWarpCG, N);
    const cudaError_t e = launch_pdl(warp_op_kernel, grid, dim3(256), 0, st, in, flow, out, C, H, W, sin, sfl, sout);
    if (e != cudaSuccess)
        return e;
    return cudaGetLastError();
}

cudaError_t launch_correlation_f64(const double* f1, const double* f2, double* out, int N, int C, int H, int W, int md,
    cudaStream_t st)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int P = 2 * md + 1;
    dim3 grid(static_cast<unsigned>((HW + 255) / 256), P * P, N);
    corr_f64_kernel<<<grid, 256, 0, st>>>(f1, f2, out, C, H, W, md);
    return cudaGetLastError();
}

cudaError_t launch_warp_op_f64(const double* in, const double* flow, double* out, int N, int C, int H, int W,
    cudaStream_t st)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    dim3 grid(static_cast<unsigned>((HW + 255) / 256), 1, N);
    warp_f64_kernel<<<grid, 256, 0, st>>>(in, flow, out, C, H, W);
    return cudaGetLastError();
}

}  // namespace vsc
