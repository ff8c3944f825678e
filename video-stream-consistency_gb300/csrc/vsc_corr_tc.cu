// Correlation on the tensor cores (tcgen05) in BF16 or FP16 with FP32
// accumulation: the reduced-precision form of custom::Correlation (the
// legacy = 0 layout of correlation.cc:45-143 / correlation_cuda.cu:97-175).
//
// For one row y of the output and a segment of kTcM = 128 pixels starting at
// x0, and one displacement row dy, the 2 md + 1 correlations of every pixel
// are a band of the product
//     D_dy[m][n] = sum_c f1[c][y][x0 + m] * f2[c][y + dy][x0 - md + n],
// m < 128, n < kTcN = 144 (>= 128 + 2 md): pixel m's value for displacement
// dx is D_dy[m][m + dx + md].  Each D_dy is one M = 128, N = 144 MMA chain
// over K = channels (padded to a multiple of 16 with zeros), accumulated in
// Tensor Memory; both operands come from shared memory, staged by one 5-D TMA
// load each from the features in a "chunked" layout
//     [n][y][c / 8][x][c % 8]  (16-bit elements, channels padded to Cp),
// which the TMA box {8, pixels, Cp / 8} turns directly into the operand's
// 8-row x 16-byte core-matrix grid (K-adjacent core matrices pixels x 16 B
// apart, M/N-adjacent ones 128 B apart).  Rows y + dy and columns outside
// the map are zero-filled by the TMA, which is the operator's zero outside.
// The epilogue reads each warp's 32 lanes x 48 columns of D_dy out of Tensor
// Memory, stages them in shared memory and picks the diagonal band.
//
// Per-level scaling: each operand is multiplied by a power of two 2^k chosen
// from its largest magnitude (|f| 2^k in [2^13, 2^14)) before the 16-bit
// conversion, which keeps FP16 clear of overflow and of its subnormal range;
// the sums are multiplied by 2^-(k1 + k2) afterwards (exact).
#include "vsc_internal.h"
#include "vsc_math.cuh"
#include "vsc_ptx.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <mutex>

namespace vsc {
namespace {

constexpr int kTcM = 128;        // pixels per tile (MMA M, TMEM lanes)
constexpr int kTcN = 144;        // f2 window per displacement row (MMA N)
constexpr int kTcCols = 48;      // TMEM columns one warp reads per row: 32 + 2 md
constexpr int kTcPitch = 52;     // staging row pitch (floats): 53 * lane spreads the diagonal over all banks
constexpr int kTcThreads = 128;  // 4 warps, one per 32 TMEM lanes
constexpr uint32_t kTmemCols = 256;
constexpr int kTcWaitSpins = 1 << 22;  // bounded mbarrier waits (about a second)
constexpr int kTcStageBytes = 4 * 32 * kTcPitch * 4;
// At least this much dynamic shared memory per CTA, so that at most two CTAs
// share an SM and their Tensor Memory (2 x 256 of 512 columns) never waits.
constexpr int kTcMinSmem = 100 * 1024;
static_assert(kTcN >= kTcM + 2 * kTcMaxMd && kTcN % 16 == 0 && kTcN <= 256, "MMA N");
static_assert(32 * 3 + kTcCols <= kTcN, "epilogue columns inside the accumulator");
static_assert(kTcCols >= 32 + 2 * kTcMaxMd, "epilogue columns cover the band");

__host__ __device__ constexpr uint32_t align1k(uint32_t v) { return (v + 1023u) & ~1023u; }

__host__ __device__ constexpr uint32_t tc_smem_bytes(int cp)
{
    return 1024 + align1k(kTcM * cp * 2) + 2 * align1k(kTcN * cp * 2) + kTcStageBytes + 64;
}

__global__ void __launch_bounds__(kTcThreads, 1)
    corr_tc_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB,
        float* __restrict__ out, const float* __restrict__ scales, int H, int W, int Cp, int md, uint32_t idesc,
        int* __restrict__ timeout_flag)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sA = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~static_cast<uintptr_t>(1023));
    const uint32_t bytesA = kTcM * Cp * 2;
    const uint32_t bytesB = kTcN * Cp * 2;
    unsigned char* sB[2];
    sB[0] = sA + align1k(bytesA);
    sB[1] = sB[0] + align1k(bytesB);
    float* stage = reinterpret_cast<float*>(sB[1] + align1k(bytesB));
    uint64_t* bars = reinterpret_cast<uint64_t*>(stage + 4 * 32 * kTcPitch);  // A, B0, B1, MMA
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 4);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x0 = blockIdx.x * kTcM, y = blockIdx.y, n = blockIdx.z;
    const int P = 2 * md + 1;

    if (warp == 0) {
        ptx::tmem_alloc(tmem_slot, kTmemCols);
        ptx::tmem_relinquish();
    }
    if (tid == 0) {
        *abort_flag = 0;
        for (int i = 0; i < 4; ++i)
            ptx::mbar_init(&bars[i], 1);
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // thread 0 owns the pipeline: loads in flight per B buffer and phase parities
    bool a_pending = false;
    bool b_pending[2] = {false, false};
    uint32_t b_par[2] = {0, 0};
    bool mma_pending = false;
    uint32_t mma_par = 0;
    if (tid == 0) {
        ptx::mbar_expect_tx(&bars[0], bytesA);
        ptx::tma_load_5d(sA, &mA, 0, x0, 0, y, n, &bars[0]);
        a_pending = true;
        for (int d = 0; d < 2 && d < P; ++d) {
            ptx::mbar_expect_tx(&bars[1 + d], bytesB);
            ptx::tma_load_5d(sB[d], &mB, 0, x0 - md, 0, y + d - md, n, &bars[1 + d]);
            b_pending[d] = true;
        }
    }
    const float inv_scale = 1.0f / (scales[0] * scales[1]);  // powers of two: exact
    float* st = stage + warp * 32 * kTcPitch;
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int x = x0 + warp * 32 + lane;
    float* obase = out + static_cast<int64_t>(n) * P * P * HW + static_cast<int64_t>(y) * W + x;
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;

    for (int d = 0; d < P; ++d) {
        const int buf = d & 1;
        if (tid == 0) {
            bool ok = true;
            if (a_pending) {
                ok = ptx::mbar_wait_bounded(&bars[0], 0, kTcWaitSpins);
                a_pending = !ok;
            }
            if (ok) {
                ok = ptx::mbar_wait_bounded(&bars[1 + buf], b_par[buf], kTcWaitSpins);
                if (ok) {
                    b_pending[buf] = false;
                    b_par[buf] ^= 1u;
                }
            }
            if (ok) {
                ptx::tc_fence_after();
                const uint32_t a0 = ptx::smem_u32(sA), b0 = ptx::smem_u32(sB[buf]);
                for (int kk = 0; kk < Cp / 16; ++kk) {
                    const uint64_t ad = ptx::umma_desc_kmajor(a0 + kk * 2 * kTcM * 16, kTcM * 16, 128);
                    const uint64_t bd = ptx::umma_desc_kmajor(b0 + kk * 2 * kTcN * 16, kTcN * 16, 128);
                    ptx::umma_f16(tmem, ad, bd, idesc, kk > 0);
                }
                ptx::umma_commit(&bars[3]);
                mma_pending = true;
                mma_par = static_cast<uint32_t>(d & 1);
                ok = ptx::mbar_wait_bounded(&bars[3], d & 1, kTcWaitSpins);
                if (ok) {
                    mma_pending = false;
                    if (d + 2 < P) {  // the MMA has read this buffer: refill it
                        ptx::mbar_expect_tx(&bars[1 + buf], bytesB);
                        ptx::tma_load_5d(sB[buf], &mB, 0, x0 - md, 0, y + d + 2 - md, n, &bars[1 + buf]);
                        b_pending[buf] = true;
                    }
                }
            }
            if (!ok)
                *abort_flag = 1;
        }
        __syncthreads();
        if (*abort_flag)
            break;
        ptx::tc_fence_after();
        uint32_t v0[32], v1[16];
        ptx::tmem_ld32(tmem + lane_base + warp * 32, v0);
        ptx::tmem_ld16(tmem + lane_base + warp * 32 + 32, v1);
        ptx::tmem_ld_wait();
        float4* row = reinterpret_cast<float4*>(st + lane * kTcPitch);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            row[j] = make_float4(__uint_as_float(v0[4 * j]), __uint_as_float(v0[4 * j + 1]),
                __uint_as_float(v0[4 * j + 2]), __uint_as_float(v0[4 * j + 3]));
#pragma unroll
        for (int j = 0; j < 4; ++j)
            row[8 + j] = make_float4(__uint_as_float(v1[4 * j]), __uint_as_float(v1[4 * j + 1]),
                __uint_as_float(v1[4 * j + 2]), __uint_as_float(v1[4 * j + 3]));
        __syncwarp();
        if (x < W) {
            float* o = obase + static_cast<int64_t>(d) * P * HW;
            const float* srow = st + lane * kTcPitch + lane;
            for (int k = 0; k < P; ++k)
                o[k * HW] = srow[k] * inv_scale;
        }
        __syncwarp();
        ptx::tc_fence_before();
        __syncthreads();
    }

    if (tid == 0 && *abort_flag) {
        atomicExch(timeout_flag, 1);
        // let the copies and the MMA still in flight land before the CTA exits
        if (a_pending)
            ptx::mbar_wait_bounded(&bars[0], 0, kTcWaitSpins);
        for (int b = 0; b < 2; ++b)
            if (b_pending[b])
                ptx::mbar_wait_bounded(&bars[1 + b], b_par[b], kTcWaitSpins);
        if (mma_pending)
            ptx::mbar_wait_bounded(&bars[3], mma_par, kTcWaitSpins);
    }
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, kTmemCols);
    }
}

// ---- operand preparation ---------------------------------------------------------
// |max| of a tensor as the bits of a non-negative float (ordered like uint).
__global__ void absmax_kernel(const float* __restrict__ a, int64_t n, unsigned int* __restrict__ result)
{
    float m = 0.0f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        m = fmaxf(m, fabsf(a[i]));
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(result, __float_as_uint(m));
}

// scale = 2^k with |max| * 2^k in [2^13, 2^14); 1 for zero or non-finite maxima.
__global__ void scales_kernel(const unsigned int* __restrict__ maxbits, float* __restrict__ scales)
{
    const int i = threadIdx.x;
    if (i >= 2)
        return;
    const float m = __uint_as_float(maxbits[i]);
    float s = 1.0f;
    if (m > 0.0f && m <= 3.4e38f) {
        int e;
        frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
        s = ldexpf(1.0f, min(60, max(-60, 14 - e)));
    }
    scales[i] = s;
}

template <bool kBf16>
__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    if (kBf16) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    } else {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
}

// NCHW float -> chunked 16-bit [n][y][c / 8][x][c % 8], scaled, zero-padded
// to chunks * 8 channels.  One thread per pixel; reads coalesced along x
// for every channel, one 16-byte store per chunk.
template <bool kBf16>
__global__ void to_chunked_kernel(const float* __restrict__ in, uint4* __restrict__ out, const float* __restrict__ scale,
    int C, int H, int W, int chunks)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W)
        return;
    const int y = blockIdx.y, n = blockIdx.z;
    const float s = *scale;
    const int64_t HW = static_cast<int64_t>(H) * W;
    const float* src = in + static_cast<int64_t>(n) * C * HW + static_cast<int64_t>(y) * W + x;
    uint4* dst = out + (static_cast<int64_t>(n) * H + y) * chunks * W + x;
    for (int q = 0; q < chunks; ++q) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = q * 8 + j;
            v[j] = c < C ? src[c * HW] * s : 0.0f;
        }
        dst[static_cast<int64_t>(q) * W] = make_uint4(pack2<kBf16>(v[0], v[1]), pack2<kBf16>(v[2], v[3]),
            pack2<kBf16>(v[4], v[5]), pack2<kBf16>(v[6], v[7]));
    }
}

// custom::Warp (the single-precision arithmetic of warp_op_kernel) writing
// the chunked 16-bit operand layout directly, scaled by *scale: the warped
// second-frame features of the flow estimator go straight to the tensor-core
// correlation.  One thread per pixel and chunk of 8 channels.
template <bool kBf16>
__global__ void warp_to_chunked_kernel(const float* __restrict__ in, const float* __restrict__ flow,
    uint4* __restrict__ out, const float* __restrict__ scale, int C, int H, int W, int chunks, int64_t sin,
    int64_t sfl, int64_t sout)
{
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= HW)
        return;
    const int q = blockIdx.y, n = blockIdx.z;
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
    const float s = *scale;
    float v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int c = q * 8 + j;
        float val = 0.0f;
        if (take && c < C) {
            const float* src = in + n * sin + static_cast<int64_t>(c) * HW;
            val += tl ? wTL * __ldg(src + oTL) : 0.0f;
            val += tr ? wTR * __ldg(src + oTL + 1) : 0.0f;
            val += bl ? wBL * __ldg(src + oTL + W) : 0.0f;
            val += br ? wBR * __ldg(src + oTL + W + 1) : 0.0f;
        }
        v[j] = val * s;
    }
    out[n * sout + (static_cast<int64_t>(y) * chunks + q) * W + x] =
        make_uint4(pack2<kBf16>(v[0], v[1]), pack2<kBf16>(v[2], v[3]), pack2<kBf16>(v[4], v[5]), pack2<kBf16>(v[6], v[7]));
}

// 5-D map over a chunked tensor: {c % 8, x, c / 8, y, n}, box {8, pixels, cp / 8, 1, 1}.
bool encode_chunked_map(CUtensorMap* m, const void* base, int N, int H, int W, int cp, int box_pixels)
{
    EncodeTiledFn fn = tensor_map_encoder();
    if (!fn)
        return false;
    const cuuint64_t q = static_cast<cuuint64_t>(cp / 8);
    const cuuint64_t dims[5] = {8, static_cast<cuuint64_t>(W), q, static_cast<cuuint64_t>(H),
        static_cast<cuuint64_t>(N)};
    const cuuint64_t strides[4] = {16, static_cast<cuuint64_t>(W) * 16, q * W * 16, static_cast<cuuint64_t>(H) * q * W * 16};
    const cuuint32_t box[5] = {8, static_cast<cuuint32_t>(box_pixels), static_cast<cuuint32_t>(q), 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 5, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The dynamic shared memory opt-in is a per-device function attribute.
cudaError_t tc_prepare_device()
{
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!done[dev]) {
        e = cudaFuncSetAttribute(corr_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(tc_smem_bytes(kTcMaxChannelsPadded)));
        if (e != cudaSuccess)
            return e;
        done[dev] = true;
    }
    return cudaSuccess;
}

}  // namespace

int tc_padded_channels(int C) { return (C + 15) / 16 * 16; }

size_t corr_tc_workspace_bytes(int N, int C, int H, int W)
{
    const size_t chunked = static_cast<size_t>(N) * H * W * tc_padded_channels(C) * 2;
    return 256 + 2 * ((chunked + 255) / 256 * 256);
}

cudaError_t launch_corr_tc_chunked(const void* f1c, const void* f2c, float* out, const float* scales, int N, int Cp,
    int H, int W, int md, bool bf16, cudaStream_t st)
{
    if (Cp % 16 != 0 || Cp > kTcMaxChannelsPadded || md < 0 || md > kTcMaxMd)
        return cudaErrorInvalidValue;
    cudaError_t e = tc_prepare_device();
    if (e != cudaSuccess)
        return e;
    int* flag = nullptr;
    if ((e = device_timeout_flag(&flag)) != cudaSuccess)
        return e;
    CUtensorMap mA, mB;
    if (!encode_chunked_map(&mA, f1c, N, H, W, Cp, kTcM) || !encode_chunked_map(&mB, f2c, N, H, W, Cp, kTcN))
        return cudaErrorInvalidValue;
    const uint32_t smem = std::max<uint32_t>(tc_smem_bytes(Cp), kTcMinSmem);
    const dim3 grid((W + kTcM - 1) / kTcM, H, N);
    corr_tc_kernel<<<grid, kTcThreads, smem, st>>>(mA, mB, out, scales, H, W, Cp, md,
        ptx::umma_idesc_f16(bf16, kTcM, kTcN), flag);
    return cudaGetLastError();
}

cudaError_t launch_to_chunked(const float* in, void* out, const float* scale, int N, int C, int H, int W, bool bf16,
    cudaStream_t st)
{
    const int chunks = tc_padded_channels(C) / 8;
    const dim3 g((W + 127) / 128, H, N);
    if (bf16)
        to_chunked_kernel<true><<<g, 128, 0, st>>>(in, static_cast<uint4*>(out), scale, C, H, W, chunks);
    else
        to_chunked_kernel<false><<<g, 128, 0, st>>>(in, static_cast<uint4*>(out), scale, C, H, W, chunks);
    return cudaGetLastError();
}

cudaError_t launch_warp_to_chunked(const float* in, const float* flow, void* out, const float* scale, int N, int C,
    int H, int W, int64_t sin, int64_t sfl, int64_t sout_bytes, bool bf16, cudaStream_t st)
{
    const int chunks = tc_padded_channels(C) / 8;
    const int64_t HW = static_cast<int64_t>(H) * W;
    const dim3 g(static_cast<unsigned>((HW + 255) / 256), chunks, N);
    const int64_t so = sout_bytes / 16;
    if (bf16)
        warp_to_chunked_kernel<true><<<g, 256, 0, st>>>(in, flow, static_cast<uint4*>(out), scale, C, H, W, chunks,
            sin, sfl, so);
    else
        warp_to_chunked_kernel<false><<<g, 256, 0, st>>>(in, flow, static_cast<uint4*>(out), scale, C, H, W, chunks,
            sin, sfl, so);
    return cudaGetLastError();
}

cudaError_t launch_corr_tc(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md,
    bool bf16, void* workspace, cudaStream_t st)
{
    const int cp = tc_padded_channels(C);
    const size_t chunked = static_cast<size_t>(N) * H * W * cp * 2;
    const size_t chunked_al = (chunked + 255) / 256 * 256;
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    unsigned int* maxbits = reinterpret_cast<unsigned int*>(ws);
    float* scales = reinterpret_cast<float*>(ws + 16);
    uint4* c1 = reinterpret_cast<uint4*>(ws + 256);
    uint4* c2 = reinterpret_cast<uint4*>(ws + 256 + chunked_al);
    cudaError_t e = cudaMemsetAsync(maxbits, 0, 8, st);
    if (e != cudaSuccess)
        return e;
    const int64_t total = static_cast<int64_t>(N) * C * H * W;
    const unsigned blocks = static_cast<unsigned>(std::min<int64_t>((total + 255) / 256, 4096));
    absmax_kernel<<<blocks, 256, 0, st>>>(f1, total, maxbits);
    absmax_kernel<<<blocks, 256, 0, st>>>(f2, total, maxbits + 1);
    scales_kernel<<<1, 32, 0, st>>>(maxbits, scales);
    const int chunks = cp / 8;
    const dim3 g((W + 127) / 128, H, N);
    if (bf16) {
        to_chunked_kernel<true><<<g, 128, 0, st>>>(f1, c1, scales, C, H, W, chunks);
        to_chunked_kernel<true><<<g, 128, 0, st>>>(f2, c2, scales + 1, C, H, W, chunks);
    } else {
        to_chunked_kernel<false><<<g, 128, 0, st>>>(f1, c1, scales, C, H, W, chunks);
        to_chunked_kernel<false><<<g, 128, 0, st>>>(f2, c2, scales + 1, C, H, W, chunks);
    }
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    return launch_corr_tc_chunked(c1, c2, out, scales, N, cp, H, W, md, bf16, st);
}

}  // namespace vsc
