// Inference of the learned flow upsampler on the tensor cores (tcgen05).
//
// Each 3x3 convolution (zero padding) is an implicit GEMM.  For one output
// row y and a segment of kUpM = 128 pixels starting at x0,
//     D[m][o] = sum over taps t = (ty, tx) and input channels c of
//               act[c][y + ty - 1][x0 + m + tx - 1] * w[o][t][c],
// which is nine MMA chains (one per tap, K = input channels in steps of 16)
// into one accumulator of M = 128 pixels x N output channels in Tensor
// Memory.  Activations are FP16 in a chunked planar layout
//     [n][c / 8][y][x][c % 8],
// so one TMA box {8, 130, kUpR + 2, chunks} brings a band of kUpR + 2 rows x
// 130 pixels (the segment with its one-pixel halo; zero-filled outside the
// image, which is the convolution's zero padding) into shared memory as
// [chunk][row][pixel][8].  The A operand of tap (ty, tx) for output row r is
// that buffer seen from (row r + ty, pixel tx): 8 consecutive pixels x 16
// bytes are one core matrix, M-adjacent core matrices 128 bytes apart,
// K-adjacent ones one chunk plane apart.  Weights [tap][chunk][out][8] (FP16,
// out padded to the MMA's N, in to the K chunks) stay in shared memory for the
// whole launch.  The first layer's three input channels (base flow u, v and
// luma) occupy one chunk; its second K chunk is a zero plane that is never
// loaded.
//
// Persistent and warp-specialised: warp 0 issues the TMA loads (a ring of
// band buffers), warp 1 the MMAs (and owns Tensor Memory; two accumulator
// sets of kUpR rows), warps 2-5 the epilogue, one per 32 Tensor Memory lanes:
// bias, ReLU, FP16 and the chunked store for the inner layers; for the last
// layer the residual test and the finished flow (base + r where
// max(|r_u|, |r_v|) <= max_residual, else base).  Every mbarrier wait is
// bounded; a wait that runs out stops all roles and sets the device timeout
// flag.
#include "vsc_internal.h"
#include "vsc_math.cuh"
#include "vsc_ptx.cuh"

#include <cuda_fp16.h>

#include <mutex>

namespace vsc {
namespace {

constexpr int kUpM = 128;               // pixels per segment (MMA M, Tensor Memory lanes)
constexpr int kUpR = 4;                 // output rows per band
constexpr int kUpTW = kUpM + 2;         // band width with the halo
constexpr int kUpStages = 3;            // band buffers
constexpr uint32_t kUpTmemCols = 256;   // two accumulator sets of kUpR x 32 columns
constexpr int kUpWaitSpins = 1 << 22;   // bounded mbarrier waits (about a second)
constexpr int kUpThreads = 6 * 32;
constexpr int kUpPlaneBytes = (kUpR + 2) * kUpTW * 16;  // one chunk plane of a band
constexpr int kUpSmemLimit = 232448;
constexpr uint32_t kUpMinSmem = 120 * 1024;
static_assert(kUpPlaneBytes % 16 == 0, "chunk planes on the 16-byte grid");
static_assert(2 * kUpR * 32 <= static_cast<int>(kUpTmemCols), "accumulators inside the allocation");

__host__ __device__ constexpr uint32_t up_align1k(uint32_t v) { return (v + 1023u) & ~1023u; }

// Per-layer shape: kch K chunks of 8 channels (lch of them loaded, the rest
// zero), no output columns of the MMA.
struct TcLayer {
    int kch, lch, no, ci, co;
    size_t wt_off;  // byte offset of the layer's packed weights
};
constexpr TcLayer kTcLayers[4] = {{2, 1, 32, 3, 32, 0}, {4, 4, 32, 32, 32, 9216}, {4, 4, 32, 32, 32, 27648},
    {4, 4, 16, 32, 2, 46080}};
constexpr size_t kTcWeightBytes = 55296;
static_assert(kTcLayers[3].wt_off + 9 * 4 * 16 * 16 == kTcWeightBytes, "packed weight layout");

__host__ __device__ constexpr uint32_t up_weight_bytes(int kch, int no) { return 9u * kch * no * 16u; }

__host__ __device__ constexpr uint32_t up_smem_bytes(int kch, int no)
{
    return 1024 + kUpStages * up_align1k(kch * kUpPlaneBytes) + up_align1k(up_weight_bytes(kch, no)) + 32 * 4 + 256;
}

// Bounded wait that also gives up when another role has aborted; a wait that
// runs out raises the abort for everyone.
__device__ __forceinline__ bool up_wait(uint64_t* bar, uint32_t parity, volatile int* abort)
{
    for (int i = 0; i < kUpWaitSpins; ++i) {
        if (ptx::mbar_try_wait(bar, parity))
            return true;
        if ((i & 63) == 63 && *abort)
            return false;
        if (i > 256)
            __nanosleep(64);
    }
    *abort = 1;
    return false;
}

// ---- the convolution --------------------------------------------------------------
// KCH / LCH / NO as TcLayer; kFinish: last layer (residual test and flow out).
template <int KCH, int LCH, int NO, bool kFinish>
__global__ void __launch_bounds__(kUpThreads, 1)
    up_conv_tc_kernel(const __grid_constant__ CUtensorMap mIn, const uint4* __restrict__ wpk,
        const float* __restrict__ bias, int co, __half* __restrict__ out, const float* __restrict__ input,
        float* __restrict__ flow, int64_t s_out, float max_residual, int N, int H, int W,
        int* __restrict__ timeout_flag)
{
    constexpr uint32_t kStageBytes = up_align1k(KCH * kUpPlaneBytes);
    constexpr uint32_t kWBytes = up_weight_bytes(KCH, NO);
    constexpr uint32_t idesc = ptx::umma_idesc_f16(false, kUpM, NO);
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    unsigned char* stages = base;
    unsigned char* wts = stages + kUpStages * kStageBytes;
    float* sbias = reinterpret_cast<float*>(wts + up_align1k(kWBytes));
    uint64_t* bars = reinterpret_cast<uint64_t*>(sbias + 32);
    uint64_t* full = bars;            // [kUpStages]
    uint64_t* empty = bars + 3;       // [kUpStages]
    uint64_t* dfull = bars + 6;       // [2]
    uint64_t* dempty = bars + 8;      // [2]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 10);
    volatile int* abort = reinterpret_cast<volatile int*>(bars + 11);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nseg = (W + kUpM - 1) / kUpM, nband = (H + kUpR - 1) / kUpR;
    const int items = N * nband * nseg;

    // weights and bias into shared memory; the K chunks that are never loaded are zero
    for (uint32_t i = threadIdx.x; i < kWBytes / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(wts)[i] = wpk[i];
    for (int i = threadIdx.x; i < NO; i += blockDim.x)
        sbias[i] = i < co ? bias[i] : 0.0f;
    if (LCH < KCH) {
        for (int s = 0; s < kUpStages; ++s) {
            uint4* z = reinterpret_cast<uint4*>(stages + s * kStageBytes + LCH * kUpPlaneBytes);
            for (int i = threadIdx.x; i < (KCH - LCH) * kUpPlaneBytes / 16; i += blockDim.x)
                z[i] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor-core reads
    if (warp == 1) {
        ptx::tmem_alloc(tmem_slot, kUpTmemCols);
        ptx::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        *abort = 0;
        for (int i = 0; i < kUpStages; ++i) {
            ptx::mbar_init(&full[i], 1);
            ptx::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            ptx::mbar_init(&dfull[i], 1);
            ptx::mbar_init(&dempty[i], 4);  // one arrival per epilogue warp
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---- TMA producer -------------------------------------------------------------
        if (lane == 0) {
            int u = 0;
            for (int it = blockIdx.x; it < items; it += gridDim.x) {
                const int seg = it % nseg, rest = it / nseg;
                const int band = rest % nband, n = rest / nband;
                const int s = u % kUpStages;
                if (!up_wait(&empty[s], ((u / kUpStages) & 1) ^ 1, abort))
                    break;
                ptx::mbar_expect_tx(&full[s], LCH * kUpPlaneBytes);
                ptx::tma_load_5d(stages + s * kStageBytes, &mIn, 0, seg * kUpM - 1, band * kUpR - 1, 0, n, &full[s]);
                ++u;
            }
            if (*abort)  // let every copy issued land before the CTA exits
                for (int i = 0; i < kUpStages && i < u; ++i) {
                    const int v = u - 1 - i;
                    ptx::mbar_wait_bounded(&full[v % kUpStages], (v / kUpStages) & 1, kUpWaitSpins);
                }
        }
    } else if (warp == 1) {
        // ---- MMA issuer ---------------------------------------------------------------
        if (lane == 0) {
            int u = 0, ud = 0;
            const uint32_t w0 = ptx::smem_u32(wts);
            for (int it = blockIdx.x; it < items; it += gridDim.x) {
                const int s = u % kUpStages, b = ud & 1;
                if (!up_wait(&full[s], (u / kUpStages) & 1, abort))
                    break;
                if (!up_wait(&dempty[b], ((ud >> 1) & 1) ^ 1, abort))
                    break;
                ptx::tc_fence_after();
                const uint32_t a0 = ptx::smem_u32(stages + s * kStageBytes);
                for (int r = 0; r < kUpR; ++r) {
                    const uint32_t dcol = tmem + b * (kUpR * NO) + r * NO;
#pragma unroll
                    for (int t = 0; t < 9; ++t) {
                        const int ty = t / 3, tx = t % 3;
#pragma unroll
                        for (int k = 0; k < KCH / 2; ++k) {
                            const uint64_t ad = ptx::umma_desc_kmajor(
                                a0 + 2 * k * kUpPlaneBytes + ((r + ty) * kUpTW + tx) * 16, kUpPlaneBytes, 128);
                            const uint64_t bd = ptx::umma_desc_kmajor(w0 + (t * KCH + 2 * k) * NO * 16, NO * 16, 128);
                            ptx::umma_f16(dcol, ad, bd, idesc, t > 0 || k > 0);
                        }
                    }
                }
                ptx::umma_commit(&dfull[b]);   // accumulators ready
                ptx::umma_commit(&empty[s]);   // band buffer read
                ++u;
                ++ud;
            }
            if (*abort && ud > 0) {  // the MMAs in flight finish before Tensor Memory is freed
                const int v = ud - 1;
                ptx::mbar_wait_bounded(&dfull[v & 1], (v >> 1) & 1, kUpWaitSpins);
            }
        }
    } else {
        // ---- epilogue: Tensor Memory -> registers -> global ------------------------------
        const int q = warp & 3;  // this warp's 32 Tensor Memory lanes
        const uint32_t lane_base = static_cast<uint32_t>(q * 32) << 16;
        const int64_t HW = static_cast<int64_t>(H) * W;
        int ud = 0;
        for (int it = blockIdx.x; it < items; it += gridDim.x, ++ud) {
            const int seg = it % nseg, rest = it / nseg;
            const int band = rest % nband, n = rest / nband;
            const int b = ud & 1;
            // warp-uniform outcome: the Tensor Memory loads below are warp-collective
            if (!__all_sync(0xffffffffu, up_wait(&dfull[b], (ud >> 1) & 1, abort)))
                break;
            ptx::tc_fence_after();
            const int x = seg * kUpM + q * 32 + lane;
            for (int r = 0; r < kUpR; ++r) {
                const int y = band * kUpR + r;
                const uint32_t ta = tmem + lane_base + b * (kUpR * NO) + r * NO;
                const bool inside = x < W && y < H;
                const int64_t p = static_cast<int64_t>(y) * W + x;
                if (!kFinish) {
                    uint32_t v[32];
                    ptx::tmem_ld32(ta, v);
                    ptx::tmem_ld_wait();
                    if (inside) {
#pragma unroll
                        for (int c8 = 0; c8 < 4; ++c8) {
                            uint32_t h[4];
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                const int o = c8 * 8 + 2 * j;
                                const float lo = fmaxf(__uint_as_float(v[o]) + sbias[o], 0.0f);
                                const float hi = fmaxf(__uint_as_float(v[o + 1]) + sbias[o + 1], 0.0f);
                                const __half2 hv = __floats2half2_rn(lo, hi);
                                h[j] = *reinterpret_cast<const uint32_t*>(&hv);
                            }
                            reinterpret_cast<uint4*>(out)[(static_cast<int64_t>(n) * 4 + c8) * HW + p] =
                                make_uint4(h[0], h[1], h[2], h[3]);
                        }
                    }
                } else {
                    uint32_t v[16];
                    ptx::tmem_ld16(ta, v);
                    ptx::tmem_ld_wait();
                    if (inside) {
                        const float ru = __uint_as_float(v[0]) + sbias[0];
                        const float rv = __uint_as_float(v[1]) + sbias[1];
                        const float* in = input + (static_cast<int64_t>(n) * HW + p) * 3;
                        const bool take = fmaxf(fabsf(ru), fabsf(rv)) <= max_residual;
                        float* o = flow + n * s_out + p * 3;
                        o[0] = take ? in[0] + ru : in[0];
                        o[1] = take ? in[1] + rv : in[1];
                        o[2] = 0.0f;
                    }
                }
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0)
                ptx::mbar_arrive(&dempty[b]);  // the accumulators may be overwritten
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, kUpTmemCols);
    }
    if (threadIdx.x == 0 && *abort)
        atomicExch(timeout_flag, 1);
}

// ---- operand preparation ------------------------------------------------------------
// One layer's FP32 weights [out][tap][in] -> [tap][chunk][out][8] in FP16,
// zero for padded input and output channels.
__global__ void up_pack_weights_kernel(const float* __restrict__ w, int ci, int co, int kch, int no,
    __half* __restrict__ wtc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * kch * no * 8)
        return;
    const int j = i % 8, o = (i / 8) % no, c8 = (i / (8 * no)) % kch, t = i / (8 * no * kch);
    const int c = c8 * 8 + j;
    wtc[i] = __float2half_rn(o < co && c < ci ? w[(o * 9 + t) * ci + c] : 0.0f);
}

// prepared input (u, v, luma as floats) -> the first layer's chunk plane (FP16, 5 zero channels)
__global__ void up_input_half_kernel(const float* __restrict__ input, uint4* __restrict__ in16, int64_t npx)
{
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= npx)
        return;
    const __half2 a = __floats2half2_rn(input[p * 3], input[p * 3 + 1]);
    const __half2 b = __floats2half2_rn(input[p * 3 + 2], 0.0f);
    in16[p] = make_uint4(*reinterpret_cast<const uint32_t*>(&a), *reinterpret_cast<const uint32_t*>(&b), 0u, 0u);
}

bool encode_act_map(CUtensorMap* m, const void* base, int N, int H, int W, int chunks)
{
    EncodeTiledFn fn = tensor_map_encoder();
    if (!fn)
        return false;
    const cuuint64_t dims[5] = {8, static_cast<cuuint64_t>(W), static_cast<cuuint64_t>(H),
        static_cast<cuuint64_t>(chunks), static_cast<cuuint64_t>(N)};
    const cuuint64_t plane = static_cast<cuuint64_t>(H) * W * 16;
    const cuuint64_t strides[4] = {16, static_cast<cuuint64_t>(W) * 16, plane, plane * chunks};
    const cuuint32_t box[5] = {8, kUpTW, kUpR + 2, static_cast<cuuint32_t>(chunks), 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int KCH, int LCH, int NO, bool kFinish>
cudaError_t run_layer(int l, const void* wtc, const float* prm, const void* in, __half* out, const float* input,
    float* flow, int64_t s_out, float max_residual, int N, int H, int W, int sms, int* flag, cudaStream_t st)
{
    // at least kUpMinSmem, so that one CTA (and one Tensor Memory allocation) occupies an SM
    constexpr uint32_t smem = up_smem_bytes(KCH, NO) > kUpMinSmem ? up_smem_bytes(KCH, NO) : kUpMinSmem;
    static_assert(smem <= static_cast<uint32_t>(kUpSmemLimit), "shared memory per CTA");
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(up_conv_tc_kernel<KCH, LCH, NO, kFinish>,
            cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    });
    if (attr != cudaSuccess)
        return attr;
    CUtensorMap m;
    if (!encode_act_map(&m, in, N, H, W, LCH))
        return cudaErrorInvalidValue;
    const int items = N * ((H + kUpR - 1) / kUpR) * ((W + kUpM - 1) / kUpM);
    up_conv_tc_kernel<KCH, LCH, NO, kFinish><<<std::min(items, sms), kUpThreads, smem, st>>>(m,
        reinterpret_cast<const uint4*>(static_cast<const unsigned char*>(wtc) + kTcLayers[l].wt_off),
        prm + kUpLayers[l].b_off, kUpLayers[l].co, out, input, flow, s_out, max_residual, N, H, W, flag);
    return cudaGetLastError();
}

}  // namespace

size_t upsampler_tc_weight_bytes() { return kTcWeightBytes; }

// first layer's input plane (16 B/px) and two activation maps (64 B/px each)
size_t upsampler_tc_work_bytes(int N, int H, int W) { return static_cast<size_t>(N) * H * W * (16 + 64 + 64); }

cudaError_t launch_upsampler_tc_pack(const float* prm, void* wtc, cudaStream_t st)
{
    for (int l = 0; l < 4; ++l) {
        const TcLayer& L = kTcLayers[l];
        const int n = 9 * L.kch * L.no * 8;
        up_pack_weights_kernel<<<(n + 255) / 256, 256, 0, st>>>(prm + kUpLayers[l].w_off, L.ci, L.co, L.kch, L.no,
            reinterpret_cast<__half*>(static_cast<unsigned char*>(wtc) + L.wt_off));
    }
    return cudaGetLastError();
}

cudaError_t launch_upsampler_tc(const void* wtc, const float* prm, const float* input, void* work, float* flow, int N,
    int H, int W, float max_residual, int64_t s_out, cudaStream_t st, int* launches)
{
    if (N <= 0 || H <= 0 || W <= 0)
        return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int* flag = nullptr;
    if (e == cudaSuccess)
        e = device_timeout_flag(&flag);
    if (e != cudaSuccess)
        return e;
    const int64_t npx = static_cast<int64_t>(N) * H * W;
    unsigned char* wb = static_cast<unsigned char*>(work);
    __half* in16 = reinterpret_cast<__half*>(wb);
    __half* actA = reinterpret_cast<__half*>(wb + npx * 16);
    __half* actB = reinterpret_cast<__half*>(wb + npx * 80);
    up_input_half_kernel<<<static_cast<unsigned>((npx + 255) / 256), 256, 0, st>>>(input, reinterpret_cast<uint4*>(in16),
        npx);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    if ((e = run_layer<2, 1, 32, false>(0, wtc, prm, in16, actA, nullptr, nullptr, 0, 0.0f, N, H, W, sms, flag, st)) !=
        cudaSuccess)
        return e;
    if ((e = run_layer<4, 4, 32, false>(1, wtc, prm, actA, actB, nullptr, nullptr, 0, 0.0f, N, H, W, sms, flag, st)) !=
        cudaSuccess)
        return e;
    if ((e = run_layer<4, 4, 32, false>(2, wtc, prm, actB, actA, nullptr, nullptr, 0, 0.0f, N, H, W, sms, flag, st)) !=
        cudaSuccess)
        return e;
    e = run_layer<4, 4, 16, true>(3, wtc, prm, actA, nullptr, input, flow, s_out, max_residual, N, H, W, sms, flag, st);
    if (launches)
        *launches += 5;
    return e;
}

}  // namespace vsc
