// Inference of the learned flow upsampler on the tensor cores (tcgen05).
//
// Each 3x3 convolution (zero padding) is an implicit GEMM.  Activations are
// FP16 in a chunked planar layout [n][c / 8][y][x][c % 8].  For a segment of
// kUpM = 128 output positions x0 ... x0 + 127, output row y is
//     out[o][y][x] = sum over ty, tx and input channels c of
//                    act[c][y + ty - 1][x + tx - 1] * w[o][ty][tx][c] + bias.
// Input row j contributes to output rows j + 1 (ty = 0), j (ty = 1) and
// j - 1 (ty = 2).  Output rows are accumulated in groups of kUpGR = 8 in one
// Tensor Memory slot of 8 NO columns, output row y0 + t at columns
// NO (7 - t), so the three rows an input row feeds are adjacent columns in
// ty order, which is the order of the packed weights: one MMA chain per
// input row (M = 128 positions, N = NO times the number of its rows inside
// the group, K = input channels x horizontal taps in steps of 16) writes
// straight into its rows' columns.  A slot is cleared by one MMA of zero
// operands and every later MMA accumulates; once its ten input rows are in,
// the epilogue reads it once and frees it.  A tcgen05.mma of M = 128, K = 16
// costs about max(45, N / 2) cycles on GB300, so a group of 8 rows costs
// about 351 cycles per row, and with two slots the MMAs of one group overlap
// the epilogue of the other: the layer is bound by HBM, not by the
// accumulator ring.
//
// A work item is a segment of kUpRC = 16 output rows (two groups); each
// group's ten input rows stream through a ring of row buffers (one TMA box
// {8, 130, 1, chunks} per row: the segment with its one-pixel halo,
// zero-filled outside the image, which is the convolution's zero padding);
// the two rows the groups share are loaded for each, so that every buffer has
// one reader.  The A operand is
// a row buffer seen from position tx (8 positions x 16 bytes per core
// matrix, M-adjacent core matrices 128 bytes apart, K-adjacent ones a chunk
// plane apart).  Weights [tx][chunk][ty * NO + o][8] (FP16, output channels
// padded to NO, input channels to the K chunks) stay in shared memory for the
// launch.  The first layer's three input channels (base flow u, v and luma)
// occupy one chunk; its second K chunk is a zero plane that is never loaded.
//
// Persistent and warp-specialised: warp 0 issues the TMA loads; warp 1 (which
// owns Tensor Memory) issues the MMAs of every item's first group and warp 18
// those of its second (one thread issues an MMA about every 90 cycles, twice
// the tensor pipe's time for these shapes); warps 2-17 are the epilogue, four
// per 32 Tensor Memory lanes, each taking two output rows of a group.  Epilogue:
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

constexpr int kUpM = 128;                // output positions per segment (MMA M, Tensor Memory lanes)
constexpr int kUpGR = 8;                 // output rows per accumulator group
constexpr int kUpRC = 16;                // output rows per work item
constexpr int kUpGPI = kUpRC / kUpGR;    // groups per work item
constexpr int kUpGRows = kUpGR + 2;      // input rows per group
constexpr int kUpLoads = kUpGPI * kUpGRows;  // row loads per work item (each group has its own)
constexpr int kUpTW = kUpM + 2;          // positions loaded per row (one-pixel halo)
constexpr int kUpRowBufs = 22;           // row buffers in shared memory (more than an item's 18 rows)
constexpr int kUpSlots = 2;              // group accumulators in Tensor Memory
constexpr uint32_t kUpTmemCols = 512;
constexpr int kUpEpiWarps = 16;          // 4 lane quarters x 4 pairs of a group's rows
constexpr int kUpWaitSpins = 1 << 22;    // bounded mbarrier waits (about a second)
constexpr int kUpIssuerWarp1 = 2 + kUpEpiWarps;  // the second group's MMA issuer (the first: warp 1)
constexpr int kUpThreads = (3 + kUpEpiWarps) * 32;
constexpr int kUpPlaneBytes = kUpTW * 16;  // one chunk plane of a row buffer
constexpr uint32_t kUpZeroBytes = 8192;  // zero operands of the slot-clearing MMA (A 4 KB, B 8 KB overlapped)
constexpr int kUpSmemLimit = 232448;
constexpr uint32_t kUpMinSmem = 120 * 1024;
static_assert(kUpRC % kUpGR == 0 && kUpEpiWarps == 4 * (kUpGR / 2), "epilogue rows");
static_assert(kUpRowBufs >= kUpLoads + 2 && kUpGPI == kUpSlots, "row buffers; one slot and issuer per group");

__host__ __device__ constexpr uint32_t up_align1k(uint32_t v) { return (v + 1023u) & ~1023u; }
// a row buffer: the TMA destination and the MMA operands need 128-byte alignment
__host__ __device__ constexpr uint32_t up_row_bytes(int kch) { return (kch * kUpPlaneBytes + 127u) & ~127u; }

// Per-layer shape: kch K chunks of 8 channels (lch of them loaded, the rest
// zero), no output channels per vertical tap in the MMA (N = 3 no).
struct TcLayer {
    int kch, lch, no, ci, co;
    size_t wt_off;  // byte offset of the layer's packed weights
};
constexpr TcLayer kTcLayers[4] = {{2, 1, 32, 3, 32, 0}, {4, 4, 32, 32, 32, 9216}, {4, 4, 32, 32, 32, 27648},
    {4, 4, 16, 32, 2, 46080}};
constexpr size_t kTcWeightBytes = 55296;

__host__ __device__ constexpr uint32_t up_weight_bytes(int kch, int no) { return 3u * kch * 3u * no * 16u; }
static_assert(kTcLayers[3].wt_off + up_weight_bytes(4, 16) == kTcWeightBytes, "packed weight layout");

// row buffers, weights, the zero operands, bias, barriers (full / empty per row
// buffer, full / empty per slot, the drain barrier, the Tensor Memory address and
// the abort flag)
constexpr uint32_t kBarBytes = (2 * kUpRowBufs + 3 * kUpSlots + 2) * 8;
__host__ __device__ constexpr uint32_t up_smem_bytes(int kch, int no)
{
    return 1024 + up_align1k(kUpRowBufs * up_row_bytes(kch)) + up_align1k(up_weight_bytes(kch, no)) +
           kUpZeroBytes + 32 * 4 + kBarBytes;
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
    constexpr int N3 = 3 * NO;                      // the weights' N rows: three vertical taps
    constexpr int kSlotCols = kUpGR * NO;           // one group's accumulator
    constexpr uint32_t kRowBytes = up_row_bytes(KCH);
    constexpr uint32_t kWBytes = up_weight_bytes(KCH, NO);
    constexpr uint32_t idesc1 = ptx::umma_idesc_f16(false, kUpM, NO);
    constexpr uint32_t idesc2 = ptx::umma_idesc_f16(false, kUpM, 2 * NO);
    constexpr uint32_t idesc3 = ptx::umma_idesc_f16(false, kUpM, N3);
    constexpr uint32_t idesc0 = ptx::umma_idesc_f16(false, kUpM, kSlotCols);
    static_assert(NO % 16 == 0 && kSlotCols <= 256 && kUpSlots * kSlotCols <= static_cast<int>(kUpTmemCols),
        "MMA N and the accumulator ring");
    static_assert(2 * 2048 <= kUpZeroBytes && 2 * kSlotCols * 16 <= static_cast<int>(kUpZeroBytes),
        "zero operands (A: 128 x 16, B: kSlotCols x 16 halves)");
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    unsigned char* rows = base;
    unsigned char* wts = rows + up_align1k(kUpRowBufs * kRowBytes);
    unsigned char* zero = wts + up_align1k(kWBytes);
    float* sbias = reinterpret_cast<float*>(zero + kUpZeroBytes);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sbias + 32);
    uint64_t* full = bars;                        // [kUpRowBufs]
    uint64_t* empty = full + kUpRowBufs;          // [kUpRowBufs]
    uint64_t* sfull = empty + kUpRowBufs;         // [kUpSlots]
    uint64_t* sempty = sfull + kUpSlots;          // [kUpSlots]
    uint64_t* drain = sempty + kUpSlots;          // [kUpSlots] each MMA issuer's last commit on abort
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + kUpSlots);
    volatile int* abort = reinterpret_cast<volatile int*>(drain + kUpSlots + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nseg = (W + kUpM - 1) / kUpM, nchunk = (H + kUpRC - 1) / kUpRC;
    const int items = N * nchunk * nseg;

    // weights and bias into shared memory; the zero operands and the K chunks that
    // are never loaded are zero
    for (uint32_t i = threadIdx.x; i < kWBytes / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(wts)[i] = wpk[i];
    for (uint32_t i = threadIdx.x; i < kUpZeroBytes / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(zero)[i] = make_uint4(0u, 0u, 0u, 0u);
    for (int i = threadIdx.x; i < 32; i += blockDim.x)
        sbias[i] = i < co ? bias[i] : 0.0f;
    if (LCH < KCH) {
        for (int b = 0; b < kUpRowBufs; ++b) {
            uint4* z = reinterpret_cast<uint4*>(rows + b * kRowBytes + LCH * kUpPlaneBytes);
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
        for (int i = 0; i < kUpRowBufs; ++i) {
            ptx::mbar_init(&full[i], 1);
            ptx::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < kUpSlots; ++i) {
            ptx::mbar_init(&sfull[i], 1);
            ptx::mbar_init(&sempty[i], kUpEpiWarps);  // every epilogue warp reads each group once
            ptx::mbar_init(&drain[i], 1);
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // row loads are counted over the whole CTA (u): row buffer u % kUpRowBufs; item
    // k of the CTA owns loads k * kUpLoads ..., group g's ten input rows from
    // k * kUpLoads + g * kUpGRows (the two rows the groups share are loaded for
    // each).  Group g of every item is issued by its own thread (warp 1 for g = 0,
    // warp kUpIssuerWarp1 for g = 1) into Tensor Memory slot g; the epilogue
    // counts groups over the CTA (G), slot G % kUpSlots = g.
    if (warp == 0) {
        // ---- TMA producer -------------------------------------------------------------
        if (lane == 0) {
            int u = 0;
            bool ok = true;
            for (int it = blockIdx.x; ok && it < items; it += gridDim.x) {
                const int seg = it % nseg, rest = it / nseg;
                const int chunk = rest % nchunk, n = rest / nchunk;
                for (int j = 0; j < kUpLoads; ++j, ++u) {
                    const int b = u % kUpRowBufs;
                    if (!(ok = up_wait(&empty[b], ((u / kUpRowBufs) & 1) ^ 1, abort)))
                        break;
                    const int y = chunk * kUpRC - 1 + (j / kUpGRows) * kUpGR + j % kUpGRows;
                    ptx::mbar_expect_tx(&full[b], LCH * kUpPlaneBytes);
                    ptx::tma_load_5d(rows + b * kRowBytes, &mIn, 0, seg * kUpM - 1, y, 0, n, &full[b]);
                }
            }
            if (*abort)  // let every copy issued land before the CTA exits
                for (int i = 0; i < kUpRowBufs && i < u; ++i) {
                    const int v = u - 1 - i;
                    ptx::mbar_wait_bounded(&full[v % kUpRowBufs], (v / kUpRowBufs) & 1, kUpWaitSpins);
                }
        }
    } else if (warp == 1 || warp == kUpIssuerWarp1) {
        // ---- MMA issuers: group g of every item ------------------------------------------
        if (lane == 0) {
            const int g = warp == 1 ? 0 : 1;
            int m = 0;  // items done by this issuer (slot g's uses)
            bool ok = true;
            // Descriptors are built once; an operand at byte offset d from its base is
            // the base descriptor + d / 16 (the start-address field, which cannot carry:
            // shared memory stays below 256 KB).
            const uint64_t adesc0 = ptx::umma_desc_kmajor(ptx::smem_u32(rows), kUpPlaneBytes, 128);
            const uint64_t bdesc0 = ptx::umma_desc_kmajor(ptx::smem_u32(wts), N3 * 16, 128);
            const uint64_t zadesc = ptx::umma_desc_kmajor(ptx::smem_u32(zero), 2048, 128);
            const uint64_t zbdesc = ptx::umma_desc_kmajor(ptx::smem_u32(zero), kSlotCols * 16, 128);
            const uint32_t dslot = tmem + g * kSlotCols;
            for (int it = blockIdx.x; ok && it < items; it += gridDim.x, ++m) {
                if (!(ok = up_wait(&sempty[g], (m & 1) ^ 1, abort)))
                    break;
                ptx::tc_fence_after();
                ptx::umma_f16(dslot, zadesc, zbdesc, idesc0, false);  // clear the group's accumulator
                // the group's output rows 0 ... 7 read its input rows r = 0 ... 9
                for (int r = 0; r < kUpGRows; ++r) {
                    const int u = m * kUpLoads + g * kUpGRows + r, b = u % kUpRowBufs;
                    if (!(ok = up_wait(&full[b], (u / kUpRowBufs) & 1, abort)))
                        break;
                    ptx::tc_fence_after();
                    // input row r feeds output row t = r - ty for ty = 0, 1, 2 where
                    // 0 <= t < kUpGR: ty_lo ... ty_hi, at columns NO (kUpGR - 1 - t)
                    const int ty_lo = r > kUpGR - 1 ? r - (kUpGR - 1) : 0;
                    const int ty_hi = r < 2 ? r : 2;
                    const int nt = ty_hi - ty_lo + 1;
                    const uint32_t idesc = nt == 3 ? idesc3 : (nt == 2 ? idesc2 : idesc1);
                    const uint32_t dcol = dslot + NO * (kUpGR - 1 - r + ty_lo);
                    const uint64_t ab = adesc0 + ((b * kRowBytes) >> 4);
                    const uint64_t bb = bdesc0 + ((ty_lo * NO * 16) >> 4);
#pragma unroll
                    for (int tx = 0; tx < 3; ++tx) {
#pragma unroll
                        for (int k = 0; k < KCH / 2; ++k) {
                            const uint64_t ad = ab + ((2 * k * kUpPlaneBytes + tx * 16) >> 4);
                            const uint64_t bd = bb + (((tx * KCH + 2 * k) * N3 * 16) >> 4);
                            ptx::umma_f16(dcol, ad, bd, idesc, true);
                        }
                    }
                    ptx::umma_commit(&empty[b]);  // the row buffer is read once the MMAs finish
                }
                if (ok)
                    ptx::umma_commit(&sfull[g]);  // the group's accumulator is complete
            }
            if (*abort) {  // the MMAs in flight finish before Tensor Memory is freed
                ptx::umma_commit(&drain[g]);
                ptx::mbar_wait_bounded(&drain[g], 0, kUpWaitSpins);
            }
        }
    } else {
        // ---- epilogue: a group accumulator -> registers -> global -----------------------
        const int e = warp - 2;
        const int q = warp & 3;                   // this warp's 32 Tensor Memory lanes
        const int rp = e >> 2;                    // its rows of a group: 2 rp, 2 rp + 1
        const uint32_t lane_base = static_cast<uint32_t>(q * 32) << 16;
        const int64_t HW = static_cast<int64_t>(H) * W;
        int G = 0;
        bool ok = true;
        for (int it = blockIdx.x; ok && it < items; it += gridDim.x) {
            const int seg = it % nseg, rest = it / nseg;
            const int chunk = rest % nchunk, n = rest / nchunk;
            const int x = seg * kUpM + q * 32 + lane;
            for (int g = 0; g < kUpGPI; ++g, ++G) {
                const int sl = G % kUpSlots;
                // warp-uniform outcome: the Tensor Memory loads below are warp-collective
                ok = __all_sync(0xffffffffu, up_wait(&sfull[sl], (G / kUpSlots) & 1, abort));
                if (!ok)
                    break;
                ptx::tc_fence_after();
                constexpr int KC = kFinish ? 16 : 32;  // columns read per row (the last layer needs 2 of 16)
                float acc[2][KC];
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const int t = 2 * rp + r;
                    const uint32_t ta = tmem + lane_base + sl * kSlotCols + NO * (kUpGR - 1 - t);
                    uint32_t v[KC];
                    if constexpr (KC == 32)
                        ptx::tmem_ld32(ta, v);
                    else
                        ptx::tmem_ld16(ta, v);
                    ptx::tmem_ld_wait();
#pragma unroll
                    for (int o = 0; o < KC; ++o)
                        acc[r][o] = __uint_as_float(v[o]);
                }
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0)
                    ptx::mbar_arrive(&sempty[sl]);
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    const int y = chunk * kUpRC + g * kUpGR + 2 * rp + r;
                    if (x >= W || y >= H)
                        continue;
                    const int64_t p = static_cast<int64_t>(y) * W + x;
                    if (!kFinish) {
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            uint32_t h[4];
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                const int o = c * 8 + 2 * j;
                                const __half2 hv = __floats2half2_rn(fmaxf(acc[r][o] + sbias[o], 0.0f),
                                    fmaxf(acc[r][o + 1] + sbias[o + 1], 0.0f));
                                h[j] = *reinterpret_cast<const uint32_t*>(&hv);
                            }
                            reinterpret_cast<uint4*>(out)[(static_cast<int64_t>(n) * 4 + c) * HW + p] =
                                make_uint4(h[0], h[1], h[2], h[3]);
                        }
                    } else {
                        const float ru = acc[r][0] + sbias[0], rv = acc[r][1] + sbias[1];
                        const float* in = input + (static_cast<int64_t>(n) * HW + p) * 3;
                        const bool take = fmaxf(fabsf(ru), fabsf(rv)) <= max_residual;
                        float* o = flow + n * s_out + p * 3;
                        o[0] = take ? in[0] + ru : in[0];
                        o[1] = take ? in[1] + rv : in[1];
                        o[2] = 0.0f;
                    }
                }
            }
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
// One layer's FP32 weights [out][tap][in] -> [tx][chunk][ty * no + out][8] in
// FP16, zero for padded input and output channels.
__global__ void up_pack_weights_kernel(const float* __restrict__ w, int ci, int co, int kch, int no,
    __half* __restrict__ wtc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n3 = 3 * no;
    if (i >= 3 * kch * n3 * 8)
        return;
    const int j = i % 8, nr = (i / 8) % n3, c8 = (i / (8 * n3)) % kch, tx = i / (8 * n3 * kch);
    const int ty = nr / no, o = nr % no, t = ty * 3 + tx, c = c8 * 8 + j;
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
    const cuuint32_t box[5] = {8, kUpTW, 1, static_cast<cuuint32_t>(chunks), 1};
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
    const int items = N * ((H + kUpRC - 1) / kUpRC) * ((W + kUpM - 1) / kUpM);
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
        const int n = static_cast<int>(up_weight_bytes(L.kch, L.no) / 2);
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
