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
//     [n][y][c / 16][x][c % 16]  (16-bit elements, channels padded to Cp),
// which the TMA box {16, pixels, Cp / 16} with the 32-byte swizzle turns
// directly into the K-major operand layout of that swizzle: one chunk plane
// per MMA K step (pixels x 32 bytes), every box row one 32-byte L2 sector.
// Rows y + dy and columns outside the map are zero-filled by the TMA, which
// is the operator's zero outside.
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
// warps: 0 TMA producer, 1 MMA issuer + Tensor Memory owner, then 1..3
// epilogue groups of four warps (one per 32 TMEM lanes); group g drains the
// accumulators of rows u with u % groups == g
constexpr int kMaxEpiGroups = 3;
constexpr int kMaxStagesA = 2, kMaxStagesB = 4, kStagesD = 3;
constexpr uint32_t kTmemCols = 512;    // three accumulators
constexpr uint32_t kDStride = 160;     // TMEM columns between accumulators (>= kTcN, multiple of 32)
constexpr int kTcWaitSpins = 1 << 22;  // bounded mbarrier waits (about a second)
constexpr int kTcGroupStageBytes = 4 * 32 * kTcPitch * 4;  // one epilogue group's staging
constexpr int kTcBarBytes = 256;
constexpr int kTcSmemLimit = 232448;   // dynamic shared memory per CTA on sm_103
// at least this much dynamic shared memory, so that one CTA (and one
// 512-column Tensor Memory allocation) occupies an SM
constexpr int kTcMinSmem = 120 * 1024;
static_assert(kTcN >= kTcM + 2 * kTcMaxMd && kTcN % 16 == 0 && kTcN <= 256, "MMA N");
static_assert(32 * 3 + kTcCols <= kTcN, "epilogue columns inside the accumulator");
static_assert(kTcCols >= 32 + 2 * kTcMaxMd, "epilogue columns cover the band");
static_assert((kStagesD - 1) * kDStride + kTcN <= kTmemCols, "accumulators inside the allocation");

__host__ __device__ constexpr uint32_t align1k(uint32_t v) { return (v + 1023u) & ~1023u; }

struct TcPlan {
    int stages_a, stages_b, groups;
    uint32_t smem;
};

__host__ uint32_t tc_smem_need(int cp, int sa, int sb, int g)
{
    return 1024 + sa * align1k(kTcM * cp * 2) + sb * align1k(kTcN * cp * 2) + g * kTcGroupStageBytes + kTcBarBytes;
}

// Buffers that fit in shared memory for Cp channels: three epilogue groups,
// two A tiles and four B rows when they fit; B rows, then A tiles, then
// epilogue groups are given up in that order (208 channels: 1, 2, 2).
__host__ TcPlan tc_plan(int cp)
{
    TcPlan p{kMaxStagesA, kMaxStagesB, kMaxEpiGroups, 0};
    while (tc_smem_need(cp, p.stages_a, p.stages_b, p.groups) > static_cast<uint32_t>(kTcSmemLimit)) {
        if (p.stages_b > 2)
            --p.stages_b;
        else if (p.stages_a > 1)
            --p.stages_a;
        else if (p.groups > 1)
            --p.groups;
        else
            break;
    }
    p.smem = std::max<uint32_t>(tc_smem_need(cp, p.stages_a, p.stages_b, p.groups), kTcMinSmem);
    return p;
}

// Base + stride, not arrays of pointers: indexed by run-time stage numbers,
// arrays would live in local memory and every access would wait on it.
struct TcShared {
    unsigned char* a;  // stage i at a + i * a_stride
    unsigned char* b;
    uint32_t a_stride, b_stride;
    float* stage;
    uint64_t *full_a, *empty_a, *full_b, *empty_b, *full_d, *empty_d;
    uint32_t* tmem_slot;
    volatile int* abort;
};

// Bounded wait that also gives up when another role has aborted; a wait that
// runs out raises the abort for everyone.
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* abort)
{
    for (int i = 0; i < kTcWaitSpins; ++i) {
        if (ptx::mbar_try_wait(bar, parity))
            return true;
        if ((i & 63) == 63 && *abort)
            return false;
        if (i > 256)  // hand-offs are short: poll first, then back off
            __nanosleep(64);
    }
    *abort = 1;
    return false;
}

// Persistent, warp-specialised: work item = (batch n, row y, 128-pixel
// segment); every CTA walks items blockIdx.x, +gridDim.x, ...  Rings:
// A tiles (producer -> MMA, freed by the MMA's commit after the item's last
// row), B rows (freed by the commit of the MMA that read them), accumulators
// in Tensor Memory (MMA -> epilogue, freed by the four epilogue warps as soon
// as their columns are in registers, before the shared-memory and global
// part of the epilogue).
__global__ void __launch_bounds__((2 + 4 * kMaxEpiGroups) * 32, 1)
    corr_tc_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB,
        float* __restrict__ out, const __grid_constant__ CUtensorMap mA2, const __grid_constant__ CUtensorMap mB2,
        float* __restrict__ out2, int nprob, const float* __restrict__ scales, int N, int H, int W, int Cp, int md,
        uint32_t idesc, int stages_a, int stages_b, int groups, int ndyg, int* __restrict__ timeout_flag)
{
    extern __shared__ unsigned char smem_raw[];
    const uint32_t bytesA = kTcM * Cp * 2;
    const uint32_t bytesB = kTcN * Cp * 2;
    TcShared sh;
    {
        unsigned char* p = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                            ~static_cast<uintptr_t>(1023));
        sh.a_stride = align1k(bytesA);
        sh.b_stride = align1k(bytesB);
        sh.a = p;
        p += stages_a * sh.a_stride;
        sh.b = p;
        p += stages_b * sh.b_stride;
        sh.stage = reinterpret_cast<float*>(p);
        uint64_t* bars = reinterpret_cast<uint64_t*>(p + groups * kTcGroupStageBytes);
        sh.full_a = bars;
        sh.empty_a = bars + 2;
        sh.full_b = bars + 4;
        sh.empty_b = bars + 8;
        sh.full_d = bars + 12;
        sh.empty_d = bars + 15;
        sh.tmem_slot = reinterpret_cast<uint32_t*>(bars + 18);
        sh.abort = reinterpret_cast<volatile int*>(bars + 19);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int P = 2 * md + 1;
    const int nseg = (W + kTcM - 1) / kTcM;
    // work item: (n, segment, row y, group of displacement rows); small maps
    // split the 2 md + 1 displacement rows over ndyg items to fill the GPU
    const int rpg = (P + ndyg - 1) / ndyg;
    // nprob independent correlations of the same shape (the flow's two
    // directions) share the launch: item it belongs to problem it / items_per
    const int items_per = N * H * nseg * ndyg;
    const int items = items_per * nprob;

    if (warp == 1) {
        ptx::tmem_alloc(sh.tmem_slot, kTmemCols);
        ptx::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        *sh.abort = 0;
        for (int i = 0; i < 2; ++i) {
            ptx::mbar_init(&sh.full_a[i], 1);
            ptx::mbar_init(&sh.empty_a[i], 1);
        }
        for (int i = 0; i < 4; ++i) {
            ptx::mbar_init(&sh.full_b[i], 1);
            ptx::mbar_init(&sh.empty_b[i], 1);
        }
        for (int i = 0; i < kStagesD; ++i) {
            ptx::mbar_init(&sh.full_d[i], 1);
            ptx::mbar_init(&sh.empty_d[i], 4);  // one arrival per epilogue warp
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *sh.tmem_slot;
    // the setup above (Tensor Memory, barriers) overlaps the previous
    // kernel's tail; its outputs (this launch's operands) are read from here
    pdl_enter();

    if (warp == 0) {
        // ---- TMA producer ------------------------------------------------------
        if (lane == 0) {
            int ua = 0, ub = 0;
            bool ok = true;
            for (int it = blockIdx.x; ok && it < items; it += gridDim.x) {
                const int prob = it / items_per, il = it - prob * items_per;
                const CUtensorMap* ma = prob ? &mA2 : &mA;
                const CUtensorMap* mb = prob ? &mB2 : &mB;
                const int dyg = il % ndyg, r = il / ndyg;
                const int y = r % H, seg = (r / H) % nseg, n = r / (H * nseg);
                const int d0 = dyg * rpg, d1 = min(P, d0 + rpg);
                const int x0 = seg * kTcM;
                const int sa = ua % stages_a;
                if (!(ok = tc_wait(&sh.empty_a[sa], ((ua / stages_a) & 1) ^ 1, sh.abort)))
                    break;
                ptx::mbar_expect_tx(&sh.full_a[sa], bytesA);
                ptx::tma_load_5d(sh.a + sa * sh.a_stride, ma, 0, x0, 0, y, n, &sh.full_a[sa]);
                ++ua;
                for (int d = d0; d < d1; ++d) {
                    const int sb = ub % stages_b;
                    if (!(ok = tc_wait(&sh.empty_b[sb], ((ub / stages_b) & 1) ^ 1, sh.abort)))
                        break;
                    ptx::mbar_expect_tx(&sh.full_b[sb], bytesB);
                    ptx::tma_load_5d(sh.b + sb * sh.b_stride, mb, 0, x0 - md, 0, y + d - md, n, &sh.full_b[sb]);
                    ++ub;
                }
            }
            if (*sh.abort) {  // let every copy issued land before the CTA exits
                for (int i = 0; i < stages_a && i < ua; ++i) {
                    const int u = ua - 1 - i;
                    ptx::mbar_wait_bounded(&sh.full_a[u % stages_a], (u / stages_a) & 1, kTcWaitSpins);
                }
                for (int i = 0; i < stages_b && i < ub; ++i) {
                    const int u = ub - 1 - i;
                    ptx::mbar_wait_bounded(&sh.full_b[u % stages_b], (u / stages_b) & 1, kTcWaitSpins);
                }
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer ----------------------------------------------------------
        if (lane == 0) {
            int ua = 0, ub = 0, ud = 0;
            bool ok = true;
            for (int it = blockIdx.x; ok && it < items; it += gridDim.x) {
                const int dyg = (it % items_per) % ndyg;
                const int d0 = dyg * rpg, d1 = min(P, d0 + rpg);
                const int sa = ua % stages_a;
                if (!(ok = tc_wait(&sh.full_a[sa], (ua / stages_a) & 1, sh.abort)))
                    break;
                for (int d = d0; d < d1; ++d) {
                    const int sb = ub % stages_b, sd = ud % kStagesD;
                    if (!(ok = tc_wait(&sh.full_b[sb], (ub / stages_b) & 1, sh.abort)))
                        break;
                    if (!(ok = tc_wait(&sh.empty_d[sd], ((ud / kStagesD) & 1) ^ 1, sh.abort)))
                        break;
                    ptx::tc_fence_after();
                    const uint32_t a0 = ptx::smem_u32(sh.a + sa * sh.a_stride), b0 = ptx::smem_u32(sh.b + sb * sh.b_stride);
                    const uint32_t dcol = tmem + sd * kDStride;
                    for (int kk = 0; kk < Cp / 16; ++kk) {
                        // K step kk = the tile's chunk plane kk (rows x 32 bytes, swizzled)
                        const uint64_t ad = ptx::umma_desc_kmajor_sw32(a0 + kk * kTcM * 32);
                        const uint64_t bd = ptx::umma_desc_kmajor_sw32(b0 + kk * kTcN * 32);
                        ptx::umma_f16(dcol, ad, bd, idesc, kk > 0);
                    }
                    ptx::umma_commit(&sh.full_d[sd]);   // accumulator ready
                    ptx::umma_commit(&sh.empty_b[sb]);  // B row read
                    ++ub;
                    ++ud;
                }
                if (!ok)
                    break;
                ptx::umma_commit(&sh.empty_a[sa]);  // A tile read by every row of the item
                ++ua;
            }
            if (*sh.abort && ud > 0) {  // the MMAs still in flight finish before Tensor Memory is freed
                const int u = ud - 1;
                ptx::mbar_wait_bounded(&sh.full_d[u % kStagesD], (u / kStagesD) & 1, kTcWaitSpins);
            }
        }
    } else {
        // ---- epilogue: TMEM -> registers -> shared (diagonal) -> global -----------
        const int q = warp & 3;          // this warp's 32 TMEM lanes (the warp's rank in its warpgroup)
        const int grp = (warp - 2) >> 2;  // epilogue group
        const uint32_t lane_base = static_cast<uint32_t>(q * 32) << 16;
        float* st = sh.stage + (warp - 2) * 32 * kTcPitch;
        const float inv_scale = 1.0f / (scales[0] * scales[1]);  // powers of two: exact
        const int64_t HW = static_cast<int64_t>(H) * W;
        int ud = 0;  // accumulator use index, counted over every row of the CTA
        bool ok = true;
        for (int it = blockIdx.x; ok && it < items; it += gridDim.x) {
            const int prob = it / items_per, il = it - prob * items_per;
            const int dyg = il % ndyg, r = il / ndyg;
            const int y = r % H, seg = (r / H) % nseg, n = r / (H * nseg);
            const int d0 = dyg * rpg, d1 = min(P, d0 + rpg);
            const int x = seg * kTcM + q * 32 + lane;
            float* obase = (prob ? out2 : out) + static_cast<int64_t>(n) * P * P * HW + static_cast<int64_t>(y) * W + x;
            for (int d = d0; d < d1; ++d, ++ud) {
                if (ud % groups != grp)
                    continue;
                const int sd = ud % kStagesD;
                // warp-uniform outcome: the Tensor Memory loads below are warp-collective
                ok = __all_sync(0xffffffffu, tc_wait(&sh.full_d[sd], (ud / kStagesD) & 1, sh.abort));
                if (!ok)
                    break;
                ptx::tc_fence_after();
                uint32_t v0[32], v1[16];
                const uint32_t ta = tmem + lane_base + sd * kDStride + q * 32;
                ptx::tmem_ld32(ta, v0);
                ptx::tmem_ld16(ta + 32, v1);
                ptx::tmem_ld_wait();
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0)
                    ptx::mbar_arrive(&sh.empty_d[sd]);  // the accumulator may be overwritten
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
            }
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, kTmemCols);
    }
    if (threadIdx.x == 0 && *sh.abort)
        atomicExch(timeout_flag, 1);
}

// ---- operand preparation ---------------------------------------------------------
// |max| of a tensor as the bits of a non-negative float (ordered like uint).
// max |a| as float bits (non-negative floats order like their bit patterns):
// a grid-stride pass, a warp and then a block reduction, one atomic per
// block (blockDim.x == 256)
__global__ void __launch_bounds__(256) absmax_kernel(const float* __restrict__ a, int64_t n,
    unsigned int* __restrict__ result)
{
    __shared__ float wm[8];
    float m = 0.0f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        m = fmaxf(m, fabsf(a[i]));
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0)
        wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < 8 ? wm[threadIdx.x] : 0.0f;
        for (int o = 4; o > 0; o >>= 1)
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0)
            atomicMax(result, __float_as_uint(m));
    }
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

// The chunked 16-bit layout [n][y][c / 16][x][c % 16]: row (n, y) of the
// map, 16-channel chunks, each pixel's 16 channels 32 bytes.  A thread that
// packs 8 channels (chunk8 q of `chunks8`) writes the uint4 at this index.
__device__ __forceinline__ int64_t chunked_index(int64_t row, int q, int x, int W, int chunks8)
{
    return ((row * (chunks8 >> 1) + (q >> 1)) * W + x) * 2 + (q & 1);
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

// NCHW float -> chunked 16-bit [n][y][c / 16][x][c % 16], scaled,
// zero-padded to chunks * 8 channels.  One thread per pixel and 8 channels
// (the small pyramid levels have few pixels and up to 26 such groups);
// reads coalesced along x for every channel, one 16-byte store.
template <bool kBf16>
__global__ void to_chunked_kernel(const float* __restrict__ in, uint4* __restrict__ out, const float* __restrict__ scale,
    int C, int H, int W, int chunks)
{
    pdl_enter();
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= HW)
        return;
    const int q = blockIdx.y, n = blockIdx.z;
    const int y = HW < (int64_t(1) << 31) ? static_cast<int>(p) / W : static_cast<int>(p / W);
    const int x = static_cast<int>(p - static_cast<int64_t>(y) * W);
    const float s = *scale;
    const float* src = in + static_cast<int64_t>(n) * C * HW + p;
    float v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int c = q * 8 + j;
        v[j] = c < C ? src[c * HW] * s : 0.0f;
    }
    out[chunked_index(static_cast<int64_t>(n) * H + y, q, x, W, chunks)] = make_uint4(pack2<kBf16>(v[0], v[1]),
        pack2<kBf16>(v[2], v[3]), pack2<kBf16>(v[4], v[5]), pack2<kBf16>(v[6], v[7]));
}

// to_chunked_kernel for the five levels of a feature pyramid (N = 1) in one
// launch: a flat list of (128-pixel block, chunk) pairs, level after level.
constexpr int kChunkLevelsMax = 5;
struct ChunkLevels {
    const float* in[kChunkLevelsMax];
    uint4* out[kChunkLevelsMax];
    int C[kChunkLevelsMax], H[kChunkLevelsMax], W[kChunkLevelsMax], chunks[kChunkLevelsMax];
    int block0[kChunkLevelsMax + 1];
    int count;
};

template <bool kBf16>
__global__ void to_chunked_levels_kernel(const __grid_constant__ ChunkLevels cl, const float* __restrict__ scale)
{
    pdl_enter();
    int l = 0;
    while (l + 1 < cl.count && static_cast<int>(blockIdx.x) >= cl.block0[l + 1])
        ++l;
    const int W = cl.W[l], H = cl.H[l], C = cl.C[l], chunks = cl.chunks[l];
    const int HW = H * W, nhw = (HW + 127) / 128;
    const int b = blockIdx.x - cl.block0[l];
    const int p = (b % nhw) * 128 + threadIdx.x, q = b / nhw;
    if (p >= HW)
        return;
    const int y = p / W, x = p - y * W;
    const float s = *scale;
    const float* src = cl.in[l] + p;
    float v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int c = q * 8 + j;
        v[j] = c < C ? src[static_cast<int64_t>(c) * HW] * s : 0.0f;
    }
    cl.out[l][chunked_index(y, q, x, W, chunks)] = make_uint4(pack2<kBf16>(v[0], v[1]),
        pack2<kBf16>(v[2], v[3]), pack2<kBf16>(v[4], v[5]), pack2<kBf16>(v[6], v[7]));
}

// custom::Warp (the single-precision arithmetic of warp_op_kernel) writing
// the chunked 16-bit operand layout directly, scaled by *scale: the warped
// second-frame features of the flow estimator go straight to the tensor-core
// correlation.  One thread per pixel and chunk of 8 channels.  kUp: `flow`
// is the estimator's coarser cw x chh level, upsampled 2x here (up2_sample)
// instead of read from an upsampled copy.
template <bool kBf16, bool kUp>
__global__ void warp_to_chunked_kernel(const float* __restrict__ in, const float* __restrict__ flow,
    uint4* __restrict__ out, const float* __restrict__ scale, int C, int H, int W, int chunks, int64_t sin,
    int64_t sfl, int64_t sout, int cw, int chh)
{
    pdl_enter();
    const int64_t HW = static_cast<int64_t>(H) * W;
    const int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (p >= HW)
        return;
    const int q = blockIdx.y, n = blockIdx.z;
    // 32-bit division where the plane allows (a 64-bit one is a software routine)
    const int y = HW < (int64_t(1) << 31) ? static_cast<int>(p) / W : static_cast<int>(p / W);
    const int x = static_cast<int>(p - static_cast<int64_t>(y) * W);
    const float* fl = flow + n * sfl;
    const float xf = static_cast<float>(x) + (kUp ? up2_sample(fl, cw, chh, x, y, 0) : __ldg(fl + p));
    const float yf = static_cast<float>(y) + (kUp ? up2_sample(fl, cw, chh, x, y, 1) : __ldg(fl + HW + p));
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
    out[n * sout + chunked_index(y, q, x, W, chunks)] =
        make_uint4(pack2<kBf16>(v[0], v[1]), pack2<kBf16>(v[2], v[3]), pack2<kBf16>(v[4], v[5]), pack2<kBf16>(v[6], v[7]));
}

// 5-D map over a chunked tensor: {c % 16, x, c / 16, y, n}, box {16, pixels,
// cp / 16, 1, 1}, 32-byte swizzle: each box row is one 32-byte sector and
// the tile lands in the operand layout umma_desc_kmajor_sw32 describes.
bool encode_chunked_map(CUtensorMap* m, const void* base, int N, int H, int W, int cp, int box_pixels)
{
    EncodeTiledFn fn = tensor_map_encoder();
    if (!fn)
        return false;
    const cuuint64_t q = static_cast<cuuint64_t>(cp / 16);
    const cuuint64_t dims[5] = {16, static_cast<cuuint64_t>(W), q, static_cast<cuuint64_t>(H),
        static_cast<cuuint64_t>(N)};
    const cuuint64_t strides[4] = {32, static_cast<cuuint64_t>(W) * 32, q * W * 32, static_cast<cuuint64_t>(H) * q * W * 32};
    const cuuint32_t box[5] = {16, static_cast<cuuint32_t>(box_pixels), static_cast<cuuint32_t>(q), 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 5, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The dynamic shared memory opt-in is a per-device function attribute; the
// persistent grid is sized by the device's SM count.
cudaError_t tc_prepare_device(int* sms)
{
    static std::mutex mu;
    static int count[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!count[dev]) {
        if ((e = cudaFuncSetAttribute(corr_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemLimit)) !=
            cudaSuccess)
            return e;
        if ((e = cudaDeviceGetAttribute(&count[dev], cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            return e;
    }
    *sms = count[dev];
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
    return launch_corr_tc_chunked2(f1c, f2c, out, nullptr, nullptr, nullptr, scales, N, Cp, H, W, md, bf16, st);
}

cudaError_t launch_corr_tc_chunked2(const void* f1c, const void* f2c, float* out, const void* g1c, const void* g2c,
    float* out2, const float* scales, int N, int Cp, int H, int W, int md, bool bf16, cudaStream_t st)
{
    const int nprob = g1c ? 2 : 1;
    if (Cp % 16 != 0 || Cp > kTcMaxChannelsPadded || md < 0 || md > kTcMaxMd)
        return cudaErrorInvalidValue;
    int sms = 0;
    cudaError_t e = tc_prepare_device(&sms);
    if (e != cudaSuccess)
        return e;
    int* flag = nullptr;
    if ((e = device_timeout_flag(&flag)) != cudaSuccess)
        return e;
    CUtensorMap mA, mB, mA2, mB2;
    if (!encode_chunked_map(&mA, f1c, N, H, W, Cp, kTcM) || !encode_chunked_map(&mB, f2c, N, H, W, Cp, kTcN))
        return cudaErrorInvalidValue;
    if (nprob == 2 &&
        (!encode_chunked_map(&mA2, g1c, N, H, W, Cp, kTcM) || !encode_chunked_map(&mB2, g2c, N, H, W, Cp, kTcN)))
        return cudaErrorInvalidValue;
    if (nprob == 1) {
        mA2 = mA;
        mB2 = mB;
    }
    const TcPlan plan = tc_plan(Cp);
    const int P = 2 * md + 1;
    const int base = nprob * N * H * ((W + kTcM - 1) / kTcM);
    int ndyg = 1;  // split the displacement rows until there are two items per SM
    while (ndyg < P && base * ndyg < 2 * sms)
        ++ndyg;
    const int items = base * ndyg;
    const cudaError_t el = launch_pdl(corr_tc_kernel, dim3(std::min(items, sms)), dim3((2 + 4 * plan.groups) * 32),
        plan.smem, st, mA, mB, out, mA2, mB2, nprob == 2 ? out2 : out, nprob, scales, N, H, W, Cp, md,
        ptx::umma_idesc_f16(bf16, kTcM, kTcN), plan.stages_a, plan.stages_b, plan.groups, ndyg, flag);
    return el != cudaSuccess ? el : cudaGetLastError();
}

cudaError_t launch_to_chunked(const float* in, void* out, const float* scale, int N, int C, int H, int W, bool bf16,
    cudaStream_t st)
{
    const int chunks = tc_padded_channels(C) / 8;
    const int64_t HW = static_cast<int64_t>(H) * W;
    const dim3 g(static_cast<unsigned>((HW + 127) / 128), chunks, N);
    const cudaError_t e = launch_pdl(bf16 ? to_chunked_kernel<true> : to_chunked_kernel<false>, g, dim3(128), 0, st, in,
        static_cast<uint4*>(out), scale, C, H, W, chunks);
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_to_chunked_levels(const float* const* in, void* const* out, const int* C, const int* H,
    const int* W, int n, const float* scale, bool bf16, cudaStream_t st)
{
    if (n < 1 || n > kChunkLevelsMax)
        return cudaErrorInvalidValue;
    ChunkLevels cl{};
    cl.count = n;
    cl.block0[0] = 0;
    for (int l = 0; l < n; ++l) {
        if (static_cast<int64_t>(H[l]) * W[l] >= (int64_t(1) << 31))
            return cudaErrorInvalidValue;
        cl.in[l] = in[l];
        cl.out[l] = static_cast<uint4*>(out[l]);
        cl.C[l] = C[l];
        cl.H[l] = H[l];
        cl.W[l] = W[l];
        cl.chunks[l] = tc_padded_channels(C[l]) / 8;
        cl.block0[l + 1] = cl.block0[l] + ((H[l] * W[l] + 127) / 128) * cl.chunks[l];
    }
    const cudaError_t e = launch_pdl(bf16 ? to_chunked_levels_kernel<true> : to_chunked_levels_kernel<false>,
        dim3(cl.block0[n]), dim3(128), 0, st, cl, scale);
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_warp_to_chunked(const float* in, const float* flow, void* out, const float* scale, int N, int C,
    int H, int W, int64_t sin, int64_t sfl, int64_t sout_bytes, bool bf16, cudaStream_t st, int cw, int chh)
{
    const int chunks = tc_padded_channels(C) / 8;
    const int64_t HW = static_cast<int64_t>(H) * W;
    const dim3 g(static_cast<unsigned>((HW + 255) / 256), chunks, N);
    const int64_t so = sout_bytes / 16;
    const bool up = cw > 0 && chh > 0;
    auto k = bf16 ? (up ? warp_to_chunked_kernel<true, true> : warp_to_chunked_kernel<true, false>)
                  : (up ? warp_to_chunked_kernel<false, true> : warp_to_chunked_kernel<false, false>);
    const cudaError_t e = launch_pdl(k, g, dim3(256), 0, st, in, flow, static_cast<uint4*>(out), scale, C, H, W,
        chunks, sin, sfl, so, cw, chh);
    return e != cudaSuccess ? e : cudaGetLastError();
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
    // a few blocks per SM, each thread striding over ~2^4+ values
    const unsigned blocks = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((total + 4095) / 4096, 1216)));
    absmax_kernel<<<blocks, 256, 0, st>>>(f1, total, maxbits);
    absmax_kernel<<<blocks, 256, 0, st>>>(f2, total, maxbits + 1);
    scales_kernel<<<1, 32, 0, st>>>(maxbits, scales);
    const int chunks = cp / 8;
    const dim3 g(static_cast<unsigned>((static_cast<int64_t>(H) * W + 127) / 128), chunks, N);
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
