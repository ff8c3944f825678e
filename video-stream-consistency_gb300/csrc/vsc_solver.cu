// The blend solver of the stabilization pass (reference: kernel_consist_out
// and get_consist_out, src/stabilization/flowconsistency.cu:193-258, :350-374).
//
// Differences from the reference's schedule (results are the CPU
// restatement's, bit for bit except that a zero may carry the other sign,
// see jacobi_px):
//   - Jacobi iteration: the reference updates consisOut in place
//     (flowconsistency.cu:370), so neighbours read a timing-dependent mix of
//     old and new values; here every pixel reads the previous iterate;
//   - the Laplacian of the processed image, which the reference recomputes in
//     every iteration, is computed once per solve (same expression, same bits);
//   - several iterations per launch on register-resident tiles (temporal
//     blocking) instead of one launch per iteration.
#include "vsc_internal.h"
#include "vsc_math.cuh"

#include <cuda.h>  // CUtensorMap (the encoder is fetched from the driver at run time)

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace vsc {
namespace {

inline dim3 grid2d(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

// ---- kernel_consist_out (flowconsistency.cu:193-258) ------------------------
// Laplacian of the processed image with the reference's neighbour rule and
// summation order (right, left, bottom, top, then - cnt * centre).
__global__ void lap_pr_kernel(const float* __restrict__ P, float* __restrict__ L, int w, int h)
{
    pdl_enter();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h)
        return;
    const int64_t i0 = pix_index(x, y, w) * 3;
    const int64_t rs = static_cast<int64_t>(w) * 3;
    for (int c = 0; c < 3; ++c) {
        const int64_t i = i0 + c;
        int cnt = 0;
        float lap = 0.0f;
        if ((x + 1) < (w - 1)) {
            lap += P[i + 3];
            cnt += 1;
        }
        if ((x - 1) >= 0) {
            lap += P[i - 3];
            cnt += 1;
        }
        if ((y + 1) < (h - 1)) {
            lap += P[i + rs];
            cnt += 1;
        }
        if ((y - 1) >= 0) {
            lap += P[i - rs];
            cnt += 1;
        }
        lap -= static_cast<float>(cnt) * P[i];
        L[i] = lap;
    }
}

// ---- temporally blocked solver --------------------------------------------
// kTbT Jacobi iterations per launch on a kTbEX x kTbEY extended tile; the
// interior (the tile minus a kTbT-wide ring) is exact after kTbT iterations
// and is written back.  Each of the 512 threads owns a 2x2 pixel block and
// keeps its state (O, U) and the per-pixel constants (lap P, A, consWt) in
// registers; O is published to shared memory (double-buffered) for the rows
// of the neighbouring warps, and horizontal neighbours travel by warp
// shuffle (one warp spans the full tile width).  Tiles away from the image
// border skip the reference's neighbour-validity selects.  The result equals
// the one-iteration-per-launch Jacobi bit for bit.
#ifndef VSC_SOLVER_T
#define VSC_SOLVER_T 8
#endif
constexpr int kTbEX = 64;
constexpr int kTbEY = 32;
constexpr int kTbT = VSC_SOLVER_T;             // iterations per launch
constexpr int kTbPX = kTbEX + 4;               // shared row pitch (2-column apron each side)
constexpr int kTbPlane = kTbPX * (kTbEY + 2);  // one colour plane with a 1-row apron
constexpr int kTbSmem = 2 * 3 * kTbPlane * static_cast<int>(sizeof(float));
static_assert(2 * kTbT < kTbEY, "tile too small for the iteration count");

// One Jacobi step of one pixel (kernel_consist_out's expression).  With kAll
// every neighbour is valid (cnt = 4) and the validity selects are skipped.
template <bool kAll>
__device__ __forceinline__ float jacobi_px(float o, float& u, float a, float wt, float lp, float right, float left,
    float down, float up, bool vr, bool vl, bool vd, bool vu, float cnt, float step, float mom, bool mom_on)
{
    // The reference sums the neighbours onto 0.0f; starting from the first
    // term drops one addition per pixel and channel.  0 + x equals x except
    // for x = -0 (0 + -0 = +0), so the two sums differ at most in the sign of
    // a zero, and no later operation of the pass (sums, products, squares,
    // fabs, comparisons) turns a zero's sign into a different non-zero value
    // or output byte.
    float lap;
    if (kAll) {
        lap = right + left;
        lap += down;
        lap += up;
    } else {
        lap = vr ? right : 0.0f;
        lap += vl ? left : 0.0f;
        lap += vd ? down : 0.0f;
        lap += vu ? up : 0.0f;
    }
    // with every neighbour valid cnt is 4 and 4 * o is exact (|o| < 2^125),
    // so one fused multiply-add rounds as the reference's multiply, subtract
    if (kAll)
        lap = __fmaf_rn(-4.0f, o, lap);
    else
        lap -= cnt * o;
    const float tmp_1 = wt * (o - a);
    const float tmp_2 = lap - lp;
    const float sg = step * (tmp_2 - tmp_1);
    float out = o + sg;
    if (mom_on)
        out = out + mom * u;
    u = sg;
    return out;
}

struct TbState {
    float o[4][3], u[4][3], a[4][3], wt[4][3], lp[4][3];  // [pixel q = 2*row + col][channel]
};

// One Jacobi step of a thread's 2x2 block, all three channels: reads the
// previous iterate from shared buffer `cur` (vertical neighbours) and the
// neighbouring lanes (horizontal ones), publishes the new one to `cur ^ 1`.
template <bool kAll>
__device__ __forceinline__ void tb_step(TbState& s, const bool (&vr)[4], const bool (&vl)[4], const bool (&vd)[4],
    const bool (&vu)[4], const float (&cnt)[4], float* smem, int cur, bool mom_on, float step, float mom, int px0,
    int py0)
{
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float* S = smem + (cur * 3 + ch) * kTbPlane;
        const float2 up = *reinterpret_cast<const float2*>(&S[py0 * kTbPX + px0 + 2]);
        const float2 dn = *reinterpret_cast<const float2*>(&S[(py0 + 3) * kTbPX + px0 + 2]);
        const float o0 = s.o[0][ch], o1 = s.o[1][ch], o2 = s.o[2][ch], o3 = s.o[3][ch];
        const float l0 = __shfl_up_sync(0xffffffffu, o1, 1);
        const float l1 = __shfl_up_sync(0xffffffffu, o3, 1);
        const float r0 = __shfl_down_sync(0xffffffffu, o0, 1);
        const float r1 = __shfl_down_sync(0xffffffffu, o2, 1);
        const float n0 = jacobi_px<kAll>(o0, s.u[0][ch], s.a[0][ch], s.wt[0][ch], s.lp[0][ch], o1, l0, o2, up.x,
            vr[0], vl[0], vd[0], vu[0], cnt[0], step, mom, mom_on);
        const float n1 = jacobi_px<kAll>(o1, s.u[1][ch], s.a[1][ch], s.wt[1][ch], s.lp[1][ch], r0, o0, o3, up.y,
            vr[1], vl[1], vd[1], vu[1], cnt[1], step, mom, mom_on);
        const float n2 = jacobi_px<kAll>(o2, s.u[2][ch], s.a[2][ch], s.wt[2][ch], s.lp[2][ch], o3, l1, dn.x, o0,
            vr[2], vl[2], vd[2], vu[2], cnt[2], step, mom, mom_on);
        const float n3 = jacobi_px<kAll>(o3, s.u[3][ch], s.a[3][ch], s.wt[3][ch], s.lp[3][ch], r1, o2, dn.y, o1,
            vr[3], vl[3], vd[3], vu[3], cnt[3], step, mom, mom_on);
        s.o[0][ch] = n0;
        s.o[1][ch] = n1;
        s.o[2][ch] = n2;
        s.o[3][ch] = n3;
        float* D = smem + ((cur ^ 1) * 3 + ch) * kTbPlane;
        *reinterpret_cast<float2*>(&D[(py0 + 1) * kTbPX + px0 + 2]) = make_float2(n0, n1);
        *reinterpret_cast<float2*>(&D[(py0 + 2) * kTbPX + px0 + 2]) = make_float2(n2, n3);
    }
}

// `ring` is the width of the ring around the rows written back (the rows
// [ring, kTbEY - ring) are exact after the T iterations).  Iteration k only
// has to be right on rows [ring - T + k + 1, kTbEY - ring + T - k - 1), one
// row fewer on each side per iteration, so a warp (two rows) whose rows all
// lie outside skips it: the rows it would have published are read only by
// rows that are themselves outside the next iteration's range.  A launch of
// the full kTbT iterations after the first step of the solve (momentum on
// throughout) runs fully unrolled; others take the general loop.
template <bool kAll>
__device__ __forceinline__ void tb_iterate(TbState& s, const bool (&vr)[4], const bool (&vl)[4],
    const bool (&vd)[4], const bool (&vu)[4], const float (&cnt)[4], float* smem, int T, int ring, int k0,
    float step, float mom, int px0, int py0)
{
    if (T == kTbT && ring == kTbT) {
        // full launches, unrolled; momentum is off only in the first step of a solve
        const bool later = k0 > 0;
#pragma unroll
        for (int k = 0; k < kTbT; ++k) {
            const int lo = k + 1, hi = kTbEY - k - 1;  // the general bounds with ring == T == kTbT
            if (!(py0 + 1 < lo || py0 >= hi))  // warp-uniform: py0 = 2 * threadIdx.y
                tb_step<kAll>(s, vr, vl, vd, vu, cnt, smem, k & 1, k > 0 || later, step, mom, px0, py0);
            __syncthreads();
        }
        return;
    }
    for (int k = 0; k < T; ++k) {
        const int lo = ring - T + k + 1, hi = kTbEY - ring + T - k - 1;
        if (!(py0 + 1 < lo || py0 >= hi))
            tb_step<kAll>(s, vr, vl, vd, vu, cnt, smem, k & 1, (k0 + k) > 0, step, mom, px0, py0);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kTbEX / 2 * kTbEY / 2, 1)
    solver_tb_kernel(const float* __restrict__ Oin, float* __restrict__ Oout, const float* __restrict__ Uin,
        float* __restrict__ Uout, const float* __restrict__ L, const float* __restrict__ A,
        const float* __restrict__ Wt, int w, int h, int T, int k0, float step, float mom, uint8_t* __restrict__ rgba)
{
    extern __shared__ __align__(16) float smem[];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tx;
    const int ox = blockIdx.x * (kTbEX - 2 * T) - T;
    const int oy = blockIdx.y * (kTbEY - 2 * T) - T;
    const int px0 = 2 * tx, py0 = 2 * ty;

    // both buffers start at zero, aprons included (apron cells are only read
    // by pixels of the outermost ring, whose results are never written back)
    for (int i = tid; i < 2 * 3 * kTbPlane; i += blockDim.x * blockDim.y)
        smem[i] = 0.0f;
    __syncthreads();

    TbState s;
    float cnt[4];
    bool vr[4], vl[4], vd[4], vu[4], inimg[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int gx = ox + px0 + (q & 1);
        const int gy = oy + py0 + (q >> 1);
        inimg[q] = gx >= 0 && gx < w && gy >= 0 && gy < h;
        vr[q] = (gx + 1) < (w - 1);
        vl[q] = (gx - 1) >= 0;
        vd[q] = (gy + 1) < (h - 1);
        vu[q] = (gy - 1) >= 0;
        cnt[q] = static_cast<float>(static_cast<int>(vr[q]) + static_cast<int>(vl[q]) + static_cast<int>(vd[q]) +
                                    static_cast<int>(vu[q]));
        const int64_t idx = inimg[q] ? pix_index(gx, gy, w) * 3 : 0;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            s.o[q][ch] = inimg[q] ? Oin[idx + ch] : 0.0f;
            s.u[q][ch] = inimg[q] ? Uin[idx + ch] : 0.0f;
            s.a[q][ch] = inimg[q] ? A[idx + ch] : 0.0f;
            s.wt[q][ch] = inimg[q] ? Wt[idx + ch] : 0.0f;
            s.lp[q][ch] = inimg[q] ? L[idx + ch] : 0.0f;
        }
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        float* S = smem + ch * kTbPlane;
        *reinterpret_cast<float2*>(&S[(py0 + 1) * kTbPX + px0 + 2]) = make_float2(s.o[0][ch], s.o[1][ch]);
        *reinterpret_cast<float2*>(&S[(py0 + 2) * kTbPX + px0 + 2]) = make_float2(s.o[2][ch], s.o[3][ch]);
    }
    __syncthreads();

    // tiles whose every pixel has all four neighbours skip the validity selects
    const bool interior = ox >= 1 && oy >= 1 && ox + kTbEX - 1 <= w - 3 && oy + kTbEY - 1 <= h - 3;
    if (interior)
        tb_iterate<true>(s, vr, vl, vd, vu, cnt, smem, T, T, k0, step, mom, px0, py0);
    else
        tb_iterate<false>(s, vr, vl, vd, vu, cnt, smem, T, T, k0, step, mom, px0, py0);

#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int r = q >> 1, c = q & 1;
        const int px = px0 + c, py = py0 + r;
        if (!inimg[q] || px < T || px >= kTbEX - T || py < T || py >= kTbEY - T)
            continue;
        const int64_t p = pix_index(ox + px, oy + py, w);
        float ov[3];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            ov[ch] = s.o[q][ch];
            Oout[p * 3 + ch] = ov[ch];
            Uout[p * 3 + ch] = s.u[q][ch];
        }
        if (rgba)
            reinterpret_cast<uint32_t*>(rgba)[p] = pack_rgba(ov[0], ov[1], ov[2]);
    }
}

// ---- persistent, TMA-fed solver ----------------------------------------------
// Same tile, same per-pixel arithmetic as solver_tb_kernel, but one CTA per
// SM walks a list of tiles and the five input tiles (O, U, A, consWt, lap P:
// 32 rows x 192 floats of the interleaved images each) of its NEXT tile are
// fetched by TMA into shared memory while the current tile iterates, so
// global-memory latency no longer serialises with the compute.  The tile
// origin is fixed by the 8-pixel ring (kTbT), whatever the iteration count
// of the launch, which keeps the TMA x coordinate (3 * origin floats) on the
// 16-byte grid.  Needs width % 4 == 0 (16-byte row pitch) and 16-byte
// aligned images; other sizes use solver_tb_kernel.
constexpr int kIW = kTbEX - 2 * kTbT;                  // interior width  (48)
constexpr int kIH = kTbEY - 2 * kTbT;                  // interior height (16)
constexpr int kStageFloats = kTbEY * kTbEX * 3;        // one input tile
constexpr int kStageBytes = kStageFloats * static_cast<int>(sizeof(float));
constexpr int kPsSmem = 5 * kStageBytes + kTbSmem + 16;
constexpr int kWaitSpins = 1 << 22;                    // bounded mbarrier wait (about a second)
static_assert((3 * kTbT) % 4 == 0 && (3 * kIW) % 4 == 0, "TMA x coordinates must be 16-byte aligned");

__device__ int g_device_timeout;  // set by a kernel whose bounded wait gave up

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Spins at most `spins` polls (with back-off); false if the phase never completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int spins)
{
    for (int i = 0; i < spins; ++i) {
        if (mbar_try_wait(bar, parity))
            return true;
        if (i > 32)
            __nanosleep(256);
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Programmatic dependent launch: a solver launch may start while the previous
// one drains (its CTAs set up shared memory and barriers meanwhile); before
// the first read of the previous launch's O and U, and before any write to
// the images it was reading, every thread waits for that launch to complete.
// The previous launch lets the next one start once each of its CTAs is on
// its last tile.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_dependent_launch() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// TMA tensor store (shared -> global) of one box; elements outside the image are clipped
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
        "r"(x), "r"(y), "r"(smem_u32(src))
        : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// this thread's bulk stores have read their shared-memory source
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// this thread's bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// The interior of a tile (after the T-pixel ring) leaves through shared memory
// and two TMA stores, one per image, instead of scalar stores of 12-byte
// pixels: `so` / `su` hold rows of 3 * kIW floats, filled by every thread,
// then one thread issues the stores; the staging is reusable after
// bulk_wait_read and a barrier.
__device__ __forceinline__ void store_interior(const CUtensorMap* mOo, const CUtensorMap* mUo, int ox, int oy,
    const float* so, const float* su)
{
    tma_store_2d(mOo, 3 * (ox + kTbT), oy + kTbT, so);
    tma_store_2d(mUo, 3 * (ox + kTbT), oy + kTbT, su);
    bulk_commit();
}

// The images of one solve, in the order of a problem's tensor maps: the five
// loaded per tile (O, U, A, consWt, lap P; tile box) and the two stored
// (O, U; interior box).
enum { kMapO, kMapU, kMapA, kMapW, kMapL, kMapOo, kMapUo, kMaps };

// The problems of one launch of a persistent solver kernel: kN images of any
// sizes (one per video stream at one pyramid level), each with its tensor
// maps, its size and its first tile in the launch's tile list.  Every problem
// runs the same iterations (T, k0, step, mom).  Passed by value as a
// __grid_constant__ parameter, so the maps stay in parameter memory, where
// TMA reads them.
template <int kN>
struct SolverGroup {
    CUtensorMap map[kN][kMaps];
    int w[kN], h[kN], tiles_x[kN];
    int tile0[kN + 1];  // first tile of problem p; tile0[count] = tiles in all
    uint8_t* rgba[kN];  // RGBA8 output of the last launch, or null
    int count;
};
constexpr int kGroupMax = 16;

struct TileLoc {
    int p;       // problem
    int ox, oy;  // tile origin (ring included)
    int w, h;
};

// tile -> problem by a scan of the first-tile table (kN <= kGroupMax)
template <int kN, int kRows>
__device__ __forceinline__ TileLoc locate(const SolverGroup<kN>& g, int tile)
{
    int p = 0;
    if (kN > 1) {
#pragma unroll 1
        while (p + 1 < g.count && tile >= g.tile0[p + 1])
            ++p;
    }
    const int t = tile - g.tile0[p];
    TileLoc l;
    l.p = p;
    l.ox = (t % g.tiles_x[p]) * kIW - kTbT;
    l.oy = (t / g.tiles_x[p]) * kRows - kTbT;
    l.w = g.w[p];
    l.h = g.h[p];
    return l;
}

// input tiles first .. last - 1 (map order) of a tile at (ox, oy), into consecutive stages
__device__ __forceinline__ void issue_tile_loads(float* stage, const CUtensorMap* m, int ox, int oy, int stage_floats,
    int first, int last, uint64_t* bar)
{
    for (int i = first; i < last; ++i)
        tma_load_2d(stage + i * stage_floats, m + i, 3 * ox, oy, bar);
}

// the five input tiles of a tile at (ox, oy), `bytes` each, into consecutive stages
__device__ __forceinline__ void issue_loads(float* stage, const CUtensorMap* m, int ox, int oy, int stage_floats,
    uint32_t bytes, uint64_t* bar)
{
    mbar_expect_tx(bar, 5 * bytes);
    issue_tile_loads(stage, m, ox, oy, stage_floats, kMapO, kMapL + 1, bar);
}

// The first tile of a launch.  A, consWt and lap P are not written by solver
// launches, so a launch after the first of a solve (k0 > 0: its predecessor
// is the previous solver launch, which itself waited for the kernels that
// wrote them) fetches them before waiting for the predecessor to complete;
// O and U, which the predecessor writes, after.
__device__ __forceinline__ void issue_first_loads(float* stage, const CUtensorMap* m, int ox, int oy,
    int stage_floats, uint32_t bytes, uint64_t* bar, bool early)
{
    if (early) {
        mbar_expect_tx(bar, 5 * bytes);
        issue_tile_loads(stage, m, ox, oy, stage_floats, kMapA, kMapL + 1, bar);
    }
    grid_dependency_wait();
    if (early)
        issue_tile_loads(stage, m, ox, oy, stage_floats, kMapO, kMapU + 1, bar);
    else
        issue_loads(stage, m, ox, oy, stage_floats, bytes, bar);
}

template <int kN>
__global__ void __launch_bounds__(kTbEX / 2 * kTbEY / 2, 1)
    solver_persistent_kernel(const __grid_constant__ SolverGroup<kN> g, int T, int k0, float step, float mom)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* stage = reinterpret_cast<float*>(smem_raw);
    float* obuf = stage + 5 * kStageFloats;
    uint64_t* bar = reinterpret_cast<uint64_t*>(obuf + 2 * 3 * kTbPlane);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tx;
    const int px0 = 2 * tx, py0 = 2 * ty;

    for (int i = tid; i < 2 * 3 * kTbPlane; i += blockDim.x * blockDim.y)
        obuf[i] = 0.0f;
    if (tid == 0)
        mbar_init(bar, 1);
    __syncthreads();
    const int ntiles = g.tile0[g.count];
    int tile = blockIdx.x;
    if (tid == 0 && tile < ntiles) {
        const TileLoc n = locate<kN, kIH>(g, tile);
        issue_first_loads(stage, g.map[n.p], n.ox, n.oy, kStageFloats, kStageBytes, bar, k0 > 0);
    }
    grid_dependency_wait();
    uint32_t parity = 0;
    for (; tile < ntiles; tile += gridDim.x) {
        if (tile + static_cast<int>(gridDim.x) >= ntiles)
            allow_dependent_launch();
        const TileLoc c = locate<kN, kIH>(g, tile);
        const int ox = c.ox, oy = c.oy, w = c.w, h = c.h;
        if (!mbar_wait_bounded(bar, parity, kWaitSpins)) {
            // the outputs are invalid and vsc_check_device reports VSC_ETIMEOUT; the
            // second bounded wait gives copies still in flight a chance to land
            // before the CTA exits
            if (tid == 0) {
                atomicExch(&g_device_timeout, 1);
                bulk_wait_all();
            }
            mbar_wait_bounded(bar, parity, kWaitSpins);
            return;
        }
        parity ^= 1;

        TbState s;
        float cnt[4];
        bool vr[4], vl[4], vd[4], vu[4], inimg[4];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int row = py0 + r;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const int q = 2 * r + c;
                const int gx = ox + px0 + c, gy = oy + row;
                inimg[q] = gx >= 0 && gx < w && gy >= 0 && gy < h;
                vr[q] = (gx + 1) < (w - 1);
                vl[q] = (gx - 1) >= 0;
                vd[q] = (gy + 1) < (h - 1);
                vu[q] = (gy - 1) >= 0;
                cnt[q] = static_cast<float>(static_cast<int>(vr[q]) + static_cast<int>(vl[q]) +
                                            static_cast<int>(vd[q]) + static_cast<int>(vu[q]));
            }
            // six consecutive floats: both pixels' RGB (TMA zero-fills outside the image)
            float(*dst[5])[3] = {s.o, s.u, s.a, s.wt, s.lp};
#pragma unroll
            for (int arr = 0; arr < 5; ++arr) {
                const float* src = stage + arr * kStageFloats + row * (3 * kTbEX) + 3 * px0;
                const float2 v01 = *reinterpret_cast<const float2*>(src);
                const float2 v23 = *reinterpret_cast<const float2*>(src + 2);
                const float2 v45 = *reinterpret_cast<const float2*>(src + 4);
                float* p0 = dst[arr][2 * r];
                float* p1 = dst[arr][2 * r + 1];
                p0[0] = v01.x;
                p0[1] = v01.y;
                p0[2] = v23.x;
                p1[0] = v23.y;
                p1[1] = v45.x;
                p1[2] = v45.y;
            }
        }
        if (tid == 0)
            bulk_wait_read();  // the previous tile's TMA stores have read the staging
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int ch = 0; ch < 3; ++ch)
                *reinterpret_cast<float2*>(&obuf[ch * kTbPlane + (py0 + r + 1) * kTbPX + px0 + 2]) =
                    make_float2(s.o[2 * r][ch], s.o[2 * r + 1][ch]);
        __syncthreads();  // staging consumed, O published
        if (tid == 0 && tile + static_cast<int>(gridDim.x) < ntiles) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const TileLoc n = locate<kN, kIH>(g, tile + gridDim.x);
            issue_loads(stage, g.map[n.p], n.ox, n.oy, kStageFloats, kStageBytes, bar);
        }

        const bool interior = ox >= 1 && oy >= 1 && ox + kTbEX - 1 <= w - 3 && oy + kTbEY - 1 <= h - 3;
        if (interior)
            tb_iterate<true>(s, vr, vl, vd, vu, cnt, obuf, T, kTbT, k0, step, mom, px0, py0);
        else
            tb_iterate<false>(s, vr, vl, vd, vu, cnt, obuf, T, kTbT, k0, step, mom, px0, py0);

        // interior out: the edge-row buffers are idle until the next tile's publish;
        // a thread's two pixels of a row are six consecutive floats
        float* so = obuf;
        float* su = obuf + kIH * 3 * kIW;
        {
            const int ix = px0 - kTbT;
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int iy = py0 + r - kTbT;
                if (ix < 0 || ix >= kIW || iy < 0 || iy >= kIH)
                    continue;
                float2* o2 = reinterpret_cast<float2*>(so + iy * 3 * kIW + 3 * ix);
                float2* u2 = reinterpret_cast<float2*>(su + iy * 3 * kIW + 3 * ix);
                const float* a = s.o[2 * r];
                const float* b = s.o[2 * r + 1];
                o2[0] = make_float2(a[0], a[1]);
                o2[1] = make_float2(a[2], b[0]);
                o2[2] = make_float2(b[1], b[2]);
                const float* c = s.u[2 * r];
                const float* d = s.u[2 * r + 1];
                u2[0] = make_float2(c[0], c[1]);
                u2[1] = make_float2(c[2], d[0]);
                u2[2] = make_float2(d[1], d[2]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0)
            store_interior(g.map[c.p] + kMapOo, g.map[c.p] + kMapUo, ox, oy, so, su);
        if (uint8_t* rgba = g.rgba[c.p]) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int px = px0 + (q & 1), py = py0 + (q >> 1);
                if (!inimg[q] || px < kTbT || px >= kTbEX - kTbT || py < kTbT || py >= kTbEY - kTbT)
                    continue;
                reinterpret_cast<uint32_t*>(rgba)[pix_index(ox + px, oy + py, w)] =
                    pack_rgba(s.o[q][0], s.o[q][1], s.o[q][2]);
            }
        }
        // the TMA stores read the staging while the next tile's copies land
    }
    if (tid == 0)
        bulk_wait_all();
}

// ---- persistent, TMA-fed solver on 64 x 48 tiles of 2 x 4 pixel blocks -------------
// Same per-pixel arithmetic as the kernels above, on a taller tile: 12 warps,
// each thread a 2-column x 4-row block (its vertical neighbours inside the
// block are its own registers), so 48 rows fit in the register budget of
// 384 threads and the interior after the 8-pixel ring is 48 x 32 (50 % of
// the tile instead of 37.5 %).  Only the top and bottom row of each warp
// are read by other warps; they are published to a compact double-buffered
// array of "slots" (slot w + 1 holds warp w's two edge rows, slots 0 and 13
// are zero aprons).  Half the shared-memory traffic per pixel of the 2 x 2
// blocking, the same shuffles per pixel.
constexpr int kPWarps = 12;
constexpr int kPThreads = 32 * kPWarps;
constexpr int kPEY = 4 * kPWarps;            // 48 tile rows
constexpr int kPIH = kPEY - 2 * kTbT;        // 32 interior rows
constexpr int kPStageFloats = kPEY * kTbEX * 3;
constexpr int kPStageBytes = kPStageFloats * static_cast<int>(sizeof(float));
constexpr int kPSlots = kPWarps + 2;
constexpr int kPPlane = kPSlots * 2 * kTbPX;  // one channel of one buffer
constexpr int kPObuf = 2 * 3 * kPPlane;
constexpr int kPSmem = 5 * kPStageBytes + kPObuf * static_cast<int>(sizeof(float)) + 16;
static_assert(kPSmem <= 232448, "dynamic shared memory per CTA");
static_assert(kPObuf >= 2 * kPIH * 3 * kIW && 2 * 3 * kTbPlane >= 2 * kIH * 3 * kIW,
    "the edge-row buffers hold a tile's interior O and U");
static_assert((kPIH * 3 * kIW * 4) % 128 == 0 && (kIH * 3 * kIW * 4) % 128 == 0 &&
    (5 * kPStageBytes) % 128 == 0 && (5 * kStageBytes) % 128 == 0, "TMA store sources on the 128-byte grid");
static_assert(2 * kTbT < kPEY, "tile too small for the iteration count");

struct P8State {
    float o[8][3], u[8][3], a[8][3], wt[8][3], lp[8][3];  // [pixel q = 2 * row + col][channel]
};

// validity of a pixel's four neighbours in the reference's rule (border tiles only)
struct Nb {
    bool vr, vl, vd, vu;
    float cnt;
};
__device__ __forceinline__ Nb nb_of(int gx, int gy, int w, int h)
{
    Nb n;
    n.vr = (gx + 1) < (w - 1);
    n.vl = (gx - 1) >= 0;
    n.vd = (gy + 1) < (h - 1);
    n.vu = (gy - 1) >= 0;
    n.cnt = static_cast<float>(static_cast<int>(n.vr) + static_cast<int>(n.vl) + static_cast<int>(n.vd) +
                               static_cast<int>(n.vu));
    return n;
}

template <bool kAll>
__device__ __forceinline__ void p8_step(P8State& s, float* obuf, int cur, bool mom_on, float step, float mom, int px0,
    int warp, int gx0, int gy0, int w, int h)
{
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float* S = obuf + (cur * 3 + ch) * kPPlane;
        const float2 up = *reinterpret_cast<const float2*>(&S[(warp * 2 + 1) * kTbPX + px0 + 2]);   // slot w, row 1
        const float2 dn = *reinterpret_cast<const float2*>(&S[((warp + 2) * 2) * kTbPX + px0 + 2]);  // slot w+2, row 0
        float ol[4], orr[4], L[4], R[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            ol[r] = s.o[2 * r][ch];
            orr[r] = s.o[2 * r + 1][ch];
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            L[r] = __shfl_up_sync(0xffffffffu, orr[r], 1);
            R[r] = __shfl_down_sync(0xffffffffu, ol[r], 1);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const float ul = r == 0 ? up.x : ol[r - 1], ur = r == 0 ? up.y : orr[r - 1];
            const float dl = r == 3 ? dn.x : ol[r + 1], dr = r == 3 ? dn.y : orr[r + 1];
            Nb a{true, true, true, true, 4.0f}, b{true, true, true, true, 4.0f};
            if (!kAll) {
                a = nb_of(gx0, gy0 + r, w, h);
                b = nb_of(gx0 + 1, gy0 + r, w, h);
            }
            const int ql = 2 * r, qr = 2 * r + 1;
            s.o[ql][ch] = jacobi_px<kAll>(ol[r], s.u[ql][ch], s.a[ql][ch], s.wt[ql][ch], s.lp[ql][ch], orr[r], L[r], dl,
                ul, a.vr, a.vl, a.vd, a.vu, a.cnt, step, mom, mom_on);
            s.o[qr][ch] = jacobi_px<kAll>(orr[r], s.u[qr][ch], s.a[qr][ch], s.wt[qr][ch], s.lp[qr][ch], R[r], ol[r],
                dr, ur, b.vr, b.vl, b.vd, b.vu, b.cnt, step, mom, mom_on);
        }
        float* D = obuf + ((cur ^ 1) * 3 + ch) * kPPlane + ((warp + 1) * 2) * kTbPX + px0 + 2;
        *reinterpret_cast<float2*>(D) = make_float2(s.o[0][ch], s.o[1][ch]);            // top row
        *reinterpret_cast<float2*>(D + kTbPX) = make_float2(s.o[6][ch], s.o[7][ch]);    // bottom row
    }
}

// Iteration k is needed on rows [ring - T + k + 1, kPEY - ring + T - k - 1);
// a warp (four rows) outside that range skips it (the argument of tb_iterate).
template <bool kAll>
__device__ __forceinline__ void p8_iterate(P8State& s, float* obuf, int T, int k0, float step, float mom, int px0,
    int warp, int gx0, int gy0, int w, int h)
{
    const int r0 = 4 * warp;
    if (T == kTbT) {
        // full launches, unrolled; momentum is off only in the first step of a solve
        const bool later = k0 > 0;
#pragma unroll
        for (int k = 0; k < kTbT; ++k) {
            if (!(r0 + 3 < k + 1 || r0 >= kPEY - k - 1))
                p8_step<kAll>(s, obuf, k & 1, k > 0 || later, step, mom, px0, warp, gx0, gy0, w, h);
            __syncthreads();
        }
        return;
    }
    for (int k = 0; k < T; ++k) {
        const int lo = kTbT - T + k + 1, hi = kPEY - kTbT + T - k - 1;
        if (!(r0 + 3 < lo || r0 >= hi))
            p8_step<kAll>(s, obuf, k & 1, (k0 + k) > 0, step, mom, px0, warp, gx0, gy0, w, h);
        __syncthreads();
    }
}

template <int kN>
__global__ void __launch_bounds__(kPThreads, 1)
    solver_tall_kernel(const __grid_constant__ SolverGroup<kN> g, int T, int k0, float step, float mom)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* stage = reinterpret_cast<float*>(smem_raw);
    float* obuf = stage + 5 * kPStageFloats;
    uint64_t* bar = reinterpret_cast<uint64_t*>(obuf + kPObuf);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px0 = 2 * lane, py0 = 4 * warp;

    for (int i = threadIdx.x; i < kPObuf; i += kPThreads)
        obuf[i] = 0.0f;  // the apron slots stay zero
    if (threadIdx.x == 0)
        mbar_init(bar, 1);
    __syncthreads();
    const int ntiles = g.tile0[g.count];
    int tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < ntiles) {
        const TileLoc n = locate<kN, kPIH>(g, tile);
        issue_first_loads(stage, g.map[n.p], n.ox, n.oy, kPStageFloats, kPStageBytes, bar, k0 > 0);
    }
    grid_dependency_wait();
    uint32_t parity = 0;
    for (; tile < ntiles; tile += gridDim.x) {
        if (tile + static_cast<int>(gridDim.x) >= ntiles)
            allow_dependent_launch();
        const TileLoc c = locate<kN, kPIH>(g, tile);
        const int ox = c.ox, oy = c.oy, w = c.w, h = c.h;
        if (!mbar_wait_bounded(bar, parity, kWaitSpins)) {
            // the outputs are invalid and vsc_check_device reports VSC_ETIMEOUT; the
            // second bounded wait gives copies still in flight a chance to land
            // before the CTA exits
            if (threadIdx.x == 0) {
                atomicExch(&g_device_timeout, 1);
                bulk_wait_all();
            }
            mbar_wait_bounded(bar, parity, kWaitSpins);
            return;
        }
        parity ^= 1;

        P8State s;
        float(*dst[5])[3] = {s.o, s.u, s.a, s.wt, s.lp};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            // six consecutive floats: both pixels' RGB (TMA zero-fills outside the image)
#pragma unroll
            for (int arr = 0; arr < 5; ++arr) {
                const float* src = stage + arr * kPStageFloats + (py0 + r) * (3 * kTbEX) + 3 * px0;
                const float2 v01 = *reinterpret_cast<const float2*>(src);
                const float2 v23 = *reinterpret_cast<const float2*>(src + 2);
                const float2 v45 = *reinterpret_cast<const float2*>(src + 4);
                float* p0 = dst[arr][2 * r];
                float* p1 = dst[arr][2 * r + 1];
                p0[0] = v01.x;
                p0[1] = v01.y;
                p0[2] = v23.x;
                p1[0] = v23.y;
                p1[1] = v45.x;
                p1[2] = v45.y;
            }
        }
        if (threadIdx.x == 0)
            bulk_wait_read();  // the previous tile's TMA stores have read the staging
        __syncthreads();
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            float* D = obuf + ch * kPPlane + ((warp + 1) * 2) * kTbPX + px0 + 2;  // buffer 0
            *reinterpret_cast<float2*>(D) = make_float2(s.o[0][ch], s.o[1][ch]);
            *reinterpret_cast<float2*>(D + kTbPX) = make_float2(s.o[6][ch], s.o[7][ch]);
        }
        __syncthreads();  // staging consumed, edge rows published
        if (threadIdx.x == 0 && tile + static_cast<int>(gridDim.x) < ntiles) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const TileLoc n = locate<kN, kPIH>(g, tile + gridDim.x);
            issue_loads(stage, g.map[n.p], n.ox, n.oy, kPStageFloats, kPStageBytes, bar);
        }

        const int gx0 = ox + px0, gy0 = oy + py0;
        const bool interior = ox >= 1 && oy >= 1 && ox + kTbEX - 1 <= w - 3 && oy + kPEY - 1 <= h - 3;
        if (interior)
            p8_iterate<true>(s, obuf, T, k0, step, mom, px0, warp, gx0, gy0, w, h);
        else
            p8_iterate<false>(s, obuf, T, k0, step, mom, px0, warp, gx0, gy0, w, h);

        // interior out: the edge-row slots are idle until the next tile's publish;
        // a thread's two pixels of a row are six consecutive floats (the
        // interior starts at an even column, so both or neither are inside)
        float* so = obuf;
        float* su = obuf + kPIH * 3 * kIW;
        {
            const int ix = px0 - kTbT;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int iy = py0 + r - kTbT;
                if (ix < 0 || ix >= kIW || iy < 0 || iy >= kPIH)
                    continue;
                float2* o2 = reinterpret_cast<float2*>(so + iy * 3 * kIW + 3 * ix);
                float2* u2 = reinterpret_cast<float2*>(su + iy * 3 * kIW + 3 * ix);
                const float* a = s.o[2 * r];
                const float* b = s.o[2 * r + 1];
                o2[0] = make_float2(a[0], a[1]);
                o2[1] = make_float2(a[2], b[0]);
                o2[2] = make_float2(b[1], b[2]);
                const float* c = s.u[2 * r];
                const float* d = s.u[2 * r + 1];
                u2[0] = make_float2(c[0], c[1]);
                u2[1] = make_float2(c[2], d[0]);
                u2[2] = make_float2(d[1], d[2]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0)
            store_interior(g.map[c.p] + kMapOo, g.map[c.p] + kMapUo, ox, oy, so, su);
        if (uint8_t* rgba = g.rgba[c.p]) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int px = px0 + (q & 1), py = py0 + (q >> 1);
                const int gx = ox + px, gy = oy + py;
                if (gx < 0 || gx >= w || gy < 0 || gy >= h || px < kTbT || px >= kTbEX - kTbT || py < kTbT ||
                    py >= kPEY - kTbT)
                    continue;
                reinterpret_cast<uint32_t*>(rgba)[pix_index(gx, gy, w)] =
                    pack_rgba(s.o[q][0], s.o[q][1], s.o[q][2]);
            }
        }
        // the TMA stores read the staging while the next tile's copies land; the
        // next tile waits for those reads before it publishes its edge rows
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

// ---- FMA form of the solver ---------------------------------------------------
// kernel_consist_out's step, g = (lap O - lap P) - w (O - A), O' = O + s g
// (+ m U), U' = s g, regrouped around two per-pixel constants computed once
// per solve (solver_prep_fma_kernel):
//   Cs = s * fma(w, A, -lap P),   nK = -(s * (cnt + w))   (cnt = valid neighbours),
// so that one step is
//   S = (left + right) + (up + down),  g = fma(nK, O, fma(s, S, Cs)),
//   O' = O + g, then O' = fma(m, U, O') after the first step,  U' = g,
// with invalid neighbours read as +0: seven FP32 operations per pixel and
// channel against twelve in the reference expression.  The rounding differs
// from the reference form's, so results agree with it within a tolerance
// (and with the restatement's FMA form, vo_consist_out_fma, bit for bit).
//
// The three colour channels of the step never interact, so the form solves
// each channel as its own image: the workspace holds O, U, Cs and nK as
// planes (channel-major, solver_to_planar / solver_from_planar convert O at
// the ends of a solve).  A tile is 128 x 72 pixels of one plane: each of the
// 384 threads keeps a 4-column x 6-row block of O, U, Cs and nK in registers
// (96 floats), a warp spans the tile's width, so the 8-pixel ring of the
// temporal blocking leaves a 112 x 56 interior (68 % of the tile; the
// interleaved 64 x 48 tile of three channels kept 50 %), horizontal
// neighbours cost two shuffles per row for four pixels, and each warp
// publishes its top and bottom row as two 16-byte stores per thread.

constexpr int kPlW = 128;                 // tile width (a warp: 32 lanes x 4 columns)
constexpr int kPlIW = kPlW - 2 * kTbT;    // interior width (112)
constexpr int kPlPX = kPlW + 8;           // edge-row pitch (a 16-byte apron each side)
constexpr int kPlWarps = 12;
constexpr int kPlThreads = 32 * kPlWarps;
constexpr int kPlRPT = 6;                 // rows per thread
constexpr int kPlRows = kPlRPT * kPlWarps;  // 72
constexpr int kPlIRows = kPlRows - 2 * kTbT;  // 56
constexpr int kPlStage = kPlRows * kPlW;  // floats of one input tile
constexpr int kPlStageBytes = kPlStage * static_cast<int>(sizeof(float));
constexpr int kPlSlotPlane = (kPlWarps + 2) * 2 * kPlPX;  // edge-row slots of one buffer
constexpr int kPlOut = kPlIRows * kPlIW;  // floats of one interior tile
constexpr int kPlSmem = 4 * kPlStageBytes + (2 * kPlSlotPlane + 2 * kPlOut) * static_cast<int>(sizeof(float)) + 16;
static_assert(kPlSmem <= 232448, "dynamic shared memory per CTA");
static_assert((kPlIW * 4) % 16 == 0 && (kTbT * 4) % 16 == 0, "TMA x coordinates must be 16-byte aligned");
static_assert((4 * kPlStageBytes) % 128 == 0 && (2 * kPlSlotPlane * 4) % 128 == 0 && (kPlOut * 4) % 128 == 0,
    "TMA sources and destinations on the 128-byte grid");

// Cs = step * fma(wt, A, -lap P) and nK = -(step * (cnt + wt)) as planes
// (lap P, cnt as lap_pr_kernel computes them); with O non-null, also O as
// planes into Op, or with Oc non-null the cw x ch image Oc upsampled to w x h
// as kernel_bilinear does (bilinear_px: the pyramid's initial solution of
// this level, written straight into the planes); with cnt non-null, the ncnt
// solve counters zeroed.
__global__ void solver_prep_fma_kernel(const float* __restrict__ P, const float* __restrict__ A,
    const float* __restrict__ Wt, const float* __restrict__ O, float* __restrict__ Cs, float* __restrict__ nK,
    float* __restrict__ Op, int w, int h, float step, unsigned* __restrict__ cnt, int ncnt,
    const float* __restrict__ Oc, int cw, int ch)
{
    pdl_enter();
    if (cnt && blockIdx.x == 0 && blockIdx.y == 0)  // the solve kernel's counters start at zero
        for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < ncnt; i += blockDim.x * blockDim.y)
            cnt[i] = 0;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h)
        return;
    const int64_t i0 = pix_index(x, y, w) * 3;
    const int64_t rs = static_cast<int64_t>(w) * 3;
    const int64_t plane = static_cast<int64_t>(w) * h;
    const int64_t q = pix_index(x, y, w);
    float up[3];
    if (Oc)
        bilinear_px(Oc, cw, ch, w, h, 3, x, y, up);
    for (int c = 0; c < 3; ++c) {
        const int64_t i = i0 + c;
        int cnt = 0;
        float lap = 0.0f;
        if ((x + 1) < (w - 1)) {
            lap += P[i + 3];
            cnt += 1;
        }
        if ((x - 1) >= 0) {
            lap += P[i - 3];
            cnt += 1;
        }
        if ((y + 1) < (h - 1)) {
            lap += P[i + rs];
            cnt += 1;
        }
        if ((y - 1) >= 0) {
            lap += P[i - rs];
            cnt += 1;
        }
        lap = __fsub_rn(lap, __fmul_rn(static_cast<float>(cnt), P[i]));
        const float wt = Wt[i];
        Cs[c * plane + q] = __fmul_rn(step, __fmaf_rn(wt, A[i], -lap));
        nK[c * plane + q] = -__fmul_rn(step, __fadd_rn(static_cast<float>(cnt), wt));
        if (Oc)
            Op[c * plane + q] = up[c];
        else if (O)
            Op[c * plane + q] = O[i];
    }
}

// Interleaved <-> planar copies of the images of up to kPlanarGroupMax solves
// (one launch per level of a multi-stream step): to_planar = 1 reads the
// interleaved src and writes dst as planes; 0 the reverse, and writes the
// RGBA8 copy when rgba is non-null.
constexpr int kPlanarGroupMax = 16;
struct PlanarGroup {
    const float* src[kPlanarGroupMax];
    float* dst[kPlanarGroupMax];
    uint8_t* rgba[kPlanarGroupMax];
    unsigned* cnt[kPlanarGroupMax];  // solve counters zeroed on the way in, or null
    int ncnt[kPlanarGroupMax];
    int64_t npix[kPlanarGroupMax];
    int block0[kPlanarGroupMax + 1];
    int count;
};

__global__ void __launch_bounds__(256) planar_group_kernel(const __grid_constant__ PlanarGroup g, int to_planar)
{
    pdl_enter();
    int p = 0;
    while (p + 1 < g.count && static_cast<int>(blockIdx.x) >= g.block0[p + 1])
        ++p;
    if (g.cnt[p] && static_cast<int>(blockIdx.x) == g.block0[p])
        for (int k = threadIdx.x; k < g.ncnt[p]; k += blockDim.x)
            g.cnt[p][k] = 0;
    const int64_t i = static_cast<int64_t>(blockIdx.x - g.block0[p]) * blockDim.x + threadIdx.x;
    const int64_t n = g.npix[p];
    if (i >= n)
        return;
    if (to_planar) {
        const float* s = g.src[p] + i * 3;
        g.dst[p][i] = s[0];
        g.dst[p][n + i] = s[1];
        g.dst[p][2 * n + i] = s[2];
        return;
    }
    const float r = g.src[p][i], gg = g.src[p][n + i], b = g.src[p][2 * n + i];
    float* d = g.dst[p] + i * 3;
    d[0] = r;
    d[1] = gg;
    d[2] = b;
    if (g.rgba[p])
        reinterpret_cast<uint32_t*>(g.rgba[p])[i] = pack_rgba(r, gg, b);
}

struct PlState {
    float4 o[kPlRPT], u[kPlRPT], c[kPlRPT], nk[kPlRPT];  // [row] = (column 0 .. 3)
};

__device__ __forceinline__ float& f4(float4& v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }
__device__ __forceinline__ float f4c(const float4& v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

// Neighbour tests of the planar step.  kernel_consist_out reads a neighbour as
// +0 unless it lies in [0, w - 2] x [0, h - 2] (left: gx - 1 >= 0, right:
// gx + 1 < w - 1, up: gy - 1 >= 0, down: gy + 1 < h - 1), so the only pixels of
// the frame with a neighbour read as +0 are column 0 (left), columns w - 2 and
// w - 1 (right), row 0 (up) and rows h - 2 and h - 1 (down); every other read
// of a pixel inside the frame is of a pixel inside the frame.  Pixels outside
// the frame (the ring of a border tile) are computed too, but no pixel inside
// the frame reads them unmasked, so their values never reach the output.
//   kPlAll:   an interior tile, no test.
//   kPlLanes: a border tile of a frame whose width, like the tile origins, is
//             a multiple of 4: column 0 is then column j = 0 of the thread
//             with gx0 = 0 and columns w - 2, w - 1 are j = 2, 3 of the thread
//             with gx0 = w - 4 (three selects a row); row 0 of a tile at
//             oy = -8 is row 2 of warp 1 and rows h - 2, h - 1 of a tile at
//             oy = h - 64 are rows 2, 3 of warp 10 (a select of a row's up or
//             down neighbours in every warp, true only in that one).  A tile
//             holding row 0, h - 2 or h - 1 elsewhere (frames of few rows)
//             takes kPlEvery.  Same bits as kPlEvery for every pixel inside
//             the frame, without its four tests a pixel.
//   kPlEvery: every neighbour tested.
enum { kPlAll, kPlLanes, kPlEvery };

// One step of a thread's 4 x 6 block: the previous iterate's edge rows of the
// neighbouring warps come from `src`, the new top and bottom rows go to `dst`.
// zl / zr (kPlLanes): this thread holds column 0 / columns w - 4 .. w - 1;
// zt / zb: its row 2 is row 0 / its rows 2 and 3 are rows h - 2 and h - 1.
template <int kMode>
__device__ __forceinline__ void pl_step(PlState& s, const float* src, float* dst, bool mom_on, float step, float mom,
    int lane, int warp, int gx0, int gy0, int w, int h, bool zl, bool zr, bool zt, bool zb)
{
    const float4 up = *reinterpret_cast<const float4*>(&src[(warp * 2 + 1) * kPlPX + 4 * lane + 4]);
    const float4 dn = *reinterpret_cast<const float4*>(&src[((warp + 2) * 2) * kPlPX + 4 * lane + 4]);
    float L[kPlRPT], R[kPlRPT];
#pragma unroll
    for (int r = 0; r < kPlRPT; ++r) {
        L[r] = __shfl_up_sync(0xffffffffu, s.o[r].w, 1);
        R[r] = __shfl_down_sync(0xffffffffu, s.o[r].x, 1);
    }
    float4 on[kPlRPT];
#pragma unroll
    for (int r = 0; r < kPlRPT; ++r) {
        const float4 o = s.o[r];
        float4 u = r == 0 ? up : s.o[r - 1];
        float4 d = r == kPlRPT - 1 ? dn : s.o[r + 1];
        if (kMode == kPlLanes && r == 2 && zt)
            u = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (kMode == kPlLanes && (r == 2 || r == 3) && zb)
            d = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bool vu = true, vd = true;
        if (kMode == kPlEvery) {
            vu = (gy0 + r - 1) >= 0;
            vd = (gy0 + r + 1) < (h - 1);
        }
        float lft = L[r], rgt = R[r], o3 = o.w;  // left of column 0, right of columns 3 and 2
        if (kMode == kPlLanes) {
            lft = zl ? 0.0f : lft;
            rgt = zr ? 0.0f : rgt;
            o3 = zr ? 0.0f : o3;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float left = j == 0 ? lft : f4c(o, j - 1);
            float right = j == 3 ? rgt : (j == 2 ? o3 : f4c(o, j + 1));
            float upv = f4c(u, j), dnv = f4c(d, j);
            if (kMode == kPlEvery) {
                const int gx = gx0 + j;
                left = (gx - 1) >= 0 ? left : 0.0f;
                right = (gx + 1) < (w - 1) ? right : 0.0f;
                upv = vu ? upv : 0.0f;
                dnv = vd ? dnv : 0.0f;
            }
            const float oj = f4c(o, j);
            const float g = __fmaf_rn(f4c(s.nk[r], j), oj,
                __fmaf_rn(step, __fadd_rn(__fadd_rn(left, right), __fadd_rn(upv, dnv)), f4c(s.c[r], j)));
            float n = __fadd_rn(oj, g);
            if (mom_on)
                n = __fmaf_rn(mom, f4c(s.u[r], j), n);
            f4(s.u[r], j) = g;
            f4(on[r], j) = n;
        }
    }
#pragma unroll
    for (int r = 0; r < kPlRPT; ++r)
        s.o[r] = on[r];
    float* D = dst + ((warp + 1) * 2) * kPlPX + 4 * lane + 4;
    *reinterpret_cast<float4*>(D) = on[0];                   // top row
    *reinterpret_cast<float4*>(D + kPlPX) = on[kPlRPT - 1];  // bottom row
}

// The planar step's test mode for a tile at (ox, oy) of a w x h frame.
__device__ __forceinline__ int pl_mode(int ox, int oy, int w, int h)
{
    if (ox >= 1 && oy >= 1 && ox + kPlW - 1 <= w - 3 && oy + kPlRows - 1 <= h - 3)
        return kPlAll;
    const bool row0 = oy <= 0 && oy + kPlRows - 1 >= 0;
    const bool last2 = oy <= h - 1 && oy + kPlRows - 1 >= h - 2;
    if ((w & 3) == 0 && (ox & 3) == 0 && (!row0 || oy == -kTbT) && (!last2 || oy == h - kPlRows + kTbT))
        return kPlLanes;
    return kPlEvery;
}

// Iteration k is needed on rows [ring - T + k + 1, kPlRows - ring + T - k - 1)
// (ring = kTbT); a warp whose rows all lie outside skips it.  idle(k) runs in
// the warps that skip the last three steps k of a full round (warps 0 and
// 11: work a caller keeps off the steps' critical path, as long as each part
// fits a step); in a shorter round idle(kTbT - 3) runs before its steps and
// the other two after them.
template <int kMode, class Idle>
__device__ __forceinline__ void pl_iterate(PlState& s, float* slots, int T, int k0, float step, float mom, int lane,
    int warp, int gx0, int gy0, int w, int h, int oy, Idle&& idle)
{
    const int r0 = kPlRPT * warp;
    const bool zl = gx0 == 0, zr = gx0 == w - 4;
    const bool zt = oy == -kTbT && warp == 1, zb = oy == h - kPlRows + kTbT && warp == 10;
    auto one = [&](int k, bool mom_on) {
        pl_step<kMode>(s, slots + (k & 1) * kPlSlotPlane, slots + ((k & 1) ^ 1) * kPlSlotPlane, mom_on, step, mom,
            lane, warp, gx0, gy0, w, h, zl, zr, zt, zb);
    };
    if (T == kTbT) {
        // full launches, unrolled; momentum is off only in the first step of a solve
        const bool later = k0 > 0;
#pragma unroll
        for (int k = 0; k < kTbT; ++k) {
            if (!(r0 + kPlRPT - 1 < k + 1 || r0 >= kPlRows - k - 1))
                one(k, k > 0 || later);
            else if (k >= kTbT - 3)
                idle(k);
            __syncthreads();
        }
        return;
    }
    idle(kTbT - 3);
    for (int k = 0; k < T; ++k) {
        const int lo = kTbT - T + k + 1, hi = kPlRows - kTbT + T - k - 1;
        if (!(r0 + kPlRPT - 1 < lo || r0 >= hi))
            one(k, (k0 + k) > 0);
        __syncthreads();
    }
    idle(kTbT - 2);
    idle(kTbT - 1);
}

int pl_tiles_x(int w) { return (w + kPlIW - 1) / kPlIW; }
int pl_tiles(int w, int h) { return 3 * pl_tiles_x(w) * ((h + kPlIRows - 1) / kPlIRows); }

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, int x, int y, int z, const void* src)
{
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
        "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
        : "memory");
}

// The planes of one solve for the plain-load form of the kernel (widths that
// are not a multiple of 4, or planes off the 16-byte grid).
struct PlPlain {
    const float *O, *U, *K, *C;
    float *Oo, *Uo;
    int w, h, tiles_x, ntiles;
};

// Stage <- tile (c, ox, oy) of the four planes, zero outside the image.
__device__ __forceinline__ void pl_plain_load(float* stage, const PlPlain& p, int c, int ox, int oy)
{
    const float* src[4] = {p.O, p.U, p.K, p.C};
    const int64_t base = static_cast<int64_t>(c) * p.w * p.h;
    for (int i = threadIdx.x; i < kPlStage; i += kPlThreads) {
        const int row = i / kPlW, col = i - row * kPlW;
        const int gy = oy + row, gx = ox + col;
        const bool in = gx >= 0 && gx < p.w && gy >= 0 && gy < p.h;
        const int64_t idx = in ? base + pix_index(gx, gy, p.w) : 0;
#pragma unroll
        for (int a = 0; a < 4; ++a)
            stage[a * kPlStage + i] = in ? src[a][idx] : 0.0f;
    }
}

// The plain-load form (widths that are not a multiple of 4, or a workspace off
// the 16-byte grid): one launch per round of up to kTbT steps, each CTA
// walking the round's tiles with plain loads and stores.
__device__ __forceinline__ void pl_plain_body(const PlPlain& pl, int T, int k0, float step, float mom)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* stage = reinterpret_cast<float*>(smem_raw);
    float* slots = stage + 4 * kPlStage;
    float* so = slots + 2 * kPlSlotPlane;
    float* su = so + kPlOut;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px0 = 4 * lane, py0 = kPlRPT * warp;

    for (int i = threadIdx.x; i < 2 * kPlSlotPlane; i += kPlThreads)
        slots[i] = 0.0f;  // the apron slots stay zero
    grid_dependency_wait();
    const int per_plane = pl.ntiles / 3;
    for (int tile = blockIdx.x; tile < pl.ntiles; tile += gridDim.x) {
        if (tile + static_cast<int>(gridDim.x) >= pl.ntiles)
            allow_dependent_launch();
        const int c = tile / per_plane, r = tile - c * per_plane;
        const int ox = (r % pl.tiles_x) * kPlIW - kTbT, oy = (r / pl.tiles_x) * kPlIRows - kTbT;
        const int w = pl.w, h = pl.h;
        __syncthreads();  // the previous tile has left the staging and the slots
        pl_plain_load(stage, pl, c, ox, oy);
        __syncthreads();
        const int gx0 = ox + px0, gy0 = oy + py0;
        const bool interior = ox >= 1 && oy >= 1 && ox + kPlW - 1 <= w - 3 && oy + kPlRows - 1 <= h - 3;

        PlState s;
#pragma unroll
        for (int rr = 0; rr < kPlRPT; ++rr) {
            const float* row = stage + (py0 + rr) * kPlW + px0;
            s.o[rr] = *reinterpret_cast<const float4*>(row);
            s.u[rr] = *reinterpret_cast<const float4*>(row + kPlStage);
            s.nk[rr] = *reinterpret_cast<const float4*>(row + 2 * kPlStage);
            s.c[rr] = *reinterpret_cast<const float4*>(row + 3 * kPlStage);
        }
        {
            float* D = slots + ((warp + 1) * 2) * kPlPX + px0 + 4;  // buffer 0
            *reinterpret_cast<float4*>(D) = s.o[0];
            *reinterpret_cast<float4*>(D + kPlPX) = s.o[kPlRPT - 1];
        }
        __syncthreads();  // edge rows published
        if (interior)
            pl_iterate<kPlAll>(s, slots, T, k0, step, mom, lane, warp, gx0, gy0, w, h, oy, [](int) {});
        else
            pl_iterate<kPlEvery>(s, slots, T, k0, step, mom, lane, warp, gx0, gy0, w, h, oy, [](int) {});
        {
            const int ix = px0 - kTbT;
#pragma unroll
            for (int rr = 0; rr < kPlRPT; ++rr) {
                const int iy = py0 + rr - kTbT;
                if (ix < 0 || ix >= kPlIW || iy < 0 || iy >= kPlIRows)
                    continue;
                *reinterpret_cast<float4*>(so + iy * kPlIW + ix) = s.o[rr];
                *reinterpret_cast<float4*>(su + iy * kPlIW + ix) = s.u[rr];
            }
        }
        __syncthreads();
        const int64_t base = static_cast<int64_t>(c) * w * h;
        for (int i = threadIdx.x; i < kPlOut; i += kPlThreads) {
            const int iy = i / kPlIW, ix = i - iy * kPlIW;
            const int gy = oy + kTbT + iy, gx = ox + kTbT + ix;
            if (gx < w && gy < h) {
                const int64_t idx = base + pix_index(gx, gy, w);
                pl.Oo[idx] = so[i];
                pl.Uo[idx] = su[i];
            }
        }
    }
}

__global__ void __launch_bounds__(kPlThreads, 1)
    solver_fma_plain_kernel(const __grid_constant__ PlPlain pl, int T, int k0, float step, float mom)
{
    pl_plain_body(pl, T, k0, step, mom);
}

// ---- the FMA form's solve in one persistent launch -----------------------------
// A solve of L launches' worth of 8-step rounds over N tiles is one kernel:
// each CTA takes (round k, tile t) tickets in order from a global counter
// (k = ticket / N, t = ticket % N), waits until the tile's 3x3 neighbourhood
// has finished round k - 1 (per-tile counters of finished rounds, released
// after the tile's TMA stores complete), runs the tile's steps and signals
// its counter.  Round k reads O[k & 1], U[k & 1] and writes O[(k + 1) & 1],
// U[(k + 1) & 1]; waiting for the neighbours' round k - 1 orders both the
// reads of round k after those writes and the writes of round k after the
// neighbours' round-(k - 1) reads of the same buffer region.  A ticket only
// waits for earlier tickets, whose CTAs already run, so the order cannot
// deadlock whatever else occupies the GPU; every wait is bounded all the
// same.  Rounds overlap: a CTA moves on to round k + 1 while the last tiles of
// round k finish elsewhere, which removes the per-launch tail (1,080 tiles
// per round at 1920x1080 leave the eighth of eight rounds 11 % full) and the
// launch boundaries.  The next ticket's loads are issued while the current
// tile iterates when its neighbours are ready (normally: they finished about
// N / #SMs tiles earlier); otherwise warp 0 looks again during the steps it
// skips, and failing that the CTA first finishes and signals its current
// tile, then waits.  The tickets' bookkeeping (decoding, neighbour checks,
// and with many tiles a round the fence that publishes a tile) runs in those
// skipped steps, not between a tile's data and its first step.
enum { kPmO0, kPmO1, kPmU0, kPmU1, kPmK, kPmC, kPmOo0, kPmOo1, kPmUo0, kPmUo1, kPlMaps };

template <int kN>
struct PlSolve {
    CUtensorMap map[kN][kPlMaps];
    unsigned* done[kN];  // per problem and tile: rounds finished (zeroed before the launch)
    int w[kN], h[kN], tiles_x[kN];
    int tile0[kN + 1];   // first tile of problem p in a round's tile list; tile0[count] = N
    int count, nround, num_iter;
    unsigned* ticket;    // the next ticket (zeroed before the launch)
};

struct PlJob {
    int k;                   // round
    int p, c, tx, ty, local;  // problem, plane, tile position, tile index within the problem
    int ox, oy, w, h;
};

template <int kN>
__device__ __forceinline__ PlJob pl_job(const PlSolve<kN>& g, int ticket)
{
    const int N = g.tile0[g.count];
    PlJob j;
    j.k = ticket / N;
    const int tile = ticket - j.k * N;
    int p = 0;
    if (kN > 1) {
        // the last problem whose first tile is <= tile (binary search: a job is
        // decoded several times per tile, partly on thread 0's critical path)
        int hi = g.count - 1;
#pragma unroll 1
        while (p < hi) {
            const int mid = (p + hi + 1) >> 1;
            if (g.tile0[mid] <= tile)
                p = mid;
            else
                hi = mid - 1;
        }
    }
    j.p = p;
    j.local = tile - g.tile0[p];
    const int per_plane = (g.tile0[p + 1] - g.tile0[p]) / 3;
    j.c = j.local / per_plane;
    const int r = j.local - j.c * per_plane;
    j.tx = r % g.tiles_x[p];
    j.ty = r / g.tiles_x[p];
    j.ox = j.tx * kPlIW - kTbT;
    j.oy = j.ty * kPlIRows - kTbT;
    j.w = g.w[p];
    j.h = g.h[p];
    // The bottom row of tiles is moved up until its interior ends on the
    // frame's last row (rows h - 2 and h - 1 then sit in warp 10, rows 2 and 3,
    // where pl_step tests them without per-pixel tests), when its 8-row top
    // ring still lies in the row of tiles above (the 3 x 3 dependency holds).
    // Its interior then overlaps that row's: both compute the shared rows from
    // the same inputs with the same arithmetic and store the same bits.
    const int ty_n = per_plane / g.tiles_x[p];
    if (j.ty == ty_n - 1 && j.ty > 0 && j.h - j.ty * kPlIRows >= kTbT)
        j.oy = j.h - kPlRows + kTbT;
    return j;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Round k - 1 finished on the tile's 3x3 neighbourhood (spins <= 1: one look).
template <int kN>
__device__ __forceinline__ bool pl_deps(const PlSolve<kN>& g, const PlJob& j, int spins)
{
    if (j.k == 0)
        return true;
    const int tx_n = g.tiles_x[j.p];
    const int per_plane = (g.tile0[j.p + 1] - g.tile0[j.p]) / 3;
    const int ty_n = per_plane / tx_n;
    const unsigned* d = g.done[j.p] + j.c * per_plane;
    for (int dy = -1; dy <= 1; ++dy) {
        const int y = j.ty + dy;
        if (y < 0 || y >= ty_n)
            continue;
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = j.tx + dx;
            if (x < 0 || x >= tx_n)
                continue;
            const unsigned* f = d + y * tx_n + x;
            int i = 0;
            while (ld_acquire_u32(f) < static_cast<unsigned>(j.k)) {
                if (++i >= spins)
                    return false;
                if (i > 32)
                    __nanosleep(256);
            }
        }
    }
    return true;
}

// the tile's four input planes for its round, after its neighbours' stores
template <int kN>
__device__ __forceinline__ void pl_job_loads(float* stage, const PlSolve<kN>& g, const PlJob& j, uint64_t* bar)
{
    asm volatile("fence.proxy.async.global;" ::: "memory");  // the acquired stores, before the async-proxy reads
    const CUtensorMap* m = g.map[j.p];
    const int par = j.k & 1;
    mbar_expect_tx(bar, 4 * kPlStageBytes);
    tma_load_3d(stage, m + (par ? kPmO1 : kPmO0), j.ox, j.oy, j.c, bar);
    tma_load_3d(stage + kPlStage, m + (par ? kPmU1 : kPmU0), j.ox, j.oy, j.c, bar);
    tma_load_3d(stage + 2 * kPlStage, m + kPmK, j.ox, j.oy, j.c, bar);
    tma_load_3d(stage + 3 * kPlStage, m + kPmC, j.ox, j.oy, j.c, bar);
}

__device__ __forceinline__ void st_relaxed_u32(unsigned* p, unsigned v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// the tile's stores are complete: publish its round (the release store
// orders the completed async-proxy writes, brought into the generic proxy
// by the proxy fence, before the counter)
template <int kN>
__device__ __forceinline__ void pl_job_signal(const PlSolve<kN>& g, const PlJob& j)
{
    bulk_wait_all();
    asm volatile("fence.proxy.async.global;" ::: "memory");
    st_release_u32(g.done[j.p] + j.local, static_cast<unsigned>(j.k + 1));
}

__device__ __forceinline__ void pl_counter_signal(unsigned* done, unsigned v)
{
    bulk_wait_all();
    asm volatile("fence.proxy.async.global;" ::: "memory");
    st_release_u32(done, v);
}

// Warp 0 looks at the 3x3 neighbourhood of job j in two halves, so that the
// L2 round trip can overlap a tile's steps.  Issue: lanes 0..8 each start one
// relaxed load of a neighbour's counter (a lane without a neighbour, or a job
// that waits for nothing, yields ~0u).
template <int kN>
__device__ __forceinline__ unsigned pl_deps_issue(const PlSolve<kN>& g, const PlJob& j, bool valid, int lane)
{
    unsigned v = ~0u;
    if (valid && j.k > 0 && lane < 9) {
        const int tx_n = g.tiles_x[j.p];
        const int per_plane = (g.tile0[j.p + 1] - g.tile0[j.p]) / 3;
        const int ty_n = per_plane / tx_n;
        const int x = j.tx + lane % 3 - 1, y = j.ty + lane / 3 - 1;
        if (x >= 0 && x < tx_n && y >= 0 && y < ty_n)
            asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];"
                         : "=r"(v)
                         : "l"(g.done[j.p] + j.c * per_plane + y * tx_n + x)
                         : "memory");
    }
    return v;
}

// Take, all lanes of warp 0: every neighbour has finished round k - 1.  A yes
// is followed by an acquire fence in the lanes that read the counters and a
// warp barrier, which order the counters' published stores before the
// warp's later accesses (lane 0's TMA loads of the job).
__device__ __forceinline__ bool pl_deps_take(unsigned v, int k)
{
    const bool ok = __all_sync(0xffffffffu, v >= static_cast<unsigned>(k));
    if (ok) {
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        __syncwarp();
    }
    return ok;
}

template <int kN>
__global__ void __launch_bounds__(kPlThreads, 1)
    solver_fma_solve_kernel(const __grid_constant__ PlSolve<kN> g, float step, float mom)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* stage = reinterpret_cast<float*>(smem_raw);
    float* slots = stage + 4 * kPlStage;
    float* so = slots + 2 * kPlSlotPlane;
    float* su = so + kPlOut;
    uint64_t* bar = reinterpret_cast<uint64_t*>(su + kPlOut);
    __shared__ int s_next, s_deferred, s_abort;
    // decoded jobs: the next tile's (read by every thread at its top) and the
    // one after it (decoded by warp 0 while the current tile runs)
    __shared__ PlJob s_job, s_job2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px0 = 4 * lane, py0 = kPlRPT * warp;
    const int total = g.tile0[g.count] * g.nround;
    // Many tiles a round (ticketed several tiles' time before their
    // dependents): a tile's round is published while the next tile runs, in
    // steps warp 0 skips, instead of on that tile's critical path.
    const bool lag = g.tile0[g.count] >= 3 * static_cast<int>(gridDim.x);

    for (int i = threadIdx.x; i < 2 * kPlSlotPlane; i += kPlThreads)
        slots[i] = 0.0f;  // the apron slots stay zero
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        s_abort = 0;
    }
    __syncthreads();
    grid_dependency_wait();
    // Tickets are taken two ahead: while a CTA runs its current tile, warp 0
    // holds the next ticket (t1, loaded during the current tile) and takes the
    // one after (t2), which it decodes and whose neighbours it checks in the
    // steps it skips; the atomic, the divisions and the counter reads stay off
    // the critical path.
    int t1 = 0;
    bool t1_ready = false;  // warp 0: t1's neighbours were seen finished
    if (warp == 0) {
        int a = 0, b = 0;
        if (lane == 0) {
            a = static_cast<int>(atomicAdd(g.ticket, 1u));
            b = static_cast<int>(atomicAdd(g.ticket, 1u));
        }
        a = __shfl_sync(0xffffffffu, a, 0);
        t1 = __shfl_sync(0xffffffffu, b, 0);
        if (lane == 0) {
            s_next = a;
            if (a < total) {
                const PlJob n = pl_job(g, a);
                s_job = n;
                if (pl_deps(g, n, kWaitSpins)) {
                    pl_job_loads(stage, g, n, bar);
                } else {
                    atomicExch(&g_device_timeout, 1);
                    s_abort = 1;
                }
            }
        }
        const bool valid = t1 < total;
        const PlJob n = valid ? pl_job(g, t1) : PlJob{};
        if (lane == 0)
            s_job2 = n;
        t1_ready = pl_deps_take(pl_deps_issue(g, n, valid, lane), n.k);
    }
    __syncthreads();
    int cur = s_next;
    uint32_t parity = 0;
    // thread 0: the counter and value of a tile whose round is not yet published
    unsigned* prev_done = nullptr;
    unsigned prev_val = 0;
    while (cur < total && !s_abort) {
        const PlJob j = s_job;
        int t2 = 0;
        if (warp == 0 && lane == 0)
            t2 = static_cast<int>(atomicAdd(g.ticket, 1u));  // used after the tile's first barrier
        if (!mbar_wait_bounded(bar, parity, kWaitSpins)) {
            // the outputs are invalid and vsc_check_device reports VSC_ETIMEOUT
            if (threadIdx.x == 0) {
                atomicExch(&g_device_timeout, 1);
                bulk_wait_all();
            }
            mbar_wait_bounded(bar, parity, kWaitSpins);  // let copies still in flight land
            return;
        }
        parity ^= 1;
        if (warp == 0 && !lag) {
            // One fence a tile, taken while the other warps stage their
            // registers: it releases the previous tile's completed stores
            // (published by the relaxed counter store after it) and acquires
            // the neighbour counters read for t1 during that tile's steps.
            // (With `lag`, the same happens in the previous tile's last step.)
            if (lane == 0 && prev_done) {
                bulk_wait_all();
                asm volatile("fence.proxy.async.global;" ::: "memory");
            }
            __syncwarp();
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            __syncwarp();
            if (lane == 0 && prev_done)
                st_relaxed_u32(prev_done, prev_val);
            prev_done = nullptr;
        }
        const int w = j.w, h = j.h;
        const int gx0 = j.ox + px0, gy0 = j.oy + py0;

        PlState s;
#pragma unroll
        for (int r = 0; r < kPlRPT; ++r) {
            const float* row = stage + (py0 + r) * kPlW + px0;
            s.o[r] = *reinterpret_cast<const float4*>(row);
            s.u[r] = *reinterpret_cast<const float4*>(row + kPlStage);
            s.nk[r] = *reinterpret_cast<const float4*>(row + 2 * kPlStage);
            s.c[r] = *reinterpret_cast<const float4*>(row + 3 * kPlStage);
        }
        if (threadIdx.x == 0)
            bulk_wait_read();  // the previous tile's TMA stores have read the out staging
        __syncthreads();       // staging consumed
        {
            float* D = slots + ((warp + 1) * 2) * kPlPX + px0 + 4;  // buffer 0
            *reinterpret_cast<float4*>(D) = s.o[0];
            *reinterpret_cast<float4*>(D + kPlPX) = s.o[kPlRPT - 1];
        }
        if (warp == 0) {
            // load the next tile now if its neighbours are finished (seen
            // across the previous tile, else one look now)
            const bool valid = t1 < total;
            const PlJob n = s_job2;  // decoded while the previous tile ran
            const bool ready = t1_ready || pl_deps_take(pl_deps_issue(g, n, valid, lane), n.k);
            if (lane == 0) {
                s_next = t1;
                s_job = n;
                s_deferred = 0;
                if (valid) {
                    if (ready) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        pl_job_loads(stage, g, n, bar);
                    } else {
                        s_deferred = 1;
                    }
                }
            }
        }
        __syncthreads();  // edge rows published
        unsigned t2_look = ~0u, t1_look = ~0u;
        int t2_round = 0;
        // warp 0, in the steps it skips: decode t2 and start reading its
        // neighbours' counters; with `lag`, wait for the previous tile's
        // stores (long complete by then); take the counters and, with `lag`,
        // one fence that acquires them (for t2's loads at the top of the next
        // tile) and releases the previous tile's stores, published after it
        auto idle = [&](int k) {
            if (warp != 0)
                return;
            if (k == kTbT - 3) {
                t2 = __shfl_sync(0xffffffffu, t2, 0);
                const bool valid = t2 < total;
                const PlJob n = valid ? pl_job(g, t2) : PlJob{};
                if (lane == 0)
                    s_job2 = n;
                t2_look = pl_deps_issue(g, n, valid, lane);
                t2_round = n.k;
                // a deferred next tile (few tiles a round): look again now
                if (!lag && s_deferred)
                    t1_look = pl_deps_issue(g, s_job, true, lane);
            } else if (k == kTbT - 2) {
                if (lag && lane == 0 && prev_done) {
                    bulk_wait_all();
                    asm volatile("fence.proxy.async.global;" ::: "memory");
                }
                if (!lag && s_deferred) {
                    // its neighbours finished during this tile's steps: load it
                    // now instead of after the tile (ordered as at the top)
                    const PlJob n = s_job;
                    if (__all_sync(0xffffffffu, t1_look >= static_cast<unsigned>(n.k))) {
                        __syncwarp();
                        asm volatile("fence.acq_rel.gpu;" ::: "memory");
                        __syncwarp();
                        if (lane == 0) {
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            pl_job_loads(stage, g, n, bar);
                            s_deferred = 0;
                        }
                    }
                }
            } else {
                t1_ready = __all_sync(0xffffffffu, t2_look >= static_cast<unsigned>(t2_round));
                if (lag) {
                    __syncwarp();
                    asm volatile("fence.acq_rel.gpu;" ::: "memory");
                    __syncwarp();
                    if (lane == 0 && prev_done)
                        st_relaxed_u32(prev_done, prev_val);
                    prev_done = nullptr;
                }
            }
        };
        const int k0 = j.k * kTbT, T = min(kTbT, g.num_iter - k0);
        const int mode = pl_mode(j.ox, j.oy, w, h);
        if (mode == kPlAll)
            pl_iterate<kPlAll>(s, slots, T, k0, step, mom, lane, warp, gx0, gy0, w, h, j.oy, idle);
        else if (mode == kPlLanes)
            pl_iterate<kPlLanes>(s, slots, T, k0, step, mom, lane, warp, gx0, gy0, w, h, j.oy, idle);
        else
            pl_iterate<kPlEvery>(s, slots, T, k0, step, mom, lane, warp, gx0, gy0, w, h, j.oy, idle);
        {
            const int ix = px0 - kTbT;
#pragma unroll
            for (int r = 0; r < kPlRPT; ++r) {
                const int iy = py0 + r - kTbT;
                if (ix < 0 || ix >= kPlIW || iy < 0 || iy >= kPlIRows)
                    continue;
                *reinterpret_cast<float4*>(so + iy * kPlIW + ix) = s.o[r];
                *reinterpret_cast<float4*>(su + iy * kPlIW + ix) = s.u[r];
            }
        }
        if (warp == 0)
            t1 = t2;  // t1_ready: taken in the last step, acquired by its fence or the next top's
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            const CUtensorMap* m = g.map[j.p];
            const int par = (j.k + 1) & 1;
            tma_store_3d(m + (par ? kPmOo1 : kPmOo0), j.ox + kTbT, j.oy + kTbT, j.c, so);
            tma_store_3d(m + (par ? kPmUo1 : kPmUo0), j.ox + kTbT, j.oy + kTbT, j.c, su);
            bulk_commit();
            prev_done = g.done[j.p] + j.local;
            prev_val = static_cast<unsigned>(j.k + 1);
            if (s_deferred) {
                // the next tile's neighbours were not finished: publish this
                // tile first (the next one may need it), then wait
                pl_job_signal(g, j);
                prev_done = nullptr;
                const PlJob n = s_job;
                if (pl_deps(g, n, kWaitSpins)) {
                    pl_job_loads(stage, g, n, bar);
                } else {
                    atomicExch(&g_device_timeout, 1);
                    s_abort = 1;
                }
            }
        }
        __syncthreads();  // s_next, s_abort
        cur = s_next;
    }
    if (threadIdx.x == 0) {
        if (prev_done)
            pl_counter_signal(prev_done, prev_val);
        bulk_wait_all();
    }
}

// An mbarrier nobody arrives on, waited for with a bounded spin: exercises
// the timeout path of the bounded waits (sets g_device_timeout, returns).
__global__ void bounded_wait_selftest_kernel(int spins)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0)
        mbar_init(&bar, 1);
    __syncthreads();
    if (!mbar_wait_bounded(&bar, 0, spins) && threadIdx.x == 0)
        atomicExch(&g_device_timeout, 1);
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// 2D map over an interleaved w x h x 3 float image: x = float index in a row.
bool encode_image_map(CUtensorMap* m, const float* base, int w, int h, int box_rows, int box_cols = 3 * kTbEX)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn)
        return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(w) * 3, static_cast<cuuint64_t>(h)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(w) * 3 * sizeof(float)};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_cols), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int kN>
bool set_group_smem()
{
    constexpr auto kAttr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    return cudaFuncSetAttribute(solver_persistent_kernel<kN>, kAttr, kPsSmem) == cudaSuccess &&
           cudaFuncSetAttribute(solver_tall_kernel<kN>, kAttr, kPSmem) == cudaSuccess &&
           cudaFuncSetAttribute(solver_fma_solve_kernel<kN>, kAttr, kPlSmem) == cudaSuccess;
}

struct DeviceInfo {
    int sms = 0;
    bool tb_smem = false, ps_smem = false;
};

// The solver kernels need more than 48 KB of dynamic shared memory; the
// opt-in is a per-device function attribute, set once per device together
// with the SM count the persistent kernel sizes its grid by.
cudaError_t device_info(DeviceInfo** out)
{
    static std::mutex mu;
    static DeviceInfo info[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    DeviceInfo& d = info[dev];
    if (!d.sms) {
        if ((e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            return e;
        if ((e = cudaFuncSetAttribute(solver_tb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTbSmem)) !=
            cudaSuccess)
            return e;
        d.ps_smem = set_group_smem<1>() && set_group_smem<4>() && set_group_smem<kGroupMax>() &&
                    cudaFuncSetAttribute(solver_fma_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                        kPlSmem) == cudaSuccess;
        cudaGetLastError();
    }
    *out = &d;
    return cudaSuccess;
}

bool aligned16p(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// ---- tile-shape autotuner ------------------------------------------------------------
// The two persistent kernels of the exact form (64 x 32 and 64 x 48 tiles)
// give the same results bit for bit; which is faster depends on how their
// tiles fill the waves of one tile per SM.  solver_group_autotune times both
// on scratch images of the sizes one launch solves (one image, or one image
// per stream of a multi-stream step) and keeps the faster per (device, form,
// sizes); sizes never tuned use a wave model: a 64 x 48 tile costs about 1.91
// times a 64 x 32 one (GB300, 1920x1080 and 960x540).  The FMA form has one
// shape, 128 x 72 pixels of one channel plane.
struct ShapeTable {
    std::mutex mu;
    std::map<std::vector<int>, int> rows;  // {device, form, w0, h0, w1, h1, ...} -> tile rows
    bool enabled = true;
};
ShapeTable& shape_table()
{
    static ShapeTable t;
    return t;
}

std::vector<int> shape_key(int dev, const int* w, const int* h, int n, int form)
{
    std::vector<int> k{dev, form};
    for (int i = 0; i < n; ++i) {
        k.push_back(w[i]);
        k.push_back(h[i]);
    }
    return k;
}

int tiles_of(int w, int h, int ir) { return ((w + kIW - 1) / kIW) * ((h + ir - 1) / ir); }

int model_rows(const int* w, const int* h, int n, int sms, int form)
{
    if (form == kSolverFma)
        return kPlRows;
    int64_t n_short = 0, n_tall = 0;
    for (int i = 0; i < n; ++i) {
        n_short += tiles_of(w[i], h[i], kIH);
        n_tall += tiles_of(w[i], h[i], kPIH);
    }
    return 1.91 * ((n_tall + sms - 1) / sms) < 1.0 * ((n_short + sms - 1) / sms) ? kPEY : kTbEY;
}

// the tile rows a launch over these sizes uses on the current device: tuned, else the model
int chosen_rows(int dev, const int* w, const int* h, int n, int sms, int form, bool* tuned = nullptr)
{
    ShapeTable& t = shape_table();
    std::lock_guard<std::mutex> lock(t.mu);
    auto it = t.rows.find(shape_key(dev, w, h, n, form));
    if (tuned)
        *tuned = it != t.rows.end();
    return it != t.rows.end() ? it->second : model_rows(w, h, n, sms, form);
}

int interior_rows(int rows) { return rows - 2 * kTbT; }

// The tensor maps of one image's solve for both ping-pong phases: O[c] / U[c]
// with the tile box (loads), Oo[c] / Uo[c] with the interior box (stores).
struct SolveMaps {
    CUtensorMap O[2], U[2], A, W, L, Oo[2], Uo[2];
};

bool encode_solve(SolveMaps* m, float* const O[2], float* const U[2], const float* A, const float* Wt,
    const float* L, int w, int h, int rows)
{
    const int ir = interior_rows(rows);
    bool ok = encode_image_map(&m->A, A, w, h, rows) && encode_image_map(&m->W, Wt, w, h, rows) &&
              encode_image_map(&m->L, L, w, h, rows);
    for (int c = 0; c < 2 && ok; ++c)
        ok = encode_image_map(&m->O[c], O[c], w, h, rows) && encode_image_map(&m->U[c], U[c], w, h, rows) &&
             encode_image_map(&m->Oo[c], O[c], w, h, ir, 3 * kIW) &&
             encode_image_map(&m->Uo[c], U[c], w, h, ir, 3 * kIW);
    return ok;
}

// 3D map over the three w x h planes of a planar image (x, y, channel).
bool encode_plane_map(CUtensorMap* m, const float* base, int w, int h, int box_w, int box_h)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn)
        return false;
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(w), static_cast<cuuint64_t>(h), 3};
    const cuuint64_t strides[2] = {static_cast<cuuint64_t>(w) * sizeof(float),
        static_cast<cuuint64_t>(w) * h * sizeof(float)};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(box_w), static_cast<cuuint32_t>(box_h), 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// problem p of a launch: launch li of the solve reads O[c] and U[li & 1] and
// writes O[c ^ 1] and U[(li + 1) & 1]
template <int kN>
void group_set(SolverGroup<kN>& g, int p, const SolveMaps& m, int c, int li, int w, int h, int rows, uint8_t* rgba)
{
    g.map[p][kMapO] = m.O[c];
    g.map[p][kMapU] = m.U[li & 1];
    g.map[p][kMapA] = m.A;
    g.map[p][kMapW] = m.W;
    g.map[p][kMapL] = m.L;
    g.map[p][kMapOo] = m.Oo[c ^ 1];
    g.map[p][kMapUo] = m.Uo[(li + 1) & 1];
    g.w[p] = w;
    g.h[p] = h;
    g.tiles_x[p] = (w + kIW - 1) / kIW;
    g.rgba[p] = rgba;
    if (p == 0)
        g.tile0[0] = 0;
    g.tile0[p + 1] = g.tile0[p] + tiles_of(w, h, interior_rows(rows));
    g.count = p + 1;
}

// One launch of a persistent kernel of the exact form (`rows`-row tiles)
// over a group's tiles, with programmatic dependent launch on the previous
// launch of the stream.
template <int kN>
cudaError_t launch_group(int rows, const SolverGroup<kN>& g, int T, int k0, float step, float mom, int sms,
    cudaStream_t st)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(std::min(g.tile0[g.count], sms));
    if (rows == kPEY) {
        cfg.blockDim = dim3(kPThreads);
        cfg.dynamicSmemBytes = kPSmem;
        return cudaLaunchKernelEx(&cfg, solver_tall_kernel<kN>, g, T, k0, step, mom);
    }
    cfg.blockDim = dim3(32, kTbEY / 2);
    cfg.dynamicSmemBytes = kPsSmem;
    return cudaLaunchKernelEx(&cfg, solver_persistent_kernel<kN>, g, T, k0, step, mom);
}

// One image of a grouped solve: its maps and where its iterate starts.
struct GroupMember {
    SolveMaps maps;
    int w, h, c0;  // c0: the ping-pong buffer the first launch reads
    uint8_t* rgba;
};

// Steps k_first .. num_iter - 1 of a solve over all members, in launches of
// T <= kTbT steps, kN problems per launch.
template <int kN>
cudaError_t launch_members(const std::vector<GroupMember>& mem, int rows, int num_iter, float step, float mom,
    int sms, cudaStream_t st, int* nl, int k_first = 0)
{
    const int nlaunch = (num_iter - k_first + kTbT - 1) / kTbT;
    SolverGroup<kN> g{};
    cudaError_t e = cudaSuccess;
    int k0 = k_first;
    for (int li = 0; li < nlaunch && e == cudaSuccess; ++li) {
        const int T = std::min(kTbT, num_iter - k0);
        for (size_t b = 0; b < mem.size() && e == cudaSuccess; b += kN) {
            const int cnt = static_cast<int>(std::min(mem.size() - b, static_cast<size_t>(kN)));
            for (int p = 0; p < cnt; ++p) {
                const GroupMember& m = mem[b + p];
                group_set(g, p, m.maps, m.c0 ^ (li & 1), li, m.w, m.h, rows, li == nlaunch - 1 ? m.rgba : nullptr);
            }
            e = launch_group(rows, g, T, k0, step, mom, sms, st);
            ++*nl;
        }
        k0 += T;
    }
    return e;
}

}  // namespace

void solver_set_autotune(bool on)
{
    ShapeTable& t = shape_table();
    std::lock_guard<std::mutex> lock(t.mu);
    t.enabled = on;
    if (!on)
        t.rows.clear();
}

int solver_group_tile_rows(const int* w, const int* h, int n, bool* tuned, int form)
{
    int dev = 0;
    DeviceInfo* di = nullptr;
    if (n < 1 || cudaGetDevice(&dev) != cudaSuccess || device_info(&di) != cudaSuccess)
        return 0;
    return chosen_rows(dev, w, h, n, di->sms, form, tuned);
}

int solver_tile_rows(int w, int h, bool* tuned, int form) { return solver_group_tile_rows(&w, &h, 1, tuned, form); }

cudaError_t solver_group_autotune(const int* w, const int* h, int n, cudaStream_t st, int* rows_out, int form)
{
    DeviceInfo* di = nullptr;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = device_info(&di);
    if (e != cudaSuccess)
        return e;
    if (n < 1)
        return cudaErrorInvalidValue;
    bool eligible = di->ps_smem && form != kSolverFma;  // the FMA form has one shape
    size_t total = 0;  // floats of one image per member, 16-byte multiples
    for (int i = 0; i < n; ++i) {
        eligible = eligible && (w[i] % 4) == 0 && w[i] >= 1 && h[i] >= 1;
        total += static_cast<size_t>(w[i]) * h[i] * 3;
    }
    ShapeTable& t = shape_table();
    const std::vector<int> key = shape_key(dev, w, h, n, form);
    {
        std::lock_guard<std::mutex> lock(t.mu);
        auto it = t.rows.find(key);
        if (it != t.rows.end() || !t.enabled || !eligible) {
            if (rows_out)
                *rows_out = it != t.rows.end() ? it->second : model_rows(w, h, n, di->sms, form);
            return cudaSuccess;
        }
    }
    // scratch images (zeros; the kernels have no data-dependent control flow):
    // per member O, O2, U0, U1, A, Wt, lap P
    float* buf = nullptr;
    if ((e = cudaMalloc(&buf, 7 * total * sizeof(float))) != cudaSuccess)
        return e;
    // Five rounds, the shapes alternating within each, one warm-up launch per
    // shape and four timed 8-step launches; each shape's best round counts (the
    // first launches after the allocation and a clock still ramping up would
    // otherwise favour whichever shape is timed last; where the shapes are
    // close, more rounds keep the choice from flipping between runs).
    cudaEvent_t ev[2] = {};
    float best_ms[2] = {1e30f, 1e30f};
    const int shapes[2] = {kTbEY, kPEY};
    std::vector<GroupMember> mem[2];
    e = cudaMemsetAsync(buf, 0, 7 * total * sizeof(float), st);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
        e = cudaEventCreate(&ev[i]);
    for (int s = 0; s < 2 && e == cudaSuccess; ++s) {
        size_t off = 0;
        for (int i = 0; i < n && e == cudaSuccess; ++i) {
            float* im[7];
            for (int k = 0; k < 7; ++k)
                im[k] = buf + k * total + off;
            off += static_cast<size_t>(w[i]) * h[i] * 3;
            GroupMember m{};
            float* const O[2] = {im[0], im[1]};
            float* const U[2] = {im[2], im[3]};
            if (!encode_solve(&m.maps, O, U, im[4], im[5], im[6], w[i], h[i], shapes[s]))
                e = cudaErrorInvalidValue;
            m.w = w[i];
            m.h = h[i];
            mem[s].push_back(m);
        }
    }
    // the kernel instantiation the solves will use: one problem, up to 4, up to 16 per launch
    auto launch = [&](const std::vector<GroupMember>& m, int rows, int num_iter, int* nl) {
        return n == 1 ? launch_members<1>(m, rows, num_iter, 0.15f, 0.15f, di->sms, st, nl, kTbT)
             : n <= 4 ? launch_members<4>(m, rows, num_iter, 0.15f, 0.15f, di->sms, st, nl, kTbT)
                      : launch_members<kGroupMax>(m, rows, num_iter, 0.15f, 0.15f, di->sms, st, nl, kTbT);
    };
    for (int round = 0; round < 5 && e == cudaSuccess; ++round) {
        for (int s = 0; s < 2 && e == cudaSuccess; ++s) {
            int nl = 0;
            // a warm-up launch, then four timed ones, all of kTbT steps with momentum
            e = launch(mem[s], shapes[s], 2 * kTbT, &nl);
            if (e == cudaSuccess)
                e = cudaEventRecord(ev[0], st);
            if (e == cudaSuccess)
                e = launch(mem[s], shapes[s], 5 * kTbT, &nl);
            float ms = 0.0f;
            if (e == cudaSuccess)
                e = cudaEventRecord(ev[1], st);
            if (e == cudaSuccess)
                e = cudaEventSynchronize(ev[1]);
            if (e == cudaSuccess)
                e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (e == cudaSuccess)
                best_ms[s] = std::min(best_ms[s], ms);
        }
    }
    for (cudaEvent_t x : ev)
        if (x)
            cudaEventDestroy(x);
    cudaFree(buf);
    if (e != cudaSuccess)
        return e;
    const int best = best_ms[1] < best_ms[0] ? shapes[1] : shapes[0];
    {
        std::lock_guard<std::mutex> lock(t.mu);
        if (t.enabled)
            t.rows[key] = best;
    }
    if (rows_out)
        *rows_out = best;
    return cudaSuccess;
}

cudaError_t solver_autotune(int w, int h, cudaStream_t st, int* rows_out, int form)
{
    return solver_group_autotune(&w, &h, 1, st, rows_out, form);
}

// The FMA form's workspace ends in the solve kernel's counters: the ticket,
// padding to 64 bytes, one finished-round counter per tile; rounded up to
// 256 bytes so that a workspace placed after it stays aligned.
int pl_counter_floats(int w, int h) { return (16 + pl_tiles(w, h) + 63) / 64 * 64; }

size_t solver_workspace_floats(int w, int h, int form)
{
    const size_t img = static_cast<size_t>(w) * h * 3;
    return form == kSolverFma ? 6 * img + pl_counter_floats(w, h) : 4 * img;
}

int solver_steps_per_launch() { return kTbT; }

namespace {

// launches of a solve, and the buffer its iterate starts in so that the last
// launch writes O: O itself for an even count, the second buffer otherwise
int solve_launches(int num_iter) { return num_iter > 0 ? (num_iter + kTbT - 1) / kTbT : 0; }

struct WsView {
    float *L, *U0, *U1, *O2;
};
WsView ws_view(float* ws, int w, int h)
{
    const size_t n = static_cast<size_t>(w) * h * 3;
    return WsView{ws, ws + n, ws + 2 * n, ws + 3 * n};
}

// The FMA form's workspace: six planar images (three w x h planes each),
// then the solve kernel's counters.
struct PlWs {
    float *C, *K, *U[2], *O[2];
    unsigned* cnt;
    int ncnt;
};
PlWs pl_view(float* ws, int w, int h)
{
    const size_t n = static_cast<size_t>(w) * h * 3;
    return PlWs{ws, ws + n, {ws + 2 * n, ws + 3 * n}, {ws + 4 * n, ws + 5 * n},
        reinterpret_cast<unsigned*>(ws + 6 * n), pl_counter_floats(w, h)};
}

bool tma_eligible(const DeviceInfo* di, int w, const float* O, const WsView& v, const float* A, const float* Wt)
{
    return di->ps_smem && (w % 4) == 0 && aligned16p(O) && aligned16p(v.O2) && aligned16p(v.U0) &&
           aligned16p(v.U1) && aligned16p(A) && aligned16p(Wt) && aligned16p(v.L);
}

// planes of a width that is a multiple of 4 in a 16-byte aligned workspace
// (each plane then starts on the 16-byte grid)
bool pl_tma_eligible(const DeviceInfo* di, int w, const float* ws) { return di->ps_smem && (w % 4) == 0 && aligned16p(ws); }

struct PlanarCopy {
    const float* src;
    float* dst;
    uint8_t* rgba;
    int64_t npix;
    unsigned* cnt = nullptr;  // solve counters to zero on the way in
    int ncnt = 0;
};

// Interleaved <-> planar copies of n images, kPlanarGroupMax per launch.
cudaError_t launch_planar(const PlanarCopy* c, int n, int to_planar, cudaStream_t st, int* nl)
{
    for (int b0 = 0; b0 < n; b0 += kPlanarGroupMax) {
        PlanarGroup g{};
        g.count = std::min(n - b0, kPlanarGroupMax);
        g.block0[0] = 0;
        for (int p = 0; p < g.count; ++p) {
            g.src[p] = c[b0 + p].src;
            g.dst[p] = c[b0 + p].dst;
            g.rgba[p] = c[b0 + p].rgba;
            g.cnt[p] = c[b0 + p].cnt;
            g.ncnt[p] = c[b0 + p].ncnt;
            g.npix[p] = c[b0 + p].npix;
            g.block0[p + 1] = g.block0[p] + static_cast<int>((c[b0 + p].npix + 255) / 256);
        }
        const cudaError_t e = launch_pdl(planar_group_kernel, dim3(g.block0[g.count]), dim3(256), 0, st, g, to_planar);
        if (e != cudaSuccess)
            return e;
        ++*nl;
    }
    return cudaGetLastError();
}

// One launch of the FMA form's solve kernel per kN members (each member's
// counters zeroed beforehand; the first member's ticket serves the launch).
template <int kN>
cudaError_t launch_solve(const std::vector<PlWs>& v, const int* w, const int* h, int n, int num_iter, float step,
    float mom, int sms, cudaStream_t st, int* nl)
{
    const int nround = solve_launches(num_iter);
    for (int b0 = 0; b0 < n; b0 += kN) {
        PlSolve<kN> g{};
        g.count = std::min(n - b0, kN);
        g.tile0[0] = 0;
        for (int p = 0; p < g.count; ++p) {
            const PlWs& m = v[b0 + p];
            const int W = w[b0 + p], H = h[b0 + p];
            CUtensorMap* mp = g.map[p];
            bool ok = true;
            for (int c = 0; c < 2 && ok; ++c)
                ok = encode_plane_map(&mp[c ? kPmO1 : kPmO0], m.O[c], W, H, kPlW, kPlRows) &&
                     encode_plane_map(&mp[c ? kPmU1 : kPmU0], m.U[c], W, H, kPlW, kPlRows) &&
                     encode_plane_map(&mp[c ? kPmOo1 : kPmOo0], m.O[c], W, H, kPlIW, kPlIRows) &&
                     encode_plane_map(&mp[c ? kPmUo1 : kPmUo0], m.U[c], W, H, kPlIW, kPlIRows);
            if (!ok || !encode_plane_map(&mp[kPmK], m.K, W, H, kPlW, kPlRows) ||
                !encode_plane_map(&mp[kPmC], m.C, W, H, kPlW, kPlRows))
                return cudaErrorInvalidValue;
            g.done[p] = m.cnt + 16;
            g.w[p] = W;
            g.h[p] = H;
            g.tiles_x[p] = pl_tiles_x(W);
            g.tile0[p + 1] = g.tile0[p] + pl_tiles(W, H);
        }
        g.nround = nround;
        g.num_iter = num_iter;
        g.ticket = v[b0].cnt;
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cfg.gridDim = dim3(static_cast<unsigned>(std::min<int64_t>(static_cast<int64_t>(g.tile0[g.count]) * nround, sms)));
        cfg.blockDim = dim3(kPlThreads);
        cfg.dynamicSmemBytes = kPlSmem;
        const cudaError_t e = cudaLaunchKernelEx(&cfg, solver_fma_solve_kernel<kN>, g, step, mom);
        if (e != cudaSuccess)
            return e;
        ++*nl;
    }
    return cudaGetLastError();
}

// The FMA form of run_solver: constants, O's planes (or the upsampled coarse
// solution Oc) and zeroed counters, the solve (one launch; per round on the
// plain-load path), O (and the RGBA8 copy) back from its planes.
cudaError_t run_solver_fma(const DeviceInfo* di, const float* P, const float* A, const float* Wt, float* O, int w,
    int h, int num_iter, float step, float mom, float* workspace, cudaStream_t st, int* nl, uint8_t* rgba_out,
    const float* Oc, int cw, int ch)
{
    const PlWs v = pl_view(workspace, w, h);
    const dim3 b(32, 8);
    cudaError_t e = launch_pdl(solver_prep_fma_kernel, grid2d(w, h, b), b, 0, st, P, A, Wt,
        static_cast<const float*>(O), v.C, v.K, v.O[0], w, h, step, v.cnt, v.ncnt, Oc, cw, ch);
    ++*nl;
    const int nlaunch = solve_launches(num_iter);
    if (e == cudaSuccess && pl_tma_eligible(di, w, workspace)) {
        const std::vector<PlWs> one(1, v);
        e = launch_solve<1>(one, &w, &h, 1, num_iter, step, mom, di->sms, st, nl);
    } else if (e == cudaSuccess) {
        // plain loads and stores (widths not a multiple of 4, an unaligned workspace)
        const int tx = pl_tiles_x(w), nt = pl_tiles(w, h);
        int k0 = 0;
        for (int li = 0; li < nlaunch && e == cudaSuccess; ++li) {
            const int T = std::min(kTbT, num_iter - k0);
            const PlPlain pl{v.O[li & 1], v.U[li & 1], v.K, v.C, v.O[(li + 1) & 1], v.U[(li + 1) & 1], w, h, tx, nt};
            e = launch_pdl(solver_fma_plain_kernel, dim3(std::min(nt, di->sms)), dim3(kPlThreads), kPlSmem, st, pl, T,
                k0, step, mom);
            ++*nl;
            k0 += T;
        }
    }
    if (e == cudaSuccess) {
        const PlanarCopy back{v.O[nlaunch & 1], O, rgba_out, static_cast<int64_t>(w) * h};
        e = launch_planar(&back, 1, 0, st, nl);
    }
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace

bool solver_tma_supported()
{
    DeviceInfo* di = nullptr;
    return device_info(&di) == cudaSuccess && di->ps_smem;
}

float* solver_start_buffer(float* O, int w, int h, int num_iter, float* workspace, int form)
{
    if (form == kSolverFma)
        return O;  // the solve copies O into its planes first
    return solve_launches(num_iter) % 2 == 0 ? O : ws_view(workspace, w, h).O2;
}

cudaError_t solver_lap(const float* P, int w, int h, float* workspace, cudaStream_t st)
{
    const dim3 b(32, 8);
    const cudaError_t e = launch_pdl(lap_pr_kernel, grid2d(w, h, b), b, 0, st, P, workspace, w, h);
    if (e != cudaSuccess)
        return e;
    return cudaGetLastError();
}

cudaError_t solver_prep(int form, const float* P, const float* A, const float* Wt, int w, int h, float step,
    float* workspace, cudaStream_t st)
{
    if (form != kSolverFma)
        return solver_lap(P, w, h, workspace, st);
    const PlWs v = pl_view(workspace, w, h);
    const dim3 b(32, 8);
    const cudaError_t e = launch_pdl(solver_prep_fma_kernel, grid2d(w, h, b), b, 0, st, P, A, Wt,
        static_cast<const float*>(nullptr), v.C, v.K, static_cast<float*>(nullptr), w, h, step,
        static_cast<unsigned*>(nullptr), 0, static_cast<const float*>(nullptr), 0, 0);
    if (e != cudaSuccess)
        return e;
    return cudaGetLastError();
}

bool solver_group_eligible(const SolverImage* im, int n, int form)
{
    DeviceInfo* di = nullptr;
    if (n < 1 || device_info(&di) != cudaSuccess)
        return false;
    for (int i = 0; i < n; ++i) {
        const bool ok = form == kSolverFma
                            ? pl_tma_eligible(di, im[i].w, im[i].workspace)
                            : tma_eligible(di, im[i].w, im[i].O, ws_view(im[i].workspace, im[i].w, im[i].h), im[i].A,
                                  im[i].Wt);
        if (!ok)
            return false;
    }
    return true;
}

cudaError_t run_solver_group(const SolverImage* im, int n, int num_iter, float step, float mom, cudaStream_t st,
    int* launches, int form)
{
    DeviceInfo* di = nullptr;
    cudaError_t e = device_info(&di);
    if (e != cudaSuccess)
        return e;
    if (!solver_group_eligible(im, n, form))
        return cudaErrorInvalidValue;
    int nl = 0;
    if (num_iter <= 0) {
        for (int i = 0; i < n && e == cudaSuccess; ++i)
            if (im[i].rgba) {
                e = launch_float_to_rgba(im[i].O, im[i].rgba, static_cast<int64_t>(im[i].w) * im[i].h, st);
                ++nl;
            }
        if (launches)
            *launches += nl;
        return e;
    }
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess)
        return e;
    std::vector<int> ws(n), hs(n);
    for (int i = 0; i < n; ++i) {
        ws[i] = im[i].w;
        hs[i] = im[i].h;
    }
    const int rows = chosen_rows(dev, ws.data(), hs.data(), n, di->sms, form);
    const bool odd = solve_launches(num_iter) % 2 == 1;
    if (form == kSolverFma) {
        // O into planes (counters zeroed), one solve launch per 16 images, O back
        std::vector<PlWs> v(n);
        std::vector<PlanarCopy> to(n), back(n);
        for (int i = 0; i < n; ++i) {
            v[i] = pl_view(im[i].workspace, im[i].w, im[i].h);
            const int64_t np = static_cast<int64_t>(im[i].w) * im[i].h;
            to[i] = PlanarCopy{im[i].O, v[i].O[0], nullptr, np, v[i].cnt, v[i].ncnt};
            back[i] = PlanarCopy{v[i].O[solve_launches(num_iter) & 1], im[i].O, im[i].rgba, np};
        }
        e = launch_planar(to.data(), n, 1, st, &nl);
        if (e == cudaSuccess)
            e = n <= 4 ? launch_solve<4>(v, ws.data(), hs.data(), n, num_iter, step, mom, di->sms, st, &nl)
                       : launch_solve<kGroupMax>(v, ws.data(), hs.data(), n, num_iter, step, mom, di->sms, st, &nl);
        if (e == cudaSuccess)
            e = launch_planar(back.data(), n, 0, st, &nl);
        if (launches)
            *launches += nl;
        return e != cudaSuccess ? e : cudaGetLastError();
    }
    std::vector<GroupMember> mem(n);
    for (int i = 0; i < n; ++i) {
        const WsView v = ws_view(im[i].workspace, im[i].w, im[i].h);
        float* const O[2] = {im[i].O, v.O2};
        float* const U[2] = {v.U0, v.U1};
        if (!encode_solve(&mem[i].maps, O, U, im[i].A, im[i].Wt, v.L, im[i].w, im[i].h, rows))
            return cudaErrorInvalidValue;
        mem[i].c0 = odd ? 1 : 0;
        mem[i].rgba = im[i].rgba;
        mem[i].w = im[i].w;
        mem[i].h = im[i].h;
    }
    e = n <= 4 ? launch_members<4>(mem, rows, num_iter, step, mom, di->sms, st, &nl)
               : launch_members<kGroupMax>(mem, rows, num_iter, step, mom, di->sms, st, &nl);
    if (launches)
        *launches += nl;
    if (e == cudaSuccess)
        e = cudaGetLastError();
    return e;
}

cudaError_t run_solver_from_coarse(const float* P, const float* A, const float* Wt, float* O, int w, int h,
    const float* Oc, int cw, int ch, int num_iter, float step, float mom, float* workspace, cudaStream_t st,
    int* launches, uint8_t* rgba_out)
{
    if (num_iter <= 0 || !Oc || cw <= 0 || ch <= 0)
        return cudaErrorInvalidValue;
    DeviceInfo* di = nullptr;
    cudaError_t e = device_info(&di);
    if (e != cudaSuccess)
        return e;
    if (!di->ps_smem)
        return cudaErrorNotSupported;
    int nl = 0;
    e = run_solver_fma(di, P, A, Wt, O, w, h, num_iter, step, mom, workspace, st, &nl, rgba_out, Oc, cw, ch);
    if (launches)
        *launches += nl;
    return e;
}

cudaError_t run_solver(const float* P, const float* A, const float* Wt, float* O, int w, int h, int num_iter,
    float step, float mom, float* workspace, cudaStream_t st, int* launches, uint8_t* rgba_out, int form)
{
    const size_t n = static_cast<size_t>(w) * h * 3;
    const WsView v = ws_view(workspace, w, h);
    int nl = 0;
    if (num_iter <= 0) {
        if (rgba_out) {
            cudaError_t e = launch_float_to_rgba(O, rgba_out, static_cast<int64_t>(w) * h, st);
            if (launches)
                *launches += 1;
            return e;
        }
        return cudaSuccess;
    }
    DeviceInfo* di = nullptr;
    cudaError_t e0 = device_info(&di);
    if (e0 != cudaSuccess)
        return e0;
    if (form == kSolverFma) {
        if (!di->ps_smem)
            return cudaErrorNotSupported;
        const cudaError_t e = run_solver_fma(di, P, A, Wt, O, w, h, num_iter, step, mom, workspace, st, &nl, rgba_out,
            nullptr, 0, 0);
        if (launches)
            *launches += nl;
        return e;
    }
    if ((e0 = solver_lap(P, w, h, v.L, st)) != cudaSuccess)
        return e0;
    ++nl;
    // Launches of up to kTbT iterations; ping-pong O between O and O2 and U
    // between its two buffers so that the last launch writes O.
    const int nlaunch = solve_launches(num_iter);
    float* cur = solver_start_buffer(O, w, h, num_iter, workspace, kSolverExact);
    if (cur != O) {
        cudaError_t e = cudaMemcpyAsync(v.O2, O, n * sizeof(float), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess)
            return e;
    }
    // TMA path: 16-byte row pitch and aligned images; the tile shape is the
    // autotuned one for this size, else the wave model's
    int dev = 0;
    if ((e0 = cudaGetDevice(&dev)) != cudaSuccess)
        return e0;
    const int rows = chosen_rows(dev, &w, &h, 1, di->sms, kSolverExact);
    GroupMember m{};
    bool tma = tma_eligible(di, w, O, v, A, Wt);
    if (tma) {
        float* const Ob[2] = {O, v.O2};
        float* const Ub[2] = {v.U0, v.U1};
        tma = encode_solve(&m.maps, Ob, Ub, A, Wt, v.L, w, h, rows);
    }
    if (tma) {
        m.w = w;
        m.h = h;
        m.c0 = cur == O ? 0 : 1;
        m.rgba = rgba_out;
        const std::vector<GroupMember> one(1, m);
        cudaError_t e = launch_members<1>(one, rows, num_iter, step, mom, di->sms, st, &nl);
        if (launches)
            *launches += nl;
        return e != cudaSuccess ? e : cudaGetLastError();
    }
    float* U[2] = {v.U0, v.U1};
    int k0 = 0;
    for (int li = 0; li < nlaunch; ++li) {
        const int T = std::min(kTbT, num_iter - k0);
        float* nxt = (cur == O) ? v.O2 : O;
        uint8_t* rg = (li == nlaunch - 1) ? rgba_out : nullptr;
        const dim3 grid((w + (kTbEX - 2 * T) - 1) / (kTbEX - 2 * T), (h + (kTbEY - 2 * T) - 1) / (kTbEY - 2 * T));
        solver_tb_kernel<<<grid, dim3(32, kTbEY / 2), kTbSmem, st>>>(cur, nxt, U[li & 1], U[(li + 1) & 1], v.L, A,
            Wt, w, h, T, k0, step, mom, rg);
        ++nl;
        k0 += T;
        cur = nxt;
    }
    if (launches)
        *launches += nl;
    return cudaGetLastError();
}

// ---- device addresses of file-scope device arrays -----------------------------
// In host code a __device__ variable's name is only a stand-in symbol, not a
// device address.  Its address is looked up with cudaGetSymbolAddress, with
// the device current, once per device and context: the address belongs to
// the module loaded into the context, so after a device reset (a new primary
// context) it is looked up again.  The context is told apart by its id
// (cuCtxGetId, fetched from the driver at run time); without that entry
// point every call looks the address up.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

bool current_context_id(unsigned long long* id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
    });
    CUcontext ctx = nullptr;
    return get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, id) == CUDA_SUCCESS;
}

struct SymbolCache {
    std::mutex mu;
    void* addr[64] = {};
    unsigned long long ctx[64] = {};
};

cudaError_t symbol_address(SymbolCache& c, const void* symbol, void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    unsigned long long id = 0;
    std::lock_guard<std::mutex> lock(c.mu);
    if (!c.addr[dev] || !current_context_id(&id) || c.ctx[dev] != id) {
        void* p = nullptr;
        if ((e = cudaGetSymbolAddress(&p, symbol)) != cudaSuccess)
            return e;
        // the lookup made the device's context current
        c.addr[dev] = p;
        c.ctx[dev] = current_context_id(&id) ? id : 0;
    }
    *out = c.addr[dev];
    return cudaSuccess;
}

// ---- solver workspace for callers that cannot allocate ------------------------
// A file-scope device array (every GPU that loads the library holds it until
// the process exits), handed to the kernels by its device address
// (symbol_address: looked up once per device and context).
static __device__ __align__(256) float g_noalloc_ws[kNoAllocWorkspaceFloats];

cudaError_t noalloc_workspace(float** out)
{
    static SymbolCache cache;
    return symbol_address(cache, g_noalloc_ws, reinterpret_cast<void**>(out));
}

cudaError_t run_solver_noalloc(const float* P, const float* A, const float* Wt, float* O, int w, int h, int num_iter,
    float step, float mom, cudaStream_t st)
{
    float* ws = nullptr;
    cudaError_t e = noalloc_workspace(&ws);
    if (e != cudaSuccess)
        return e;
    // Every workspace element (lap P, both momentum images, the second Jacobi
    // buffer) is written before it is read, so nothing is cleared.
    return run_solver(P, A, Wt, O, w, h, num_iter, step, mom, ws, st, nullptr, nullptr, kSolverExact);
}

cudaError_t device_timeout_flag(int** flag)
{
    static SymbolCache cache;
    return symbol_address(cache, &g_device_timeout, reinterpret_cast<void**>(flag));
}

cudaError_t check_device_timeout(int* flagged)
{
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_device_timeout, sizeof(int));
    if (e != cudaSuccess)
        return e;
    if (v) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(g_device_timeout, &zero, sizeof(int));
    }
    *flagged = v;
    return e;
}

cudaError_t launch_bounded_wait_selftest(int spins, cudaStream_t st)
{
    bounded_wait_selftest_kernel<<<1, 32, 0, st>>>(spins);
    return cudaGetLastError();
}

}  // namespace vsc
