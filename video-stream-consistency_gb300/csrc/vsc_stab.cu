// Stabilization-pass kernels for sm_103a (reference: src/stabilization/
// flowconsistency.cu and gpuimage.cu).
//
// Images are interleaved float HWC with 3 channels, the reference's GPUImage
// layout.  Every kernel keeps the reference's per-pixel expression order and
// is compiled with -fmad=false, so it reproduces the CPU restatement of the
// reference bit for bit.  Differences from the reference's schedule:
//   - the solver lives in vsc_solver.cu;
//   - the orchestrator uses one fused kernel for the five warps, the
//     adaptive combination and the consistency weights (the reference runs
//     seven kernels with a device synchronisation after each).
#include "vsc_internal.h"
#include "vsc_math.cuh"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace vsc {
namespace {


// ---- frame I/O (gpuimage.cu:39-67) ---------------------------------------
// float(double(v) / 255.0) equals the single-precision quotient v / 255.0f
// for every byte value (checked exhaustively by the tests), so the table is
// built with one IEEE float division per entry.
__device__ __forceinline__ void build_lut(float* lut)
{
    for (int v = threadIdx.x; v < 256; v += blockDim.x)
        lut[v] = __fdiv_rn(static_cast<float>(v), 255.0f);
    __syncthreads();
}

// 4 pixels per thread: one 16-byte RGBA load, three 16-byte float stores.
__global__ void rgba_to_float4_kernel(const uint4* __restrict__ rgba, float4* __restrict__ out, int64_t nquad)
{
    pdl_enter();
    __shared__ float lut[256];
    build_lut(lut);
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= nquad)
        return;
    const uint4 px = rgba[i];
    const uint32_t w[4] = {px.x, px.y, px.z, px.w};
    float f[12];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        f[3 * k + 0] = lut[w[k] & 0xff];
        f[3 * k + 1] = lut[(w[k] >> 8) & 0xff];
        f[3 * k + 2] = lut[(w[k] >> 16) & 0xff];
    }
    out[3 * i + 0] = make_float4(f[0], f[1], f[2], f[3]);
    out[3 * i + 1] = make_float4(f[4], f[5], f[6], f[7]);
    out[3 * i + 2] = make_float4(f[8], f[9], f[10], f[11]);
}

__global__ void rgba_to_float_kernel(const uint8_t* __restrict__ rgba, float* __restrict__ out, int64_t first,
    int64_t npix)
{
    __shared__ float lut[256];
    build_lut(lut);
    const int64_t i = first + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= npix)
        return;
    out[i * 3 + 0] = lut[rgba[i * 4 + 0]];
    out[i * 3 + 1] = lut[rgba[i * 4 + 1]];
    out[i * 3 + 2] = lut[rgba[i * 4 + 2]];
}

__global__ void float4_to_rgba_kernel(const float4* __restrict__ in, uint4* __restrict__ rgba, int64_t nquad)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= nquad)
        return;
    const float4 a = in[3 * i + 0], b = in[3 * i + 1], c = in[3 * i + 2];
    rgba[i] = make_uint4(pack_rgba(a.x, a.y, a.z), pack_rgba(a.w, b.x, b.y), pack_rgba(b.z, b.w, c.x),
        pack_rgba(c.y, c.z, c.w));
}

__global__ void float_to_rgba_kernel(const float* __restrict__ in, uint8_t* __restrict__ rgba, int64_t first,
    int64_t npix)
{
    const int64_t i = first + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= npix)
        return;
    reinterpret_cast<uint32_t*>(rgba)[i] = pack_rgba(in[i * 3 + 0], in[i * 3 + 1], in[i * 3 + 2]);
}

// ---- kernel_warp (flowconsistency.cu:77-114) --------------------------------
// I: the index type of the tap offsets (int64_t in general; int where every
// element offset of the frame fits, which saves 64-bit arithmetic).
template <class I>
struct WarpTapT {
    I q0, q1;  // pixel indices of the top-left tap of rows map_iy and map_iy+1
    I o0, o1;  // their element offsets in a 3-channel image
    float fx, fy;
};
using WarpTap = WarpTapT<int64_t>;

template <class I = int64_t>
__device__ __forceinline__ WarpTapT<I> warp_tap_uv(float flo_x, float flo_y, int x, int y, int w, int h)
{
    const float map_fx = fmaxf(0.0f, fminf(static_cast<float>(x) + flo_x, static_cast<float>(w - 3)));
    const float map_fy = fmaxf(0.0f, fminf(static_cast<float>(y) + flo_y, static_cast<float>(h - 3)));
    const int map_ix = static_cast<int>(floorf(map_fx));
    const int map_iy = static_cast<int>(floorf(map_fy));
    WarpTapT<I> t;
    t.fx = map_fx - static_cast<float>(map_ix);
    t.fy = map_fy - static_cast<float>(map_iy);
    t.q0 = static_cast<I>(map_iy) * w + map_ix;
    t.q1 = t.q0 + w;
    t.o0 = t.q0 * 3;
    t.o1 = t.q1 * 3;
    return t;
}

template <class I = int64_t>
__device__ __forceinline__ WarpTapT<I> warp_tap(const float* __restrict__ flow, int fc, int x, int y, int w, int h)
{
    const I fi = (static_cast<I>(y) * w + x) * fc;
    return warp_tap_uv<I>(flow[fi + 0], flow[fi + 1], x, y, w, h);
}

// The first two channels of a 3-channel flow of fw x fh, bilinearly sampled
// at pixel (x, y) of a w x h frame: the value kernel_bilinear's upsampling to
// w x h stores there (bilinear_px: same positions, clamps and expression,
// so the same bits), computed where it is used instead of stored.
__device__ __forceinline__ void flow_upsampled_uv(const float* __restrict__ small, int fw, int fh, int w, int h, int x,
    int y, float& u, float& v)
{
    const float xx = static_cast<float>(x) * static_cast<float>(fw) / static_cast<float>(w);
    const float yy = static_cast<float>(y) * static_cast<float>(fh) / static_cast<float>(h);
    const int ix = min(static_cast<int>(floorf(xx)), fw - 1);
    const int iy = min(static_cast<int>(floorf(yy)), fh - 1);
    const float fx = xx - static_cast<float>(ix);
    const float fy = yy - static_cast<float>(iy);
    const int ix1 = min(ix + 1, fw - 1);
    const int iy1 = min(iy + 1, fh - 1);
    const float* r0 = small + static_cast<int64_t>(iy) * fw * 3;
    const float* r1 = small + static_cast<int64_t>(iy1) * fw * 3;
    float out[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float v00 = r0[ix * 3 + k], v10 = r0[ix1 * 3 + k], v01 = r1[ix * 3 + k], v11 = r1[ix1 * 3 + k];
        out[k] = v00 * (1 - fx) * (1 - fy) + v10 * fx * (1 - fy) + v01 * (1 - fx) * fy + v11 * fx * fy;
    }
    u = out[0];
    v = out[1];
}

// the bilinear blend of the four taps, in kernel_warp's operation order
__device__ __forceinline__ float bilerp(float t00, float t01, float t10, float t11, float fx, float fy)
{
    const float tmp_1 = t00 * (1.0f - fx) + t01 * fx;
    const float tmp_2 = t10 * (1.0f - fx) + t11 * fx;
    return tmp_1 * (1.0f - fy) + tmp_2 * fy;
}

template <class I>
__device__ __forceinline__ float warp_sample(const float* __restrict__ in, const WarpTapT<I>& t, int c)
{
    return bilerp(in[t.o0 + c], in[t.o0 + 3 + c], in[t.o1 + c], in[t.o1 + 3 + c], t.fx, t.fy);
}

// I = int where every element offset of the frame fits (32-bit tap
// arithmetic).  Two pixels per thread, rows y and y + 8 of a 32 x 16 block:
// both flows are read, then all 24 taps, so a thread has two dependent
// memory round trips in flight instead of one.
template <class I>
__global__ void stab_warp_kernel(const float* __restrict__ in, const float* __restrict__ flow, int fc,
    float* __restrict__ out, int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y0 = blockIdx.y * (2 * blockDim.y) + threadIdx.y;
    if (x >= w || y0 >= h)
        return;
    const int y1 = y0 + blockDim.y;
    const bool second = y1 < h;
    const WarpTapT<I> t0 = warp_tap<I>(flow, fc, x, y0, w, h);
    const WarpTapT<I> t1 = warp_tap<I>(flow, fc, x, second ? y1 : y0, w, h);
    float v0[3], v1[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v0[c] = warp_sample(in, t0, c);
        v1[c] = warp_sample(in, t1, c);
    }
    const I o0 = (static_cast<I>(y0) * w + x) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c)
        out[o0 + c] = v0[c];
    if (second) {
        const I o1 = (static_cast<I>(y1) * w + x) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[o1 + c] = v1[c];
    }
}

// ---- kernel_adap_comb / kernel_consist_wt (flowconsistency.cu:116-191) ------
struct Comb {
    float ain, apr;
};

// mp, mn: the opt-in occlusion mask's factors for the previous and the next
// frame's weight, applied after the clamps (1, 1 = kernel_adap_comb's bits).
// kNonPos: alpha is finite and >= 0, so the exponent -alpha d^2 is <= 0 and
// expf_cw_nonpos gives the same weight (see there).
template <bool kNonPos = false>
__device__ __forceinline__ Comb adap_comb_px(float ci, float cp, float pi, float pp, float ni, float np, float ls,
    float alpha, float mp = 1.0f, float mn = 1.0f, bool masked = false)
{
    float wt_prv = kNonPos ? expf_cw_nonpos(-alpha * (ci - pi) * (ci - pi)) : expf_cw(-alpha * (ci - pi) * (ci - pi));
    float wt_nxt = kNonPos ? expf_cw_nonpos(-alpha * (ci - ni) * (ci - ni)) : expf_cw(-alpha * (ci - ni) * (ci - ni));
    if (wt_prv > 0.45f)
        wt_prv = 0.45f;
    if (wt_nxt > 0.3f)
        wt_nxt = 0.3f;
    if (wt_prv < 0.001f)
        wt_prv = 0.0f;
    if (wt_nxt < 0.001f)
        wt_nxt = 0.0f;
    if (masked) {
        wt_prv = wt_prv * mp;
        wt_nxt = wt_nxt * mn;
    }
    Comb r;
    r.ain = wt_prv * pi + wt_nxt * ni + (1.0f - (wt_prv + wt_nxt)) * ci;
    float apr = wt_prv * pp + wt_nxt * np + (1.0f - (wt_prv + wt_nxt)) * cp;
    r.apr = wt_prv * ls + (1.0f - wt_prv) * apr;
    return r;
}

// kNonPos: beta finite and >= 0 and |gamma| <= 1e30 (then gamma times
// expf_cw_nonpos's floor is below the 0.001 cut, as gamma times 0 is).
template <bool kNonPos = false>
__device__ __forceinline__ float consist_wt_px(float c, float a, float beta, float gamma)
{
    float wt = gamma * (kNonPos ? expf_cw_nonpos(-beta * (c - a) * (c - a)) : expf_cw(-beta * (c - a) * (c - a)));
    if (wt < 0.001f)
        wt = 0.0f;
    return wt;
}

__global__ void adap_comb_kernel(const float* __restrict__ ci, const float* __restrict__ cp,
    const float* __restrict__ pwi, const float* __restrict__ pwp, const float* __restrict__ nwi,
    const float* __restrict__ nwp, float* __restrict__ ai, float* __restrict__ ap, const float* __restrict__ lsw,
    const float* __restrict__ occ, float alpha, int64_t n)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    Comb r;
    if (occ)
        r = adap_comb_px(ci[i], cp[i], pwi[i], pwp[i], nwi[i], nwp[i], lsw[i], alpha, occ[(i / 3) * 2],
            occ[(i / 3) * 2 + 1], true);
    else
        r = adap_comb_px(ci[i], cp[i], pwi[i], pwp[i], nwi[i], nwp[i], lsw[i], alpha);
    ai[i] = r.ain;
    ap[i] = r.apr;
}

// ---- forward-backward flow consistency (opt-in; no counterpart in the reference)
// Flow a at (x, y) carries the pixel to p = (x + a.x, y + a.y); the opposite
// flow b is sampled there bilinearly (right/bottom taps clamped) and the
// pixel is consistent if |a + b(p)|^2 <= 0.01 (|a|^2 + |b(p)|^2) + 0.5.
// Outside the frame, or NaN: inconsistent.  Operation order as the CPU
// restatement's, so the 0/1 decisions agree bit for bit.
__device__ __forceinline__ float occl_check(const float* __restrict__ a, const float* __restrict__ b, int fc, int x,
    int y, int w, int h)
{
    const int64_t i = pix_index(x, y, w) * fc;
    const float ax = a[i], ay = a[i + 1];
    const float px = static_cast<float>(x) + ax;
    const float py = static_cast<float>(y) + ay;
    if (!(px >= 0.0f && px <= static_cast<float>(w - 1) && py >= 0.0f && py <= static_cast<float>(h - 1)))
        return 0.0f;
    const int ix = static_cast<int>(floorf(px));
    const int iy = static_cast<int>(floorf(py));
    const float fx = px - static_cast<float>(ix);
    const float fy = py - static_cast<float>(iy);
    const int ix1 = min(ix + 1, w - 1);
    const int iy1 = min(iy + 1, h - 1);
    float bv[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float b00 = b[pix_index(ix, iy, w) * fc + k];
        const float b10 = b[pix_index(ix1, iy, w) * fc + k];
        const float b01 = b[pix_index(ix, iy1, w) * fc + k];
        const float b11 = b[pix_index(ix1, iy1, w) * fc + k];
        const float t0 = b00 * (1.0f - fx) + b10 * fx;
        const float t1 = b01 * (1.0f - fx) + b11 * fx;
        bv[k] = t0 * (1.0f - fy) + t1 * fy;
    }
    const float dx = ax + bv[0];
    const float dy = ay + bv[1];
    const float lhs = dx * dx + dy * dy;
    const float rhs = 0.01f * ((ax * ax + ay * ay) + (bv[0] * bv[0] + bv[1] * bv[1])) + 0.5f;
    return lhs <= rhs ? 1.0f : 0.0f;
}

__global__ void flow_consistency_kernel(const float* __restrict__ ffwd, const float* __restrict__ fbwd, int fc,
    float* __restrict__ mask, int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h)
        return;
    const int64_t o = pix_index(x, y, w) * 2;
    mask[o] = occl_check(fbwd, ffwd, fc, x, y, w, h);
    mask[o + 1] = occl_check(ffwd, fbwd, fc, x, y, w, h);
}

template <bool kNonPos>
__global__ void consist_wt_kernel(const float* __restrict__ ci, const float* __restrict__ ai, float* __restrict__ wt,
    float beta, float gamma, int64_t first, int64_t n)
{
    const int64_t i = first + blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    wt[i] = consist_wt_px<kNonPos>(ci[i], ai[i], beta, gamma);
}

// four values per thread through 16-byte loads and stores (16-byte aligned images)
template <bool kNonPos>
__global__ void consist_wt4_kernel(const float4* __restrict__ ci, const float4* __restrict__ ai,
    float4* __restrict__ wt, float beta, float gamma, int64_t nquad)
{
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= nquad)
        return;
    const float4 c = ci[i], a = ai[i];
    wt[i] = make_float4(consist_wt_px<kNonPos>(c.x, a.x, beta, gamma), consist_wt_px<kNonPos>(c.y, a.y, beta, gamma),
        consist_wt_px<kNonPos>(c.z, a.z, beta, gamma), consist_wt_px<kNonPos>(c.w, a.w, beta, gamma));
}

// ---- kernel_bilinear (flowconsistency.cu:50-75): bilinear_px in vsc_math.cuh ----
__global__ void bilinear_kernel(const float* __restrict__ in, int iw, int ih, float* __restrict__ out, int ow, int oh,
    int c)
{
    const int ox = blockIdx.x * blockDim.x + threadIdx.x;
    const int oy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ox >= ow || oy >= oh)
        return;
    bilinear_px(in, iw, ih, ow, oh, c, ox, oy, out + pix_index(ox, oy, ow) * c);
}

// bilinear_px for four consecutive output pixels of C channels per thread:
// the row terms are computed once, the 4 C outputs leave as 16-byte stores
// when the row is 16-byte aligned (same arithmetic, same bits).
template <int C>
__device__ __forceinline__ void bilinear4_px(const float* __restrict__ in, int iw, int ih, float* __restrict__ out,
    int ow, int oh, int ox0, int oy)
{
    if (ox0 >= ow || oy >= oh)
        return;
    const float yy = static_cast<float>(oy) * static_cast<float>(ih) / static_cast<float>(oh);
    const int iy = min(static_cast<int>(floorf(yy)), ih - 1);
    const float fy = yy - static_cast<float>(iy);
    const int iy1 = min(iy + 1, ih - 1);
    float v[4 * C];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int ox = min(ox0 + j, ow - 1);
        const float xx = static_cast<float>(ox) * static_cast<float>(iw) / static_cast<float>(ow);
        const int ix = min(static_cast<int>(floorf(xx)), iw - 1);
        const float fx = xx - static_cast<float>(ix);
        const int ix1 = min(ix + 1, iw - 1);
#pragma unroll
        for (int k = 0; k < C; ++k) {
            const float v00 = in[pix_index(ix, iy, iw) * C + k];
            const float v10 = in[pix_index(ix1, iy, iw) * C + k];
            const float v01 = in[pix_index(ix, iy1, iw) * C + k];
            const float v11 = in[pix_index(ix1, iy1, iw) * C + k];
            v[j * C + k] = v00 * (1 - fx) * (1 - fy) + v10 * fx * (1 - fy) + v01 * (1 - fx) * fy + v11 * fx * fy;
        }
    }
    float* dst = out + pix_index(ox0, oy, ow) * C;
    if (ox0 + 3 < ow && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
#pragma unroll
        for (int q = 0; q < C; ++q)
            reinterpret_cast<float4*>(dst)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else {
        for (int j = 0; j < 4 && ox0 + j < ow; ++j)
#pragma unroll
            for (int k = 0; k < C; ++k)
                dst[j * C + k] = v[j * C + k];
    }
}

template <int C>
__global__ void bilinear4_kernel(const float* __restrict__ in, int iw, int ih, float* __restrict__ out, int ow, int oh)
{
    pdl_enter();
    bilinear4_px<C>(in, iw, ih, out, ow, oh, (blockIdx.x * blockDim.x + threadIdx.x) * 4,
        blockIdx.y * blockDim.y + threadIdx.y);
}

// Exact 2x upsampling of 3-channel images (ow == 2 iw, oh == 2 ih): the
// sample positions ox * iw / ow and oy * ih / oh are exactly ox / 2 and
// oy / 2, so a 128 x 8 output block (32 x 8 threads, 4 pixels each) reads
// the 65 x 5 input window that starts at (ox_b / 2, oy_b / 2).  The window is
// staged in shared memory by coalesced loads (its clamped columns and rows
// repeat the last ones, as the clamped indices of bilinear_px do), each
// output is the same expression of the same values as bilinear_px, and each
// warp's output row leaves through shared memory as coalesced 16-byte
// stores.  Same bits as bilinear4_kernel<3>.
constexpr int kB2W = 128, kB2H = 8;
constexpr int kB2InW = kB2W / 2 + 1, kB2InH = kB2H / 2 + 1;
struct Bilinear2xSmem {
    float tile[kB2InH][kB2InW * 3];
    __align__(16) float row[kB2H][kB2W * 3];
};

__device__ __forceinline__ void bilinear2x3_block(Bilinear2xSmem& sm, const float* __restrict__ in, int iw, int ih,
    float* __restrict__ out, int ow, int oh, int bx, int by)
{
    const int ox_b = bx * kB2W, oy_b = by * kB2H;
    const int ix_b = ox_b / 2, iy_b = oy_b / 2;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    for (int i = tid; i < kB2InH * kB2InW * 3; i += 32 * kB2H) {
        const int r = i / (kB2InW * 3), q = i - r * (kB2InW * 3);
        const int col = q / 3, ch = q - col * 3;
        const int iy = min(iy_b + r, ih - 1), ix = min(ix_b + col, iw - 1);
        sm.tile[r][q] = in[(static_cast<int64_t>(iy) * iw + ix) * 3 + ch];
    }
    __syncthreads();
    const int oy = oy_b + threadIdx.y;
    if (oy >= oh)
        return;  // no barrier follows
    const float yy = static_cast<float>(oy) * static_cast<float>(ih) / static_cast<float>(oh);
    const int iy = min(static_cast<int>(floorf(yy)), ih - 1);
    const float fy = yy - static_cast<float>(iy);
    const float* t0 = sm.tile[iy - iy_b];
    const float* t1 = sm.tile[iy - iy_b + 1];  // the clamped row min(iy + 1, ih - 1)
    float* rb = sm.row[threadIdx.y];
    float v[12];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int ox = min(ox_b + 4 * static_cast<int>(threadIdx.x) + j, ow - 1);
        const float xx = static_cast<float>(ox) * static_cast<float>(iw) / static_cast<float>(ow);
        const int ix = min(static_cast<int>(floorf(xx)), iw - 1);
        const float fx = xx - static_cast<float>(ix);
        const int c0 = (ix - ix_b) * 3, c1 = c0 + 3;  // column c1 is the clamped min(ix + 1, iw - 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float v00 = t0[c0 + k], v10 = t0[c1 + k], v01 = t1[c0 + k], v11 = t1[c1 + k];
            v[j * 3 + k] = v00 * (1 - fx) * (1 - fy) + v10 * fx * (1 - fy) + v01 * (1 - fx) * fy + v11 * fx * fy;
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q)  // the thread's 12 floats, 48 bytes: conflict-free 16-byte stores
        reinterpret_cast<float4*>(rb)[3 * threadIdx.x + q] =
            make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    __syncwarp();
    const int n = min(kB2W, ow - ox_b) * 3;  // floats of this row segment
    float* dst = out + (static_cast<int64_t>(oy) * ow + ox_b) * 3;
    if (n == kB2W * 3 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
#pragma unroll
        for (int q = 0; q < 3; ++q)
            reinterpret_cast<float4*>(dst)[threadIdx.x + 32 * q] =
                reinterpret_cast<const float4*>(rb)[threadIdx.x + 32 * q];
    } else {
        for (int q = threadIdx.x; q < n; q += 32)
            dst[q] = rb[q];
    }
}

__global__ void __launch_bounds__(256) bilinear2x3_kernel(const float* __restrict__ in, int iw, int ih,
    float* __restrict__ out, int ow, int oh)
{
    pdl_enter();
    __shared__ Bilinear2xSmem sm;
    bilinear2x3_block(sm, in, iw, ih, out, ow, oh, blockIdx.x, blockIdx.y);
}

// the exact-2x form applies: twice the size, and every product ox * iw and
// oy * ih exact in float (below 2^24), so the positions are exactly ox / 2, oy / 2
bool bilinear_is_2x(int iw, int ih, int ow, int oh)
{
    return ow == 2 * iw && oh == 2 * ih && static_cast<int64_t>(ow) * iw < (int64_t{1} << 24) &&
           static_cast<int64_t>(oh) * ih < (int64_t{1} << 24);
}

// bilinear4_kernel<3> over up to kBilinearGroupMax images of any sizes in one
// launch (one per stream of a multi-stream step): a flat list of 32 x 8
// blocks, each image's blocks after the previous image's.
constexpr int kBilinearGroupMax = 16;
struct BilinearGroup {
    const float* in[kBilinearGroupMax];
    float* out[kBilinearGroupMax];
    int iw[kBilinearGroupMax], ih[kBilinearGroupMax], ow[kBilinearGroupMax], oh[kBilinearGroupMax];
    int bx[kBilinearGroupMax];              // blocks per output row band
    int two_x[kBilinearGroupMax];           // bilinear_is_2x: the staged exact-2x form
    int block0[kBilinearGroupMax + 1];      // first block of each image
    int count;
};

__global__ void __launch_bounds__(256) bilinear4_group_kernel(const __grid_constant__ BilinearGroup g)
{
    __shared__ Bilinear2xSmem sm;
    int p = 0;
    while (p + 1 < g.count && static_cast<int>(blockIdx.x) >= g.block0[p + 1])
        ++p;
    const int b = blockIdx.x - g.block0[p];
    const int bx = b % g.bx[p], by = b / g.bx[p];
    if (g.two_x[p]) {
        bilinear2x3_block(sm, g.in[p], g.iw[p], g.ih[p], g.out[p], g.ow[p], g.oh[p], bx, by);
        return;
    }
    bilinear4_px<3>(g.in[p], g.iw[p], g.ih[p], g.out[p], g.ow[p], g.oh[p], (bx * 32 + threadIdx.x) * 4,
        by * 8 + threadIdx.y);
}

__global__ void pyr_down3_kernel(const float* __restrict__ P, const float* __restrict__ A,
    const float* __restrict__ Wt, int iw, int ih, float* __restrict__ Pd, float* __restrict__ Ad,
    float* __restrict__ Wd, int ow, int oh)
{
    pdl_enter();
    const int ox = blockIdx.x * blockDim.x + threadIdx.x;
    const int oy = blockIdx.y * blockDim.y + threadIdx.y;
    if (ox >= ow || oy >= oh)
        return;
    const int64_t o = pix_index(ox, oy, ow) * 3;
    bilinear_px(P, iw, ih, ow, oh, 3, ox, oy, Pd + o);
    bilinear_px(A, iw, ih, ow, oh, 3, ox, oy, Ad + o);
    bilinear_px(Wt, iw, ih, ow, oh, 3, ox, oy, Wd + o);
}

// ---- fused front end of doOneStep (videostabilizer.cpp:182-198) --------------
// kOcc: the opt-in forward-backward consistency mask, evaluated in place.
// kFast: every element offset of the frame fits an int (32-bit tap
// arithmetic), alpha and beta are finite and >= 0 and |gamma| <= 1e30
// (expf_cw_nonpos for the three weights): the same outputs bit for bit,
// about a sixth fewer instructions and fewer registers.
// kHalf (without kOcc): ffwd and fbwd are the 3-channel flows of fw x fh that
// the step upsamples bilinearly to w x h (FLOWDOWNSCALE); each pixel samples
// them with flow_upsampled_uv, the value the upsampled flow holds there, so
// the full-size flows are neither written nor read.
// kDown (w and h even): also the next pyramid level, w/2 x h/2, of the
// processed frame, adapCmbPr and consWt (pyr_down3_kernel's bilinear_px
// downsampling, whose taps are exactly the 2 x 2 group (2 ox .. 2 ox + 1,
// 2 oy .. 2 oy + 1) with zero fractions): the block's 32 x 8 pixels pass
// their values through shared memory and one thread per 2 x 2 group
// evaluates bilinear_px's expression on them.  The same bits as the
// separate pass, without reading the three full-size images again.
struct FrontDown {
    float* P;
    float* A;
    float* W;
    int ow, oh;
};

template <bool kOcc, bool kFast, bool kHalf = false, bool kDown = false>
__global__ void __launch_bounds__(256) fused_front_kernel(const float* __restrict__ o0,
    const float* __restrict__ o1,
    const float* __restrict__ o2, const float* __restrict__ p0, const float* __restrict__ p1,
    const float* __restrict__ p2, const float* __restrict__ ls, const float* __restrict__ ffwd,
    const float* __restrict__ fbwd, int fc, float* __restrict__ adap_pr, float* __restrict__ cons_wt, int w, int h,
    float alpha, float beta, float gamma, int fw, int fh, FrontDown dn)
{
    static_assert(!(kHalf && kOcc), "the occlusion mask samples the flows at warped positions");
    static_assert(!(kDown && kOcc), "the downsampling is fused into the unmasked pass only");
    pdl_enter();
    using I = typename std::conditional<kFast, int, int64_t>::type;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const bool in = x < w && y < h;
    if (!kDown && !in)
        return;
    float pv[3], av[3], wv[3];  // kDown: this pixel's P, adapCmbPr, consWt
    if (in) {
        const I o = (static_cast<I>(y) * w + x) * 3;
        prefetch_l2(o0 + o);
        prefetch_l2(p0 + o);
        prefetch_l2(ls + o);
        prefetch_l2(o2 + o);
        prefetch_l2(p2 + o);
        WarpTapT<I> tb, tf;
        if (kHalf) {
            float u, v;
            flow_upsampled_uv(fbwd, fw, fh, w, h, x, y, u, v);
            tb = warp_tap_uv<I>(u, v, x, y, w, h);
            flow_upsampled_uv(ffwd, fw, fh, w, h, x, y, u, v);
            tf = warp_tap_uv<I>(u, v, x, y, w, h);
        } else {
            tb = warp_tap<I>(fbwd, fc, x, y, w, h);
            tf = warp_tap<I>(ffwd, fc, x, y, w, h);
        }
        float mp = 1.0f, mn = 1.0f;
        if (kOcc) {
            mp = occl_check(fbwd, ffwd, fc, x, y, w, h);
            mn = occl_check(ffwd, fbwd, fc, x, y, w, h);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float pwi = warp_sample(o0, tb, c);
            const float pwp = warp_sample(p0, tb, c);
            const float nwi = warp_sample(o2, tf, c);
            const float nwp = warp_sample(p2, tf, c);
            const float lsw = warp_sample(ls, tb, c);
            const float ci = o1[o + c];
            const float cp = p1[o + c];
            const Comb r = adap_comb_px<kFast>(ci, cp, pwi, pwp, nwi, nwp, lsw, alpha, mp, mn, kOcc);
            const float wt = consist_wt_px<kFast>(ci, r.ain, beta, gamma);
            adap_pr[o + c] = r.apr;
            cons_wt[o + c] = wt;
            pv[c] = cp;
            av[c] = r.apr;
            wv[c] = wt;
        }
    }
    if (kDown) {
        __shared__ float sd[8][32][9];
        const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            sd[ty][tx][c] = in ? pv[c] : 0.0f;
            sd[ty][tx][3 + c] = in ? av[c] : 0.0f;
            sd[ty][tx][6 + c] = in ? wv[c] : 0.0f;
        }
        __syncthreads();
        if (in && !(tx & 1) && !(ty & 1)) {
            const int ox = x >> 1, oy = y >> 1;  // < w / 2, h / 2
            // bilinear_px at (ox, oy): taps 2 ox, 2 ox + 1 and 2 oy, 2 oy + 1 (inside: w, h even)
            const float xx = static_cast<float>(ox) * static_cast<float>(w) / static_cast<float>(dn.ow);
            const float yy = static_cast<float>(oy) * static_cast<float>(h) / static_cast<float>(dn.oh);
            const float fx = xx - static_cast<float>(x), fy = yy - static_cast<float>(y);
            const int64_t q = (static_cast<int64_t>(oy) * dn.ow + ox) * 3;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const float v00 = sd[ty][tx][k], v10 = sd[ty][tx + 1][k];
                const float v01 = sd[ty + 1][tx][k], v11 = sd[ty + 1][tx + 1][k];
                const float v = v00 * (1 - fx) * (1 - fy) + v10 * fx * (1 - fy) + v01 * (1 - fx) * fy + v11 * fx * fy;
                float* dst = k < 3 ? dn.P : k < 6 ? dn.A : dn.W;
                dst[q + k % 3] = v;
            }
        }
    }
}

// ---- the fused front pass on RGBA8 frames ------------------------------------------
// For callers that hold the original and processed frames as RGBA8.  Every
// value of a converted frame is lut[byte] (the float(double(v)/255.0)
// conversion), so gathering the four bilinear taps of a frame as four
// 32-bit words and converting the bytes through the same table gives the
// same tap values, and therefore the same outputs bit for bit, as
// fused_front_kernel on the converted frames: 4 bytes per tap instead of 12
// (84 instead of 124 algorithmic bytes per pixel).  The last stabilized
// frame is a float image and is gathered as such.
struct RgbaTaps {
    uint32_t t00, t01, t10, t11;
};

__device__ __forceinline__ RgbaTaps rgba_taps(const uint32_t* __restrict__ img, const WarpTap& t)
{
    return RgbaTaps{img[t.q0], img[t.q0 + 1], img[t.q1], img[t.q1 + 1]};
}

__device__ __forceinline__ float rgba_sample(const float* lut, const RgbaTaps& q, const WarpTap& t, int c)
{
    const int sh = 8 * c;
    return bilerp(lut[(q.t00 >> sh) & 0xff], lut[(q.t01 >> sh) & 0xff], lut[(q.t10 >> sh) & 0xff],
        lut[(q.t11 >> sh) & 0xff], t.fx, t.fy);
}

template <bool kOcc>
__global__ void __launch_bounds__(256) fused_front_rgba_kernel(const uint32_t* __restrict__ o0,
    const uint32_t* __restrict__ o1, const uint32_t* __restrict__ o2, const uint32_t* __restrict__ p0,
    const uint32_t* __restrict__ p1, const uint32_t* __restrict__ p2, const float* __restrict__ ls,
    const float* __restrict__ ffwd, const float* __restrict__ fbwd, int fc, float* __restrict__ adap_pr,
    float* __restrict__ cons_wt, int w, int h, float alpha, float beta, float gamma)
{
    __shared__ float lut[256];
    build_lut(lut);
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h)
        return;
    const WarpTap tb = warp_tap(fbwd, fc, x, y, w, h);
    const WarpTap tf = warp_tap(ffwd, fc, x, y, w, h);
    float mp = 1.0f, mn = 1.0f;
    if (kOcc) {
        mp = occl_check(fbwd, ffwd, fc, x, y, w, h);
        mn = occl_check(ffwd, fbwd, fc, x, y, w, h);
    }
    const RgbaTaps qoi = rgba_taps(o0, tb), qop = rgba_taps(p0, tb);
    const RgbaTaps qni = rgba_taps(o2, tf), qnp = rgba_taps(p2, tf);
    const int64_t px = pix_index(x, y, w);
    const uint32_t ci8 = o1[px], cp8 = p1[px];
    const int64_t o = px * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float pwi = rgba_sample(lut, qoi, tb, c);
        const float pwp = rgba_sample(lut, qop, tb, c);
        const float nwi = rgba_sample(lut, qni, tf, c);
        const float nwp = rgba_sample(lut, qnp, tf, c);
        const float lsw = warp_sample(ls, tb, c);
        const float ci = lut[(ci8 >> (8 * c)) & 0xff];
        const float cp = lut[(cp8 >> (8 * c)) & 0xff];
        const Comb r = adap_comb_px(ci, cp, pwi, pwp, nwi, nwp, lsw, alpha, mp, mn, kOcc);
        adap_pr[o + c] = r.apr;
        cons_wt[o + c] = consist_wt_px(ci, r.ain, beta, gamma);
    }
}

inline dim3 grid2d(int w, int h, dim3 b) { return dim3((w + b.x - 1) / b.x, (h + b.y - 1) / b.y); }

}  // namespace

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

cudaError_t launch_rgba_to_float(const uint8_t* rgba, float* out, int64_t npix, cudaStream_t st)
{
    int64_t done = 0;
    if (aligned16(rgba) && aligned16(out) && npix >= 4) {
        const int64_t nq = npix / 4;
        const cudaError_t e = launch_pdl(rgba_to_float4_kernel, dim3(static_cast<unsigned>((nq + 255) / 256)),
            dim3(256), 0, st, reinterpret_cast<const uint4*>(rgba), reinterpret_cast<float4*>(out), nq);
        if (e != cudaSuccess)
            return e;
        done = nq * 4;
    }
    if (done < npix)
        rgba_to_float_kernel<<<static_cast<unsigned>((npix - done + 255) / 256), 256, 0, st>>>(rgba, out, done, npix);
    return cudaGetLastError();
}

cudaError_t launch_float_to_rgba(const float* in, uint8_t* rgba, int64_t npix, cudaStream_t st)
{
    int64_t done = 0;
    if (aligned16(rgba) && aligned16(in) && npix >= 4) {
        const int64_t nq = npix / 4;
        float4_to_rgba_kernel<<<static_cast<unsigned>((nq + 255) / 256), 256, 0, st>>>(
            reinterpret_cast<const float4*>(in), reinterpret_cast<uint4*>(rgba), nq);
        done = nq * 4;
    }
    if (done < npix)
        float_to_rgba_kernel<<<static_cast<unsigned>((npix - done + 255) / 256), 256, 0, st>>>(in, rgba, done, npix);
    return cudaGetLastError();
}

// every element offset of a w x h frame with c <= max(3, fc) channels fits an int
static bool offsets32(int w, int h, int fc)
{
    return static_cast<int64_t>(w) * h * std::max(3, fc) + 3 * static_cast<int64_t>(w) + 6 < (int64_t(1) << 31);
}

cudaError_t launch_stab_warp(Img in, Img flow, Img out, cudaStream_t st)
{
    const dim3 b(32, 8);
    const dim3 g = grid2d(out.w, out.h, dim3(32, 16));
    if (offsets32(out.w, out.h, flow.c))
        stab_warp_kernel<int><<<g, b, 0, st>>>(in.d, flow.d, flow.c, out.d, out.w, out.h);
    else
        stab_warp_kernel<int64_t><<<g, b, 0, st>>>(in.d, flow.d, flow.c, out.d, out.w, out.h);
    return cudaGetLastError();
}

cudaError_t launch_adap_comb(Img ci, Img cp, Img pwi, Img pwp, Img nwi, Img nwp, Img ai, Img ap, Img lsw, float alpha,
    cudaStream_t st, const float* occ_mask)
{
    const int64_t n = static_cast<int64_t>(ci.w) * ci.h * 3;
    adap_comb_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(
        ci.d, cp.d, pwi.d, pwp.d, nwi.d, nwp.d, ai.d, ap.d, lsw.d, occ_mask, alpha, n);
    return cudaGetLastError();
}

cudaError_t launch_flow_consistency(Img ffwd, Img fbwd, Img mask, cudaStream_t st)
{
    const dim3 b(32, 8);
    flow_consistency_kernel<<<grid2d(mask.w, mask.h, b), b, 0, st>>>(
        ffwd.d, fbwd.d, ffwd.c, mask.d, mask.w, mask.h);
    return cudaGetLastError();
}

cudaError_t launch_consist_wt(Img ai, Img ci, Img wt, float beta, float gamma, cudaStream_t st)
{
    const int64_t n = static_cast<int64_t>(ci.w) * ci.h * 3;
    // consist_wt_px's non-positive-exponent form: beta finite and >= 0, |gamma| <= 1e30
    const bool np = std::isfinite(beta) && beta >= 0.0f && std::fabs(gamma) <= 1e30f;
    int64_t done = 0;
    if (aligned16(ci.d) && aligned16(ai.d) && aligned16(wt.d) && n >= 4) {
        const int64_t nq = n / 4;
        const unsigned g = static_cast<unsigned>((nq + 255) / 256);
        auto q = [](const float* p) { return reinterpret_cast<const float4*>(p); };
        if (np)
            consist_wt4_kernel<true><<<g, 256, 0, st>>>(q(ci.d), q(ai.d), reinterpret_cast<float4*>(wt.d), beta,
                gamma, nq);
        else
            consist_wt4_kernel<false><<<g, 256, 0, st>>>(q(ci.d), q(ai.d), reinterpret_cast<float4*>(wt.d), beta,
                gamma, nq);
        done = nq * 4;
    }
    if (done < n) {
        const unsigned g = static_cast<unsigned>((n - done + 255) / 256);
        if (np)
            consist_wt_kernel<true><<<g, 256, 0, st>>>(ci.d, ai.d, wt.d, beta, gamma, done, n);
        else
            consist_wt_kernel<false><<<g, 256, 0, st>>>(ci.d, ai.d, wt.d, beta, gamma, done, n);
    }
    return cudaGetLastError();
}

cudaError_t launch_bilinear(Img in, Img out, cudaStream_t st)
{
    const dim3 b(32, 8);
    if (out.c == 2 || out.c == 3) {
        const dim3 g((out.w + 4 * b.x - 1) / (4 * b.x), (out.h + b.y - 1) / b.y);
        if (out.c == 3 && in.c == 3 && bilinear_is_2x(in.w, in.h, out.w, out.h))
            return launch_pdl(bilinear2x3_kernel, g, b, 0, st, in.d, in.w, in.h, out.d, out.w, out.h);
        if (out.c == 3)
            return launch_pdl(bilinear4_kernel<3>, g, b, 0, st, in.d, in.w, in.h, out.d, out.w, out.h);
        else
            return launch_pdl(bilinear4_kernel<2>, g, b, 0, st, in.d, in.w, in.h, out.d, out.w, out.h);
    } else {
        bilinear_kernel<<<grid2d(out.w, out.h, b), b, 0, st>>>(in.d, in.w, in.h, out.d, out.w, out.h, out.c);
    }
    return cudaGetLastError();
}

cudaError_t launch_bilinear_group(const Img* in, const Img* out, int n, cudaStream_t st)
{
    for (int b0 = 0; b0 < n; b0 += kBilinearGroupMax) {
        BilinearGroup g{};
        g.count = std::min(n - b0, kBilinearGroupMax);
        g.block0[0] = 0;
        for (int p = 0; p < g.count; ++p) {
            const Img& i = in[b0 + p];
            const Img& o = out[b0 + p];
            if (i.c != 3 || o.c != 3)
                return cudaErrorInvalidValue;
            g.in[p] = i.d;
            g.out[p] = o.d;
            g.iw[p] = i.w;
            g.ih[p] = i.h;
            g.ow[p] = o.w;
            g.oh[p] = o.h;
            g.two_x[p] = bilinear_is_2x(i.w, i.h, o.w, o.h) ? 1 : 0;
            g.bx[p] = (o.w + 127) / 128;
            g.block0[p + 1] = g.block0[p] + g.bx[p] * ((o.h + 7) / 8);
        }
        if (g.block0[g.count] > 0)
            bilinear4_group_kernel<<<g.block0[g.count], dim3(32, 8), 0, st>>>(g);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

cudaError_t launch_pyr_down3(const float* P, const float* A, const float* Wt, int iw, int ih, float* Pd, float* Ad,
    float* Wd, int ow, int oh, cudaStream_t st)
{
    const dim3 b(32, 8);
    const cudaError_t e = launch_pdl(pyr_down3_kernel, grid2d(ow, oh, b), b, 0, st, P, A, Wt, iw, ih, Pd, Ad, Wd, ow,
        oh);
    if (e != cudaSuccess)
        return e;
    return cudaGetLastError();
}

// fused_front_kernel's fast form applies (see there)
static bool front_fast_ok(int w, int h, int fc, float alpha, float beta, float gamma)
{
    return offsets32(w, h, fc) && std::isfinite(alpha) && alpha >= 0.0f && std::isfinite(beta) && beta >= 0.0f &&
           std::fabs(gamma) <= 1e30f;
}

bool front_down_fusable(int w, int h, int ow, int oh)
{
    return w % 2 == 0 && h % 2 == 0 && ow == w / 2 && oh == h / 2 && static_cast<int64_t>(ow) * w < (int64_t{1} << 24) &&
           static_cast<int64_t>(oh) * h < (int64_t{1} << 24);
}

cudaError_t launch_fused_front(const float* o0, const float* o1, const float* o2, const float* p0, const float* p1,
    const float* p2, const float* last_stab, const float* flow_fwd, const float* flow_bwd, int fc, float* adap_pr,
    float* cons_wt, int w, int h, float alpha, float beta, float gamma, cudaStream_t st, bool occlusion_mask, int fw,
    int fh, float* down_p, float* down_a, float* down_w, int ow, int oh)
{
    const dim3 b(32, 8);
    const bool half = fw > 0 && fh > 0;
    const bool down = down_p != nullptr;
    if ((half && (occlusion_mask || fc != 3)) || (down && (occlusion_mask || !front_down_fusable(w, h, ow, oh))))
        return cudaErrorInvalidValue;
    const bool fast = front_fast_ok(w, h, fc, alpha, beta, gamma);
    using K = decltype(&fused_front_kernel<false, false>);
    K k;
    if (occlusion_mask)
        k = fast ? fused_front_kernel<true, true> : fused_front_kernel<true, false>;
    else if (half)
        k = down ? (fast ? fused_front_kernel<false, true, true, true> : fused_front_kernel<false, false, true, true>)
                 : (fast ? fused_front_kernel<false, true, true> : fused_front_kernel<false, false, true>);
    else
        k = down ? (fast ? fused_front_kernel<false, true, false, true> : fused_front_kernel<false, false, false, true>)
                 : (fast ? fused_front_kernel<false, true> : fused_front_kernel<false, false>);
    const FrontDown dn{down_p, down_a, down_w, ow, oh};
    const cudaError_t el = launch_pdl(k, grid2d(w, h, b), b, 0, st, o0, o1, o2, p0, p1, p2, last_stab, flow_fwd,
        flow_bwd, fc, adap_pr, cons_wt, w, h, alpha, beta, gamma, fw, fh, dn);
    return el != cudaSuccess ? el : cudaGetLastError();
}

cudaError_t launch_fused_front_rgba(const uint8_t* o0, const uint8_t* o1, const uint8_t* o2, const uint8_t* p0,
    const uint8_t* p1, const uint8_t* p2, const float* last_stab, const float* flow_fwd, const float* flow_bwd, int fc,
    float* adap_pr, float* cons_wt, int w, int h, float alpha, float beta, float gamma, cudaStream_t st,
    bool occlusion_mask)
{
    const dim3 b(32, 8);
    auto u = [](const uint8_t* p) { return reinterpret_cast<const uint32_t*>(p); };
    if (occlusion_mask)
        fused_front_rgba_kernel<true><<<grid2d(w, h, b), b, 0, st>>>(u(o0), u(o1), u(o2), u(p0), u(p1), u(p2),
            last_stab, flow_fwd, flow_bwd, fc, adap_pr, cons_wt, w, h, alpha, beta, gamma);
    else
        fused_front_rgba_kernel<false><<<grid2d(w, h, b), b, 0, st>>>(u(o0), u(o1), u(o2), u(p0), u(p1), u(p2),
            last_stab, flow_fwd, flow_bwd, fc, adap_pr, cons_wt, w, h, alpha, beta, gamma);
    return cudaGetLastError();
}

}  // namespace vsc
