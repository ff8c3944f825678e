/*
 * vsc_oracle.c — CPU restatement of the reference's per-frame hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA library, never part of
 * it.  Build: oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp).
 *
 * Each function cites the reference function it restates (paths relative to
 * the reference project root).  Expressions keep the reference's literal
 * single-precision evaluation order; with contraction disabled every
 * intermediate is rounded to float exactly as written.  See vsc_oracle.h for
 * the two documented deviations (exp, and the Warp op's double-precision
 * weights) and for the Jacobi definition of the solver.
 */
#include "vsc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;

void vo_set_threads(int n)
{
    g_threads = n < 1 ? 1 : n;
#ifdef _OPENMP
    omp_set_num_threads(g_threads);
#endif
}

int vo_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------------
 * exp(x) for single precision: Cody & Waite range reduction x = k ln2 + r
 * (ln2 split into a 16-bit head and a tail, both applied with fused
 * multiply-add), exp(r) by the degree-7 Taylor polynomial in Horner form
 * (|r| <= ln2/2, truncation error < 1e-8 relative), then scaling by 2^k via
 * the exponent field.  Results below 2^-126 are flushed to zero.  The CUDA
 * library carries the same function, operation for operation, so both sides
 * produce identical bits.
 * ------------------------------------------------------------------------ */
float vo_expf(float x)
{
    if (x != x)
        return x;
    if (x > 88.72283f)
        return INFINITY;
    if (x < -87.33654f)
        return 0.0f;
    const float kf = rintf(x * 1.44269502f);
    float r = fmaf(kf, -0.693145751953125f, x);
    r = fmaf(kf, -1.42860682e-6f, r);
    float p = 1.98412701e-4f; /* 1/7! */
    p = fmaf(p, r, 1.38888892e-3f); /* 1/6! */
    p = fmaf(p, r, 8.33333377e-3f); /* 1/5! */
    p = fmaf(p, r, 4.16666679e-2f); /* 1/4! */
    p = fmaf(p, r, 1.66666672e-1f); /* 1/3! */
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    int k = (int)kf;
    if (k > 127) {
        p = p * 2.0f;
        k -= 1;
    }
    union {
        uint32_t u;
        float f;
    } s;
    s.u = (uint32_t)(k + 127) << 23;
    return p * s.f;
}

/* ------------------------------------------------------------------------
 * Correlation op, legacy = 0.
 * correlation.cc:203-275 (correlation_forward) with correlate_patch
 * (:147-182) for kernel 1x1, stride 1, no padding, patch (2md+1)^2:
 *   out[n][ph][pw][h][w] = sum_c f1[n][c][h][w] * f2[n][c][h+ph-md][w+pw-md]
 * summed in channel order in the element type, zero when the displaced
 * position is outside the map.
 * ------------------------------------------------------------------------ */
#define VO_CORR_BODY(T)                                                                                   \
    const int P = 2 * md + 1;                                                                             \
    const int64_t HW = (int64_t)H * W;                                                                    \
    for (int n = 0; n < N; ++n) {                                                                         \
        const T* a = f1 + (int64_t)n * C * HW;                                                            \
        const T* b = f2 + (int64_t)n * C * HW;                                                            \
        T* o = out + (int64_t)n * P * P * HW;                                                             \
        _Pragma("omp parallel for schedule(static)") for (int pp = 0; pp < P * P; ++pp)                   \
        {                                                                                                 \
            const int ph = pp / P, pw = pp % P;                                                           \
            const int su = ph - md, sv = pw - md;                                                         \
            for (int h = 0; h < H; ++h) {                                                                 \
                for (int w = 0; w < W; ++w) {                                                             \
                    T acc = 0;                                                                            \
                    const int h2 = h + su, w2 = w + sv;                                                   \
                    if (h2 >= 0 && h2 < H && w2 >= 0 && w2 < W) {                                         \
                        for (int c = 0; c < C; ++c) {                                                     \
                            const T v1 = a[(int64_t)c * HW + (int64_t)h * W + w];                         \
                            const T v2 = b[(int64_t)c * HW + (int64_t)h2 * W + w2];                       \
                            acc += v1 * v2;                                                               \
                        }                                                                                 \
                    }                                                                                     \
                    o[(int64_t)pp * HW + (int64_t)h * W + w] = acc;                                       \
                }                                                                                         \
            }                                                                                             \
        }                                                                                                 \
    }

void vo_correlation_f32(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md)
{
    VO_CORR_BODY(float)
}

void vo_correlation_f64(const double* f1, const double* f2, double* out, int N, int C, int H, int W, int md)
{
    VO_CORR_BODY(double)
}

/* Legacy (PWC-Net original) form, correlation_cuda.cu:182-265 and :393-397:
 * output N x (2md+1)^2 x H x W with top_channel = (dy+md)*(2md+1) + (dx+md),
 * each sum divided by C (kernel_size^2 * channels with kernel_size 1). */
void vo_correlation_legacy_f32(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md)
{
    vo_correlation_f32(f1, f2, out, N, C, H, W, md);
    const int P = 2 * md + 1;
    const int64_t total = (int64_t)N * P * P * H * W;
    const float fc = (float)C;
    for (int64_t i = 0; i < total; ++i)
        out[i] = out[i] / fc;
}

/* ------------------------------------------------------------------------
 * Warp op.  warp.cc:71-133: for every (n, c, y, x)
 *   xf = x + flow[n][0][y][x], yf = y + flow[n][1][y][x]
 *   bilinear weights of the four neighbours, taps outside the map count 0,
 *   mask = sum of the in-map weights; output = bilinear sum if mask > 0.999
 *   else 0.
 * vo_warp_op_refsem keeps the reference's precision exactly: in the float
 * instantiation the weight products are double ("1.0 - alpha" is a double
 * expression) and each "+=" rounds the double sum back to float.
 * ------------------------------------------------------------------------ */
void vo_warp_op_refsem(const float* in, const float* flow, float* out, int N, int C, int H, int W)
{
    const int64_t HW = (int64_t)H * W;
    for (int n = 0; n < N; ++n) {
        _Pragma("omp parallel for schedule(static)") for (int c = 0; c < C; ++c)
        {
            const float* src = in + ((int64_t)n * C + c) * HW;
            const float* fu = flow + (int64_t)n * 2 * HW;
            const float* fv = fu + HW;
            float* dst = out + ((int64_t)n * C + c) * HW;
            for (int y = 0; y < H; ++y) {
                for (int x = 0; x < W; ++x) {
                    const float xf = (float)x + fu[(int64_t)y * W + x];
                    const float yf = (float)y + fv[(int64_t)y * W + x];
                    const float alpha = xf - floorf(xf);
                    const float beta = yf - floorf(yf);
                    const float right_edge = (float)(W - 1);
                    const float bottom_edge = (float)(H - 1);
                    const float xL = floorf(xf);
                    const float xR = (float)((double)floorf(xf) + 1.0);
                    const float yT = floorf(yf);
                    const float yB = (float)((double)floorf(yf) + 1.0);
                    const int mL = (0 <= xL && xL <= right_edge) ? 1 : 0;
                    const int mR = (0 <= xR && xR <= right_edge) ? 1 : 0;
                    const int mT = (0 <= yT && yT <= bottom_edge) ? 1 : 0;
                    const int mB = (0 <= yB && yB <= bottom_edge) ? 1 : 0;
                    float val = 0.0f;
                    float mask = 0.0f;
                    mask = (float)((double)mask + (1.0 - alpha) * (1.0 - beta) * (mT + mL == 2 ? 1.0 : 0.0));
                    mask = (float)((double)mask + (alpha) * (1.0 - beta) * (mT + mR == 2 ? 1.0 : 0.0));
                    mask = (float)((double)mask + (1.0 - alpha) * (beta) * (mB + mL == 2 ? 1.0 : 0.0));
                    mask = (float)((double)mask + (alpha) * (beta) * (mB + mR == 2 ? 1.0 : 0.0));
                    if (mask > 0.999) {
                        val = (float)((double)val + (1.0 - alpha) * (1.0 - beta) *
                                                        (mT + mL == 2 ? (double)src[(int64_t)(int)yT * W + (int)xL] : 0.0));
                        val = (float)((double)val + (alpha) * (1.0 - beta) *
                                                        (mT + mR == 2 ? (double)src[(int64_t)(int)yT * W + (int)xR] : 0.0));
                        val = (float)((double)val + (1.0 - alpha) * (beta) *
                                                        (mB + mL == 2 ? (double)src[(int64_t)(int)yB * W + (int)xL] : 0.0));
                        val = (float)((double)val + (alpha) * (beta) *
                                                        (mB + mR == 2 ? (double)src[(int64_t)(int)yB * W + (int)xR] : 0.0));
                    }
                    dst[(int64_t)y * W + x] = val;
                }
            }
        }
    }
}

void vo_warp_op_f64(const double* in, const double* flow, double* out, int N, int C, int H, int W)
{
    const int64_t HW = (int64_t)H * W;
    for (int n = 0; n < N; ++n) {
        _Pragma("omp parallel for schedule(static)") for (int c = 0; c < C; ++c)
        {
            const double* src = in + ((int64_t)n * C + c) * HW;
            const double* fu = flow + (int64_t)n * 2 * HW;
            const double* fv = fu + HW;
            double* dst = out + ((int64_t)n * C + c) * HW;
            for (int y = 0; y < H; ++y) {
                for (int x = 0; x < W; ++x) {
                    const double xf = (double)x + fu[(int64_t)y * W + x];
                    const double yf = (double)y + fv[(int64_t)y * W + x];
                    const double alpha = xf - floor(xf);
                    const double beta = yf - floor(yf);
                    const double xL = floor(xf), xR = floor(xf) + 1.0;
                    const double yT = floor(yf), yB = floor(yf) + 1.0;
                    const int mL = (0 <= xL && xL <= (double)(W - 1)) ? 1 : 0;
                    const int mR = (0 <= xR && xR <= (double)(W - 1)) ? 1 : 0;
                    const int mT = (0 <= yT && yT <= (double)(H - 1)) ? 1 : 0;
                    const int mB = (0 <= yB && yB <= (double)(H - 1)) ? 1 : 0;
                    double val = 0.0, mask = 0.0;
                    mask += (1.0 - alpha) * (1.0 - beta) * (mT + mL == 2 ? 1.0 : 0.0);
                    mask += (alpha) * (1.0 - beta) * (mT + mR == 2 ? 1.0 : 0.0);
                    mask += (1.0 - alpha) * (beta) * (mB + mL == 2 ? 1.0 : 0.0);
                    mask += (alpha) * (beta) * (mB + mR == 2 ? 1.0 : 0.0);
                    if (mask > 0.999) {
                        val += (1.0 - alpha) * (1.0 - beta) * (mT + mL == 2 ? src[(int64_t)(int)yT * W + (int)xL] : 0.0);
                        val += (alpha) * (1.0 - beta) * (mT + mR == 2 ? src[(int64_t)(int)yT * W + (int)xR] : 0.0);
                        val += (1.0 - alpha) * (beta) * (mB + mL == 2 ? src[(int64_t)(int)yB * W + (int)xL] : 0.0);
                        val += (alpha) * (beta) * (mB + mR == 2 ? src[(int64_t)(int)yB * W + (int)xR] : 0.0);
                    }
                    dst[(int64_t)y * W + x] = val;
                }
            }
        }
    }
}

/* The Warp op in single precision, the arithmetic the CUDA kernel performs:
 * same taps, masks and threshold as warp.cc:85-129, with the four weights
 * w_TL=(1-a)(1-b), w_TR=a(1-b), w_BL=(1-a)b, w_BR=ab rounded to float and
 * both sums accumulated in float in the reference's tap order. */
void vo_warp_op_f32(const float* in, const float* flow, float* out, int N, int C, int H, int W)
{
    const int64_t HW = (int64_t)H * W;
    for (int n = 0; n < N; ++n) {
        _Pragma("omp parallel for schedule(static)") for (int y = 0; y < H; ++y)
        {
            const float* fu = flow + (int64_t)n * 2 * HW;
            const float* fv = fu + HW;
            for (int x = 0; x < W; ++x) {
                const float xf = (float)x + fu[(int64_t)y * W + x];
                const float yf = (float)y + fv[(int64_t)y * W + x];
                const float fxl = floorf(xf), fyt = floorf(yf);
                const float a = xf - fxl, b = yf - fyt;
                const float xR = fxl + 1.0f, yB = fyt + 1.0f;
                const int mL = (0.0f <= fxl && fxl <= (float)(W - 1));
                const int mR = (0.0f <= xR && xR <= (float)(W - 1));
                const int mT = (0.0f <= fyt && fyt <= (float)(H - 1));
                const int mB = (0.0f <= yB && yB <= (float)(H - 1));
                const float ia = 1.0f - a, ib = 1.0f - b;
                const float wTL = ia * ib, wTR = a * ib, wBL = ia * b, wBR = a * b;
                const int tl = mT && mL, tr = mT && mR, bl = mB && mL, br = mB && mR;
                float mask = 0.0f;
                mask += tl ? wTL : 0.0f;
                mask += tr ? wTR : 0.0f;
                mask += bl ? wBL : 0.0f;
                mask += br ? wBR : 0.0f;
                const int take = mask > 0.999f;
                const int xl = (int)fxl, yt = (int)fyt;
                for (int c = 0; c < C; ++c) {
                    const float* src = in + ((int64_t)n * C + c) * HW;
                    float val = 0.0f;
                    if (take) {
                        val += tl ? wTL * src[(int64_t)yt * W + xl] : 0.0f;
                        val += tr ? wTR * src[(int64_t)yt * W + xl + 1] : 0.0f;
                        val += bl ? wBL * src[(int64_t)(yt + 1) * W + xl] : 0.0f;
                        val += br ? wBR * src[(int64_t)(yt + 1) * W + xl + 1] : 0.0f;
                    }
                    out[((int64_t)n * C + c) * HW + (int64_t)y * W + x] = val;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------
 * Frame I/O, gpuimage.cu.
 * ------------------------------------------------------------------------ */
/* kernel_to_float_image, :39-51: out = float(double(v) / 255.0); alpha unused. */
void vo_rgba_to_float(const uint8_t* rgba, float* out, int64_t npix)
{
    float lut[256];
    for (int v = 0; v < 256; ++v)
        lut[v] = (float)((double)v / 255.0);
    for (int64_t i = 0; i < npix; ++i)
        for (int c = 0; c < 3; ++c)
            out[i * 3 + c] = lut[rgba[i * 4 + c]];
}

/* kernel_to_char_image, :54-67: (uchar)__float2uint_rd(fabs(v) * 255), A = 1.
 * __float2uint_rd rounds toward -inf and saturates (NaN -> 0); the cast to
 * unsigned char keeps the low 8 bits, so 256/255 and above wrap. */
static inline uint8_t vo_quant(float v)
{
    const float f = fabsf(v) * 255.0f;
    uint32_t u;
    if (f != f)
        u = 0;
    else if (f >= 4294967296.0f)
        u = 0xFFFFFFFFu;
    else
        u = (uint32_t)floorf(f);
    return (uint8_t)u;
}

void vo_float_to_rgba(const float* in, uint8_t* rgba, int64_t npix)
{
    for (int64_t i = 0; i < npix; ++i) {
        for (int c = 0; c < 3; ++c)
            rgba[i * 4 + c] = vo_quant(in[i * 3 + c]);
        rgba[i * 4 + 3] = 1;
    }
}

/* ------------------------------------------------------------------------
 * Stabilization kernels, flowconsistency.cu.
 * ------------------------------------------------------------------------ */
/* kernel_warp, :77-114: sample position clamped to [0, w-3] x [0, h-3],
 * bilinear between floor and floor+1. */
void vo_stab_warp(const float* in, const float* flow, int fc, float* out, int w, int h)
{
    _Pragma("omp parallel for schedule(static)") for (int y = 0; y < h; ++y)
    {
        for (int x = 0; x < w; ++x) {
            const int64_t fi = ((int64_t)y * w + x) * fc;
            const float flo_x = flow[fi + 0];
            const float flo_y = flow[fi + 1];
            const float map_fx = fmaxf(0.0f, fminf((float)x + flo_x, (float)(w - 3)));
            const float map_fy = fmaxf(0.0f, fminf((float)y + flo_y, (float)(h - 3)));
            const int map_ix = (int)floorf(map_fx);
            const int map_iy = (int)floorf(map_fy);
            const float flo_fx = map_fx - (float)map_ix;
            const float flo_fy = map_fy - (float)map_iy;
            const float* r0 = in + ((int64_t)map_iy * w + map_ix) * 3;
            const float* r1 = in + ((int64_t)(map_iy + 1) * w + map_ix) * 3;
            for (int c = 0; c < 3; ++c) {
                const float tmp_1 = r0[c] * (1.0f - flo_fx) + r0[3 + c] * flo_fx;
                const float tmp_2 = r1[c] * (1.0f - flo_fx) + r1[3 + c] * flo_fx;
                out[((int64_t)y * w + x) * 3 + c] = tmp_1 * (1.0f - flo_fy) + tmp_2 * flo_fy;
            }
        }
    }
}

/* kernel_adap_comb, :116-166. */
void vo_adap_comb(const float* crnt_in, const float* crnt_pr, const float* prev_warp_in, const float* prev_warp_pr,
    const float* next_warp_in, const float* next_warp_pr, float* adap_in, float* adap_pr, const float* last_stab_warp,
    float alpha, int64_t npix)
{
    vo_adap_comb_masked(crnt_in, crnt_pr, prev_warp_in, prev_warp_pr, next_warp_in, next_warp_pr, adap_in, adap_pr,
        last_stab_warp, NULL, alpha, npix);
}

/* Forward-backward flow consistency (not in the reference; an opt-in
 * extension).  For flow a at pixel (x, y), sample the opposite flow b at the
 * point a carries the pixel to, p = (x + a.x, y + a.y) (bilinear, right and
 * bottom taps clamped to the last column/row); the pixel is consistent if
 * |a + b(p)|^2 <= 0.01 (|a|^2 + |b(p)|^2) + 0.5, the usual occlusion test
 * of forward-backward checks.  Pixels carried outside the frame, and NaN
 * flows, are inconsistent.  Returns 1 or 0. */
static float occl_check(const float* a, const float* b, int fc, int x, int y, int w, int h)
{
    const int64_t i = ((int64_t)y * w + x) * fc;
    const float ax = a[i], ay = a[i + 1];
    const float px = (float)x + ax;
    const float py = (float)y + ay;
    if (!(px >= 0.0f && px <= (float)(w - 1) && py >= 0.0f && py <= (float)(h - 1)))
        return 0.0f;
    const int ix = (int)floorf(px);
    const int iy = (int)floorf(py);
    const float fx = px - (float)ix;
    const float fy = py - (float)iy;
    const int ix1 = ix + 1 < w - 1 ? ix + 1 : w - 1;
    const int iy1 = iy + 1 < h - 1 ? iy + 1 : h - 1;
    float bv[2];
    for (int k = 0; k < 2; ++k) {
        const float b00 = b[((int64_t)iy * w + ix) * fc + k];
        const float b10 = b[((int64_t)iy * w + ix1) * fc + k];
        const float b01 = b[((int64_t)iy1 * w + ix) * fc + k];
        const float b11 = b[((int64_t)iy1 * w + ix1) * fc + k];
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

void vo_flow_consistency_mask(const float* flow_fwd, const float* flow_bwd, int fc, float* mask, int w, int h)
{
    _Pragma("omp parallel for schedule(static)") for (int y = 0; y < h; ++y)
    {
        for (int x = 0; x < w; ++x) {
            float* m = mask + ((int64_t)y * w + x) * 2;
            m[0] = occl_check(flow_bwd, flow_fwd, fc, x, y, w, h);
            m[1] = occl_check(flow_fwd, flow_bwd, fc, x, y, w, h);
        }
    }
}

/* kernel_adap_comb with the two temporal weights multiplied by a per-pixel
 * mask after their clamps (mask ch0 -> previous frame, ch1 -> next frame);
 * a NULL mask, or a mask of ones, gives kernel_adap_comb's bits. */
void vo_adap_comb_masked(const float* crnt_in, const float* crnt_pr, const float* prev_warp_in,
    const float* prev_warp_pr, const float* next_warp_in, const float* next_warp_pr, float* adap_in, float* adap_pr,
    const float* last_stab_warp, const float* occ_mask, float alpha, int64_t npix)
{
    _Pragma("omp parallel for schedule(static)") for (int64_t i = 0; i < npix * 3; ++i)
    {
        const float ci = crnt_in[i], pi = prev_warp_in[i], ni = next_warp_in[i];
        const float cp = crnt_pr[i], pp = prev_warp_pr[i], np = next_warp_pr[i];
        const float ls = last_stab_warp[i];
        float wt_prv = vo_expf(-alpha * (ci - pi) * (ci - pi));
        float wt_nxt = vo_expf(-alpha * (ci - ni) * (ci - ni));
        if (wt_prv > 0.45f)
            wt_prv = 0.45f;
        if (wt_nxt > 0.3f)
            wt_nxt = 0.3f;
        if (wt_prv < 0.001f)
            wt_prv = 0.0f;
        if (wt_nxt < 0.001f)
            wt_nxt = 0.0f;
        if (occ_mask) {
            wt_prv = wt_prv * occ_mask[(i / 3) * 2];
            wt_nxt = wt_nxt * occ_mask[(i / 3) * 2 + 1];
        }
        const float ain = wt_prv * pi + wt_nxt * ni + (1.0f - (wt_prv + wt_nxt)) * ci;
        float apr = wt_prv * pp + wt_nxt * np + (1.0f - (wt_prv + wt_nxt)) * cp;
        apr = wt_prv * ls + (1.0f - wt_prv) * apr;
        adap_in[i] = ain;
        adap_pr[i] = apr;
    }
}

/* kernel_consist_wt, :168-191. */
void vo_consist_wt(const float* crnt_in, const float* adap_in, float* cons_wt, float beta, float gamma, int64_t npix)
{
    _Pragma("omp parallel for schedule(static)") for (int64_t i = 0; i < npix * 3; ++i)
    {
        const float c = crnt_in[i], a = adap_in[i];
        float wt = gamma * vo_expf(-beta * (c - a) * (c - a));
        if (wt < 0.001f)
            wt = 0.0f;
        cons_wt[i] = wt;
    }
}

/* kernel_bilinear, :50-75: xx = ox * Win / Wout (no half-pixel offset),
 * right/bottom taps clamped to the last row/column. */
void vo_bilinear(const float* in, int iw, int ih, float* out, int ow, int oh, int c)
{
    _Pragma("omp parallel for schedule(static)") for (int oy = 0; oy < oh; ++oy)
    {
        for (int ox = 0; ox < ow; ++ox) {
            const float xx = (float)ox * (float)iw / (float)ow;
            const float yy = (float)oy * (float)ih / (float)oh;
            int ix = (int)floorf(xx);
            int iy = (int)floorf(yy);
            ix = ix < iw - 1 ? ix : iw - 1; /* index guard; xx < iw for all sizes used */
            iy = iy < ih - 1 ? iy : ih - 1;
            const float fx = xx - (float)ix;
            const float fy = yy - (float)iy;
            const int ix1 = ix + 1 < iw - 1 ? ix + 1 : iw - 1;
            const int iy1 = iy + 1 < ih - 1 ? iy + 1 : ih - 1;
            for (int k = 0; k < c; ++k) {
                const float v00 = in[((int64_t)iy * iw + ix) * c + k];
                const float v10 = in[((int64_t)iy * iw + ix1) * c + k];
                const float v01 = in[((int64_t)iy1 * iw + ix) * c + k];
                const float v11 = in[((int64_t)iy1 * iw + ix1) * c + k];
                out[((int64_t)oy * ow + ox) * c + k] =
                    v00 * (1 - fx) * (1 - fy) + v10 * fx * (1 - fy) + v01 * (1 - fx) * fy + v11 * fx * fy;
            }
        }
    }
}

/* kernel_consist_out, :193-258, iterated numIter times (:367-372), as a
 * Jacobi iteration.  Per pixel and channel:
 *   lap_X = sum of valid neighbours - cnt * X, with the right neighbour valid
 *           iff x+1 < w-1, left iff x-1 >= 0, bottom iff y+1 < h-1, top iff
 *           y-1 >= 0, added in the order right, left, bottom, top;
 *   g = (lap_O - lap_P) - wt * (O - A);
 *   O' = O + s*g (+ m*U for k > 0);  U' = s*g. */
void vo_consist_out(const float* P, const float* A, const float* wt, int num_iter, float step, float mom, float* O,
    int w, int h)
{
    const int64_t n = (int64_t)w * h * 3;
    float* U = (float*)calloc((size_t)n, sizeof(float));
    float* O2 = (float*)malloc((size_t)n * sizeof(float));
    float* cur = O;
    float* nxt = O2;
    for (int k = 0; k < num_iter; ++k) {
        _Pragma("omp parallel for schedule(static)") for (int y = 0; y < h; ++y)
        {
            for (int x = 0; x < w; ++x) {
                const int64_t p = (int64_t)y * w + x;
                for (int c = 0; c < 3; ++c) {
                    const int64_t i = p * 3 + c;
                    int cnt = 0;
                    float lap_pr = 0.0f, lap_out = 0.0f;
                    if ((x + 1) < (w - 1)) {
                        lap_pr += P[i + 3];
                        lap_out += cur[i + 3];
                        cnt += 1;
                    }
                    if ((x - 1) >= 0) {
                        lap_pr += P[i - 3];
                        lap_out += cur[i - 3];
                        cnt += 1;
                    }
                    if ((y + 1) < (h - 1)) {
                        lap_pr += P[i + (int64_t)w * 3];
                        lap_out += cur[i + (int64_t)w * 3];
                        cnt += 1;
                    }
                    if ((y - 1) >= 0) {
                        lap_pr += P[i - (int64_t)w * 3];
                        lap_out += cur[i - (int64_t)w * 3];
                        cnt += 1;
                    }
                    lap_pr -= (float)cnt * P[i];
                    lap_out -= (float)cnt * cur[i];
                    const float wt_val = wt[i];
                    const float tmp_1 = wt_val * (cur[i] - A[i]);
                    const float tmp_2 = lap_out - lap_pr;
                    const float grad_val = tmp_2 - tmp_1;
                    float out_val;
                    if (k)
                        out_val = cur[i] + step * grad_val + mom * U[i];
                    else
                        out_val = cur[i] + step * grad_val;
                    U[i] = step * grad_val;
                    nxt[i] = out_val;
                }
            }
        }
        float* t = cur;
        cur = nxt;
        nxt = t;
    }
    if (cur != O)
        memcpy(O, cur, (size_t)n * sizeof(float));
    free(U);
    free(O2);
}

/* The library's FMA form of the same Jacobi iteration (vsc_get_consist_out_fma),
 * restated for its parity tests.  kernel_consist_out's step (:193-258),
 *   g = (lap_O - lap_P) - wt * (O - A),  O' = O + s*g (+ m*U),  U' = s*g,
 * is regrouped around two per-pixel constants computed once per solve,
 *   Cs = s * fma(wt, A, -lap_P)   (lap_P as in vo_consist_out),
 *   nK = -(s * (cnt + wt)),
 * and one step reads, with invalid neighbours as +0,
 *   S = (left + right) + (up + down),
 *   g = fma(nK, O, fma(s, S, Cs)),  O' = O + g, then fma(m, U, O') for k > 0,  U' = g.
 * Algebraically the reference's step; rounded differently (fused products,
 * another summation order), so it agrees with vo_consist_out within a
 * tolerance and with the library's FMA kernels bit for bit. */
void vo_consist_out_fma(const float* P, const float* A, const float* wt, int num_iter, float step, float mom, float* O,
    int w, int h)
{
    const int64_t n = (int64_t)w * h * 3;
    const int64_t rs = (int64_t)w * 3;
    float* U = (float*)calloc((size_t)n, sizeof(float));
    float* O2 = (float*)malloc((size_t)n * sizeof(float));
    float* Cs = (float*)malloc((size_t)n * sizeof(float));
    float* nK = (float*)malloc((size_t)n * sizeof(float));
    _Pragma("omp parallel for schedule(static)") for (int y = 0; y < h; ++y)
    {
        for (int x = 0; x < w; ++x) {
            const int64_t p = (int64_t)y * w + x;
            for (int c = 0; c < 3; ++c) {
                const int64_t i = p * 3 + c;
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
                lap -= (float)cnt * P[i];
                Cs[i] = step * fmaf(wt[i], A[i], -lap);
                nK[i] = -(step * ((float)cnt + wt[i]));
            }
        }
    }
    float* cur = O;
    float* nxt = O2;
    for (int k = 0; k < num_iter; ++k) {
        _Pragma("omp parallel for schedule(static)") for (int y = 0; y < h; ++y)
        {
            for (int x = 0; x < w; ++x) {
                const int64_t p = (int64_t)y * w + x;
                for (int c = 0; c < 3; ++c) {
                    const int64_t i = p * 3 + c;
                    const float right = (x + 1) < (w - 1) ? cur[i + 3] : 0.0f;
                    const float left = (x - 1) >= 0 ? cur[i - 3] : 0.0f;
                    const float down = (y + 1) < (h - 1) ? cur[i + rs] : 0.0f;
                    const float up = (y - 1) >= 0 ? cur[i - rs] : 0.0f;
                    const float S = (left + right) + (up + down);
                    const float g = fmaf(nK[i], cur[i], fmaf(step, S, Cs[i]));
                    float o = cur[i] + g;
                    if (k)
                        o = fmaf(mom, U[i], o);
                    U[i] = g;
                    nxt[i] = o;
                }
            }
        }
        float* t = cur;
        cur = nxt;
        nxt = t;
    }
    if (cur != O)
        memcpy(O, cur, (size_t)n * sizeof(float));
    free(U);
    free(O2);
    free(Cs);
    free(nK);
}

/* videostabilizer.cpp:104-112 */
void vo_default_hyper(vo_hyper* hp)
{
    hp->alpha = 6800.0f;
    hp->beta = 6800.0f;
    hp->gamma = 2.0f;
    hp->pyramid_levels = 2;
    hp->num_iter = 150;
    hp->step_size = 0.15f;
    hp->mom_fac = 0.15f;
}

/* VideoStabilizer::doOneStep, videostabilizer.cpp:181-247: five warps, the
 * adaptive combination, the consistency weights, the multi-scale solve with
 * pyramid sizes w/2^j (integer halving, :118-128), numIter/(j+1) iterations
 * on level j (:226), solution initialised with the processed frame (:209)
 * and carried down/up with kernel_bilinear (:212-223). */
int vo_stab_pass(int w, int h, const float* const orig[3], const float* const proc[3], const float* flow_fwd,
    const float* flow_bwd, int fc, const float* last_stab, const vo_hyper* hp, float* out_f32, uint8_t* out_rgba)
{
    return vo_stab_pass_ex(w, h, orig, proc, flow_fwd, flow_bwd, fc, last_stab, hp, 0, out_f32, out_rgba);
}

int vo_stab_pass_ex(int w, int h, const float* const orig[3], const float* const proc[3], const float* flow_fwd,
    const float* flow_bwd, int fc, const float* last_stab, const vo_hyper* hp, int occlusion_mask, float* out_f32,
    uint8_t* out_rgba)
{
    return vo_stab_pass_form(w, h, orig, proc, flow_fwd, flow_bwd, fc, last_stab, hp, occlusion_mask, 0, out_f32,
        out_rgba);
}

int vo_stab_pass_form(int w, int h, const float* const orig[3], const float* const proc[3], const float* flow_fwd,
    const float* flow_bwd, int fc, const float* last_stab, const vo_hyper* hp, int occlusion_mask, int solver_form,
    float* out_f32, uint8_t* out_rgba)
{
    const int L = hp->pyramid_levels;
    if (L < 1 || L > 8 || (w >> (L - 1)) < 2 || (h >> (L - 1)) < 2)
        return -1;
    const int64_t npix = (int64_t)w * h;
    const size_t bytes = (size_t)npix * 3 * sizeof(float);
    float* prev_in = (float*)malloc(bytes);
    float* prev_pr = (float*)malloc(bytes);
    float* next_in = (float*)malloc(bytes);
    float* next_pr = (float*)malloc(bytes);
    float* last_w = (float*)malloc(bytes);
    float* adap_in = (float*)malloc(bytes);
    float* adap_pr = (float*)malloc(bytes);
    float* cons_wt = (float*)malloc(bytes);
    vo_stab_warp(orig[0], flow_bwd, fc, prev_in, w, h);
    vo_stab_warp(proc[0], flow_bwd, fc, prev_pr, w, h);
    vo_stab_warp(orig[2], flow_fwd, fc, next_in, w, h);
    vo_stab_warp(proc[2], flow_fwd, fc, next_pr, w, h);
    vo_stab_warp(last_stab, flow_bwd, fc, last_w, w, h);
    float* occ = NULL;
    if (occlusion_mask) {
        occ = (float*)malloc((size_t)npix * 2 * sizeof(float));
        vo_flow_consistency_mask(flow_fwd, flow_bwd, fc, occ, w, h);
    }
    vo_adap_comb_masked(orig[1], proc[1], prev_in, prev_pr, next_in, next_pr, adap_in, adap_pr, last_w, occ, hp->alpha,
        npix);
    free(occ);
    vo_consist_wt(orig[1], adap_in, cons_wt, hp->beta, hp->gamma, npix);

    float* pP[8];
    float* pA[8];
    float* pW[8];
    float* pO[8];
    int lw[8], lh[8];
    lw[0] = w;
    lh[0] = h;
    for (int j = 1; j < L; ++j) {
        lw[j] = lw[j - 1] / 2;
        lh[j] = lh[j - 1] / 2;
    }
    for (int j = 0; j < L; ++j) {
        const size_t b = (size_t)lw[j] * lh[j] * 3 * sizeof(float);
        pP[j] = (float*)malloc(b);
        pA[j] = (float*)malloc(b);
        pW[j] = (float*)malloc(b);
        pO[j] = (float*)malloc(b);
        if (j == 0) {
            memcpy(pP[0], proc[1], b);
            memcpy(pA[0], adap_pr, b);
            memcpy(pW[0], cons_wt, b);
            memcpy(pO[0], proc[1], b);
        } else {
            vo_bilinear(pP[j - 1], lw[j - 1], lh[j - 1], pP[j], lw[j], lh[j], 3);
            vo_bilinear(pA[j - 1], lw[j - 1], lh[j - 1], pA[j], lw[j], lh[j], 3);
            vo_bilinear(pW[j - 1], lw[j - 1], lh[j - 1], pW[j], lw[j], lh[j], 3);
            vo_bilinear(pO[j - 1], lw[j - 1], lh[j - 1], pO[j], lw[j], lh[j], 3);
        }
    }
    for (int j = L - 1; j >= 0; --j) {
        if (j != L - 1)
            vo_bilinear(pO[j + 1], lw[j + 1], lh[j + 1], pO[j], lw[j], lh[j], 3);
        (solver_form ? vo_consist_out_fma : vo_consist_out)(pP[j], pA[j], pW[j], hp->num_iter / (j + 1),
            hp->step_size, hp->mom_fac, pO[j], lw[j], lh[j]);
    }
    memcpy(out_f32, pO[0], bytes);
    if (out_rgba)
        vo_float_to_rgba(out_f32, out_rgba, npix);
    for (int j = 0; j < L; ++j) {
        free(pP[j]);
        free(pA[j]);
        free(pW[j]);
        free(pO[j]);
    }
    free(prev_in);
    free(prev_pr);
    free(next_in);
    free(next_pr);
    free(last_w);
    free(adap_in);
    free(adap_pr);
    free(cons_wt);
    return 0;
}

/* ------------------------------------------------------------------------
 * Weight-free flow estimator (stand-in for the PWC-Net graph, whose weights
 * are not available).  The PWC-Net it replaces (model-conversion/
 * pwc_pytorch/pwcnet.py:418-430, :950-967) runs, per level from 1/64 to
 * 1/4 of the 64-aligned frame (convert_onnx.py:15-20): upsample the coarser
 * flow, custom::Warp the second frame's features by it, custom::Correlation
 * (max_displacement 4) against the first frame's features, decode a flow
 * refinement.  Here the learned parts are replaced by:
 *   features  : L2-normalised random projections of 3x3x3 RGB patches (each
 *               colour channel's nine values made zero-mean) onto the PWC
 *               channel counts {32,64,96,128,196} (weights from a fixed
 *               splitmix64 stream, seeded per level), so a correlation is a
 *               normalised cross-correlation of patches;
 *   decoder   : arg-max over the 81 correlations minus a small-displacement
 *               prior, refined by a soft centroid (weights exp(20*(s-smax))
 *               of the prior-adjusted scores) over its 3x3 neighbourhood;
 *               confidence = the peak's margin over the mean correlation;
 *   smoothing : confidence-weighted 3x3 mean of each level's refinement,
 *               added to the upsampled coarser flow.
 * The prior grows 4x per level because a coarse-level pixel spans more
 * motion: {0.01, 0.04, 0.16, 0.64, 2.56} for 1/4 .. 1/64.
 * ------------------------------------------------------------------------ */
#define VO_TEMP 20.0f
#define VO_EPS 0.1f
static const int vo_level_channels[VO_FLOW_LEVELS] = {32, 64, 96, 128, 196};
static const float vo_level_prior[VO_FLOW_LEVELS] = {0.01f, 0.01f * 4.0f, 0.01f * 16.0f, 0.01f * 64.0f, 0.01f * 256.0f};

int vo_flow_level_dims(int w, int h, int level, int* lw, int* lh, int* lc)
{
    if (level < 0 || level >= VO_FLOW_LEVELS)
        return -1;
    const int pw = ((w + 63) / 64) * 64;
    const int ph = ((h + 63) / 64) * 64;
    *lw = pw >> (level + 2);
    *lh = ph >> (level + 2);
    *lc = vo_level_channels[level];
    return 0;
}

size_t vo_flow_feature_floats(int w, int h)
{
    size_t n = 0;
    for (int l = 0; l < VO_FLOW_LEVELS; ++l) {
        int lw, lh, lc;
        vo_flow_level_dims(w, h, l, &lw, &lh, &lc);
        n += (size_t)lw * lh * lc;
    }
    return n;
}

static uint64_t vo_splitmix64(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

void vo_flow_weights(int level, float* wts)
{
    uint64_t s = 0x5653432D464C4F57ULL ^ ((uint64_t)(level + 1) * 0x9E3779B97F4A7C15ULL);
    const int n = vo_level_channels[level] * 27;
    for (int i = 0; i < n; ++i) {
        const uint64_t z = vo_splitmix64(&s);
        wts[i] = (float)(uint32_t)(z >> 40) * (1.0f / 8388608.0f) - 1.0f;
    }
}

/* bilinear sample with half-pixel centres (align_corners = False) of an
 * interleaved image with c channels at source coordinate (sx, sy) */
static inline void vo_sample_hp(const float* src, int sw, int sh, int c, float sx, float sy, float* res)
{
    if (sx < 0.0f)
        sx = 0.0f;
    if (sy < 0.0f)
        sy = 0.0f;
    int x0 = (int)floorf(sx), y0 = (int)floorf(sy);
    if (x0 > sw - 1)
        x0 = sw - 1;
    if (y0 > sh - 1)
        y0 = sh - 1;
    const int x1 = x0 + 1 < sw ? x0 + 1 : sw - 1;
    const int y1 = y0 + 1 < sh ? y0 + 1 : sh - 1;
    const float lx = sx - (float)x0, ly = sy - (float)y0;
    for (int k = 0; k < c; ++k) {
        const float v00 = src[((int64_t)y0 * sw + x0) * c + k];
        const float v01 = src[((int64_t)y0 * sw + x1) * c + k];
        const float v10 = src[((int64_t)y1 * sw + x0) * c + k];
        const float v11 = src[((int64_t)y1 * sw + x1) * c + k];
        const float top = (1.0f - lx) * v00 + lx * v01;
        const float bot = (1.0f - lx) * v10 + lx * v11;
        res[k] = (1.0f - ly) * top + ly * bot;
    }
}

/* level-0 (1/4) image: 4x4 box mean of the frame resized (bilinear,
 * half-pixel centres) to the 64-aligned size; coarser levels: 2x2 means. */
static void vo_flow_images(const float* img, int w, int h, float* lev[VO_FLOW_LEVELS])
{
    int lw, lh, lc;
    vo_flow_level_dims(w, h, 0, &lw, &lh, &lc);
    const int pw = lw * 4, ph = lh * 4;
    const float scx = (float)w / (float)pw, scy = (float)h / (float)ph;
    _Pragma("omp parallel for schedule(static)") for (int y = 0; y < lh; ++y)
    {
        for (int x = 0; x < lw; ++x) {
            float acc[3] = {0.0f, 0.0f, 0.0f};
            for (int j = 0; j < 4; ++j) {
                const float sy = ((float)(y * 4 + j) + 0.5f) * scy - 0.5f;
                for (int i = 0; i < 4; ++i) {
                    const float sx = ((float)(x * 4 + i) + 0.5f) * scx - 0.5f;
                    float v[3];
                    vo_sample_hp(img, w, h, 3, sx, sy, v);
                    acc[0] += v[0];
                    acc[1] += v[1];
                    acc[2] += v[2];
                }
            }
            for (int k = 0; k < 3; ++k)
                lev[0][((int64_t)y * lw + x) * 3 + k] = acc[k] * 0.0625f;
        }
    }
    for (int l = 1; l < VO_FLOW_LEVELS; ++l) {
        int cw, chh, cc;
        vo_flow_level_dims(w, h, l, &cw, &chh, &cc);
        const int fw = cw * 2;
        const float* s = lev[l - 1];
        for (int y = 0; y < chh; ++y)
            for (int x = 0; x < cw; ++x)
                for (int k = 0; k < 3; ++k) {
                    const float a = s[((int64_t)(2 * y) * fw + 2 * x) * 3 + k];
                    const float b = s[((int64_t)(2 * y) * fw + 2 * x + 1) * 3 + k];
                    const float c = s[((int64_t)(2 * y + 1) * fw + 2 * x) * 3 + k];
                    const float d = s[((int64_t)(2 * y + 1) * fw + 2 * x + 1) * 3 + k];
                    lev[l][((int64_t)y * cw + x) * 3 + k] = ((a + b) + (c + d)) * 0.25f;
                }
    }
}

/* features of one level: f_c = sum_k W[c][k] * p_k over the 27 patch values
 * p_k = I[clamp(y+ky)][clamp(x+kx)][ch] - 0.5 (k = ((ky+1)*3 + kx+1)*3 + ch),
 * then f_c / sqrt(sum_c f_c^2 + 1e-12); output planar C x lh x lw. */
static void vo_level_features(const float* im, int lw, int lh, int lc, const float* wts, float* out)
{
    const int64_t plane = (int64_t)lw * lh;
    _Pragma("omp parallel for schedule(static)") for (int y = 0; y < lh; ++y)
    {
        for (int x = 0; x < lw; ++x) {
            float p[27];
            for (int ky = -1; ky <= 1; ++ky) {
                int yy = y + ky;
                yy = yy < 0 ? 0 : (yy > lh - 1 ? lh - 1 : yy);
                for (int kx = -1; kx <= 1; ++kx) {
                    int xx = x + kx;
                    xx = xx < 0 ? 0 : (xx > lw - 1 ? lw - 1 : xx);
                    for (int ch = 0; ch < 3; ++ch)
                        p[((ky + 1) * 3 + (kx + 1)) * 3 + ch] = im[((int64_t)yy * lw + xx) * 3 + ch] - 0.5f;
                }
            }
            for (int ch = 0; ch < 3; ++ch) {
                float m = 0.0f;
                for (int k = ch; k < 27; k += 3)
                    m += p[k];
                m = m / 9.0f;
                for (int k = ch; k < 27; k += 3)
                    p[k] = p[k] - m;
            }
            float ss = 0.0f;
            for (int c = 0; c < lc; ++c) {
                float f = 0.0f;
                for (int k = 0; k < 27; ++k)
                    f += wts[c * 27 + k] * p[k];
                out[(int64_t)c * plane + (int64_t)y * lw + x] = f;
                ss += f * f;
            }
            const float nrm = sqrtf(ss + 1e-12f);
            for (int c = 0; c < lc; ++c) {
                float* o = &out[(int64_t)c * plane + (int64_t)y * lw + x];
                *o = *o / nrm;
            }
        }
    }
}

void vo_flow_features(const float* img, int w, int h, float* feats)
{
    float* lev[VO_FLOW_LEVELS];
    for (int l = 0; l < VO_FLOW_LEVELS; ++l) {
        int lw, lh, lc;
        vo_flow_level_dims(w, h, l, &lw, &lh, &lc);
        lev[l] = (float*)malloc((size_t)lw * lh * 3 * sizeof(float));
    }
    vo_flow_images(img, w, h, lev);
    float wts[196 * 27];
    size_t off = 0;
    for (int l = 0; l < VO_FLOW_LEVELS; ++l) {
        int lw, lh, lc;
        vo_flow_level_dims(w, h, l, &lw, &lh, &lc);
        vo_flow_weights(l, wts);
        vo_level_features(lev[l], lw, lh, lc, wts, feats + off);
        off += (size_t)lw * lh * lc;
        free(lev[l]);
    }
}

/* confidence-weighted 3x3 mean (edge clamp) of the residual flow:
 * S = up + sum_k conf_k * res_k / (sum_k conf_k + VO_EPS), taps row-major. */
static void vo_flow_smooth(const float* res, const float* conf, const float* up, float* out, int lw, int lh)
{
    const int64_t plane = (int64_t)lw * lh;
    for (int y = 0; y < lh; ++y)
        for (int x = 0; x < lw; ++x) {
            float sx = 0.0f, sy = 0.0f, sw = 0.0f;
            for (int ky = -1; ky <= 1; ++ky) {
                int yy = y + ky;
                yy = yy < 0 ? 0 : (yy > lh - 1 ? lh - 1 : yy);
                for (int kx = -1; kx <= 1; ++kx) {
                    int xx = x + kx;
                    xx = xx < 0 ? 0 : (xx > lw - 1 ? lw - 1 : xx);
                    const int64_t q = (int64_t)yy * lw + xx;
                    const float c = conf[q];
                    sx += c * res[q];
                    sy += c * res[plane + q];
                    sw += c;
                }
            }
            const int64_t p = (int64_t)y * lw + x;
            const float den = sw + VO_EPS;
            out[p] = up[p] + sx / den;
            out[plane + p] = up[plane + p] + sy / den;
        }
}

/* planar 2-channel bilinear upsampling x2 (half-pixel centres), vectors x2 */
static void vo_flow_up2(const float* in, int sw, int sh, float* out, int dw, int dh)
{
    const int64_t sp = (int64_t)sw * sh, dp = (int64_t)dw * dh;
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            float sx = ((float)x + 0.5f) * 0.5f - 0.5f;
            float sy = ((float)y + 0.5f) * 0.5f - 0.5f;
            if (sx < 0.0f)
                sx = 0.0f;
            if (sy < 0.0f)
                sy = 0.0f;
            int x0 = (int)floorf(sx), y0 = (int)floorf(sy);
            if (x0 > sw - 1)
                x0 = sw - 1;
            if (y0 > sh - 1)
                y0 = sh - 1;
            const int x1 = x0 + 1 < sw ? x0 + 1 : sw - 1;
            const int y1 = y0 + 1 < sh ? y0 + 1 : sh - 1;
            const float lx = sx - (float)x0, ly = sy - (float)y0;
            for (int ch = 0; ch < 2; ++ch) {
                const float* s = in + ch * sp;
                const float top = (1.0f - lx) * s[(int64_t)y0 * sw + x0] + lx * s[(int64_t)y0 * sw + x1];
                const float bot = (1.0f - lx) * s[(int64_t)y1 * sw + x0] + lx * s[(int64_t)y1 * sw + x1];
                out[ch * dp + (int64_t)y * dw + x] = ((1.0f - ly) * top + ly * bot) * 2.0f;
            }
        }
}

/* arg-max over the (2md+1)^2 = 81 correlations minus a small-displacement
 * prior (first maximum in index order), refined by a soft 3x3 centroid; the
 * confidence is the peak's prominence over the mean correlation. */
static void vo_flow_decode(const float* cv, float* res, float* conf, int lw, int lh, float prior)
{
    const int64_t plane = (int64_t)lw * lh;
    for (int64_t p = 0; p < plane; ++p) {
        int best = 0;
        float cmax = cv[p] - prior * 32.0f;
        float csum = cv[p];
        for (int d = 1; d < 81; ++d) {
            const int ddx = d % 9 - 4, ddy = d / 9 - 4;
            const float raw = cv[(int64_t)d * plane + p];
            csum += raw;
            const float v = raw - prior * (float)(ddx * ddx + ddy * ddy);
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
                const float sc = cv[(int64_t)(ny * 9 + nx) * plane + p] - prior * (float)((nx - 4) * (nx - 4) + (ny - 4) * (ny - 4));
                const float e = vo_expf((sc - cmax) * VO_TEMP);
                sw += e;
                sx += e * (float)(nx - 4);
                sy += e * (float)(ny - 4);
            }
        }
        res[p] = sx / sw;
        res[plane + p] = sy / sw;
        float k = cv[(int64_t)best * plane + p] - csum / 81.0f;
        conf[p] = k > 0.0f ? k : 0.0f;
    }
}

void vo_flow_from_features(const float* featA, const float* featB, int w, int h, float* flow_out)
{
    size_t offs[VO_FLOW_LEVELS];
    int LW[VO_FLOW_LEVELS], LH[VO_FLOW_LEVELS], LC[VO_FLOW_LEVELS];
    size_t off = 0;
    for (int l = 0; l < VO_FLOW_LEVELS; ++l) {
        vo_flow_level_dims(w, h, l, &LW[l], &LH[l], &LC[l]);
        offs[l] = off;
        off += (size_t)LW[l] * LH[l] * LC[l];
    }
    float* smooth_prev = NULL;
    for (int l = VO_FLOW_LEVELS - 1; l >= 0; --l) {
        const int lw = LW[l], lh = LH[l], lc = LC[l];
        const int64_t plane = (int64_t)lw * lh;
        float* up = (float*)calloc((size_t)plane * 2, sizeof(float));
        float* warped = (float*)malloc((size_t)plane * lc * sizeof(float));
        float* cv = (float*)malloc((size_t)plane * 81 * sizeof(float));
        float* raw = (float*)malloc((size_t)plane * 3 * sizeof(float));
        const float* fa = featA + offs[l];
        const float* fb = featB + offs[l];
        if (smooth_prev) {
            vo_flow_up2(smooth_prev, LW[l + 1], LH[l + 1], up, lw, lh);
            vo_warp_op_f32(fb, up, warped, 1, lc, lh, lw);
            free(smooth_prev);
        } else {
            memcpy(warped, fb, (size_t)plane * lc * sizeof(float));
        }
        vo_correlation_f32(fa, warped, cv, 1, lc, lh, lw, 4);
        vo_flow_decode(cv, raw, raw + 2 * plane, lw, lh, vo_level_prior[l]);
        smooth_prev = (float*)malloc((size_t)plane * 2 * sizeof(float));
        vo_flow_smooth(raw, raw + 2 * plane, up, smooth_prev, lw, lh);
        free(up);
        free(warped);
        free(cv);
        free(raw);
    }
    /* full-size flow: bilinear (half-pixel centres) from level 0, vectors
     * scaled by the size ratio of each axis; third channel 0 (the reference's
     * computed flows are 3-channel (u, v, 0), videostabilizer.cpp:50-51). */
    const int lw = LW[0], lh = LH[0];
    const int64_t plane = (int64_t)lw * lh;
    const float rx = (float)lw / (float)w, ry = (float)lh / (float)h;
    const float gx = (float)w / (float)lw, gy = (float)h / (float)lh;
    _Pragma("omp parallel for schedule(static)") for (int y = 0; y < h; ++y)
    {
        for (int x = 0; x < w; ++x) {
            float sx = ((float)x + 0.5f) * rx - 0.5f;
            float sy = ((float)y + 0.5f) * ry - 0.5f;
            if (sx < 0.0f)
                sx = 0.0f;
            if (sy < 0.0f)
                sy = 0.0f;
            int x0 = (int)floorf(sx), y0 = (int)floorf(sy);
            if (x0 > lw - 1)
                x0 = lw - 1;
            if (y0 > lh - 1)
                y0 = lh - 1;
            const int x1 = x0 + 1 < lw ? x0 + 1 : lw - 1;
            const int y1 = y0 + 1 < lh ? y0 + 1 : lh - 1;
            const float lx = sx - (float)x0, ly = sy - (float)y0;
            float r[2];
            for (int ch = 0; ch < 2; ++ch) {
                const float* s = smooth_prev + ch * plane;
                const float top = (1.0f - lx) * s[(int64_t)y0 * lw + x0] + lx * s[(int64_t)y0 * lw + x1];
                const float bot = (1.0f - lx) * s[(int64_t)y1 * lw + x0] + lx * s[(int64_t)y1 * lw + x1];
                r[ch] = (1.0f - ly) * top + ly * bot;
            }
            float* o = flow_out + ((int64_t)y * w + x) * 3;
            o[0] = r[0] * gx;
            o[1] = r[1] * gy;
            o[2] = 0.0f;
        }
    }
    free(smooth_prev);
}

void vo_flow_estimate(const float* imgA, const float* imgB, int w, int h, float* flow_out)
{
    const size_t nf = vo_flow_feature_floats(w, h);
    float* fa = (float*)malloc(nf * sizeof(float));
    float* fb = (float*)malloc(nf * sizeof(float));
    vo_flow_features(imgA, w, h, fa);
    vo_flow_features(imgB, w, h, fb);
    vo_flow_from_features(fa, fb, w, h, flow_out);
    free(fa);
    free(fb);
}
