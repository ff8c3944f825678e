/*
 * vsc_oracle — CPU restatement of the reference's per-frame hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests, the smoke
 * check and the CPU-baseline leg of bench.py call it; the product library
 * never links, loads or falls back to it.
 *
 * Every function restates one reference function and cites it
 * (paths relative to the reference project root).  Arithmetic is written in
 * the reference's literal single-precision operation order, compiled without
 * floating-point contraction (-ffp-contract=off), so that the CUDA kernels of
 * this project — compiled with -fmad=false and the same order — reproduce it
 * bit for bit.  Two documented exceptions:
 *   - exp(): both sides use vo_expf(), a Cody–Waite reduced, degree-7 Taylor
 *     exponential written for this project (the reference calls CUDA's expf,
 *     whose last-ulp behaviour cannot be reproduced on a CPU);
 *   - the reference's CPU Warp op computes its weights in double precision
 *     (warp.cc:109-126).  vo_warp_op_refsem() restates that exactly;
 *     vo_warp_op_f32() is the single-precision form the GPU computes, pinned
 *     against it by a stated tolerance.
 * The stabilization solver is restated as a Jacobi iteration (every pixel
 * reads the previous iterate); the reference GPU kernel updates in place
 * (flowconsistency.cu:370), which makes its result depend on thread timing.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- elementary ---------------------------------------------------------- */
float vo_expf(float x);
void vo_set_threads(int n); /* OpenMP threads for the row-parallel loops (1 = serial) */
int vo_get_threads(void);

/* ---- custom ops (src/ort_custom_ops) -------------------------------------- */
/* correlation.cc:147-275 (legacy=0): out[n][dy][dx][h][w], NCHW inputs. */
void vo_correlation_f32(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md);
void vo_correlation_f64(const double* f1, const double* f2, double* out, int N, int C, int H, int W, int md);
/* correlation_cuda.cu:182-265 (legacy=1): same sums divided by C, laid out
 * N x (2md+1)^2 x H x W; channel sum taken in channel order. */
void vo_correlation_legacy_f32(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md);
/* warp.cc:71-133 with its double-precision weight arithmetic (bit-exact). */
void vo_warp_op_refsem(const float* in, const float* flow, float* out, int N, int C, int H, int W);
void vo_warp_op_f64(const double* in, const double* flow, double* out, int N, int C, int H, int W);
/* The same operator evaluated in single precision: the form the CUDA kernel computes. */
void vo_warp_op_f32(const float* in, const float* flow, float* out, int N, int C, int H, int W);

/* ---- frame I/O (src/stabilization/gpuimage.cu) ----------------------------- */
void vo_rgba_to_float(const uint8_t* rgba, float* out, int64_t npix);  /* :39-51 */
void vo_float_to_rgba(const float* in, uint8_t* rgba, int64_t npix);   /* :54-67 */

/* ---- stabilization kernels (src/stabilization/flowconsistency.cu) ----------
 * Images are interleaved float HWC with 3 channels; flows have fc (2 or 3). */
void vo_stab_warp(const float* in, const float* flow, int fc, float* out, int w, int h); /* :77-114 */
void vo_adap_comb(const float* crnt_in, const float* crnt_pr, const float* prev_warp_in, const float* prev_warp_pr,
    const float* next_warp_in, const float* next_warp_pr, float* adap_in, float* adap_pr, const float* last_stab_warp,
    float alpha, int64_t npix); /* :116-166 */
/* Opt-in extension (no counterpart in the reference): forward-backward flow
 * consistency.  mask is HWC2: ch0 = 1 where the backward flow is confirmed by
 * the forward flow (the previous frame's warp), ch1 = 1 where the forward
 * flow is confirmed by the backward flow (the next frame's warp), else 0. */
void vo_flow_consistency_mask(const float* flow_fwd, const float* flow_bwd, int fc, float* mask, int w, int h);
/* vo_adap_comb with wt_prv, wt_nxt multiplied by occ_mask ch0, ch1 after the
 * clamps; occ_mask == NULL is vo_adap_comb. */
void vo_adap_comb_masked(const float* crnt_in, const float* crnt_pr, const float* prev_warp_in,
    const float* prev_warp_pr, const float* next_warp_in, const float* next_warp_pr, float* adap_in, float* adap_pr,
    const float* last_stab_warp, const float* occ_mask, float alpha, int64_t npix);
void vo_consist_wt(const float* crnt_in, const float* adap_in, float* cons_wt, float beta, float gamma,
    int64_t npix); /* :168-191 */
void vo_bilinear(const float* in, int iw, int ih, float* out, int ow, int oh, int c); /* :50-75 */
/* :193-258 + :350-374, Jacobi; O holds the initial solution and receives the result. */
void vo_consist_out(const float* P, const float* A, const float* wt, int num_iter, float step, float mom, float* O,
    int w, int h);
/* The FMA form of the solver (the library's vsc_get_consist_out_fma). */
void vo_consist_out_fma(const float* P, const float* A, const float* wt, int num_iter, float step, float mom, float* O,
    int w, int h);

typedef struct vo_hyper {
    float alpha, beta, gamma;
    int pyramid_levels, num_iter;
    float step_size, mom_fac;
} vo_hyper;
void vo_default_hyper(vo_hyper* hp); /* videostabilizer.cpp:104-112 */

/* One stabilization pass, videostabilizer.cpp:181-247.  orig/proc are the
 * frames t-1, t, t+1 (float HWC3); flows have fc channels; last_stab is the
 * previous stabilized frame.  Writes the FP32 result (consisOut) and, if
 * out_rgba != NULL, its RGBA8 quantisation.  Returns 0, or -1 on bad sizes. */
int vo_stab_pass(int w, int h, const float* const orig[3], const float* const proc[3], const float* flow_fwd,
    const float* flow_bwd, int fc, const float* last_stab, const vo_hyper* hp, float* out_f32, uint8_t* out_rgba);
/* vo_stab_pass with the opt-in forward-backward consistency mask applied to
 * the temporal weights when occlusion_mask != 0. */
int vo_stab_pass_ex(int w, int h, const float* const orig[3], const float* const proc[3], const float* flow_fwd,
    const float* flow_bwd, int fc, const float* last_stab, const vo_hyper* hp, int occlusion_mask, float* out_f32,
    uint8_t* out_rgba);
/* vo_stab_pass_ex with the solver in the exact (0) or the FMA form (1). */
int vo_stab_pass_form(int w, int h, const float* const orig[3], const float* const proc[3], const float* flow_fwd,
    const float* flow_bwd, int fc, const float* last_stab, const vo_hyper* hp, int occlusion_mask, int solver_form,
    float* out_f32, uint8_t* out_rgba);

/* ---- weight-free flow estimator built from the two ops ---------------------
 * A coarse-to-fine stand-in for the missing PWC-Net weights: random-projection
 * patch features on the PWC channel pyramid {32,64,96,128,196} at 1/4..1/64 of
 * the 64-aligned frame, Warp + Correlation(md=4) per level, arg-max with a
 * local soft refinement, smoothing, and bilinear upsampling to full size. */
#define VO_FLOW_LEVELS 5
int vo_flow_level_dims(int w, int h, int level, int* lw, int* lh, int* lc); /* level 0..4 = 1/4 .. 1/64 */
size_t vo_flow_feature_floats(int w, int h);                               /* all levels, one frame */
void vo_flow_weights(int level, float* wts);                               /* lc x 27, row-major */
void vo_flow_features(const float* img, int w, int h, float* feats);       /* img: float HWC3 */
/* flow from frame A to frame B: out is HWC3 (u, v, 0) at w x h */
void vo_flow_from_features(const float* featA, const float* featB, int w, int h, float* flow_out);
void vo_flow_estimate(const float* imgA, const float* imgB, int w, int h, float* flow_out);

#ifdef __cplusplus
}
#endif
