// Internal declarations shared by the library's translation units.
//
// Kernels live in the .cu files; the launchers declared here validate
// nothing (the C-ABI layer in vsc_api.cpp does) and only enqueue work on the
// given stream, returning the launch error.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/vsc.h"

namespace vsc {

// A kernel launch with programmatic stream serialization: the kernel may be
// scheduled while the stream's previous kernel drains; it must call
// pdl_enter() (vsc_math.cuh) before touching memory.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
    Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// ---- error plumbing (vsc_api.cpp) ----------------------------------------
vsc_status set_error(vsc_status st, const char* fmt, ...);
vsc_status check_cuda(cudaError_t e, const char* what);
void clear_error();

// ---- ops (vsc_ops.cu) -----------------------------------------------------
// Batch n of each tensor starts at base + n * stride (elements; may be
// negative).  Strides of -1 mean contiguous N x C x H x W batches.
cudaError_t launch_correlation(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md,
    int legacy, cudaStream_t st, int64_t s1 = -1, int64_t s2 = -1, int64_t so = -1);
cudaError_t launch_warp_op(const float* in, const float* flow, float* out, int N, int C, int H, int W,
    cudaStream_t st, int64_t sin = -1, int64_t sfl = -1, int64_t sout = -1);
// Double-precision ops (the DOUBLE branches of correlation.cc / warp.cc;
// the CPU op has no legacy form).
cudaError_t launch_correlation_f64(const double* f1, const double* f2, double* out, int N, int C, int H, int W, int md,
    cudaStream_t st);
cudaError_t launch_warp_op_f64(const double* in, const double* flow, double* out, int N, int C, int H, int W,
    cudaStream_t st);

// ---- tensor-core correlation (vsc_corr_tc.cu) --------------------------------
// BF16 / FP16 operands on tcgen05 with FP32 accumulation, legacy = 0 layout.
constexpr int kTcMaxMd = 8;                 // max_displacement limit of the tile
constexpr int kTcMaxChannelsPadded = 208;   // channels, padded to a multiple of 16
int tc_padded_channels(int C);
size_t corr_tc_workspace_bytes(int N, int C, int H, int W);
// From float NCHW (scaled per tensor, converted in the workspace).
cudaError_t launch_corr_tc(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md,
    bool bf16, void* workspace, cudaStream_t st);
// From operands already in the chunked 16-bit layout [n][y][c / 16][x][c % 16]
// (Cp channels) with their scales (2 floats: f1, f2) on the device.
cudaError_t launch_corr_tc_chunked(const void* f1c, const void* f2c, float* out, const float* scales, int N, int Cp,
    int H, int W, int md, bool bf16, cudaStream_t st);
// two correlations of the same shape in one launch (f1c / f2c -> out and g1c / g2c -> out2)
cudaError_t launch_corr_tc_chunked2(const void* f1c, const void* f2c, float* out, const void* g1c, const void* g2c,
    float* out2, const float* scales, int N, int Cp, int H, int W, int md, bool bf16, cudaStream_t st);

// float NCHW -> chunked 16-bit operand layout, multiplied by *scale.
cudaError_t launch_to_chunked(const float* in, void* out, const float* scale, int N, int C, int H, int W, bool bf16,
    cudaStream_t st);
// the same for up to 5 tensors of one image each (a feature pyramid's levels) in one launch
cudaError_t launch_to_chunked_levels(const float* const* in, void* const* out, const int* C, const int* H,
    const int* W, int n, const float* scale, bool bf16, cudaStream_t st);
// custom::Warp (single precision) with the chunked 16-bit layout as output;
// batch n reads in + n * sin, flow + n * sfl (floats), writes out + n * sout_bytes.
// With cw, chh > 0 the flow is the flow estimator's coarser cw x chh level,
// upsampled 2x where it is read (the estimator's upsampled flow's values).
cudaError_t launch_warp_to_chunked(const float* in, const float* flow, void* out, const float* scale, int N, int C,
    int H, int W, int64_t sin, int64_t sfl, int64_t sout_bytes, bool bf16, cudaStream_t st, int cw = 0, int chh = 0);

// ---- learned flow upsampler (vsc_upsampler.cu, vsc_upsampler_tc.cu) ----------------
// Layer table: input / output channels, offsets of the weights (laid out
// [out][tap][in], tap = 3 (dy + 1) + dx + 1) and of the biases in the
// parameter vector.
struct UpLayer {
    int ci, co, w_off, b_off;
};
constexpr UpLayer kUpLayers[4] = {{3, 32, 0, 864}, {32, 32, 896, 896 + 9216}, {32, 32, 10144, 10144 + 9216},
    {32, 2, 19392, 19392 + 576}};
int upsampler_param_count();
void upsampler_init_params(float* host, uint64_t seed);
size_t upsampler_train_work_floats(int N, int H, int W);   // activations and gradients of a batch
// input (N x h x w x 3): the coarse flows bilinearly upsampled with their vectors
// scaled to the full grid, and the frames' luma; batch n at base + n * stride
cudaError_t launch_upsampler_prepare(const float* coarse, int cw, int ch, int cfc, const float* img, float* input,
    int w, int h, int N, int64_t s_coarse, int64_t s_img, int64_t s_in, cudaStream_t st);
// Tensor-core inference (tcgen05 implicit-GEMM convolutions, FP16 operands,
// FP32 accumulation).  Packed weights: upsampler_tc_weight_bytes() bytes,
// written from the FP32 parameters by launch_upsampler_tc_pack.  Work:
// upsampler_tc_work_bytes(N, H, W) bytes, 16-byte aligned.  Writes the
// finished flows (u, v, 0) of every batch image (flow + n * s_out floats)
// from the prepared input (launch_upsampler_prepare's layout).
size_t upsampler_tc_weight_bytes();
size_t upsampler_tc_work_bytes(int N, int H, int W);
cudaError_t launch_upsampler_tc_pack(const float* prm, void* wtc, cudaStream_t st);
cudaError_t launch_upsampler_tc(const void* wtc, const float* prm, const float* input, void* work, float* flow, int N,
    int H, int W, float max_residual, int64_t s_out, cudaStream_t st, int* launches);
cudaError_t upsampler_train_step(float* prm, float* grad, float* m, float* v, int step, const float* input,
    const float* target, int N, int H, int W, float lr, float* work, float* loss_dev, cudaStream_t st);

// Device address of the flag a kernel sets when one of its bounded waits gave up.
cudaError_t device_timeout_flag(int** flag);

// ---- stabilization (vsc_stab.cu) -------------------------------------------
struct Img {
    float* d;
    int w, h, c;
};
cudaError_t launch_rgba_to_float(const uint8_t* rgba, float* out, int64_t npix, cudaStream_t st);
cudaError_t launch_float_to_rgba(const float* in, uint8_t* rgba, int64_t npix, cudaStream_t st);
cudaError_t launch_stab_warp(Img in, Img flow, Img out, cudaStream_t st);
// occ_mask: optional HWC2 forward-backward consistency mask multiplied into
// the previous/next frame weights after their clamps (nullptr: none).
cudaError_t launch_adap_comb(Img ci, Img cp, Img pwi, Img pwp, Img nwi, Img nwp, Img ai, Img ap, Img lsw, float alpha,
    cudaStream_t st, const float* occ_mask = nullptr);
// Forward-backward flow consistency mask (HWC2 of 0/1: ch0 previous frame,
// ch1 next frame); an opt-in extension with no counterpart in the reference.
cudaError_t launch_flow_consistency(Img ffwd, Img fbwd, Img mask, cudaStream_t st);
cudaError_t launch_consist_wt(Img ai, Img ci, Img wt, float beta, float gamma, cudaStream_t st);
cudaError_t launch_bilinear(Img in, Img out, cudaStream_t st);
// launch_bilinear for n 3-channel images in one launch per 16 (same bits)
cudaError_t launch_bilinear_group(const Img* in, const Img* out, int n, cudaStream_t st);
// Solver.
//   kSolverExact: kernel_consist_out's expression, bit for bit; workspace:
//                 the Laplacian of the processed image, two momentum images
//                 and the second Jacobi buffer, 4 * w*h*3 floats;
//   kSolverFma:   the same step regrouped around per-solve constants with
//                 fused multiply-adds, each channel solved as its own plane
//                 (within a tolerance of the exact form; equal to the
//                 restatement's FMA form); workspace: the constants Cs and
//                 nK, two momentum images and two iterates, all as planes,
//                 6 * w*h*3 floats.
enum SolverForm { kSolverExact = 0, kSolverFma = 1 };
size_t solver_workspace_floats(int w, int h, int form = kSolverExact);
int solver_steps_per_launch();  // Jacobi steps one solver launch performs (temporal blocking)
// Tile-shape autotuner of the persistent solver kernels (same results either
// way): solver_autotune times both shapes at (w, h) on scratch images and
// keeps the faster for the current device (synchronises `st`; not during
// stream capture); solver_tile_rows reports the rows of the tile a solve at
// (w, h) uses (tuned, or the wave model's choice); per solver form.
cudaError_t solver_autotune(int w, int h, cudaStream_t st, int* rows_out, int form = kSolverExact);
int solver_tile_rows(int w, int h, bool* tuned, int form = kSolverExact);
void solver_set_autotune(bool on);
// The same for the sizes one grouped launch solves together (one image per
// stream of a multi-stream step), keyed by the whole list.
cudaError_t solver_group_autotune(const int* w, const int* h, int n, cudaStream_t st, int* rows_out,
    int form = kSolverExact);
int solver_group_tile_rows(const int* w, const int* h, int n, bool* tuned, int form = kSolverExact);
// Runs num_iter iterations; O holds the initial solution and receives the
// result.  Returns the number of kernels launched through *launches.
cudaError_t run_solver(const float* P, const float* A, const float* Wt, float* O, int w, int h, int num_iter,
    float step, float mom, float* workspace, cudaStream_t st, int* launches, uint8_t* rgba_out = nullptr,
    int form = kSolverExact);
// The FMA form started from the cw x ch solution Oc upsampled to w x h with
// kernel_bilinear's expression (the pyramid's next level), the upsampling
// fused into the solve's setup; O receives the result only.  num_iter >= 1.
cudaError_t run_solver_from_coarse(const float* P, const float* A, const float* Wt, float* O, int w, int h,
    const float* Oc, int cw, int ch, int num_iter, float step, float mom, float* workspace, cudaStream_t st,
    int* launches, uint8_t* rgba_out);

// Grouped solve: n images of any sizes, the same iterations, each launch of
// the persistent kernel walking the tiles of all of them (up to 16 images
// per launch).  Per image, before run_solver_group on the same stream:
// solver_prep(form, ...) into its workspace, and the initial solution written to
// solver_start_buffer(O, ...) (O itself or the workspace's second buffer,
// whichever makes the last launch write O).  Needs solver_group_eligible
// (width % 4 == 0 and 16-byte aligned images, the TMA path).
struct SolverImage {
    const float* P;
    const float* A;
    const float* Wt;
    float* O;
    int w, h;
    float* workspace;  // solver_workspace_floats(w, h, form)
    uint8_t* rgba;     // RGBA8 copy of the result, or null
};
float* solver_start_buffer(float* O, int w, int h, int num_iter, float* workspace, int form = kSolverExact);
bool solver_tma_supported();  // the persistent TMA kernels run on the current device
cudaError_t solver_lap(const float* P, int w, int h, float* workspace, cudaStream_t st);
// the per-solve precomputation of a form: lap P (exact) or Cs (FMA), into the workspace
cudaError_t solver_prep(int form, const float* P, const float* A, const float* Wt, int w, int h, float step,
    float* workspace, cudaStream_t st);
bool solver_group_eligible(const SolverImage* im, int n, int form = kSolverExact);
cudaError_t run_solver_group(const SolverImage* im, int n, int num_iter, float step, float mom, cudaStream_t st,
    int* launches, int form = kSolverExact);

// Device-side bounded waits record a timeout in a device flag instead of
// hanging; this reads and clears it for the current device.
cudaError_t check_device_timeout(int* flagged);
// A kernel whose bounded wait on an mbarrier that nobody arrives on gives up
// after `spins` polls (the timeout path, without any fault).
cudaError_t launch_bounded_wait_selftest(int spins, cudaStream_t st);

// Solver with its workspace in a file-scope device array instead of caller
// or pool memory (no allocation).  Images up to kNoAllocMaxPixels pixels.
constexpr size_t kNoAllocWorkspaceFloats = size_t(1) << 22;  // 16 MiB
constexpr size_t kNoAllocMaxPixels = kNoAllocWorkspaceFloats / 12;
cudaError_t run_solver_noalloc(const float* P, const float* A, const float* Wt, float* O, int w, int h, int num_iter,
    float step, float mom, cudaStream_t st);

// Fused five-warp + adaptive combination + consistency weights for the
// orchestrator: writes adapCmbPr and consWt only.  With fw, fh > 0 the flows
// are the 3-channel fw x fh flows that the step upsamples bilinearly to
// w x h, sampled where they are used (same outputs as upsampling them first);
// not with the occlusion mask.
// With down_p non-null (no occlusion mask, front_down_fusable) it also writes
// the next pyramid level's P, A, Wt (ow x oh = w/2 x h/2), pyr_down3's values.
cudaError_t launch_fused_front(const float* o0, const float* o1, const float* o2, const float* p0, const float* p1,
    const float* p2, const float* last_stab, const float* flow_fwd, const float* flow_bwd, int fc, float* adap_pr,
    float* cons_wt, int w, int h, float alpha, float beta, float gamma, cudaStream_t st, bool occlusion_mask = false,
    int fw = 0, int fh = 0, float* down_p = nullptr, float* down_a = nullptr, float* down_w = nullptr, int ow = 0,
    int oh = 0);
// the pyramid's first downsampling can be fused into the front pass (exact 2x)
bool front_down_fusable(int w, int h, int ow, int oh);
// fused_front on the RGBA8 words of the six frames (4-byte aligned, w x h
// words each); same outputs bit for bit
cudaError_t launch_fused_front_rgba(const uint8_t* o0, const uint8_t* o1, const uint8_t* o2, const uint8_t* p0,
    const uint8_t* p1, const uint8_t* p2, const float* last_stab, const float* flow_fwd, const float* flow_bwd, int fc,
    float* adap_pr, float* cons_wt, int w, int h, float alpha, float beta, float gamma, cudaStream_t st,
    bool occlusion_mask);
// P, A, Wt of the next coarser pyramid level, one launch.
cudaError_t launch_pyr_down3(const float* P, const float* A, const float* Wt, int iw, int ih, float* Pd, float* Ad,
    float* Wd, int ow, int oh, cudaStream_t st);

// ---- flow estimator (vsc_flow.cu) ------------------------------------------
constexpr int kFlowLevels = 5;
struct FlowDims {
    int lw[kFlowLevels], lh[kFlowLevels], lc[kFlowLevels];
    size_t off[kFlowLevels];  // float offset of each level's features
    size_t feat_floats;       // all levels, one frame
    size_t max_plane;         // largest lw*lh
    int max_c;
};
FlowDims flow_dims(int w, int h);
cudaError_t flow_upload_weights();
// scratch for one frame's feature extraction: level images
size_t flow_feature_scratch_floats(const FlowDims& d);
// With `full` non-null the w x h image is the nearest-neighbour resize of the
// FW x FH frame `full` (FLOWDOWNSCALE) and `img` is not read.
cudaError_t launch_flow_features(const float* img, int w, int h, const FlowDims& d, float* feats, float* scratch,
    cudaStream_t st, int* launches, const float* full = nullptr, int FW = 0, int FH = 0);
// The tensor-core form of the estimator's correlations: each frame's
// features also kept in the chunked 16-bit layout (level l at byte offset
// tc_level_offset(d, l)), scaled by scales[0] (|f| <= 1 after the features'
// L2 normalisation, so a fixed power of two serves every level).
size_t tc_level_offset(const FlowDims& d, int level);
size_t tc_frame_bytes(const FlowDims& d);
size_t tc_warped_bytes(const FlowDims& d);  // one direction's warped operand at the largest level
cudaError_t launch_flow_features_chunked(const float* feats, const FlowDims& d, void* chunked, const float* scale,
    bool bf16, cudaStream_t st, int* launches);
struct FlowTc {
    const void* a[2];  // chunked features of the first frame of direction 0 / 1
    const void* b[2];  // chunked features of the second frame (used at the coarsest level)
    void* warped;      // 2 x tc_warped_bytes of scratch
    const float* scales;
    bool bf16;
};
// scratch for one flow direction: up/raw/smooth flows, warped features, cost volume
size_t flow_estimate_scratch_floats(const FlowDims& d);
// Two flows in the same launches (batch index z): direction n runs A_n =
// featA + n*sA against B_n = featB + n*sB and writes flow_out + n*s_out
// (w x h x 3).  scratch holds 2 * flow_estimate_scratch_floats(d).
cudaError_t launch_flow_pair(const float* featA, int64_t sA, const float* featB, int64_t sB, int w, int h,
    const FlowDims& d, float* flow_out, int64_t s_out, float* scratch, cudaStream_t st, int* launches,
    const FlowTc* tc = nullptr);

}  // namespace vsc
