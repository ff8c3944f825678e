/*
 * vsc.h — C ABI of the GB300 (sm_103a) implementation of the per-frame hot
 * path of video-stream-consistency: the Correlation and Warp optical-flow
 * operators and the per-frame stabilization pass.
 *
 * Every entry point:
 *   - takes plain device (or, where stated, host) pointers, sizes and a CUDA
 *     stream (vsc_stream_t is a cudaStream_t; NULL is the legacy default
 *     stream), enqueues its work on that stream and returns without
 *     synchronising the device;
 *   - returns a vsc_status, never exits or throws; vsc_last_error() gives
 *     the calling thread's message for the last failure;
 *   - is reentrant: no entry point keeps hidden per-call state, so calls from
 *     several threads on several streams may run concurrently — except
 *     vsc_get_consist_out_noalloc, whose calls share one built-in workspace
 *     (see there).
 *
 * Each declaration names the reference interface (file:line, relative to
 * the reference project root) it replaces.
 */
#ifndef VSC_H
#define VSC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define VSC_API __declspec(dllexport)
#else
#define VSC_API __attribute__((visibility("default")))
#endif

typedef enum vsc_status {
    VSC_OK = 0,
    VSC_EINVAL = 1,        /* bad pointer, shape, attribute or size */
    VSC_ECUDA = 2,         /* a CUDA runtime call or launch failed */
    VSC_ETIMEOUT = 3,      /* a bounded device-side wait gave up */
    VSC_ENOMEM = 4,        /* device or workspace memory exhausted / too small */
    VSC_EUNSUPPORTED = 5,  /* valid request this build does not implement */
    VSC_ESTATE = 6         /* call out of order (e.g. step before the frame window is full) */
} vsc_status;

typedef void* vsc_stream_t;

/* Message of the calling thread's last failure ("" after success). */
VSC_API const char* vsc_last_error(void);
/* 10000*major + 100*minor + patch */
VSC_API int vsc_version(void);

/* Device-side waits in this library are bounded: a kernel that gives up
 * records it in a device flag and returns instead of hanging.  Reads and
 * clears the flag of the current device (synchronous): VSC_ETIMEOUT if a
 * kernel gave up since the last call, whose outputs are then invalid.
 * No reference counterpart: the reference exits the process on CUDA errors
 * (flowconsistency.cu:25-31). */
VSC_API vsc_status vsc_check_device(void);

/* Self-test of that path: one CTA waits at most `spins` polls on a barrier
 * nothing completes, then records the timeout; vsc_check_device then
 * returns VSC_ETIMEOUT.  No fault, trap or hang is involved. */
VSC_API vsc_status vsc_selftest_bounded_wait(int32_t spins, vsc_stream_t stream);

/* Jacobi steps of the blend solver per kernel launch (temporal blocking);
 * a property of the build, for profiling tools. */
VSC_API int32_t vsc_solver_steps_per_launch(void);

/* Tile-shape autotuner of the blend solver (vsc_get_consist_out and the
 * stabilizer).  Its two persistent kernels, on 64 x 32 and 64 x 48 pixel
 * tiles, give the same results bit for bit; which is faster at a size
 * depends on how the tiles fill the GPU's waves.  vsc_solver_autotune times
 * both at width x height on scratch images and keeps the faster for the
 * current device (it synchronises the stream and is refused while the stream
 * is being captured); vsc_stabilizer_create tunes its pyramid's sizes.
 * vsc_solver_tile_rows returns the tile rows (32 or 48) a solve at that size
 * uses, with *tuned = 1 when they were measured (else the wave model's
 * choice).  vsc_solver_set_autotune(0) forgets the measurements and stops
 * tuning; (1) resumes.  No counterpart in the reference. */
VSC_API vsc_status vsc_solver_autotune(int32_t width, int32_t height, vsc_stream_t stream, int32_t* tile_rows);
VSC_API int32_t vsc_solver_tile_rows(int32_t width, int32_t height, int32_t* tuned);
VSC_API void vsc_solver_set_autotune(int32_t on);

/* Forms of the blend solver (no counterpart in the reference, whose one form
 * is VSC_SOLVER_EXACT):
 *   VSC_SOLVER_EXACT  kernel_consist_out's expression (flowconsistency.cu:
 *                     193-258), rounded as the reference rounds it;
 *   VSC_SOLVER_FMA    the same Jacobi step regrouped around two per-pixel
 *                     constants computed once per solve, Cs = s*(w*A - lap P)
 *                     and nK = -s*(cnt + w):  g = fma(nK, O, fma(s, S, Cs))
 *                     with S the sum of the valid neighbours, O' = O + g
 *                     (+ m*U), U' = g: seven FP32 operations per pixel and
 *                     channel instead of twelve, each channel solved as its
 *                     own plane.  Differs from the exact form by rounding only: at
 *                     1920x1080 over a 150-iteration solve within 1e-6
 *                     absolute (images in [0, 1]), > 100 dB PSNR, and RGBA8
 *                     bytes differing on about 1e-5 of the values.
 * The autotuner chooses the exact form's tile shape (32 or 48 rows); the
 * FMA form has one (72 rows of a plane), which vsc_solver_autotune_form
 * reports without measuring. */
#define VSC_SOLVER_EXACT 0
#define VSC_SOLVER_FMA 1
VSC_API vsc_status vsc_solver_autotune_form(int32_t width, int32_t height, int32_t form, vsc_stream_t stream,
    int32_t* tile_rows);
VSC_API int32_t vsc_solver_tile_rows_form(int32_t width, int32_t height, int32_t form, int32_t* tuned);

/* ========================================================================
 * ONNX Runtime custom ops (domain "custom")
 * ======================================================================== */

/* custom::Correlation.  Replaces CorrelationKernel::Compute /
 * ComputeCUDA (src/ort_custom_ops/include/ort_custom_ops/opticalflow/
 * correlation.h:35-50, src/ort_custom_ops/src/opticalflow/correlation_cuda.cc:29-137,
 * correlation_cuda.cu:333-442; CPU semantics correlation.cc:45-275).
 *   f1, f2 : device, N x C x H x W float (NCHW)
 *   out    : device, legacy = 0: N x P x P x H x W, out[n][i][j][h][w] =
 *            sum_c f1[n][c][h][w] * f2[n][c][h+i-md][w+j-md] (0 outside);
 *            legacy = 1: N x P*P x H x W, the same sums divided by C
 *            (the original PWC-Net layer, correlation_cuda.cu:182-331);
 *            P = 2*max_displacement + 1.
 * The channel sum is taken in channel order with separately rounded
 * products and sums, so legacy = 0 equals the reference CPU op bit for bit.
 * No workspace: the NCHW->NHWC temporaries of the reference
 * (correlation_cuda.cu:365-391) are folded into the kernel's tile loads. */
VSC_API vsc_status vsc_correlation_fwd(const float* f1, const float* f2, float* out, int64_t N, int64_t C, int64_t H,
    int64_t W, int64_t max_displacement, int64_t legacy, vsc_stream_t stream);

/* custom::Warp.  Replaces WarpKernel::Compute / ComputeCUDA
 * (warp.h:18-31, warp_cuda.cc:28-77, warp_cuda.cu:28-98; CPU semantics
 * warp.cc:25-133).
 *   input : device, N x C x H x W float;  flow : device, N x 2 x H x W
 *   (channel 0 = x displacement, 1 = y);  out : device, N x C x H x W.
 * Bilinear backward warp with zero padding; an output is 0 unless the
 * bilinear weight of its in-map taps exceeds 0.999.  Single-precision
 * weights: within 2^-21 * max|input| of the reference's double-weight CPU op. */
VSC_API vsc_status vsc_warp_fwd(const float* input, const float* flow, float* out, int64_t N, int64_t C, int64_t H,
    int64_t W, vsc_stream_t stream);

/* Operand types of the reduced-precision correlation. */
typedef enum vsc_dtype { VSC_DTYPE_F32 = 0, VSC_DTYPE_BF16 = 1, VSC_DTYPE_F16 = 2 } vsc_dtype;

/* custom::Correlation (legacy = 0 layout) on the tensor cores: f1 and f2 are
 * each scaled by a power of two chosen from their largest magnitude (per
 * call, i.e. per pyramid level), rounded to BF16 or FP16, multiplied with FP32
 * accumulation, and the sums scaled back exactly.  Error against the exact
 * sum S = sum_c f1 f2: |out - S| <= (2u + u^2) sum_c |f1 f2| with u = 2^-8
 * (BF16) or 2^-11 (FP16), plus the FP32 rounding of the sum.  No counterpart
 * in the reference (whose op is FP32 only); max_displacement <= 8 and at most
 * 208 channels.  workspace: device memory of
 * vsc_correlation_lowp_workspace_size bytes, 256-byte aligned, or NULL to
 * let the library take it from its stream-ordered pool. */
VSC_API size_t vsc_correlation_lowp_workspace_size(int64_t N, int64_t C, int64_t H, int64_t W);
VSC_API vsc_status vsc_correlation_fwd_lowp(const float* f1, const float* f2, float* out, int64_t N, int64_t C,
    int64_t H, int64_t W, int64_t max_displacement, int32_t dtype, void* workspace, size_t workspace_bytes,
    vsc_stream_t stream);

/* The DOUBLE branches of the reference's CPU ops (correlation.cc:115-139,
 * warp.cc:48-58; the op schemas declare FLOAT, the kernels also take
 * double).  Same layouts and semantics as vsc_correlation_fwd (legacy = 0;
 * the CPU op has no legacy form) and vsc_warp_fwd, computed in double with
 * the reference's operation order: bit-exact to correlation.cc / warp.cc
 * on double tensors. */
VSC_API vsc_status vsc_correlation_fwd_f64(const double* f1, const double* f2, double* out, int64_t N, int64_t C,
    int64_t H, int64_t W, int64_t max_displacement, vsc_stream_t stream);
VSC_API vsc_status vsc_warp_fwd_f64(const double* input, const double* flow, double* out, int64_t N, int64_t C,
    int64_t H, int64_t W, vsc_stream_t stream);

/* ========================================================================
 * Stabilization kernels (src/stabilization/flowconsistency.cuh:3-50)
 * ======================================================================== */

/* A device image: interleaved float, element (x, y, c) at
 * data[(y*width + x)*channels + c].  Mirrors GPUImage / GPUImageWrapper
 * (src/stabilization/gpuimage.h:8-31, gpuimagewrapper.h:8-25). */
typedef struct vsc_image {
    float* data;
    int32_t width;
    int32_t height;
    int32_t channels;
} vsc_image;

/* RGBA8 (device) -> 3-channel float image, value = float(double(v)/255.0).
 * Replaces kernel_to_float_image / char_to_cuda_float_image (gpuimage.cu:39-104). */
VSC_API vsc_status vsc_char_to_float_image(const uint8_t* rgba, const vsc_image* out, vsc_stream_t stream);

/* 3-channel float image -> RGBA8 (device), (uint8)floor(|v|*255) with the
 * reference's mod-256 wrap, alpha = 1.  Replaces kernel_to_char_image /
 * cuda_float_to_char_image (gpuimage.cu:54-67, :107-135). */
VSC_API vsc_status vsc_float_to_char_image(const vsc_image* in, uint8_t* rgba, vsc_stream_t stream);

/* Backward warp of a 3-channel image by a 2- or 3-channel flow, sample
 * position clamped to [0,w-3] x [0,h-3].  Replaces get_warp_result /
 * kernel_warp (flowconsistency.cu:77-114, :301-312). */
VSC_API vsc_status vsc_get_warp_result(const vsc_image* input, const vsc_image* flow, const vsc_image* input_warp,
    vsc_stream_t stream);

/* Adaptive temporal combination.  Replaces get_adap_comb / kernel_adap_comb
 * (flowconsistency.cu:116-166, :314-333). */
VSC_API vsc_status vsc_get_adap_comb(const vsc_image* crnt_in, const vsc_image* crnt_pr, const vsc_image* prev_warp_in,
    const vsc_image* prev_warp_pr, const vsc_image* next_warp_in, const vsc_image* next_warp_pr,
    const vsc_image* adap_cmb_in, const vsc_image* adap_cmb_pr, const vsc_image* last_stab_warp, float alpha,
    vsc_stream_t stream);

/* Opt-in extension, no counterpart in the reference (the reference weights
 * the previous and next frames by colour similarity only,
 * flowconsistency.cu:146-154).  Forward-backward flow consistency: for a
 * flow a at a pixel, the opposite flow b is sampled bilinearly where a carries
 * the pixel, p; the pixel is consistent when
 * |a + b(p)|^2 <= 0.01 (|a|^2 + |b(p)|^2) + 0.5 and p lies in the frame.
 * occ_mask (2 channels, same size): ch0 = 1 where flow_bwd is confirmed by
 * flow_fwd (the previous frame's warp), ch1 = 1 where flow_fwd is confirmed
 * by flow_bwd (the next frame's warp), else 0.  Flows: 2 or 3 channels. */
VSC_API vsc_status vsc_get_flow_consistency_mask(const vsc_image* flow_fwd, const vsc_image* flow_bwd,
    const vsc_image* occ_mask, vsc_stream_t stream);

/* vsc_get_adap_comb with the previous/next frame weights multiplied by
 * occ_mask ch0/ch1 after their clamps (a mask of ones gives
 * vsc_get_adap_comb's bits).  Opt-in extension, no counterpart in the reference. */
VSC_API vsc_status vsc_get_adap_comb_masked(const vsc_image* crnt_in, const vsc_image* crnt_pr,
    const vsc_image* prev_warp_in, const vsc_image* prev_warp_pr, const vsc_image* next_warp_in,
    const vsc_image* next_warp_pr, const vsc_image* adap_cmb_in, const vsc_image* adap_cmb_pr,
    const vsc_image* last_stab_warp, const vsc_image* occ_mask, float alpha, vsc_stream_t stream);

/* The library's flow estimator on one frame pair (what FlowModel::run
 * provides in compute mode, flowmodel.cpp:121-168, here built from the two
 * ops): img_a, img_b float HWC3 in [0, 1]; flow_ab (a -> b) and flow_ba
 * (b -> a) HWC3 (u, v, 0) of the same size.  Workspace from the library's
 * stream-ordered pool. */
VSC_API vsc_status vsc_flow_estimate(const vsc_image* img_a, const vsc_image* img_b, const vsc_image* flow_ab,
    const vsc_image* flow_ba, vsc_stream_t stream);

/* The front half of doOneStep (videostabilizer.cpp:182-198) in one pass:
 * the five get_warp_result calls (previous original and processed frames and
 * the last stabilized frame along flow_bwd, next original and processed
 * frames along flow_fwd), get_adap_comb and get_consist_wt, writing only
 * adapCmbPr and consWt (the intermediates never reach memory).  Results
 * equal the separate calls bit for bit; occlusion_mask != 0 applies the
 * opt-in forward-backward mask.  No single counterpart in the reference. */
VSC_API vsc_status vsc_stab_front(const vsc_image* orig_prev, const vsc_image* orig_cur, const vsc_image* orig_next,
    const vsc_image* proc_prev, const vsc_image* proc_cur, const vsc_image* proc_next, const vsc_image* last_stab,
    const vsc_image* flow_fwd, const vsc_image* flow_bwd, const vsc_image* adap_cmb_pr, const vsc_image* consis_wt,
    float alpha, float beta, float gamma, int32_t occlusion_mask, vsc_stream_t stream);

/* vsc_stab_front with the six original / processed frames given as the
 * RGBA8 device frames they are converted from (w x h 32-bit words each,
 * 4-byte aligned; alpha ignored): the bilinear taps are gathered as 4-byte
 * words and converted with vsc_char_to_float_image's exact conversion, so
 * the outputs equal vsc_stab_front's on the converted frames bit for bit
 * with 84 instead of 124 bytes of traffic per pixel.  No single counterpart in the
 * reference (videostabilizer.cpp:182-198 on the frames of gpuimage.cu:39-51). */
VSC_API vsc_status vsc_stab_front_rgba(const uint8_t* orig_prev, const uint8_t* orig_cur, const uint8_t* orig_next,
    const uint8_t* proc_prev, const uint8_t* proc_cur, const uint8_t* proc_next, const vsc_image* last_stab,
    const vsc_image* flow_fwd, const vsc_image* flow_bwd, const vsc_image* adap_cmb_pr, const vsc_image* consis_wt,
    float alpha, float beta, float gamma, int32_t occlusion_mask, vsc_stream_t stream);

/* Consistency weights gamma*exp(-beta*(I - adapCmbIn)^2), < 0.001 -> 0.
 * Replaces get_consist_wt / kernel_consist_wt (flowconsistency.cu:168-191, :335-348). */
VSC_API vsc_status vsc_get_consist_wt(const vsc_image* adap_cmb_in, const vsc_image* crnt_in,
    const vsc_image* consis_wt, float beta, float gamma, vsc_stream_t stream);

/* Bilinear resample, source coordinate ox*Win/Wout, edge taps clamped.
 * Replaces get_bilinear / kernel_bilinear (flowconsistency.cu:50-75, :288-299). */
VSC_API vsc_status vsc_get_bilinear(const vsc_image* input, const vsc_image* output, vsc_stream_t stream);

/* Bytes of device workspace vsc_get_consist_out needs for a width x height image. */
VSC_API size_t vsc_consist_out_workspace_size(int32_t width, int32_t height);

/* num_iter gradient-descent steps with momentum on the blend energy
 * (Jacobi form; consis_out holds the initial solution and receives the
 * result).  Replaces get_consist_out / kernel_consist_out
 * (flowconsistency.cu:193-258, :350-374).  workspace: device memory of at
 * least vsc_consist_out_workspace_size bytes, or NULL to let the library
 * take it from the stream-ordered memory pool of the current device. */
VSC_API vsc_status vsc_get_consist_out(const vsc_image* crnt_pr, const vsc_image* prev_stab_warp,
    const vsc_image* cons_wt, int32_t num_iter, float step_size, float mom_fac, const vsc_image* consis_out,
    void* workspace, size_t workspace_bytes, vsc_stream_t stream);

/* vsc_get_consist_out in the VSC_SOLVER_FMA form: same arguments; its
 * workspace (vsc_consist_out_fma_workspace_size bytes, 16-byte aligned, or
 * NULL for the library's stream-ordered pool) holds the solve as planes, 18
 * floats a pixel.  Results within the tolerance stated at VSC_SOLVER_FMA of
 * vsc_get_consist_out's.  No counterpart in the reference. */
VSC_API size_t vsc_consist_out_fma_workspace_size(int32_t width, int32_t height);
VSC_API vsc_status vsc_get_consist_out_fma(const vsc_image* crnt_pr, const vsc_image* prev_stab_warp,
    const vsc_image* cons_wt, int32_t num_iter, float step_size, float mom_fac, const vsc_image* consis_out,
    void* workspace, size_t workspace_bytes, vsc_stream_t stream);

/* Largest image (width * height) vsc_get_consist_out_noalloc accepts. */
#define VSC_NOALLOC_MAX_PIXELS 349525u

/* vsc_get_consist_out for callers that must not allocate device memory:
 * code recording a CUDA graph by stream capture, where allocation calls
 * cannot be captured; real-time frame loops, where cudaMalloc or cudaFree
 * can stall on a device-wide synchronisation; and plugins whose host
 * application owns all device memory.  No counterpart in the reference (its
 * get_consist_out allocates two images on every call,
 * flowconsistency.cu:363-365).
 * Same arguments, arithmetic and results as vsc_get_consist_out.  The
 * workspace is a 16 MiB array inside the library (each GPU that loads the
 * library holds it until the process exits), so images are limited to
 * VSC_NOALLOC_MAX_PIXELS pixels (720 x 480 fits); larger ones get VSC_EINVAL.
 * Every call shares that array and leaves its contents behind (nothing in
 * it needs to start at zero), so calls that overlap on the GPU — on two
 * streams, or from two threads — race and must be serialised by the caller.
 * The first call on a device looks up the array's device address (once per
 * device, with that device current; again after a device reset, which gives
 * the device a new context); make that first call before any stream
 * capture. */
VSC_API vsc_status vsc_get_consist_out_noalloc(const vsc_image* crnt_pr, const vsc_image* prev_stab_warp,
    const vsc_image* cons_wt, int32_t num_iter, float step_size, float mom_fac, const vsc_image* consis_out,
    vsc_stream_t stream);

/* ========================================================================
 * Per-frame orchestrator (src/stabilization/videostabilizer.{h,cpp})
 * ======================================================================== */

/* Mirrors hyperParams (videostabilizer.h:38-46). */
typedef struct vsc_hyper_params {
    float alpha;
    float beta;
    float gamma;
    int32_t pyramid_levels;
    int32_t num_iter;
    float step_size;
    float mom_fac;
} vsc_hyper_params;

/* VideoStabilizer::initHyperParams defaults (videostabilizer.cpp:104-112). */
VSC_API void vsc_default_hyper_params(vsc_hyper_params* hp);

typedef struct vsc_stabilizer vsc_stabilizer;

typedef struct vsc_stabilizer_config {
    int32_t width;
    int32_t height;
    int32_t batch_size;     /* flow batch (-b); this build supports 1 */
    int32_t compute_flow;   /* 1: flows computed from the original frames by the
                               library's flow estimator (built on the two ops);
                               0: flows supplied with vsc_stabilizer_set_flows */
    int32_t flow_downscale; /* FLOWDOWNSCALE (videostabilizer.cpp:74-98); 1 = full size */
    int32_t flow_channels;  /* channels (2 or 3) of supplied flows when compute_flow = 0 */
    int32_t use_graphs;     /* 1: after the first step, each step replays a CUDA graph
                               captured on first use (needs a non-default stream);
                               the graph is re-captured when the hyper-parameters or
                               the device output pointer change; steps run without
                               a graph while stage timing is on */
    int32_t corr_dtype;     /* operand type of the flow estimator's correlations:
                               VSC_DTYPE_F32 (0, the plain method), VSC_DTYPE_BF16 or
                               VSC_DTYPE_F16 (tensor cores, FP32 accumulation); the
                               warps, mask and blend stay FP32 */
} vsc_stabilizer_config;

/* Replaces the VideoStabilizer constructor (videostabilizer.cpp:46-102).
 * All device memory is allocated here, once; the stream is used for every
 * later call on this stabilizer. */
VSC_API vsc_status vsc_stabilizer_create(const vsc_stabilizer_config* cfg, vsc_stream_t stream,
    vsc_stabilizer** out);
VSC_API vsc_status vsc_stabilizer_destroy(vsc_stabilizer* s);

/* The live hyper-parameters (getHyperParams, videostabilizer.h:110). */
VSC_API vsc_hyper_params* vsc_stabilizer_hyper_params(vsc_stabilizer* s);

/* Append frame i to the window (loadFrame + imageToGPU, stabilizefiles.cpp:72-96):
 * RGBA8 original and per-frame processed images, width x height x 4, on the
 * host (on_device = 0) or device.  Pageable host frames are copied before the
 * call returns; pinned host frames and device frames are read asynchronously
 * (host frames on a copy stream of the stabilizer, so the upload overlaps the
 * work already enqueued; the stabilizer's stream waits for it), so keep them
 * unchanged until the stabilizer's stream has passed the load (a later
 * vsc_stabilizer_step with a synchronous host output, or
 * vsc_stabilizer_synchronize). */
VSC_API vsc_status vsc_stabilizer_load_frame(vsc_stabilizer* s, const uint8_t* orig_rgba, const uint8_t* proc_rgba,
    int32_t on_device);

/* Flows for the next step when compute_flow = 0 (FileStabilizer::retrieveOpticalFlow,
 * stabilizefiles.cpp:134-149): fwd = flow of frame t to t+1, bwd = flow of t to t-1,
 * width x height x flow_channels float, host or device. */
VSC_API vsc_status vsc_stabilizer_set_flows(vsc_stabilizer* s, const float* fwd, const float* bwd,
    int32_t on_device);

/* One frame: doOneStep (videostabilizer.cpp:167-265) for the middle frame of
 * the 3-frame window; writes its RGBA8 stabilized image to out_rgba, keeps
 * the FP32 result as the next step's previous stabilized frame, and drops
 * the oldest frame from the window.  out_on_device: 1 = device pointer
 * (stream-ordered); 0 = host pointer, copied before the call returns;
 * VSC_OUT_HOST_ASYNC = host pointer, the copy is enqueued and the call
 * returns at once: read out_rgba after vsc_stabilizer_wait_output or
 * vsc_stabilizer_synchronize.  Host copies run on a download stream of the
 * stabilizer from one of two device buffers that alternate, so with
 * page-locked memory a copy overlaps the caller's next load_frame and step. */
#define VSC_OUT_HOST_ASYNC 2
VSC_API vsc_status vsc_stabilizer_step(vsc_stabilizer* s, uint8_t* out_rgba, int32_t out_on_device);
/* Waits for the host copy of the last step with a host output (which = 0) or
 * of the one before it (which = 1); no-op if there was none. */
VSC_API vsc_status vsc_stabilizer_wait_output(vsc_stabilizer* s, int32_t which);
/* Waits until everything enqueued by the stabilizer (steps, loads, host
 * copies) has finished. */
VSC_API vsc_status vsc_stabilizer_synchronize(vsc_stabilizer* s);

/* Device pointers to internal state, for inspection (valid until the next call):
 * which = 0: last stabilized frame (float HWC3), 1: forward flow, 2: backward flow
 * (float HWC, 3 channels when computed), 3: adapCmbPr, 4: consWt.  With
 * flow_downscale > 1 and bilinear upsampling (no learned upsampler, no
 * occlusion mask) a step's front pass samples the coarse flows directly; the
 * first request for 1 or 2 after such a step upsamples them (the values the
 * step used) and waits for the stabilizer's stream. */
VSC_API vsc_status vsc_stabilizer_buffer(vsc_stabilizer* s, int32_t which, const float** dev_ptr);

/* Number of kernels the last vsc_stabilizer_step (or load_frame) enqueued. */
VSC_API int32_t vsc_stabilizer_last_launches(vsc_stabilizer* s);

/* Per-stage device timing, the counterpart of the reference's load / optflow /
 * stabilize accumulators (videostabilizer.h:72-76, stabilizefiles.cpp:121-128).
 * Off by default; when on, CUDA events are recorded between the stages. */
/* Opt-in (off by default; no counterpart in the reference): apply the
 * forward-backward flow consistency mask of vsc_get_flow_consistency_mask to
 * the temporal weights of every following step. */
VSC_API vsc_status vsc_stabilizer_set_occlusion_mask(vsc_stabilizer* s, int32_t on);

/* The solver form of every following step: VSC_SOLVER_EXACT (the default,
 * the reference's arithmetic) or VSC_SOLVER_FMA (see there).  Tunes the
 * form's tile shape for the pyramid's sizes on the stabilizer's stream
 * (synchronising it) unless the stream is being captured.  No counterpart
 * in the reference. */
VSC_API vsc_status vsc_stabilizer_set_solver_form(vsc_stabilizer* s, int32_t form);

VSC_API vsc_status vsc_stabilizer_enable_timing(vsc_stabilizer* s, int32_t on);
/* ms[0] last load_frame (upload, conversion, flow features), ms[1] flow
 * (forward + backward), ms[2] warps + adaptive combination + consistency
 * weights + pyramid, ms[3] coarse pyramid levels of the solve, ms[4]
 * full-resolution solve and RGBA8 output; n >= 5.  Synchronises the stream. */
VSC_API vsc_status vsc_stabilizer_stage_ms(vsc_stabilizer* s, float* ms, int32_t n);

/* ---- learned flow upsampler (no counterpart in the reference) ----------------
 * For the FLOWDOWNSCALE = 2 fast mode: a 4-layer 3x3 convolutional net
 * (3 -> 32 -> 32 -> 32 -> 2 channels, ReLU between, 19,970 parameters)
 * predicts a residual r on top of the bilinearly upsampled coarse flow with
 * its vectors scaled to the full-resolution grid ("base"), from the base
 * flow and the frame's luma; output = base + r where max(|r_u|, |r_v|) <=
 * the maximum residual (0.5 px by default), else base.  Trained by
 * vsc_upsampler_train_step (L1 loss against the full-resolution flow, Adam);
 * inference rounds the weights to FP16.  Parameter order: per layer the
 * weights [out][ky][kx][in], then the biases. */
typedef struct vsc_upsampler vsc_upsampler;
VSC_API int32_t vsc_upsampler_param_count(void);
/* params: host array of vsc_upsampler_param_count floats, or NULL for a
 * seeded initialisation (the last layer near zero: output = base). */
VSC_API vsc_status vsc_upsampler_create(const float* params, vsc_upsampler** out);
VSC_API vsc_status vsc_upsampler_destroy(vsc_upsampler* u);
VSC_API vsc_status vsc_upsampler_get_params(vsc_upsampler* u, float* host_params);
VSC_API vsc_status vsc_upsampler_set_max_residual(vsc_upsampler* u, float px);
/* input (frame size, 3 channels): base u, base v, luma. */
VSC_API vsc_status vsc_upsampler_prepare(const vsc_image* coarse_flow, const vsc_image* frame, const vsc_image* input,
    vsc_stream_t stream);
/* One Adam step on a batch: input n x h x w x 3 (from vsc_upsampler_prepare),
 * target n x h x w x 2 (the full-resolution flow), device pointers; the
 * batch's mean L1 loss in *loss_out (synchronises) when non-null. */
VSC_API vsc_status vsc_upsampler_train_step(vsc_upsampler* u, const float* input, const float* target, int32_t n,
    int32_t h, int32_t w, float lr, float* loss_out, vsc_stream_t stream);
/* flow_out (frame size, 3 channels (u, v, 0)) from a coarse flow and the frame. */
VSC_API vsc_status vsc_upsampler_apply(vsc_upsampler* u, const vsc_image* coarse_flow, const vsc_image* frame,
    const vsc_image* flow_out, vsc_stream_t stream);
/* Use u instead of bilinear upsampling in a stabilizer with flow_downscale > 1
 * (NULL: back to bilinear, the reference's fast mode). */
VSC_API vsc_status vsc_stabilizer_set_upsampler(vsc_stabilizer* s, vsc_upsampler* u);

/* ---- several streams per frame step (no counterpart in the reference) -------
 * Stabilizes n independent videos of any sizes in lockstep: each step runs
 * every stream's doOneStep.  Each video's flows, warps, combination and
 * pyramid run on a CUDA stream of its own, forked from `stream`; the solves
 * are grouped: per pyramid level, each launch of the persistent solver
 * kernel (8 Jacobi steps) walks the tiles of every video's image, so one
 * launch sequence on `stream` solves all videos (up to 16 per launch), with
 * the tile shape autotuned at creation for the list of sizes.  From the
 * second step on the whole step is replayed as one CUDA graph (captured once
 * per window position).  Flows are computed by the library (compute_flow =
 * 1); every stream shares the hyper-parameters of
 * vsc_multistream_hyper_params.  Results equal those of independent
 * stabilizers bit for bit, grouped or not. */
typedef struct vsc_stream_desc {
    int32_t width, height;
    int32_t flow_downscale; /* 0 or 1: none */
    int32_t corr_dtype;     /* as vsc_stabilizer_config.corr_dtype */
} vsc_stream_desc;
typedef struct vsc_multistream vsc_multistream;

VSC_API vsc_status vsc_multistream_create(const vsc_stream_desc* streams, int32_t n, vsc_stream_t stream,
    vsc_multistream** out);
VSC_API vsc_status vsc_multistream_destroy(vsc_multistream* m);
VSC_API vsc_hyper_params* vsc_multistream_hyper_params(vsc_multistream* m);
/* One frame per stream: orig[i], proc[i] RGBA8 of stream i's size. */
VSC_API vsc_status vsc_multistream_load_frames(vsc_multistream* m, const uint8_t* const* orig,
    const uint8_t* const* proc, int32_t on_device);
/* out[i]: stream i's stabilized RGBA8 frame (NULL entries skip the copy). */
VSC_API vsc_status vsc_multistream_step(vsc_multistream* m, uint8_t* const* out, int32_t out_on_device);
VSC_API int32_t vsc_multistream_last_launches(vsc_multistream* m);
/* Grouped solves on (default) or off (each video's solve on its own CUDA
 * stream, as a lone stabilizer runs it).  Grouping needs every pyramid
 * level's width to be a multiple of 4; otherwise the step runs ungrouped.
 * vsc_multistream_fused: 1 if a step with the current hyper-parameters runs
 * grouped. */
VSC_API vsc_status vsc_multistream_set_fused(vsc_multistream* m, int32_t on);
VSC_API int32_t vsc_multistream_fused(vsc_multistream* m);
/* The solver form (VSC_SOLVER_EXACT or VSC_SOLVER_FMA) of every stream's
 * solves, grouped or not; tunes the form's tile shapes (synchronises the
 * multistream's stream).  No counterpart in the reference. */
VSC_API vsc_status vsc_multistream_set_solver_form(vsc_multistream* m, int32_t form);
/* The learned flow upsampler for stream `index` (-1: every stream created
 * with flow_downscale > 1), as vsc_stabilizer_set_upsampler; NULL: bilinear.
 * Synchronises `stream`. */
VSC_API vsc_status vsc_multistream_set_upsampler(vsc_multistream* m, int32_t index, vsc_upsampler* u);

/* ---- frame directories (FileStabilizer, stabilizefiles.cpp:37-149) ----------
 * Image files: PNG (8-bit gray, gray+alpha, RGB or RGBA, not interlaced),
 * binary PPM (P6, maxval 255) and baseline JPEG (sequential DCT, Huffman
 * coding, 8-bit, grey or YCbCr, any sampling factors, restart markers; as the
 * reference reads *.jpg through Qt; progressive JPEG is VSC_EUNSUPPORTED),
 * read into RGBA8 host buffers (alpha 255 where the file has none).  A JPEG
 * decoder's output is not fixed by the standard: pixels can differ by a few
 * levels from another decoder's.  Flow files: Middlebury .flo (flowIO.cpp). */
VSC_API vsc_status vsc_image_file_info(const char* path, int32_t* width, int32_t* height);
VSC_API vsc_status vsc_read_image_file(const char* path, uint8_t* rgba, int32_t width, int32_t height);
/* Writes an 8-bit RGB PNG (the alpha of rgba is dropped). */
VSC_API vsc_status vsc_write_png(const char* path, const uint8_t* rgba, int32_t width, int32_t height);
VSC_API vsc_status vsc_flo_info(const char* path, int32_t* width, int32_t* height);
/* flow: width x height x 2 floats (u, v); the file must have exactly that
 * size (initializeFlowImage, imagehelpers.cpp:42-50). */
VSC_API vsc_status vsc_read_flo(const char* path, float* flow, int32_t width, int32_t height);
VSC_API vsc_status vsc_write_flo(const char* path, const float* flow, int32_t width, int32_t height);

/* Writes width x height RGBA8 (alpha ignored) as a baseline JFIF JPEG:
 * quality 1..100 scales the standard's example quantisation tables as the
 * IJG library does; flags bit 0: 4:4:4 chroma (else 4:2:0), bit 1: a
 * restart marker after every MCU row, bit 2: one grey component (the
 * luma).  Replaces the reference's
 * QImage::save(".jpg") of its output frames (stabilizefiles.cpp:104-106). */
VSC_API vsc_status vsc_write_jpeg(const char* path, const uint8_t* rgba, int32_t width, int32_t height,
    int32_t quality, int32_t flags);

typedef struct vsc_files_config {
    const char* original_dir;  /* original frames, *.png / *.jpg / *.jpeg / *.ppm in name order */
    const char* processed_dir; /* per-frame processed frames, same count */
    const char* output_dir;    /* created if missing; receives 000000.png ... */
    const char* flow_dir;      /* NULL: flows computed by the library; else
                                  frame_<i+1>.flo (i -> i+1) and frame_<i>_bwd.flo
                                  (i -> i-1) per frame i, six-digit indices (-f) */
    int32_t width, height;     /* frames are resized (nearest) to this size;
                                  0: the first original frame's size */
    int32_t flow_downscale;    /* FLOWDOWNSCALE, computed flows only; 0 or 1 = none */
    int32_t corr_dtype;        /* vsc_stabilizer_config.corr_dtype */
    const vsc_hyper_params* hyper; /* NULL: the defaults */
    int32_t jpeg_quality;      /* 0: PNG outputs (lossless); 1..100: .jpg outputs at
                                  that quality, as the reference writes its frames
                                  (QImage::save, stabilizefiles.cpp:104-106; Qt's
                                  default quality is 75) */
} vsc_files_config;

/* Stabilizes every frame of the directories: frame 0 is the processed frame,
 * frames 1 .. n-2 the stabilized ones, frame n-1 the processed frame again
 * (preloadProcessedFrames / outputFinalFrames), all written through the
 * float conversion and back as the reference's gpuToImage does.  Needs at
 * least three frames.  frames_written (optional) receives the count. */
VSC_API vsc_status vsc_stabilize_files(const vsc_files_config* cfg, int32_t* frames_written);

#ifdef __cplusplus
}
#endif

#endif /* VSC_H */
