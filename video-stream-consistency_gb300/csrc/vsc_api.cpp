// C ABI of the library (declared in include/vsc.h): argument validation,
// error reporting, workspace handling and the per-frame orchestrator.
//
// The orchestrator mirrors VideoStabilizer (src/stabilization/
// videostabilizer.{h,cpp}) without Qt: a 3-frame window (k = 1, batch 1) of
// original and processed frames kept on the device as float HWC3, flows
// either computed by the library's estimator or supplied by the caller, the
// FP32 feedback of the previous stabilized frame, and the multi-scale solve.
// All device memory is allocated once at creation; a step enqueues its
// kernels on the stabilizer's stream and synchronises only when the caller
// asked for the result in host memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "vsc_internal.h"

static_assert(VSC_NOALLOC_MAX_PIXELS == vsc::kNoAllocMaxPixels, "header limit out of date");

namespace vsc {

namespace {
thread_local std::string g_err;
}

void clear_error() { g_err.clear(); }

vsc_status set_error(vsc_status st, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

vsc_status check_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess)
        return VSC_OK;
    cudaGetLastError();  // clear a sticky launch-configuration error
    return set_error(e == cudaErrorMemoryAllocation ? VSC_ENOMEM : VSC_ECUDA, "%s: %s (%d)", what,
        cudaGetErrorString(e), static_cast<int>(e));
}

namespace {

constexpr int64_t kMaxDim = 1 << 16;

bool dims_ok(int64_t v) { return v > 0 && v <= kMaxDim; }

vsc_status check_image(const vsc_image* im, const char* name, int channels_lo, int channels_hi)
{
    if (!im)
        return set_error(VSC_EINVAL, "%s: null image descriptor", name);
    if (!im->data)
        return set_error(VSC_EINVAL, "%s: null data pointer", name);
    if (!dims_ok(im->width) || !dims_ok(im->height))
        return set_error(VSC_EINVAL, "%s: invalid size %dx%d", name, im->width, im->height);
    if (im->channels < channels_lo || im->channels > channels_hi)
        return set_error(VSC_EINVAL, "%s: %d channels (expected %d..%d)", name, im->channels, channels_lo,
            channels_hi);
    return VSC_OK;
}

vsc_status same_size(const vsc_image* a, const vsc_image* b, const char* name)
{
    if (a->width != b->width || a->height != b->height)
        return set_error(VSC_EINVAL, "%s: size %dx%d differs from %dx%d", name, b->width, b->height, a->width,
            a->height);
    return VSC_OK;
}

Img img(const vsc_image* i) { return Img{i->data, i->width, i->height, i->channels}; }

cudaStream_t cs(vsc_stream_t s) { return static_cast<cudaStream_t>(s); }

// Private stream-ordered pool per device for workspaces the caller did not provide.
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t st)
{
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= 64)
        return cudaErrorInvalidDevice;
    cudaMemPool_t pool;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!pools[dev]) {
            cudaMemPoolProps props;
            std::memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            e = cudaMemPoolCreate(&pools[dev], &props);
            if (e != cudaSuccess)
                return e;
            uint64_t keep = ~0ULL;
            cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

}  // namespace
}  // namespace vsc

using namespace vsc;

extern "C" {

VSC_API const char* vsc_last_error(void) { return vsc::g_err.c_str(); }

VSC_API int vsc_version(void) { return 100; }

// ---- ops ------------------------------------------------------------------

VSC_API vsc_status vsc_correlation_fwd(const float* f1, const float* f2, float* out, int64_t N, int64_t C, int64_t H,
    int64_t W, int64_t max_displacement, int64_t legacy, vsc_stream_t stream)
{
    clear_error();
    if (!f1 || !f2 || !out)
        return set_error(VSC_EINVAL, "correlation: null pointer");
    if (!dims_ok(N) || !dims_ok(C) || !dims_ok(H) || !dims_ok(W))
        return set_error(VSC_EINVAL, "correlation: invalid shape %lldx%lldx%lldx%lld", (long long)N, (long long)C,
            (long long)H, (long long)W);
    if (max_displacement < 0 || max_displacement > 32)
        return set_error(VSC_EINVAL, "correlation: max_displacement %lld outside [0, 32]", (long long)max_displacement);
    if (legacy != 0 && legacy != 1)
        return set_error(VSC_EINVAL, "correlation: legacy must be 0 or 1");
    if (N > 65535 || H * W > (int64_t(1) << 31) / 4)
        return set_error(VSC_EINVAL, "correlation: shape too large");
    return check_cuda(launch_correlation(f1, f2, out, (int)N, (int)C, (int)H, (int)W, (int)max_displacement,
                          (int)legacy, cs(stream)),
        "correlation launch");
}

VSC_API vsc_status vsc_warp_fwd(const float* input, const float* flow, float* out, int64_t N, int64_t C, int64_t H,
    int64_t W, vsc_stream_t stream)
{
    clear_error();
    if (!input || !flow || !out)
        return set_error(VSC_EINVAL, "warp: null pointer");
    if (!dims_ok(N) || !dims_ok(C) || !dims_ok(H) || !dims_ok(W))
        return set_error(VSC_EINVAL, "warp: invalid shape %lldx%lldx%lldx%lld", (long long)N, (long long)C,
            (long long)H, (long long)W);
    if (N > 65535 || (C + 7) / 8 > 65535 || H * W > (int64_t(1) << 31))
        return set_error(VSC_EINVAL, "warp: shape too large");
    return check_cuda(launch_warp_op(input, flow, out, (int)N, (int)C, (int)H, (int)W, cs(stream)), "warp launch");
}

VSC_API size_t vsc_correlation_lowp_workspace_size(int64_t N, int64_t C, int64_t H, int64_t W)
{
    if (!dims_ok(N) || !dims_ok(C) || !dims_ok(H) || !dims_ok(W))
        return 0;
    return corr_tc_workspace_bytes(static_cast<int>(N), static_cast<int>(C), static_cast<int>(H), static_cast<int>(W));
}

VSC_API vsc_status vsc_correlation_fwd_lowp(const float* f1, const float* f2, float* out, int64_t N, int64_t C,
    int64_t H, int64_t W, int64_t max_displacement, int32_t dtype, void* workspace, size_t workspace_bytes,
    vsc_stream_t stream)
{
    clear_error();
    if (!f1 || !f2 || !out)
        return set_error(VSC_EINVAL, "correlation_lowp: null pointer");
    if (!dims_ok(N) || !dims_ok(C) || !dims_ok(H) || !dims_ok(W))
        return set_error(VSC_EINVAL, "correlation_lowp: invalid shape %lldx%lldx%lldx%lld", (long long)N, (long long)C,
            (long long)H, (long long)W);
    if (dtype != VSC_DTYPE_BF16 && dtype != VSC_DTYPE_F16)
        return set_error(VSC_EINVAL, "correlation_lowp: dtype must be VSC_DTYPE_BF16 or VSC_DTYPE_F16");
    if (max_displacement < 0 || max_displacement > kTcMaxMd)
        return set_error(VSC_EUNSUPPORTED, "correlation_lowp: max_displacement %lld outside [0, %d]",
            (long long)max_displacement, kTcMaxMd);
    if (tc_padded_channels(static_cast<int>(C)) > kTcMaxChannelsPadded)
        return set_error(VSC_EUNSUPPORTED, "correlation_lowp: %lld channels, at most %d", (long long)C,
            kTcMaxChannelsPadded);
    if (N > 65535 || H > 65535 || H * W > (int64_t(1) << 31) / 4)
        return set_error(VSC_EINVAL, "correlation_lowp: shape too large");
    const size_t need = corr_tc_workspace_bytes((int)N, (int)C, (int)H, (int)W);
    void* ws = workspace;
    bool pooled = false;
    vsc_status s;
    if (ws) {
        if (workspace_bytes < need)
            return set_error(VSC_ENOMEM, "correlation_lowp: workspace of %zu bytes, need %zu", workspace_bytes, need);
        if (reinterpret_cast<uintptr_t>(ws) & 255)
            return set_error(VSC_EINVAL, "correlation_lowp: workspace not 256-byte aligned");
    } else {
        if ((s = check_cuda(pool_alloc(&ws, need, cs(stream)), "correlation_lowp workspace")))
            return s;
        pooled = true;
    }
    cudaError_t e = launch_corr_tc(f1, f2, out, (int)N, (int)C, (int)H, (int)W, (int)max_displacement,
        dtype == VSC_DTYPE_BF16, ws, cs(stream));
    if (pooled)
        cudaFreeAsync(ws, cs(stream));
    return check_cuda(e, "correlation_lowp launch");
}

VSC_API vsc_status vsc_correlation_fwd_f64(const double* f1, const double* f2, double* out, int64_t N, int64_t C,
    int64_t H, int64_t W, int64_t max_displacement, vsc_stream_t stream)
{
    clear_error();
    if (!f1 || !f2 || !out)
        return set_error(VSC_EINVAL, "correlation_f64: null pointer");
    if (!dims_ok(N) || !dims_ok(C) || !dims_ok(H) || !dims_ok(W))
        return set_error(VSC_EINVAL, "correlation_f64: invalid shape %lldx%lldx%lldx%lld", (long long)N, (long long)C,
            (long long)H, (long long)W);
    if (max_displacement < 0 || max_displacement > 32)
        return set_error(VSC_EINVAL, "correlation_f64: max_displacement %lld outside [0, 32]",
            (long long)max_displacement);
    if (N > 65535 || H * W > (int64_t(1) << 31))
        return set_error(VSC_EINVAL, "correlation_f64: shape too large");
    return check_cuda(launch_correlation_f64(f1, f2, out, (int)N, (int)C, (int)H, (int)W, (int)max_displacement,
                          cs(stream)),
        "correlation_f64 launch");
}

VSC_API vsc_status vsc_warp_fwd_f64(const double* input, const double* flow, double* out, int64_t N, int64_t C,
    int64_t H, int64_t W, vsc_stream_t stream)
{
    clear_error();
    if (!input || !flow || !out)
        return set_error(VSC_EINVAL, "warp_f64: null pointer");
    if (!dims_ok(N) || !dims_ok(C) || !dims_ok(H) || !dims_ok(W))
        return set_error(VSC_EINVAL, "warp_f64: invalid shape %lldx%lldx%lldx%lld", (long long)N, (long long)C,
            (long long)H, (long long)W);
    if (N > 65535 || H * W > (int64_t(1) << 31))
        return set_error(VSC_EINVAL, "warp_f64: shape too large");
    return check_cuda(launch_warp_op_f64(input, flow, out, (int)N, (int)C, (int)H, (int)W, cs(stream)),
        "warp_f64 launch");
}

// ---- stabilization kernels -------------------------------------------------

VSC_API vsc_status vsc_char_to_float_image(const uint8_t* rgba, const vsc_image* out, vsc_stream_t stream)
{
    clear_error();
    vsc_status s = check_image(out, "out", 3, 3);
    if (s)
        return s;
    if (!rgba || (reinterpret_cast<uintptr_t>(rgba) & 3))
        return set_error(VSC_EINVAL, "rgba: null or not 4-byte aligned");
    return check_cuda(launch_rgba_to_float(rgba, out->data, (int64_t)out->width * out->height, cs(stream)),
        "to_float launch");
}

VSC_API vsc_status vsc_float_to_char_image(const vsc_image* in, uint8_t* rgba, vsc_stream_t stream)
{
    clear_error();
    vsc_status s = check_image(in, "in", 3, 3);
    if (s)
        return s;
    if (!rgba || (reinterpret_cast<uintptr_t>(rgba) & 3))
        return set_error(VSC_EINVAL, "rgba: null or not 4-byte aligned");
    return check_cuda(launch_float_to_rgba(in->data, rgba, (int64_t)in->width * in->height, cs(stream)),
        "to_char launch");
}

VSC_API vsc_status vsc_get_warp_result(const vsc_image* input, const vsc_image* flow, const vsc_image* input_warp,
    vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if ((s = check_image(input, "input", 3, 3)) || (s = check_image(flow, "flow", 2, 3)) ||
        (s = check_image(input_warp, "input_warp", 3, 3)) || (s = same_size(input, flow, "flow")) ||
        (s = same_size(input, input_warp, "input_warp")))
        return s;
    if (input->width < 2 || input->height < 2)
        return set_error(VSC_EINVAL, "warp_result: image must be at least 2x2");
    return check_cuda(launch_stab_warp(img(input), img(flow), img(input_warp), cs(stream)), "warp_result launch");
}

namespace {
vsc_status adap_comb_impl(const vsc_image* crnt_in, const vsc_image* crnt_pr, const vsc_image* prev_warp_in,
    const vsc_image* prev_warp_pr, const vsc_image* next_warp_in, const vsc_image* next_warp_pr,
    const vsc_image* adap_cmb_in, const vsc_image* adap_cmb_pr, const vsc_image* last_stab_warp,
    const vsc_image* occ_mask, float alpha, vsc_stream_t stream)
{
    clear_error();
    if (occ_mask) {
        vsc_status s;
        if ((s = check_image(occ_mask, "occMask", 2, 2)) || (s = check_image(crnt_in, "crntIn", 3, 3)) ||
            (s = same_size(crnt_in, occ_mask, "occMask")))
            return s;
    }
    const vsc_image* all[9] = {crnt_in, crnt_pr, prev_warp_in, prev_warp_pr, next_warp_in, next_warp_pr, adap_cmb_in,
        adap_cmb_pr, last_stab_warp};
    static const char* names[9] = {"crntIn", "crntPr", "prevWarpIn", "prevWarpPr", "nextWarpIn", "nextWarpPr",
        "adapCmbIn", "adapCmbPr", "lastStabWarp"};
    for (int i = 0; i < 9; ++i) {
        vsc_status s = check_image(all[i], names[i], 3, 3);
        if (s)
            return s;
        if ((s = same_size(crnt_in, all[i], names[i])))
            return s;
    }
    return check_cuda(launch_adap_comb(img(crnt_in), img(crnt_pr), img(prev_warp_in), img(prev_warp_pr),
                          img(next_warp_in), img(next_warp_pr), img(adap_cmb_in), img(adap_cmb_pr),
                          img(last_stab_warp), alpha, cs(stream), occ_mask ? occ_mask->data : nullptr),
        "adap_comb launch");
}
}  // namespace

VSC_API vsc_status vsc_get_adap_comb(const vsc_image* crnt_in, const vsc_image* crnt_pr, const vsc_image* prev_warp_in,
    const vsc_image* prev_warp_pr, const vsc_image* next_warp_in, const vsc_image* next_warp_pr,
    const vsc_image* adap_cmb_in, const vsc_image* adap_cmb_pr, const vsc_image* last_stab_warp, float alpha,
    vsc_stream_t stream)
{
    return adap_comb_impl(crnt_in, crnt_pr, prev_warp_in, prev_warp_pr, next_warp_in, next_warp_pr, adap_cmb_in,
        adap_cmb_pr, last_stab_warp, nullptr, alpha, stream);
}

VSC_API vsc_status vsc_get_adap_comb_masked(const vsc_image* crnt_in, const vsc_image* crnt_pr,
    const vsc_image* prev_warp_in, const vsc_image* prev_warp_pr, const vsc_image* next_warp_in,
    const vsc_image* next_warp_pr, const vsc_image* adap_cmb_in, const vsc_image* adap_cmb_pr,
    const vsc_image* last_stab_warp, const vsc_image* occ_mask, float alpha, vsc_stream_t stream)
{
    if (!occ_mask) {
        clear_error();
        return set_error(VSC_EINVAL, "adap_comb_masked: null occMask descriptor");
    }
    return adap_comb_impl(crnt_in, crnt_pr, prev_warp_in, prev_warp_pr, next_warp_in, next_warp_pr, adap_cmb_in,
        adap_cmb_pr, last_stab_warp, occ_mask, alpha, stream);
}

VSC_API vsc_status vsc_get_flow_consistency_mask(const vsc_image* flow_fwd, const vsc_image* flow_bwd,
    const vsc_image* occ_mask, vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if ((s = check_image(flow_fwd, "flowFwd", 2, 3)) || (s = check_image(flow_bwd, "flowBwd", 2, 3)) ||
        (s = check_image(occ_mask, "occMask", 2, 2)) || (s = same_size(flow_fwd, flow_bwd, "flowBwd")) ||
        (s = same_size(flow_fwd, occ_mask, "occMask")))
        return s;
    if (flow_fwd->channels != flow_bwd->channels)
        return set_error(VSC_EINVAL, "flow_consistency_mask: flows have %d and %d channels", flow_fwd->channels,
            flow_bwd->channels);
    return check_cuda(launch_flow_consistency(img(flow_fwd), img(flow_bwd), img(occ_mask), cs(stream)),
        "flow_consistency_mask launch");
}

VSC_API vsc_status vsc_flow_estimate(const vsc_image* img_a, const vsc_image* img_b, const vsc_image* flow_ab,
    const vsc_image* flow_ba, vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if ((s = check_image(img_a, "imgA", 3, 3)) || (s = check_image(img_b, "imgB", 3, 3)) ||
        (s = check_image(flow_ab, "flowAB", 3, 3)) || (s = check_image(flow_ba, "flowBA", 3, 3)) ||
        (s = same_size(img_a, img_b, "imgB")) || (s = same_size(img_a, flow_ab, "flowAB")) ||
        (s = same_size(img_a, flow_ba, "flowBA")))
        return s;
    const int w = img_a->width, h = img_a->height;
    if (w < 8 || h < 8)
        return set_error(VSC_EINVAL, "flow_estimate: image must be at least 8x8");
    cudaStream_t st = cs(stream);
    const FlowDims d = flow_dims(w, h);
    if ((s = check_cuda(flow_upload_weights(), "flow_estimate weights")))
        return s;
    // two feature pyramids (contiguous: the pair addresses them as a strided
    // batch), the feature scratch, the pair's scratch and the two flows
    const size_t nf = d.feat_floats, nfs = flow_feature_scratch_floats(d), nps = 2 * flow_estimate_scratch_floats(d);
    const size_t n3 = static_cast<size_t>(w) * h * 3;
    void* ws = nullptr;
    if ((s = check_cuda(pool_alloc(&ws, (2 * nf + nfs + nps + 2 * n3) * sizeof(float), st), "flow_estimate workspace")))
        return s;
    float* fa = static_cast<float*>(ws);
    float* fb = fa + nf;
    float* fsc = fb + nf;
    float* psc = fsc + nfs;
    float* flows = psc + nps;
    cudaError_t e = launch_flow_features(img_a->data, w, h, d, fa, fsc, st, nullptr);
    if (e == cudaSuccess)
        e = launch_flow_features(img_b->data, w, h, d, fb, fsc, st, nullptr);
    if (e == cudaSuccess)
        e = launch_flow_pair(fa, fb - fa, fb, fa - fb, w, h, d, flows, static_cast<int64_t>(n3), psc, st, nullptr);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(flow_ab->data, flows, n3 * sizeof(float), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(flow_ba->data, flows + n3, n3 * sizeof(float), cudaMemcpyDeviceToDevice, st);
    cudaFreeAsync(ws, st);
    return check_cuda(e, "flow_estimate");
}

VSC_API vsc_status vsc_stab_front(const vsc_image* orig_prev, const vsc_image* orig_cur, const vsc_image* orig_next,
    const vsc_image* proc_prev, const vsc_image* proc_cur, const vsc_image* proc_next, const vsc_image* last_stab,
    const vsc_image* flow_fwd, const vsc_image* flow_bwd, const vsc_image* adap_cmb_pr, const vsc_image* consis_wt,
    float alpha, float beta, float gamma, int32_t occlusion_mask, vsc_stream_t stream)
{
    clear_error();
    const vsc_image* im[9] = {orig_prev, orig_cur, orig_next, proc_prev, proc_cur, proc_next, last_stab, adap_cmb_pr,
        consis_wt};
    static const char* names[9] = {"origPrev", "origCur", "origNext", "procPrev", "procCur", "procNext", "lastStab",
        "adapCmbPr", "consisWt"};
    vsc_status s;
    for (int i = 0; i < 9; ++i)
        if ((s = check_image(im[i], names[i], 3, 3)) || (s = same_size(orig_cur, im[i], names[i])))
            return s;
    if ((s = check_image(flow_fwd, "flowFwd", 2, 3)) || (s = check_image(flow_bwd, "flowBwd", 2, 3)) ||
        (s = same_size(orig_cur, flow_fwd, "flowFwd")) || (s = same_size(orig_cur, flow_bwd, "flowBwd")))
        return s;
    if (flow_fwd->channels != flow_bwd->channels)
        return set_error(VSC_EINVAL, "stab_front: flows have %d and %d channels", flow_fwd->channels,
            flow_bwd->channels);
    if (orig_cur->width < 3 || orig_cur->height < 3)
        return set_error(VSC_EINVAL, "stab_front: image must be at least 3x3");
    return check_cuda(launch_fused_front(orig_prev->data, orig_cur->data, orig_next->data, proc_prev->data,
                          proc_cur->data, proc_next->data, last_stab->data, flow_fwd->data, flow_bwd->data,
                          flow_fwd->channels, adap_cmb_pr->data, consis_wt->data, orig_cur->width, orig_cur->height,
                          alpha, beta, gamma, cs(stream), occlusion_mask != 0),
        "stab_front launch");
}

VSC_API vsc_status vsc_stab_front_rgba(const uint8_t* orig_prev, const uint8_t* orig_cur, const uint8_t* orig_next,
    const uint8_t* proc_prev, const uint8_t* proc_cur, const uint8_t* proc_next, const vsc_image* last_stab,
    const vsc_image* flow_fwd, const vsc_image* flow_bwd, const vsc_image* adap_cmb_pr, const vsc_image* consis_wt,
    float alpha, float beta, float gamma, int32_t occlusion_mask, vsc_stream_t stream)
{
    clear_error();
    const uint8_t* fr[6] = {orig_prev, orig_cur, orig_next, proc_prev, proc_cur, proc_next};
    for (int i = 0; i < 6; ++i) {
        if (!fr[i])
            return set_error(VSC_EINVAL, "stab_front_rgba: frame %d is null", i);
        if (reinterpret_cast<uintptr_t>(fr[i]) & 3)
            return set_error(VSC_EINVAL, "stab_front_rgba: frame %d is not 4-byte aligned", i);
    }
    const vsc_image* im[3] = {last_stab, adap_cmb_pr, consis_wt};
    static const char* names[3] = {"lastStab", "adapCmbPr", "consisWt"};
    vsc_status s;
    for (int i = 0; i < 3; ++i)
        if ((s = check_image(im[i], names[i], 3, 3)) || (s = same_size(last_stab, im[i], names[i])))
            return s;
    if ((s = check_image(flow_fwd, "flowFwd", 2, 3)) || (s = check_image(flow_bwd, "flowBwd", 2, 3)) ||
        (s = same_size(last_stab, flow_fwd, "flowFwd")) || (s = same_size(last_stab, flow_bwd, "flowBwd")))
        return s;
    if (flow_fwd->channels != flow_bwd->channels)
        return set_error(VSC_EINVAL, "stab_front_rgba: flows have %d and %d channels", flow_fwd->channels,
            flow_bwd->channels);
    if (last_stab->width < 3 || last_stab->height < 3)
        return set_error(VSC_EINVAL, "stab_front_rgba: image must be at least 3x3");
    return check_cuda(launch_fused_front_rgba(orig_prev, orig_cur, orig_next, proc_prev, proc_cur, proc_next,
                          last_stab->data, flow_fwd->data, flow_bwd->data, flow_fwd->channels, adap_cmb_pr->data,
                          consis_wt->data, last_stab->width, last_stab->height, alpha, beta, gamma, cs(stream),
                          occlusion_mask != 0),
        "stab_front_rgba launch");
}

VSC_API vsc_status vsc_get_consist_wt(const vsc_image* adap_cmb_in, const vsc_image* crnt_in,
    const vsc_image* consis_wt, float beta, float gamma, vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if ((s = check_image(adap_cmb_in, "adapCmbIn", 3, 3)) || (s = check_image(crnt_in, "crntIn", 3, 3)) ||
        (s = check_image(consis_wt, "consisWt", 3, 3)) || (s = same_size(crnt_in, adap_cmb_in, "adapCmbIn")) ||
        (s = same_size(crnt_in, consis_wt, "consisWt")))
        return s;
    return check_cuda(
        launch_consist_wt(img(adap_cmb_in), img(crnt_in), img(consis_wt), beta, gamma, cs(stream)),
        "consist_wt launch");
}

VSC_API vsc_status vsc_get_bilinear(const vsc_image* input, const vsc_image* output, vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if ((s = check_image(input, "input", 1, 4)) || (s = check_image(output, "output", 1, 4)))
        return s;
    if (input->channels != output->channels)
        return set_error(VSC_EINVAL, "bilinear: channel count differs (%d vs %d)", input->channels,
            output->channels);
    return check_cuda(launch_bilinear(img(input), img(output), cs(stream)), "bilinear launch");
}

VSC_API size_t vsc_consist_out_workspace_size(int32_t width, int32_t height)
{
    if (!dims_ok(width) || !dims_ok(height))
        return 0;
    return solver_workspace_floats(width, height, kSolverExact) * sizeof(float);
}

VSC_API size_t vsc_consist_out_fma_workspace_size(int32_t width, int32_t height)
{
    if (!dims_ok(width) || !dims_ok(height))
        return 0;
    return solver_workspace_floats(width, height, kSolverFma) * sizeof(float);
}

namespace {

vsc_status consist_out_form(int form, const vsc_image* crnt_pr, const vsc_image* prev_stab_warp,
    const vsc_image* cons_wt, int32_t num_iter, float step_size, float mom_fac, const vsc_image* consis_out,
    void* workspace, size_t workspace_bytes, vsc_stream_t stream)
{
    vsc_status s;
    if ((s = check_image(crnt_pr, "crntPr", 3, 3)) || (s = check_image(prev_stab_warp, "prevStabWarp", 3, 3)) ||
        (s = check_image(cons_wt, "consWt", 3, 3)) || (s = check_image(consis_out, "consisOut", 3, 3)) ||
        (s = same_size(consis_out, crnt_pr, "crntPr")) || (s = same_size(consis_out, prev_stab_warp, "prevStabWarp")) ||
        (s = same_size(consis_out, cons_wt, "consWt")))
        return s;
    if (num_iter < 0)
        return set_error(VSC_EINVAL, "consist_out: negative iteration count");
    const int w = consis_out->width, h = consis_out->height;
    const size_t need = solver_workspace_floats(w, h, form) * sizeof(float);
    void* ws = workspace;
    bool pooled = false;
    if (ws) {
        if (workspace_bytes < need)
            return set_error(VSC_ENOMEM, "consist_out: workspace of %zu bytes, need %zu", workspace_bytes, need);
        if (reinterpret_cast<uintptr_t>(ws) & 15)
            return set_error(VSC_EINVAL, "consist_out: workspace not 16-byte aligned");
    } else if (num_iter > 0) {
        if ((s = check_cuda(pool_alloc(&ws, need, cs(stream)), "consist_out workspace")))
            return s;
        pooled = true;
    }
    cudaError_t e = run_solver(crnt_pr->data, prev_stab_warp->data, cons_wt->data, consis_out->data, w, h, num_iter,
        step_size, mom_fac, static_cast<float*>(ws), cs(stream), nullptr, nullptr, form);
    if (pooled)
        cudaFreeAsync(ws, cs(stream));
    return check_cuda(e, "consist_out launch");
}

}  // namespace

VSC_API vsc_status vsc_get_consist_out(const vsc_image* crnt_pr, const vsc_image* prev_stab_warp,
    const vsc_image* cons_wt, int32_t num_iter, float step_size, float mom_fac, const vsc_image* consis_out,
    void* workspace, size_t workspace_bytes, vsc_stream_t stream)
{
    clear_error();
    return consist_out_form(kSolverExact, crnt_pr, prev_stab_warp, cons_wt, num_iter, step_size, mom_fac, consis_out,
        workspace, workspace_bytes, stream);
}

VSC_API vsc_status vsc_get_consist_out_fma(const vsc_image* crnt_pr, const vsc_image* prev_stab_warp,
    const vsc_image* cons_wt, int32_t num_iter, float step_size, float mom_fac, const vsc_image* consis_out,
    void* workspace, size_t workspace_bytes, vsc_stream_t stream)
{
    clear_error();
    return consist_out_form(kSolverFma, crnt_pr, prev_stab_warp, cons_wt, num_iter, step_size, mom_fac, consis_out,
        workspace, workspace_bytes, stream);
}

VSC_API int32_t vsc_solver_steps_per_launch(void) { return solver_steps_per_launch(); }

VSC_API vsc_status vsc_solver_autotune(int32_t width, int32_t height, vsc_stream_t stream, int32_t* tile_rows)
{
    return vsc_solver_autotune_form(width, height, VSC_SOLVER_EXACT, stream, tile_rows);
}

VSC_API vsc_status vsc_solver_autotune_form(int32_t width, int32_t height, int32_t form, vsc_stream_t stream,
    int32_t* tile_rows)
{
    clear_error();
    if (width < 1 || height < 1)
        return set_error(VSC_EINVAL, "solver_autotune: size %dx%d", width, height);
    if (form != VSC_SOLVER_EXACT && form != VSC_SOLVER_FMA)
        return set_error(VSC_EINVAL, "solver_autotune: unknown solver form %d", form);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    vsc_status s = check_cuda(cudaStreamIsCapturing(cs(stream), &cap), "solver_autotune");
    if (s)
        return s;
    if (cap != cudaStreamCaptureStatusNone)
        return set_error(VSC_ESTATE, "solver_autotune: the stream is being captured");
    int rows = 0;
    s = check_cuda(solver_autotune(width, height, cs(stream), &rows, form), "solver_autotune");
    if (!s && tile_rows)
        *tile_rows = rows;
    return s;
}

VSC_API int32_t vsc_solver_tile_rows(int32_t width, int32_t height, int32_t* tuned)
{
    return vsc_solver_tile_rows_form(width, height, VSC_SOLVER_EXACT, tuned);
}

VSC_API int32_t vsc_solver_tile_rows_form(int32_t width, int32_t height, int32_t form, int32_t* tuned)
{
    bool t = false;
    const bool ok = width > 0 && height > 0 && (form == VSC_SOLVER_EXACT || form == VSC_SOLVER_FMA);
    const int rows = ok ? solver_tile_rows(width, height, &t, form) : 0;
    if (tuned)
        *tuned = t ? 1 : 0;
    return rows;
}

VSC_API void vsc_solver_set_autotune(int32_t on) { solver_set_autotune(on != 0); }

VSC_API vsc_status vsc_check_device(void)
{
    clear_error();
    int flagged = 0;
    vsc_status st = check_cuda(check_device_timeout(&flagged), "check_device");
    if (st)
        return st;
    if (flagged)
        return set_error(VSC_ETIMEOUT, "a kernel's bounded wait gave up (its results are invalid)");
    return VSC_OK;
}

VSC_API vsc_status vsc_selftest_bounded_wait(int32_t spins, vsc_stream_t stream)
{
    clear_error();
    if (spins < 1 || spins > (1 << 20))
        return set_error(VSC_EINVAL, "selftest_bounded_wait: spins outside [1, 2^20]");
    return check_cuda(launch_bounded_wait_selftest(spins, cs(stream)), "selftest launch");
}

VSC_API vsc_status vsc_get_consist_out_noalloc(const vsc_image* crnt_pr, const vsc_image* prev_stab_warp,
    const vsc_image* cons_wt, int32_t num_iter, float step_size, float mom_fac, const vsc_image* consis_out,
    vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if ((s = check_image(crnt_pr, "crntPr", 3, 3)) || (s = check_image(prev_stab_warp, "prevStabWarp", 3, 3)) ||
        (s = check_image(cons_wt, "consWt", 3, 3)) || (s = check_image(consis_out, "consisOut", 3, 3)) ||
        (s = same_size(consis_out, crnt_pr, "crntPr")) || (s = same_size(consis_out, prev_stab_warp, "prevStabWarp")) ||
        (s = same_size(consis_out, cons_wt, "consWt")))
        return s;
    if (num_iter < 0)
        return set_error(VSC_EINVAL, "consist_out_noalloc: negative iteration count");
    const int w = consis_out->width, h = consis_out->height;
    const size_t pixels = static_cast<size_t>(w) * h;
    if (pixels > VSC_NOALLOC_MAX_PIXELS)
        return set_error(VSC_EINVAL,
            "consist_out_noalloc: %dx%d image (%zu pixels) exceeds the %zu-pixel limit of the built-in workspace; "
            "use vsc_get_consist_out",
            w, h, pixels, static_cast<size_t>(VSC_NOALLOC_MAX_PIXELS));
    if (num_iter == 0)
        return VSC_OK;
    return check_cuda(run_solver_noalloc(crnt_pr->data, prev_stab_warp->data, cons_wt->data, consis_out->data, w, h,
                          num_iter, step_size, mom_fac, cs(stream)),
        "consist_out_noalloc launch");
}

VSC_API void vsc_default_hyper_params(vsc_hyper_params* hp)
{
    if (!hp)
        return;
    hp->alpha = 6800.0f;
    hp->beta = 6800.0f;
    hp->gamma = 2.0f;
    hp->pyramid_levels = 2;
    hp->num_iter = 150;
    hp->step_size = 0.15f;
    hp->mom_fac = 0.15f;
}

}  // extern "C"

// ---- orchestrator -----------------------------------------------------------

struct vsc_stabilizer {
    int w = 0, h = 0, fc = 3;
    bool compute_flow = true;
    int downscale = 1, fw = 0, fh = 0;  // flow size
    int device = 0;
    cudaStream_t st = nullptr;
    vsc_hyper_params hp{};
    int levels_alloc = 0;

    float* orig[3] = {};
    float* proc[3] = {};
    float* feat[3] = {};
    int head = 0, count = 0;
    bool started = false;
    bool flows_set = false;

    uint8_t* stage[2] = {};  // device staging for host RGBA uploads
    // host uploads run on a copy stream: staged[k] = stage[k] filled,
    // consumed[k] = its conversion done (the next upload into it waits)
    cudaStream_t cst = nullptr;
    cudaEvent_t staged[2] = {}, consumed[2] = {};
    uint8_t* out_rgba = nullptr;    // device copy of a host-destined output (buffer 0 of two)
    uint8_t* out_rgba_b = nullptr;  // buffer 1: a step writes one while the other is copied back
    int out_par = 0;
    // host outputs are copied back on a download stream: step_done orders the copy
    // after its step, d2h_done[p] marks buffer p's copy finished
    cudaStream_t dst = nullptr;
    cudaEvent_t step_done = nullptr, d2h_done[2] = {};
    int d2h_last = -1, d2h_prev = -1;  // buffers of the last two host copies
    float* flow_fwd = nullptr;
    float* flow_bwd = nullptr;
    float* flow_small = nullptr;  // flow at the flow size before upsampling
    float* last_stab[2] = {};
    int ls_cur = 0;
    float* adap_pr = nullptr;
    float* cons_wt = nullptr;
    float* pyrP[8] = {};
    float* pyrA[8] = {};
    float* pyrW[8] = {};
    float* pyrO[8] = {};
    int lw[8] = {}, lh[8] = {};
    float* solver_ws = nullptr;
    float* feat_scratch = nullptr;
    float* flow_scratch = nullptr;
    // tensor-core correlations (corr_dtype BF16 / F16): chunked 16-bit
    // features of the three frames, the warped operand, the operand scales
    int corr_dtype = VSC_DTYPE_F32;
    unsigned char* feat_tc[3] = {};
    unsigned char* warped_tc = nullptr;
    float* tc_scales = nullptr;
    FlowDims fd{};
    int last_launches = 0;
    bool occlusion = false;  // opt-in forward-backward consistency mask
    // the last step's front pass sampled the coarse flows (bilinear
    // FLOWDOWNSCALE): flow_fwd / flow_bwd are upsampled only on request
    bool flows_pending = false;
    int solver_form = kSolverExact;  // VSC_SOLVER_EXACT / VSC_SOLVER_FMA
    // learned flow upsampling (flow_downscale > 1); null: bilinear
    vsc_upsampler* upsampler = nullptr;
    float* up_work = nullptr;  // input (2 x w x h x 3), activations, residual
    // stage timing (off by default): events around load_frame and the stages of a step
    bool timing = false;
    cudaEvent_t ev[7] = {};
    // CUDA graphs of the step, one per ring position / feedback parity /
    // output / hyper-parameters / timing combination
    bool use_graphs = false;
    struct GraphEntry {
        bool valid = false;
        int head = 0, ls_cur = 0, nl = 0;
        uint8_t* rgba = nullptr;
        vsc_hyper_params hp{};
        bool timing = false, occlusion = false;
        int solver_form = kSolverExact;
        const vsc_upsampler* upsampler = nullptr;
        cudaGraphExec_t exec = nullptr;
        uint64_t used = 0;
    } graphs[12];  // 3 ring positions x 2 feedback buffers x 2 output buffers
    uint64_t graph_clock = 0;
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev)
            cudaSetDevice(dev);
        else
            prev = -1;
    }
    ~DeviceGuard()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
};

enum { kEvLoad0, kEvLoad1, kEvStep0, kEvFlow, kEvFront, kEvCoarse, kEvStep1 };

// FLOWDOWNSCALE with bilinear upsampling (flowmodel.cpp:158-161) and no
// occlusion mask: the front pass samples the coarse 3-channel flows where it
// uses them, with the upsampling's expression, instead of reading upsampled
// copies (the same values; the full-size flows are not written).
bool front_samples_small_flows(const vsc_stabilizer* s)
{
    return s->compute_flow && s->downscale > 1 && !s->upsampler && !s->occlusion && s->fc == 3;
}

void mark(vsc_stabilizer* s, int which)
{
    if (s->timing)
        cudaEventRecord(s->ev[which], s->st);
}

template <typename T>
cudaError_t dalloc(T** p, size_t elems)
{
    return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(elems, 1) * sizeof(T));
}

void free_all(vsc_stabilizer* s)
{
    auto f = [](void* p) {
        if (p)
            cudaFree(p);
    };
    for (int i = 0; i < 3; ++i) {
        f(s->orig[i]);
        f(s->proc[i]);
    }
    f(s->feat[0]);
    f(s->stage[0]);
    f(s->stage[1]);
    f(s->out_rgba);
    f(s->out_rgba_b);
    f(s->flow_fwd);
    f(s->flow_small);
    f(s->last_stab[0]);
    f(s->last_stab[1]);
    f(s->adap_pr);
    f(s->cons_wt);
    for (int j = 0; j < 8; ++j) {
        f(s->pyrP[j]);
        f(s->pyrA[j]);
        f(s->pyrW[j]);
        f(s->pyrO[j]);
    }
    f(s->solver_ws);
    f(s->feat_scratch);
    f(s->flow_scratch);
    f(s->feat_tc[0]);
    f(s->warped_tc);
    f(s->tc_scales);
    f(s->up_work);
    for (cudaEvent_t& e : s->ev)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    for (int k = 0; k < 2; ++k) {
        if (s->staged[k])
            cudaEventDestroy(s->staged[k]);
        if (s->consumed[k])
            cudaEventDestroy(s->consumed[k]);
        s->staged[k] = s->consumed[k] = nullptr;
    }
    if (s->cst) {
        cudaStreamDestroy(s->cst);
        s->cst = nullptr;
    }
    for (cudaEvent_t& e : s->d2h_done)
        if (e) {
            cudaEventDestroy(e);
            e = nullptr;
        }
    if (s->step_done) {
        cudaEventDestroy(s->step_done);
        s->step_done = nullptr;
    }
    if (s->dst) {
        cudaStreamDestroy(s->dst);
        s->dst = nullptr;
    }
    for (auto& g : s->graphs)
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
            g.valid = false;
        }
}

vsc_status alloc_all(vsc_stabilizer* s)
{
    const size_t n3 = static_cast<size_t>(s->w) * s->h * 3;
    cudaError_t e = cudaSuccess;
    auto A = [&](cudaError_t r) {
        if (e == cudaSuccess)
            e = r;
    };
    for (int i = 0; i < 3; ++i) {
        A(dalloc(&s->orig[i], n3));
        A(dalloc(&s->proc[i], n3));
    }
    A(dalloc(&s->stage[0], static_cast<size_t>(s->w) * s->h * 4));
    A(dalloc(&s->stage[1], static_cast<size_t>(s->w) * s->h * 4));
    A(cudaStreamCreateWithFlags(&s->cst, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
        A(cudaEventCreateWithFlags(&s->staged[k], cudaEventDisableTiming));
        A(cudaEventCreateWithFlags(&s->consumed[k], cudaEventDisableTiming));
    }
    A(dalloc(&s->out_rgba, static_cast<size_t>(s->w) * s->h * 4));
    A(dalloc(&s->out_rgba_b, static_cast<size_t>(s->w) * s->h * 4));
    A(cudaStreamCreateWithFlags(&s->dst, cudaStreamNonBlocking));
    A(cudaEventCreateWithFlags(&s->step_done, cudaEventDisableTiming));
    for (int k = 0; k < 2; ++k)
        A(cudaEventCreateWithFlags(&s->d2h_done[k], cudaEventDisableTiming));
    // forward and backward flow contiguous: the estimator writes both in one launch
    A(dalloc(&s->flow_fwd, 2 * static_cast<size_t>(s->w) * s->h * s->fc));
    if (e == cudaSuccess)
        s->flow_bwd = s->flow_fwd + static_cast<size_t>(s->w) * s->h * s->fc;
    A(dalloc(&s->last_stab[0], n3));
    A(dalloc(&s->last_stab[1], n3));
    A(dalloc(&s->adap_pr, n3));
    A(dalloc(&s->cons_wt, n3));
    s->levels_alloc = 8;
    s->lw[0] = s->w;
    s->lh[0] = s->h;
    for (int j = 1; j < 8; ++j) {
        s->lw[j] = s->lw[j - 1] / 2;
        s->lh[j] = s->lh[j - 1] / 2;
    }
    for (int j = 1; j < 8; ++j) {
        if (s->lw[j] < 2 || s->lh[j] < 2) {
            s->levels_alloc = j;
            break;
        }
        const size_t m = static_cast<size_t>(s->lw[j]) * s->lh[j] * 3;
        A(dalloc(&s->pyrP[j], m));
        A(dalloc(&s->pyrA[j], m));
        A(dalloc(&s->pyrW[j], m));
        A(dalloc(&s->pyrO[j], m));
    }
    A(dalloc(&s->solver_ws, solver_workspace_floats(s->w, s->h, kSolverFma)));  // room for either form
    if (s->compute_flow) {
        s->fd = flow_dims(s->fw, s->fh);
        // the three frames' features in one allocation, so a flow pair can
        // address them as a strided batch
        A(dalloc(&s->feat[0], 3 * s->fd.feat_floats));
        if (e == cudaSuccess) {
            s->feat[1] = s->feat[0] + s->fd.feat_floats;
            s->feat[2] = s->feat[1] + s->fd.feat_floats;
        }
        A(dalloc(&s->feat_scratch, flow_feature_scratch_floats(s->fd)));
        A(dalloc(&s->flow_scratch, 2 * flow_estimate_scratch_floats(s->fd)));
        if (s->corr_dtype != VSC_DTYPE_F32) {
            const size_t fb = tc_frame_bytes(s->fd);
            A(dalloc(&s->feat_tc[0], 3 * fb));
            if (e == cudaSuccess) {
                s->feat_tc[1] = s->feat_tc[0] + fb;
                s->feat_tc[2] = s->feat_tc[1] + fb;
            }
            A(dalloc(&s->warped_tc, 2 * tc_warped_bytes(s->fd)));
            A(dalloc(&s->tc_scales, 2));
            // |feature| <= 1 (L2-normalised): 2^14 keeps FP16 below its
            // maximum with every level's values in its normal range
            const float sc[2] = {16384.0f, 16384.0f};
            if (e == cudaSuccess)
                A(cudaMemcpy(s->tc_scales, sc, sizeof(sc), cudaMemcpyHostToDevice));
        }
        if (s->downscale > 1) {
            A(dalloc(&s->flow_small, 2 * static_cast<size_t>(s->fw) * s->fh * 3));
        }
        A(flow_upload_weights());
    }
    return check_cuda(e, "stabilizer allocation");
}

// The solver's tile shape of a form for the pyramid's sizes (a stream being
// captured keeps the wave model; a failed measurement too).
void tune_pyramid(vsc_stabilizer* s, int form)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s->st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone)
        for (int j = 0; j < std::min(s->levels_alloc, 4); ++j)
            if (solver_autotune(s->lw[j], s->lh[j], s->st, nullptr, form) != cudaSuccess) {
                cudaGetLastError();
                break;
            }
}

}  // namespace

extern "C" {

VSC_API vsc_status vsc_stabilizer_create(const vsc_stabilizer_config* cfg, vsc_stream_t stream, vsc_stabilizer** out)
{
    clear_error();
    if (!cfg || !out)
        return set_error(VSC_EINVAL, "stabilizer_create: null argument");
    *out = nullptr;
    if (cfg->width < 8 || cfg->height < 8 || cfg->width > 16384 || cfg->height > 16384)
        return set_error(VSC_EINVAL, "stabilizer_create: size %dx%d outside [8, 16384]", cfg->width, cfg->height);
    if (cfg->batch_size != 1)
        return set_error(VSC_EUNSUPPORTED, "stabilizer_create: batch_size %d (only 1 is supported)", cfg->batch_size);
    if (cfg->flow_downscale < 1 || cfg->flow_downscale > 8)
        return set_error(VSC_EINVAL, "stabilizer_create: flow_downscale %d outside [1, 8]", cfg->flow_downscale);
    if (!cfg->compute_flow && cfg->flow_channels != 2 && cfg->flow_channels != 3)
        return set_error(VSC_EINVAL, "stabilizer_create: flow_channels must be 2 or 3");
    if (cfg->corr_dtype != VSC_DTYPE_F32 && cfg->corr_dtype != VSC_DTYPE_BF16 && cfg->corr_dtype != VSC_DTYPE_F16)
        return set_error(VSC_EINVAL, "stabilizer_create: corr_dtype %d unknown", cfg->corr_dtype);
    vsc_stabilizer* s = new (std::nothrow) vsc_stabilizer();
    if (!s)
        return set_error(VSC_ENOMEM, "stabilizer_create: out of host memory");
    s->w = cfg->width;
    s->h = cfg->height;
    s->compute_flow = cfg->compute_flow != 0;
    s->fc = s->compute_flow ? 3 : cfg->flow_channels;
    s->downscale = s->compute_flow ? cfg->flow_downscale : 1;
    // videostabilizer.cpp:92-94: round(width / factor)
    s->fw = static_cast<int>(std::lround(static_cast<float>(s->w) / static_cast<float>(s->downscale)));
    s->fh = static_cast<int>(std::lround(static_cast<float>(s->h) / static_cast<float>(s->downscale)));
    s->st = cs(stream);
    s->use_graphs = cfg->use_graphs != 0;
    s->corr_dtype = cfg->corr_dtype;
    cudaGetDevice(&s->device);
    vsc_default_hyper_params(&s->hp);
    vsc_status st = alloc_all(s);
    if (st != VSC_OK) {
        free_all(s);
        delete s;
        return st;
    }
    tune_pyramid(s, kSolverExact);
    *out = s;
    return VSC_OK;
}

VSC_API vsc_status vsc_stabilizer_destroy(vsc_stabilizer* s)
{
    clear_error();
    if (!s)
        return VSC_OK;
    DeviceGuard g(s->device);
    // the compute stream, then the upload and download streams (an
    // asynchronous host read-back may still be running on the latter)
    cudaStreamSynchronize(s->st);
    if (s->cst)
        cudaStreamSynchronize(s->cst);
    if (s->dst)
        cudaStreamSynchronize(s->dst);
    free_all(s);
    delete s;
    return VSC_OK;
}

VSC_API vsc_hyper_params* vsc_stabilizer_hyper_params(vsc_stabilizer* s) { return s ? &s->hp : nullptr; }

VSC_API vsc_status vsc_stabilizer_load_frame(vsc_stabilizer* s, const uint8_t* orig_rgba, const uint8_t* proc_rgba,
    int32_t on_device)
{
    clear_error();
    if (!s || !orig_rgba || !proc_rgba)
        return set_error(VSC_EINVAL, "load_frame: null argument");
    if (s->count >= 3)
        return set_error(VSC_ESTATE, "load_frame: window full; call vsc_stabilizer_step first");
    if (on_device && ((reinterpret_cast<uintptr_t>(orig_rgba) & 3) || (reinterpret_cast<uintptr_t>(proc_rgba) & 3)))
        return set_error(VSC_EINVAL, "load_frame: device frames must be 4-byte aligned");
    DeviceGuard g(s->device);
    const int slot = (s->head + s->count) % 3;
    const int64_t npix = static_cast<int64_t>(s->w) * s->h;
    mark(s, kEvLoad0);
    const uint8_t* src[2] = {orig_rgba, proc_rgba};
    float* dst[2] = {s->orig[slot], s->proc[slot]};
    int nl = 0;
    for (int k = 0; k < 2; ++k) {
        const uint8_t* dsrc = src[k];
        if (!on_device) {
            // upload on the copy stream once the previous conversion has read
            // the staging buffer; the stabilizer's stream waits for the upload
            vsc_status st = check_cuda(cudaStreamWaitEvent(s->cst, s->consumed[k], 0), "load_frame upload");
            if (!st)
                st = check_cuda(cudaMemcpyAsync(s->stage[k], src[k], static_cast<size_t>(npix) * 4,
                                    cudaMemcpyHostToDevice, s->cst),
                    "load_frame upload");
            if (!st)
                st = check_cuda(cudaEventRecord(s->staged[k], s->cst), "load_frame upload");
            if (!st)
                st = check_cuda(cudaStreamWaitEvent(s->st, s->staged[k], 0), "load_frame upload");
            if (st)
                return st;
            dsrc = s->stage[k];
        }
        vsc_status st = check_cuda(launch_rgba_to_float(dsrc, dst[k], npix, s->st), "load_frame convert");
        if (!st && !on_device)
            st = check_cuda(cudaEventRecord(s->consumed[k], s->st), "load_frame convert");
        if (st)
            return st;
        ++nl;
    }
    if (s->compute_flow) {
        // FLOWDOWNSCALE (flowmodel.cpp:126-133): the pyramid reads the frame
        // through the nearest-neighbour resize mapping, no resized copy
        const bool small = s->downscale > 1;
        vsc_status st = check_cuda(launch_flow_features(s->orig[slot], s->fw, s->fh, s->fd, s->feat[slot],
                                       s->feat_scratch, s->st, &nl, small ? s->orig[slot] : nullptr, s->w, s->h),
            "load_frame features");
        if (st)
            return st;
        if (s->corr_dtype != VSC_DTYPE_F32 &&
            (st = check_cuda(launch_flow_features_chunked(s->feat[slot], s->fd, s->feat_tc[slot], s->tc_scales,
                                 s->corr_dtype == VSC_DTYPE_BF16, s->st, &nl),
                 "load_frame features (16-bit)")))
            return st;
    }
    mark(s, kEvLoad1);
    s->count += 1;
    s->last_launches = nl;
    return VSC_OK;
}

VSC_API vsc_status vsc_stabilizer_set_flows(vsc_stabilizer* s, const float* fwd, const float* bwd, int32_t on_device)
{
    clear_error();
    if (!s || !fwd || !bwd)
        return set_error(VSC_EINVAL, "set_flows: null argument");
    if (s->compute_flow)
        return set_error(VSC_ESTATE, "set_flows: this stabilizer computes its own flow");
    DeviceGuard g(s->device);
    const size_t bytes = static_cast<size_t>(s->w) * s->h * s->fc * sizeof(float);
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    vsc_status st = check_cuda(cudaMemcpyAsync(s->flow_fwd, fwd, bytes, kind, s->st), "set_flows fwd");
    if (st)
        return st;
    st = check_cuda(cudaMemcpyAsync(s->flow_bwd, bwd, bytes, kind, s->st), "set_flows bwd");
    if (st)
        return st;
    s->flows_set = true;
    return VSC_OK;
}

}  // extern "C"

namespace {

// All device work of one doOneStep, enqueued on the stabilizer's stream.
// ---- learned flow upsampler state -----------------------------------------------------
}  // namespace
struct vsc_upsampler {
    int device = 0;
    float* prm = nullptr;  // FP32 master parameters
    float* grad = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    void* wtc = nullptr;  // FP16 weights packed for the tensor-core inference
    bool wtc_valid = false;
    int step = 0;
    float* work = nullptr;
    size_t work_floats = 0;
    float* loss = nullptr;
    float max_residual = 0.5f;
};
namespace {

cudaError_t upsampler_sync_weights(vsc_upsampler* u, cudaStream_t st)
{
    if (u->wtc_valid)
        return cudaSuccess;
    cudaError_t e = launch_upsampler_tc_pack(u->prm, u->wtc, st);
    u->wtc_valid = e == cudaSuccess;
    return e;
}

// the tensor-core work area follows the prepared input, on the 16-byte grid
unsigned char* up_tc_work(float* input, int64_t input_floats)
{
    return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(input + input_floats) + 15) &
                                            ~static_cast<uintptr_t>(15));
}

// both flows of a step: coarse flows (fw x fh) -> full-size flows
cudaError_t upsampler_apply_pair(vsc_stabilizer* s, cudaStream_t st, int* nl)
{
    const int64_t npx = static_cast<int64_t>(s->w) * s->h;
    const int64_t fs = static_cast<int64_t>(s->fw) * s->fh * 3;
    float* input = s->up_work;
    cudaError_t e = upsampler_sync_weights(s->upsampler, st);
    if (e == cudaSuccess)
        e = launch_upsampler_prepare(s->flow_small, s->fw, s->fh, 3, s->orig[(s->head + 1) % 3], input, s->w, s->h, 2,
            fs, s->orig[(s->head + 2) % 3] - s->orig[(s->head + 1) % 3], npx * 3, st);
    *nl += 1;
    if (e == cudaSuccess)
        e = launch_upsampler_tc(s->upsampler->wtc, s->upsampler->prm, input, up_tc_work(input, 2 * npx * 3),
            s->flow_fwd, 2, s->h, s->w, s->upsampler->max_residual, s->flow_bwd - s->flow_fwd, st, nl);
    return e;
}

// The images of the solve at each pyramid level of a step.
struct LevelImages {
    float* P[8];
    float* A[8];
    float* W[8];
    float* O[8];
};

// A step up to the solves: flows, the fused front pass (warps, adaptive
// combination, consistency weights) and the pyramid of the solve's inputs.
cudaError_t enqueue_pre_solve(vsc_stabilizer* s, const vsc_hyper_params& hp, LevelImages* lv, int* launches)
{
    const int L = hp.pyramid_levels;
    const int s0 = s->head, s1 = (s->head + 1) % 3, s2 = (s->head + 2) % 3;
    const size_t n3b = static_cast<size_t>(s->w) * s->h * 3 * sizeof(float);
    cudaStream_t st = s->st;
    int nl = 0;
    cudaError_t e = cudaSuccess;
    auto run = [&](cudaError_t r) {
        if (e == cudaSuccess)
            e = r;
    };

    mark(s, kEvStep0);
    // preloadProcessedFrames (videostabilizer.cpp:152): the first previous
    // stabilized frame is the processed image of the last preloaded frame.
    if (!s->started)
        run(cudaMemcpyAsync(s->last_stab[s->ls_cur], s->proc[s2], n3b, cudaMemcpyDeviceToDevice, st));

    // retrieveOpticalFlow (videostabilizer.cpp:267-279): forward flow runs
    // frame pair (t, t+1); the "backward" flow runs (t+1, t) (flowmodel.cpp:139-143).
    if (s->compute_flow) {
        const bool small = s->downscale > 1;
        const int64_t fs = static_cast<int64_t>(s->fw) * s->fh * 3;
        FlowTc tc{};
        if (s->corr_dtype != VSC_DTYPE_F32) {
            tc.a[0] = s->feat_tc[s1];
            tc.a[1] = s->feat_tc[s2];
            tc.b[0] = s->feat_tc[s2];
            tc.b[1] = s->feat_tc[s1];
            tc.warped = s->warped_tc;
            tc.scales = s->tc_scales;
            tc.bf16 = s->corr_dtype == VSC_DTYPE_BF16;
        }
        run(launch_flow_pair(s->feat[s1], s->feat[s2] - s->feat[s1], s->feat[s2], s->feat[s1] - s->feat[s2], s->fw,
            s->fh, s->fd, small ? s->flow_small : s->flow_fwd, small ? fs : s->flow_bwd - s->flow_fwd,
            s->flow_scratch, st, &nl, s->corr_dtype != VSC_DTYPE_F32 ? &tc : nullptr));
        if (small && s->upsampler) {
            // learned upsampling of both flows in one batch (the luma of
            // frame t for the forward flow, of frame t+1 for the backward one)
            run(upsampler_apply_pair(s, st, &nl));
        } else if (small && !front_samples_small_flows(s)) {
            // flowmodel.cpp:158-161: bilinear upsampling, vectors not rescaled
            run(launch_bilinear(Img{s->flow_small, s->fw, s->fh, 3}, Img{s->flow_fwd, s->w, s->h, 3}, st));
            run(launch_bilinear(Img{s->flow_small + fs, s->fw, s->fh, 3}, Img{s->flow_bwd, s->w, s->h, 3}, st));
            nl += 2;
        }
    }

    mark(s, kEvFlow);
    float* ls_in = s->last_stab[s->ls_cur];
    float* ls_out = s->last_stab[s->ls_cur ^ 1];
    // the pyramid's first level (videostabilizer.cpp:203-217) comes out of the
    // front pass when it is an exact half (same values as pyr_down3)
    const bool down = L > 1 && !s->occlusion && front_down_fusable(s->w, s->h, s->lw[1], s->lh[1]);
    float* dP = down ? s->pyrP[1] : nullptr;
    float* dA = down ? s->pyrA[1] : nullptr;
    float* dW = down ? s->pyrW[1] : nullptr;
    if (front_samples_small_flows(s)) {
        // the upsampling of both flows happens inside the front pass
        const int64_t fs = static_cast<int64_t>(s->fw) * s->fh * 3;
        run(launch_fused_front(s->orig[s0], s->orig[s1], s->orig[s2], s->proc[s0], s->proc[s1], s->proc[s2], ls_in,
            s->flow_small, s->flow_small + fs, 3, s->adap_pr, s->cons_wt, s->w, s->h, hp.alpha, hp.beta, hp.gamma,
            st, false, s->fw, s->fh, dP, dA, dW, s->lw[1], s->lh[1]));
    } else {
        run(launch_fused_front(s->orig[s0], s->orig[s1], s->orig[s2], s->proc[s0], s->proc[s1], s->proc[s2], ls_in,
            s->flow_fwd, s->flow_bwd, s->fc, s->adap_pr, s->cons_wt, s->w, s->h, hp.alpha, hp.beta, hp.gamma, st,
            s->occlusion, 0, 0, dP, dA, dW, s->lw[1], s->lh[1]));
    }
    ++nl;

    // pyramid (videostabilizer.cpp:203-217)
    float** P = lv->P;
    float** A = lv->A;
    float** W = lv->W;
    float** O = lv->O;
    P[0] = s->proc[s1];
    A[0] = s->adap_pr;
    W[0] = s->cons_wt;
    O[0] = ls_out;
    for (int j = 1; j < L; ++j) {
        P[j] = s->pyrP[j];
        A[j] = s->pyrA[j];
        W[j] = s->pyrW[j];
        O[j] = s->pyrO[j];
        if (j == 1 && down)
            continue;  // written by the front pass
        run(launch_pyr_down3(P[j - 1], A[j - 1], W[j - 1], s->lw[j - 1], s->lh[j - 1], P[j], A[j], W[j], s->lw[j],
            s->lh[j], st));
        ++nl;
    }
    *launches += nl;
    return e;
}

cudaError_t enqueue_step(vsc_stabilizer* s, const vsc_hyper_params& hp, uint8_t* rgba_dev, int* launches)
{
    const int L = hp.pyramid_levels;
    cudaStream_t st = s->st;
    int nl = 0;
    LevelImages lv;
    cudaError_t e = enqueue_pre_solve(s, hp, &lv, &nl);
    auto run = [&](cudaError_t r) {
        if (e == cudaSuccess)
            e = r;
    };
    float** P = lv.P;
    float** A = lv.A;
    float** W = lv.W;
    float** O = lv.O;
    // The solution is initialised with the processed frame and carried down
    // with the same bilinear chain, so at the coarsest level it equals P.
    run(cudaMemcpyAsync(O[L - 1], P[L - 1], static_cast<size_t>(s->lw[L - 1]) * s->lh[L - 1] * 3 * sizeof(float),
        cudaMemcpyDeviceToDevice, st));
    mark(s, kEvFront);
    for (int j = L - 1; j >= 0; --j) {
        if (j == 0)
            mark(s, kEvCoarse);
        const int iters = hp.num_iter / (j + 1);
        uint8_t* rgba = j == 0 ? rgba_dev : nullptr;
        if (j != L - 1 && s->solver_form == kSolverFma && iters > 0) {
            // the FMA form upsamples the coarser solution in its setup pass
            run(run_solver_from_coarse(P[j], A[j], W[j], O[j], s->lw[j], s->lh[j], O[j + 1], s->lw[j + 1],
                s->lh[j + 1], iters, hp.step_size, hp.mom_fac, s->solver_ws, st, &nl, rgba));
            continue;
        }
        if (j != L - 1) {
            run(launch_bilinear(Img{O[j + 1], s->lw[j + 1], s->lh[j + 1], 3}, Img{O[j], s->lw[j], s->lh[j], 3}, st));
            ++nl;
        }
        run(run_solver(P[j], A[j], W[j], O[j], s->lw[j], s->lh[j], iters, hp.step_size, hp.mom_fac, s->solver_ws, st,
            &nl, rgba, s->solver_form));
    }
    mark(s, kEvStep1);
    *launches = nl;
    return e;
}

bool same_hp(const vsc_hyper_params& a, const vsc_hyper_params& b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

// Replays (capturing on first use) the step graph for the current state.
// Returns false when graphs cannot be used; the caller then enqueues directly.
bool launch_step_graph(vsc_stabilizer* s, const vsc_hyper_params& hp, uint8_t* rgba_dev, int* launches,
    cudaError_t* err)
{
    *err = cudaSuccess;
    auto* hit = static_cast<vsc_stabilizer::GraphEntry*>(nullptr);
    for (auto& g : s->graphs)
        if (g.valid && g.head == s->head && g.ls_cur == s->ls_cur && g.rgba == rgba_dev && g.timing == s->timing &&
            g.occlusion == s->occlusion && g.solver_form == s->solver_form && g.upsampler == s->upsampler &&
            same_hp(g.hp, hp))
            hit = &g;
    if (!hit) {
        auto* slot = &s->graphs[0];
        for (auto& g : s->graphs)
            if (!g.valid || g.used < slot->used)
                slot = &g;
        if (slot->exec) {
            cudaGraphExecDestroy(slot->exec);
            slot->exec = nullptr;
        }
        slot->valid = false;
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        int nl = 0;
        const cudaError_t ee = enqueue_step(s, hp, rgba_dev, &nl);
        const cudaError_t ec = cudaStreamEndCapture(s->st, &graph);
        if (ee != cudaSuccess || ec != cudaSuccess || !graph) {
            if (graph)
                cudaGraphDestroy(graph);
            cudaGetLastError();
            return false;
        }
        const cudaError_t ei = cudaGraphInstantiate(&slot->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            cudaGetLastError();
            slot->exec = nullptr;
            return false;
        }
        slot->valid = true;
        slot->head = s->head;
        slot->ls_cur = s->ls_cur;
        slot->rgba = rgba_dev;
        slot->timing = s->timing;
        slot->occlusion = s->occlusion;
        slot->solver_form = s->solver_form;
        slot->upsampler = s->upsampler;
        slot->hp = hp;
        slot->nl = nl;
        hit = slot;
    }
    hit->used = ++s->graph_clock;
    *launches = hit->nl;
    *err = cudaGraphLaunch(hit->exec, s->st);
    return true;
}

// The window advances after a step: the feedback frame flips, the oldest
// frame leaves the ring (doOneStep's pop_front, videostabilizer.cpp:247-252).
void finish_step(vsc_stabilizer* s, int launches)
{
    s->ls_cur ^= 1;
    s->started = true;
    s->flows_set = false;
    s->head = (s->head + 1) % 3;
    s->count -= 1;
    s->last_launches = launches;
    s->flows_pending = front_samples_small_flows(s);
}

vsc_status step_preconditions(vsc_stabilizer* s, const vsc_hyper_params& hp)
{
    if (s->count < 3)
        return set_error(VSC_ESTATE, "step: window holds %d of 3 frames", s->count);
    if (!s->compute_flow && !s->flows_set)
        return set_error(VSC_ESTATE, "step: flows not set for this step");
    if (hp.pyramid_levels < 1 || hp.pyramid_levels > s->levels_alloc)
        return set_error(VSC_EINVAL, "step: pyramid_levels %d outside [1, %d]", hp.pyramid_levels, s->levels_alloc);
    if (hp.num_iter < 0)
        return set_error(VSC_EINVAL, "step: negative num_iter");
    return VSC_OK;
}

}  // namespace

extern "C" {

VSC_API vsc_status vsc_stabilizer_step(vsc_stabilizer* s, uint8_t* out_rgba, int32_t out_on_device)
{
    clear_error();
    if (!s)
        return set_error(VSC_EINVAL, "step: null stabilizer");
    if (s->count < 3)
        return set_error(VSC_ESTATE, "step: window holds %d of 3 frames", s->count);
    if (!s->compute_flow && !s->flows_set)
        return set_error(VSC_ESTATE, "step: flows not set for this step");
    const vsc_hyper_params hp = s->hp;
    const int L = hp.pyramid_levels;
    if (L < 1 || L > s->levels_alloc)
        return set_error(VSC_EINVAL, "step: pyramid_levels %d outside [1, %d]", L, s->levels_alloc);
    if (hp.num_iter < 0)
        return set_error(VSC_EINVAL, "step: negative num_iter");
    if (out_on_device < 0 || out_on_device > VSC_OUT_HOST_ASYNC)
        return set_error(VSC_EINVAL, "step: out_on_device %d is not 0, 1 or VSC_OUT_HOST_ASYNC", out_on_device);
    if (out_rgba && out_on_device == 1 && (reinterpret_cast<uintptr_t>(out_rgba) & 3))
        return set_error(VSC_EINVAL, "step: device output must be 4-byte aligned");
    DeviceGuard g(s->device);
    const bool host_out = out_rgba && out_on_device != 1;
    uint8_t* rgba_dev = (out_rgba && out_on_device == 1) ? out_rgba : s->out_rgba;
    int par = 0;
    if (host_out) {
        // alternate device buffers: this step writes one while the previous
        // step's copy back reads the other; the copy from this buffer two host
        // outputs ago must have finished
        par = s->out_par;
        rgba_dev = par ? s->out_rgba_b : s->out_rgba;
        vsc_status w = check_cuda(cudaStreamWaitEvent(s->st, s->d2h_done[par], 0), "step");
        if (w)
            return w;
    }
    int nl = 0;
    cudaError_t e = cudaSuccess;
    // The first step (which seeds the feedback frame) runs directly; later
    // steps replay a captured graph when the stream allows capture.
    // (stage timing records plain events, so timed steps are not captured)
    const bool graphed = s->use_graphs && !s->timing && s->started && s->st != nullptr &&
                         launch_step_graph(s, hp, rgba_dev, &nl, &e);
    if (!graphed)
        e = enqueue_step(s, hp, rgba_dev, &nl);
    vsc_status stt = check_cuda(e, "step");
    if (stt)
        return stt;
    finish_step(s, nl);
    if (host_out) {
        // the copy back runs on the download stream, after the step, beside the
        // caller's next load_frame and step
        s->out_par ^= 1;
        stt = check_cuda(cudaEventRecord(s->step_done, s->st), "step download");
        if (!stt)
            stt = check_cuda(cudaStreamWaitEvent(s->dst, s->step_done, 0), "step download");
        if (!stt)
            stt = check_cuda(cudaMemcpyAsync(out_rgba, rgba_dev, static_cast<size_t>(s->w) * s->h * 4,
                                 cudaMemcpyDeviceToHost, s->dst),
                "step download");
        if (!stt)
            stt = check_cuda(cudaEventRecord(s->d2h_done[par], s->dst), "step download");
        if (stt)
            return stt;
        s->d2h_prev = s->d2h_last;
        s->d2h_last = par;
        if (out_on_device == VSC_OUT_HOST_ASYNC)
            return VSC_OK;
        return check_cuda(cudaEventSynchronize(s->d2h_done[par]), "step synchronize");
    }
    return VSC_OK;
}

VSC_API vsc_status vsc_stabilizer_wait_output(vsc_stabilizer* s, int32_t which)
{
    clear_error();
    if (!s || which < 0 || which > 1)
        return set_error(VSC_EINVAL, "wait_output: null stabilizer or which not 0 or 1");
    const int par = which == 0 ? s->d2h_last : s->d2h_prev;
    if (par < 0)
        return VSC_OK;
    DeviceGuard g(s->device);
    return check_cuda(cudaEventSynchronize(s->d2h_done[par]), "wait_output");
}

VSC_API vsc_status vsc_stabilizer_synchronize(vsc_stabilizer* s)
{
    clear_error();
    if (!s)
        return set_error(VSC_EINVAL, "synchronize: null stabilizer");
    DeviceGuard g(s->device);
    vsc_status st = check_cuda(cudaStreamSynchronize(s->st), "synchronize");
    if (!st)
        st = check_cuda(cudaStreamSynchronize(s->dst), "synchronize");
    return st;
}

VSC_API vsc_status vsc_stabilizer_buffer(vsc_stabilizer* s, int32_t which, const float** dev_ptr)
{
    clear_error();
    if (!s || !dev_ptr)
        return set_error(VSC_EINVAL, "buffer: null argument");
    if ((which == 1 || which == 2) && s->flows_pending) {
        // the last step sampled the coarse flows in its front pass: upsample
        // them now (the values the step used), in stream order
        DeviceGuard g(s->device);
        const int64_t fs = static_cast<int64_t>(s->fw) * s->fh * 3;
        vsc_status st = check_cuda(
            launch_bilinear(Img{s->flow_small, s->fw, s->fh, 3}, Img{s->flow_fwd, s->w, s->h, 3}, s->st), "buffer");
        if (!st)
            st = check_cuda(launch_bilinear(Img{s->flow_small + fs, s->fw, s->fh, 3}, Img{s->flow_bwd, s->w, s->h, 3},
                                s->st),
                "buffer");
        if (!st)
            st = check_cuda(cudaStreamSynchronize(s->st), "buffer");
        if (st)
            return st;
        s->flows_pending = false;
    }
    switch (which) {
        case 0:
            *dev_ptr = s->last_stab[s->ls_cur];
            return VSC_OK;
        case 1:
            *dev_ptr = s->flow_fwd;
            return VSC_OK;
        case 2:
            *dev_ptr = s->flow_bwd;
            return VSC_OK;
        case 3:
            *dev_ptr = s->adap_pr;
            return VSC_OK;
        case 4:
            *dev_ptr = s->cons_wt;
            return VSC_OK;
        default:
            return set_error(VSC_EINVAL, "buffer: unknown buffer %d", which);
    }
}

VSC_API int32_t vsc_stabilizer_last_launches(vsc_stabilizer* s) { return s ? s->last_launches : 0; }

VSC_API int32_t vsc_upsampler_param_count(void) { return upsampler_param_count(); }

VSC_API vsc_status vsc_upsampler_create(const float* params, vsc_upsampler** out)
{
    clear_error();
    if (!out)
        return set_error(VSC_EINVAL, "upsampler_create: null argument");
    *out = nullptr;
    vsc_upsampler* u = new (std::nothrow) vsc_upsampler();
    if (!u)
        return set_error(VSC_ENOMEM, "upsampler_create: out of host memory");
    cudaGetDevice(&u->device);
    const int n = upsampler_param_count();
    std::vector<float> host(n);
    if (params)
        std::memcpy(host.data(), params, n * sizeof(float));
    else
        upsampler_init_params(host.data(), 0x55505341'4D504C45ULL);  // seeded He-uniform
    cudaError_t e = dalloc(&u->prm, n);
    if (e == cudaSuccess)
        e = dalloc(&u->grad, n);
    if (e == cudaSuccess)
        e = dalloc(&u->m, n);
    if (e == cudaSuccess)
        e = dalloc(&u->v, n);
    if (e == cudaSuccess)
        e = cudaMalloc(&u->wtc, upsampler_tc_weight_bytes());
    if (e == cudaSuccess)
        e = dalloc(&u->loss, 1);
    if (e == cudaSuccess)
        e = cudaMemcpy(u->prm, host.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemset(u->m, 0, n * sizeof(float));
    if (e == cudaSuccess)
        e = cudaMemset(u->v, 0, n * sizeof(float));
    if (e != cudaSuccess) {
        vsc_upsampler_destroy(u);
        return check_cuda(e, "upsampler_create");
    }
    *out = u;
    return VSC_OK;
}

VSC_API vsc_status vsc_upsampler_destroy(vsc_upsampler* u)
{
    if (!u)
        return VSC_OK;
    DeviceGuard g(u->device);
    cudaDeviceSynchronize();
    for (void* p : {static_cast<void*>(u->prm), static_cast<void*>(u->grad), static_cast<void*>(u->m),
             static_cast<void*>(u->v), u->wtc, static_cast<void*>(u->work),
             static_cast<void*>(u->loss)})
        if (p)
            cudaFree(p);
    delete u;
    return VSC_OK;
}

VSC_API vsc_status vsc_upsampler_get_params(vsc_upsampler* u, float* host_params)
{
    clear_error();
    if (!u || !host_params)
        return set_error(VSC_EINVAL, "upsampler_get_params: null argument");
    DeviceGuard g(u->device);
    return check_cuda(cudaMemcpy(host_params, u->prm, upsampler_param_count() * sizeof(float), cudaMemcpyDeviceToHost),
        "upsampler_get_params");
}

VSC_API vsc_status vsc_upsampler_set_max_residual(vsc_upsampler* u, float px)
{
    clear_error();
    if (!u || !(px >= 0.0f))
        return set_error(VSC_EINVAL, "upsampler_set_max_residual: bad argument");
    u->max_residual = px;
    return VSC_OK;
}

VSC_API vsc_status vsc_upsampler_prepare(const vsc_image* coarse_flow, const vsc_image* frame, const vsc_image* input,
    vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if ((s = check_image(coarse_flow, "coarseFlow", 2, 3)) || (s = check_image(frame, "frame", 3, 3)) ||
        (s = check_image(input, "input", 3, 3)) || (s = same_size(frame, input, "input")))
        return s;
    return check_cuda(launch_upsampler_prepare(coarse_flow->data, coarse_flow->width, coarse_flow->height,
                          coarse_flow->channels, frame->data, input->data, frame->width, frame->height, 1, 0, 0, 0,
                          cs(stream)),
        "upsampler_prepare");
}

VSC_API vsc_status vsc_upsampler_train_step(vsc_upsampler* u, const float* input, const float* target, int32_t n,
    int32_t h, int32_t w, float lr, float* loss_out, vsc_stream_t stream)
{
    clear_error();
    if (!u || !input || !target || n < 1 || h < 1 || w < 1 || n > 65535 || static_cast<int64_t>(n) * h * w > (1 << 26))
        return set_error(VSC_EINVAL, "upsampler_train_step: bad arguments");
    DeviceGuard g(u->device);
    cudaStream_t st = cs(stream);
    const size_t need = upsampler_train_work_floats(n, h, w);
    if (need > u->work_floats) {
        cudaStreamSynchronize(st);
        if (u->work)
            cudaFree(u->work);
        u->work = nullptr;
        u->work_floats = 0;
        vsc_status s = check_cuda(dalloc(&u->work, need), "upsampler_train_step workspace");
        if (s)
            return s;
        u->work_floats = need;
    }
    u->wtc_valid = false;
    vsc_status s = check_cuda(upsampler_train_step(u->prm, u->grad, u->m, u->v, ++u->step, input, target, n, h, w, lr,
                                  u->work, u->loss, st),
        "upsampler_train_step");
    if (s || !loss_out)
        return s;
    s = check_cuda(cudaMemcpyAsync(loss_out, u->loss, sizeof(float), cudaMemcpyDeviceToHost, st), "upsampler loss");
    return s ? s : check_cuda(cudaStreamSynchronize(st), "upsampler loss");
}

VSC_API vsc_status vsc_upsampler_apply(vsc_upsampler* u, const vsc_image* coarse_flow, const vsc_image* frame,
    const vsc_image* flow_out, vsc_stream_t stream)
{
    clear_error();
    vsc_status s;
    if (!u)
        return set_error(VSC_EINVAL, "upsampler_apply: null upsampler");
    if ((s = check_image(coarse_flow, "coarseFlow", 2, 3)) || (s = check_image(frame, "frame", 3, 3)) ||
        (s = check_image(flow_out, "flowOut", 3, 3)) || (s = same_size(frame, flow_out, "flowOut")))
        return s;
    DeviceGuard g(u->device);
    cudaStream_t st = cs(stream);
    const int w = frame->width, h = frame->height;
    const int64_t npx = static_cast<int64_t>(w) * h;
    void* ws = nullptr;
    if ((s = check_cuda(pool_alloc(&ws, npx * 3 * sizeof(float) + 16 + upsampler_tc_work_bytes(1, h, w), st),
             "upsampler_apply workspace")))
        return s;
    float* input = static_cast<float*>(ws);
    cudaError_t e = upsampler_sync_weights(u, st);
    if (e == cudaSuccess)
        e = launch_upsampler_prepare(coarse_flow->data, coarse_flow->width, coarse_flow->height, coarse_flow->channels,
            frame->data, input, w, h, 1, 0, 0, 0, st);
    if (e == cudaSuccess)
        e = launch_upsampler_tc(u->wtc, u->prm, input, up_tc_work(input, npx * 3), flow_out->data, 1, h, w,
            u->max_residual, 0, st, nullptr);
    cudaFreeAsync(ws, st);
    return check_cuda(e, "upsampler_apply");
}

VSC_API vsc_status vsc_stabilizer_set_upsampler(vsc_stabilizer* s, vsc_upsampler* u)
{
    clear_error();
    if (!s)
        return set_error(VSC_EINVAL, "set_upsampler: null stabilizer");
    if (u && !(s->compute_flow && s->downscale > 1))
        return set_error(VSC_ESTATE, "set_upsampler: the stabilizer computes no downscaled flow");
    DeviceGuard g(s->device);
    if (u && !s->up_work) {
        const size_t npx = static_cast<size_t>(s->w) * s->h;
        vsc_status st = check_cuda(
            dalloc(&s->up_work, 2 * npx * 3 + 4 + upsampler_tc_work_bytes(2, s->h, s->w) / sizeof(float)),
            "set_upsampler workspace");
        if (st)
            return st;
    }
    s->upsampler = u;
    return VSC_OK;
}

VSC_API vsc_status vsc_stabilizer_set_occlusion_mask(vsc_stabilizer* s, int32_t on)
{
    clear_error();
    if (!s)
        return set_error(VSC_EINVAL, "set_occlusion_mask: null stabilizer");
    s->occlusion = on != 0;
    return VSC_OK;
}

VSC_API vsc_status vsc_stabilizer_set_solver_form(vsc_stabilizer* s, int32_t form)
{
    clear_error();
    if (!s)
        return set_error(VSC_EINVAL, "set_solver_form: null stabilizer");
    if (form != VSC_SOLVER_EXACT && form != VSC_SOLVER_FMA)
        return set_error(VSC_EINVAL, "set_solver_form: unknown solver form %d", form);
    DeviceGuard g(s->device);
    if (form == VSC_SOLVER_FMA && !solver_tma_supported())
        return set_error(VSC_EUNSUPPORTED, "set_solver_form: the FMA form needs the solver's shared-memory opt-in");
    if (form != s->solver_form)
        tune_pyramid(s, form);
    s->solver_form = form;
    return VSC_OK;
}

VSC_API vsc_status vsc_stabilizer_enable_timing(vsc_stabilizer* s, int32_t on)
{
    clear_error();
    if (!s)
        return set_error(VSC_EINVAL, "enable_timing: null stabilizer");
    DeviceGuard g(s->device);
    if (on && !s->ev[0])
        for (cudaEvent_t& e : s->ev) {
            vsc_status st = check_cuda(cudaEventCreate(&e), "enable_timing");
            if (st)
                return st;
        }
    s->timing = on != 0;
    return VSC_OK;
}

VSC_API vsc_status vsc_stabilizer_stage_ms(vsc_stabilizer* s, float* ms, int32_t n)
{
    clear_error();
    if (!s || !ms || n < 5)
        return set_error(VSC_EINVAL, "stage_ms: null argument or n < 5");
    if (!s->timing)
        return set_error(VSC_ESTATE, "stage_ms: timing not enabled");
    DeviceGuard g(s->device);
    vsc_status st = check_cuda(cudaStreamSynchronize(s->st), "stage_ms");
    if (st)
        return st;
    const int pairs[5][2] = {{kEvLoad0, kEvLoad1}, {kEvStep0, kEvFlow}, {kEvFlow, kEvFront}, {kEvFront, kEvCoarse},
        {kEvCoarse, kEvStep1}};
    for (int i = 0; i < 5; ++i)
        if ((st = check_cuda(cudaEventElapsedTime(&ms[i], s->ev[pairs[i][0]], s->ev[pairs[i][1]]), "stage_ms")))
            return st;
    return VSC_OK;
}

}  // extern "C"

// ---- several streams in one graph launch per frame step -------------------------
// Each stream is a stabilizer on its own CUDA stream; a frame step forks from
// the caller's stream into every stabilizer's stream, enqueues its step there,
// and joins back, so the steps of small and large frames overlap on the
// device.  After the first step the whole fork/join is captured once per
// window position as one CUDA graph (all streams advance in lockstep).
struct vsc_multistream {
    std::vector<vsc_stabilizer*> st;
    // grouped solves: one persistent-kernel launch per 8 Jacobi steps walks
    // the tiles of every stream's image at a pyramid level
    bool fused = true;      // requested (vsc_multistream_set_fused)
    bool fused_ok = false;  // every stream's level sizes take the TMA path
    std::vector<float*> lvl_ws;  // per stream: solver workspaces of levels 1 ..
    int tuned_levels = 0;        // levels whose group tile shape was autotuned
    int solver_form = kSolverExact;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> loaded, joined;
    cudaEvent_t fork = nullptr, done = nullptr;
    cudaStream_t main = nullptr;
    bool own_main = false;
    int device = 0;
    vsc_hyper_params hp{};
    int last_launches = 0;
    struct Graph {
        bool valid = false;
        int head = 0, ls_cur = 0, nl = 0;
        std::vector<uint8_t*> outs;
        vsc_hyper_params hp{};
        cudaGraphExec_t exec = nullptr;
        uint64_t used = 0;
    } graphs[6];
    uint64_t clock = 0;
};

namespace {

void ms_free(vsc_multistream* m)
{
    for (float* p : m->lvl_ws)
        if (p)
            cudaFree(p);
    m->lvl_ws.clear();
    for (auto& g : m->graphs)
        if (g.exec)
            cudaGraphExecDestroy(g.exec);
    for (vsc_stabilizer* s : m->st)
        vsc_stabilizer_destroy(s);
    for (cudaStream_t x : m->side)
        if (x)
            cudaStreamDestroy(x);
    for (cudaEvent_t e : m->loaded)
        if (e)
            cudaEventDestroy(e);
    for (cudaEvent_t e : m->joined)
        if (e)
            cudaEventDestroy(e);
    if (m->fork)
        cudaEventDestroy(m->fork);
    if (m->done)
        cudaEventDestroy(m->done);
    if (m->own_main && m->main)
        cudaStreamDestroy(m->main);
}

// fork -> every stream's step -> join, on m->main; counts launches
cudaError_t ms_enqueue(vsc_multistream* m, const std::vector<uint8_t*>& outs, int* launches)
{
    cudaError_t e = cudaEventRecord(m->fork, m->main);
    int nl = 0;
    for (size_t i = 0; i < m->st.size() && e == cudaSuccess; ++i) {
        if ((e = cudaStreamWaitEvent(m->side[i], m->fork, 0)) != cudaSuccess)
            break;
        int n = 0;
        if ((e = enqueue_step(m->st[i], m->hp, outs[i], &n)) != cudaSuccess)
            break;
        nl += n;
        if ((e = cudaEventRecord(m->joined[i], m->side[i])) == cudaSuccess)
            e = cudaStreamWaitEvent(m->main, m->joined[i], 0);
    }
    *launches = nl;
    return e;
}

// Level j's solver workspace of stream i: the stabilizer's own at level 0,
// the multistream's per-level ones above (every level's Laplacian is
// computed before the first grouped solve).
float* ms_level_ws(vsc_multistream* m, size_t i, int j)
{
    vsc_stabilizer* s = m->st[i];
    if (j == 0)
        return s->solver_ws;
    float* p = m->lvl_ws[i];
    for (int k = 1; k < j; ++k)
        p += solver_workspace_floats(s->lw[k], s->lh[k], kSolverFma);
    return p;
}

// The step with grouped solves: each stream's flows, front pass, pyramid and
// Laplacians on its own CUDA stream; then, on the multistream's stream, per
// pyramid level one bilinear launch over all streams and the level's solve
// as launches of the persistent kernel over every stream's tiles.
cudaError_t ms_enqueue_fused(vsc_multistream* m, const std::vector<uint8_t*>& outs, int* launches)
{
    const vsc_hyper_params& hp = m->hp;
    const int L = hp.pyramid_levels;
    const size_t n = m->st.size();
    std::vector<LevelImages> lv(n);
    cudaError_t e = cudaEventRecord(m->fork, m->main);
    int nl = 0;
    for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
        vsc_stabilizer* s = m->st[i];
        if ((e = cudaStreamWaitEvent(m->side[i], m->fork, 0)) != cudaSuccess)
            break;
        e = enqueue_pre_solve(s, hp, &lv[i], &nl);
        for (int j = 0; j < L && e == cudaSuccess; ++j) {
            e = solver_prep(m->solver_form, lv[i].P[j], lv[i].A[j], lv[i].W[j], s->lw[j], s->lh[j], hp.step_size,
                ms_level_ws(m, i, j), s->st);
            ++nl;
        }
        // videostabilizer.cpp:212-217: the coarsest level starts from P
        const int it = hp.num_iter / L;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(solver_start_buffer(lv[i].O[L - 1], s->lw[L - 1], s->lh[L - 1], it,
                                    ms_level_ws(m, i, L - 1), m->solver_form),
                lv[i].P[L - 1], static_cast<size_t>(s->lw[L - 1]) * s->lh[L - 1] * 3 * sizeof(float),
                cudaMemcpyDeviceToDevice, s->st);
        if (e == cudaSuccess && (e = cudaEventRecord(m->joined[i], m->side[i])) == cudaSuccess)
            e = cudaStreamWaitEvent(m->main, m->joined[i], 0);
    }
    std::vector<SolverImage> im(n);
    std::vector<Img> up_in(n), up_out(n);
    for (int j = L - 1; j >= 0 && e == cudaSuccess; --j) {
        const int it = hp.num_iter / (j + 1);
        for (size_t i = 0; i < n; ++i) {
            vsc_stabilizer* s = m->st[i];
            float* ws = ms_level_ws(m, i, j);
            im[i] = SolverImage{lv[i].P[j], lv[i].A[j], lv[i].W[j], lv[i].O[j], s->lw[j], s->lh[j], ws,
                j == 0 ? outs[i] : nullptr};
            if (j != L - 1) {
                up_in[i] = Img{lv[i].O[j + 1], s->lw[j + 1], s->lh[j + 1], 3};
                up_out[i] = Img{solver_start_buffer(lv[i].O[j], s->lw[j], s->lh[j], it, ws, m->solver_form), s->lw[j],
                    s->lh[j], 3};
            }
        }
        if (j != L - 1) {
            e = launch_bilinear_group(up_in.data(), up_out.data(), static_cast<int>(n), m->main);
            nl += static_cast<int>((n + 15) / 16);
        }
        if (e == cudaSuccess)
            e = run_solver_group(im.data(), static_cast<int>(n), it, hp.step_size, hp.mom_fac, m->main, &nl,
                m->solver_form);
    }
    *launches = nl;
    return e;
}

// the grouped form when requested and possible for the current
// hyper-parameters: the device runs the TMA kernels and every level width
// is a multiple of 4 (buffers come from cudaMalloc, offsets are 16-byte
// multiples then)
bool ms_use_fused(vsc_multistream* m)
{
    if (!m->fused || !m->fused_ok || !solver_tma_supported())
        return false;
    for (vsc_stabilizer* s : m->st) {
        if (m->hp.pyramid_levels > s->levels_alloc)
            return false;
        for (int j = 0; j < m->hp.pyramid_levels; ++j)
            if (s->lw[j] % 4 != 0)
                return false;
    }
    return true;
}

// The tile shape of each level's group for a solver form (a stream being
// captured, or a failed measurement, keeps the wave model).
void ms_tune(vsc_multistream* m, int form)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(m->main, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
        return;
    int levels = 4;
    for (vsc_stabilizer* st : m->st)
        levels = std::min(levels, st->levels_alloc);
    std::vector<int> ws(m->st.size()), hs(m->st.size());
    for (int j = 0; j < levels; ++j) {
        bool eligible = true;
        for (size_t i = 0; i < m->st.size(); ++i) {
            ws[i] = m->st[i]->lw[j];
            hs[i] = m->st[i]->lh[j];
            eligible = eligible && ws[i] % 4 == 0;
        }
        if (!eligible)
            break;
        if (solver_group_autotune(ws.data(), hs.data(), static_cast<int>(ws.size()), m->main, nullptr, form) !=
            cudaSuccess) {
            cudaGetLastError();
            break;
        }
    }
}

void ms_drop_graphs(vsc_multistream* m)
{
    for (auto& g : m->graphs) {
        if (g.exec)
            cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        g.valid = false;
    }
}

cudaError_t ms_step_enqueue(vsc_multistream* m, const std::vector<uint8_t*>& outs, int* launches)
{
    return ms_use_fused(m) ? ms_enqueue_fused(m, outs, launches) : ms_enqueue(m, outs, launches);
}

bool ms_launch_graph(vsc_multistream* m, const std::vector<uint8_t*>& outs, int* launches, cudaError_t* err)
{
    *err = cudaSuccess;
    vsc_stabilizer* s0 = m->st[0];
    vsc_multistream::Graph* hit = nullptr;
    for (auto& g : m->graphs)
        if (g.valid && g.head == s0->head && g.ls_cur == s0->ls_cur && g.outs == outs && same_hp(g.hp, m->hp))
            hit = &g;
    if (!hit) {
        auto* slot = &m->graphs[0];
        for (auto& g : m->graphs)
            if (!g.valid || g.used < slot->used)
                slot = &g;
        if (slot->exec) {
            cudaGraphExecDestroy(slot->exec);
            slot->exec = nullptr;
        }
        slot->valid = false;
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(m->main, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        int nl = 0;
        const cudaError_t ee = ms_step_enqueue(m, outs, &nl);
        const cudaError_t ec = cudaStreamEndCapture(m->main, &graph);
        if (ee != cudaSuccess || ec != cudaSuccess || !graph) {
            if (graph)
                cudaGraphDestroy(graph);
            cudaGetLastError();
            return false;
        }
        const cudaError_t ei = cudaGraphInstantiate(&slot->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            cudaGetLastError();
            slot->exec = nullptr;
            return false;
        }
        slot->valid = true;
        slot->head = s0->head;
        slot->ls_cur = s0->ls_cur;
        slot->outs = outs;
        slot->hp = m->hp;
        slot->nl = nl;
        hit = slot;
    }
    hit->used = ++m->clock;
    *launches = hit->nl;
    *err = cudaGraphLaunch(hit->exec, m->main);
    return true;
}

}  // namespace

extern "C" {

VSC_API vsc_status vsc_multistream_create(const vsc_stream_desc* desc, int32_t n, vsc_stream_t stream,
    vsc_multistream** out)
{
    clear_error();
    if (!desc || !out || n < 1 || n > 256)
        return set_error(VSC_EINVAL, "multistream_create: bad arguments (1..256 streams)");
    *out = nullptr;
    vsc_multistream* m = new (std::nothrow) vsc_multistream();
    if (!m)
        return set_error(VSC_ENOMEM, "multistream_create: out of host memory");
    cudaGetDevice(&m->device);
    vsc_default_hyper_params(&m->hp);
    vsc_status s = VSC_OK;
    cudaError_t e = cudaSuccess;
    m->main = cs(stream);
    if (!m->main) {  // capture needs a stream other than the legacy default one
        e = cudaStreamCreateWithFlags(&m->main, cudaStreamNonBlocking);
        m->own_main = e == cudaSuccess;
    }
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&m->done, cudaEventDisableTiming);
    for (int i = 0; i < n && e == cudaSuccess && !s; ++i) {
        cudaStream_t x = nullptr;
        cudaEvent_t a = nullptr, b = nullptr;
        e = cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            m->side.push_back(x);
        if (e == cudaSuccess && (e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming)) == cudaSuccess)
            m->loaded.push_back(a);
        if (e == cudaSuccess && (e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming)) == cudaSuccess)
            m->joined.push_back(b);
        if (e != cudaSuccess)
            break;
        vsc_stabilizer_config cfg{};
        cfg.width = desc[i].width;
        cfg.height = desc[i].height;
        cfg.batch_size = 1;
        cfg.compute_flow = 1;
        cfg.flow_downscale = desc[i].flow_downscale > 0 ? desc[i].flow_downscale : 1;
        cfg.flow_channels = 3;
        cfg.use_graphs = 0;  // the multistream object captures the whole step itself
        cfg.corr_dtype = desc[i].corr_dtype;
        vsc_stabilizer* st = nullptr;
        if ((s = vsc_stabilizer_create(&cfg, x, &st)) == VSC_OK)
            m->st.push_back(st);
    }
    if (!s && e != cudaSuccess)
        s = check_cuda(e, "multistream_create");
    // grouped solves: per-level workspaces above level 0, and the tile shape
    // of each level's group (a stream being captured keeps the wave model)
    m->fused_ok = !s;
    for (size_t i = 0; i < m->st.size() && !s; ++i) {
        vsc_stabilizer* st = m->st[i];
        size_t floats = 0;
        for (int j = 1; j < st->levels_alloc; ++j)
            floats += solver_workspace_floats(st->lw[j], st->lh[j], kSolverFma);  // room for either form
        float* p = nullptr;
        if (floats && (s = check_cuda(dalloc(&p, floats), "multistream_create level workspaces")))
            break;
        m->lvl_ws.push_back(p);
    }
    if (!s)
        ms_tune(m, kSolverExact);
    if (s) {
        const std::string msg = vsc_last_error();
        ms_free(m);
        delete m;
        return set_error(s, "%s", msg.c_str());
    }
    *out = m;
    return VSC_OK;
}

VSC_API vsc_status vsc_multistream_destroy(vsc_multistream* m)
{
    clear_error();
    if (!m)
        return VSC_OK;
    DeviceGuard g(m->device);
    cudaStreamSynchronize(m->main);
    ms_free(m);
    delete m;
    return VSC_OK;
}

VSC_API vsc_hyper_params* vsc_multistream_hyper_params(vsc_multistream* m) { return m ? &m->hp : nullptr; }

VSC_API int32_t vsc_multistream_last_launches(vsc_multistream* m) { return m ? m->last_launches : 0; }

VSC_API vsc_status vsc_multistream_set_fused(vsc_multistream* m, int32_t on)
{
    clear_error();
    if (!m)
        return set_error(VSC_EINVAL, "multistream_set_fused: null argument");
    DeviceGuard g(m->device);
    if (m->fused != (on != 0)) {
        cudaStreamSynchronize(m->main);  // a graph being replayed is not destroyed under it
        ms_drop_graphs(m);
    }
    m->fused = on != 0;
    return VSC_OK;
}

VSC_API int32_t vsc_multistream_fused(vsc_multistream* m) { return m && ms_use_fused(m) ? 1 : 0; }

VSC_API vsc_status vsc_multistream_set_solver_form(vsc_multistream* m, int32_t form)
{
    clear_error();
    if (!m)
        return set_error(VSC_EINVAL, "multistream_set_solver_form: null argument");
    if (form != VSC_SOLVER_EXACT && form != VSC_SOLVER_FMA)
        return set_error(VSC_EINVAL, "multistream_set_solver_form: unknown solver form %d", form);
    DeviceGuard g(m->device);
    vsc_status s = check_cuda(cudaStreamSynchronize(m->main), "multistream_set_solver_form");
    for (size_t i = 0; i < m->st.size() && !s; ++i)
        s = vsc_stabilizer_set_solver_form(m->st[i], form);
    if (s)
        return s;
    if (form != m->solver_form)
        ms_tune(m, form);
    m->solver_form = form;
    ms_drop_graphs(m);
    return VSC_OK;
}

VSC_API vsc_status vsc_multistream_set_upsampler(vsc_multistream* m, int32_t index, vsc_upsampler* u)
{
    clear_error();
    if (!m)
        return set_error(VSC_EINVAL, "multistream_set_upsampler: null argument");
    if (index < -1 || index >= static_cast<int32_t>(m->st.size()))
        return set_error(VSC_EINVAL, "multistream_set_upsampler: stream %d outside [-1, %zu)", index, m->st.size());
    DeviceGuard g(m->device);
    vsc_status s = check_cuda(cudaStreamSynchronize(m->main), "multistream_set_upsampler");
    if (s)
        return s;
    // the FP16 weights are packed here, once, not inside a captured step
    if (u && (s = check_cuda(upsampler_sync_weights(u, m->main), "multistream_set_upsampler weights")))
        return s;
    if ((s = check_cuda(cudaStreamSynchronize(m->main), "multistream_set_upsampler")))
        return s;
    for (size_t i = 0; i < m->st.size() && !s; ++i) {
        vsc_stabilizer* st = m->st[i];
        if (index >= 0 ? static_cast<int32_t>(i) == index : (st->compute_flow && st->downscale > 1))
            s = vsc_stabilizer_set_upsampler(st, u);
    }
    ms_drop_graphs(m);
    return s;
}

VSC_API vsc_status vsc_multistream_load_frames(vsc_multistream* m, const uint8_t* const* orig,
    const uint8_t* const* proc, int32_t on_device)
{
    clear_error();
    if (!m || !orig || !proc)
        return set_error(VSC_EINVAL, "multistream_load_frames: null argument");
    DeviceGuard g(m->device);
    vsc_status s = check_cuda(cudaEventRecord(m->done, m->main), "multistream_load_frames");
    for (size_t i = 0; i < m->st.size() && !s; ++i) {
        // the previous step, which reads the window, completes first
        if ((s = check_cuda(cudaStreamWaitEvent(m->side[i], m->done, 0), "multistream_load_frames")))
            break;
        if ((s = vsc_stabilizer_load_frame(m->st[i], orig[i], proc[i], on_device)))
            break;
        s = check_cuda(cudaEventRecord(m->loaded[i], m->side[i]), "multistream_load_frames");
    }
    return s;
}

VSC_API vsc_status vsc_multistream_step(vsc_multistream* m, uint8_t* const* out, int32_t out_on_device)
{
    clear_error();
    if (!m)
        return set_error(VSC_EINVAL, "multistream_step: null argument");
    DeviceGuard g(m->device);
    vsc_status s;
    for (vsc_stabilizer* st : m->st)
        if ((s = step_preconditions(st, m->hp)))
            return s;
    const size_t n = m->st.size();
    std::vector<uint8_t*> outs(n);
    for (size_t i = 0; i < n; ++i) {
        outs[i] = (out && out[i] && out_on_device) ? out[i] : m->st[i]->out_rgba;
        if (reinterpret_cast<uintptr_t>(outs[i]) & 3)
            return set_error(VSC_EINVAL, "multistream_step: device output %zu not 4-byte aligned", i);
    }
    for (size_t i = 0; i < n; ++i)  // the frames just loaded are in place
        if ((s = check_cuda(cudaStreamWaitEvent(m->main, m->loaded[i], 0), "multistream_step")))
            return s;
    int nl = 0;
    cudaError_t e = cudaSuccess;
    bool started = true;
    for (vsc_stabilizer* st : m->st)
        started = started && st->started;
    if (!(started && ms_launch_graph(m, outs, &nl, &e)))
        e = ms_step_enqueue(m, outs, &nl);
    if ((s = check_cuda(e, "multistream_step")))
        return s;
    for (vsc_stabilizer* st : m->st)
        finish_step(st, 0);
    m->last_launches = nl;
    if (out && !out_on_device) {
        for (size_t i = 0; i < n; ++i)
            if (out[i] &&
                (s = check_cuda(cudaMemcpyAsync(out[i], outs[i], static_cast<size_t>(m->st[i]->w) * m->st[i]->h * 4,
                                    cudaMemcpyDeviceToHost, m->main),
                     "multistream_step download")))
                return s;
        return check_cuda(cudaStreamSynchronize(m->main), "multistream_step synchronize");
    }
    return VSC_OK;
}

}  // extern "C"

