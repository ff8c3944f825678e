/*
 * TEST INFRASTRUCTURE ONLY — runs the reference's own CUDA kernels.
 *
 * The kernels come from cubins compiled in place from the reference tree
 * (oracle/ref_gpu/ref_kernels.cu, "make refgpu"); this harness loads one with
 * the driver API, finds each kernel by name, and launches it with the
 * geometry and the call sequence of the reference's host launchers:
 *   flowconsistency.cu:262-374   get_warp_result, get_adap_comb, get_consist_wt,
 *                                get_bilinear, get_consist_out (32x32 blocks,
 *                                grid (n+32)/32, cudaDeviceSynchronize after each,
 *                                get_consist_out allocating its temporaries and
 *                                updating consisOut in place, :363-372)
 *   gpuimage.cu:70-135           the RGBA8 conversions
 *   correlation_cuda.cu:333-442  rearrange to NHWC temporaries, 1 block per output pixel
 *                                (legacy = 0); legacy = 1 (:182-331, :350-400): temporaries
 *                                padded by 4, CorrelateData_old's geometry
 *   warp_cuda.cu:86-98           one 32-thread block row per channel
 *   videostabilizer.cpp:182-238  the order of one doOneStep pass
 * Used by the tests to pin the CPU restatement against the reference's GPU
 * code and by bench.py to time the reference's schedule on the same GPU.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

// Outside the unnamed namespace: the exported functions take it by value,
// and a parameter type with internal linkage would make them internal too.
struct Img {  // layout of GPUImageWrapper (gpuimagewrapper.h:8-24)
    float* data;
    int width, height, channels;
};

namespace {

CUmodule g_mod = nullptr;
std::string g_err;
enum K { kWarp, kAdap, kWt, kOut, kBil, kToF, kToC, kCorr, kRearr, kWarpOp, kCorrOld, kCount };
CUfunction g_fn[kCount] = {};
// Kernels are found by their source name inside the mangled name: the
// Itanium ABI writes <length><name> (then "If" for the float instantiation
// of the templated op kernels).
const char* const kNames[kCount] = {"kernel_warp", "kernel_adap_comb", "kernel_consist_wt", "kernel_consist_out",
    "kernel_bilinear", "kernel_to_float_image", "kernel_to_char_image", "correlation_cuda_forward_kernel",
    "blob_rearrange_kernel", "warp_forward_kernel", "correlation_old_kernel"};
const bool kTemplated[kCount] = {false, false, false, false, false, false, false, true, true, true, true};

std::string mangled_key(int k)
{
    return std::to_string(std::strlen(kNames[k])) + kNames[k] + (kTemplated[k] ? "If" : "");
}

int fail(const char* what, CUresult r)
{
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "?");
    return -1;
}

int launch(K k, dim3 grid, dim3 block, void** args, CUstream st, unsigned smem = 0)
{
    CUresult r = cuLaunchKernel(g_fn[k], grid.x, grid.y, grid.z, block.x, block.y, block.z, smem, st, args, nullptr);
    return r == CUDA_SUCCESS ? 0 : fail(kNames[k], r);
}

dim3 grid_of(int w, int h) { return dim3((w + 32) / 32, (h + 32) / 32, 1); }  // getGrid, flowconsistency.cu:262-266

int sync() { return cudaDeviceSynchronize() == cudaSuccess ? 0 : (g_err = "sync", -1); }

}  // namespace

extern "C" {

const char* rg_last_error(void) { return g_err.c_str(); }

int rg_init(const char* cubin)
{
    cudaFree(nullptr);  // make the runtime's primary context current
    CUresult r = cuModuleLoad(&g_mod, cubin);
    if (r != CUDA_SUCCESS)
        return fail("cuModuleLoad", r);
    unsigned n = 0;
    if ((r = cuModuleGetFunctionCount(&n, g_mod)) != CUDA_SUCCESS)
        return fail("cuModuleGetFunctionCount", r);
    std::vector<CUfunction> fns(n);
    if ((r = cuModuleEnumerateFunctions(fns.data(), n, g_mod)) != CUDA_SUCCESS)
        return fail("cuModuleEnumerateFunctions", r);
    for (CUfunction f : fns) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name)
            continue;
        for (int k = 0; k < kCount; ++k)
            if (std::strstr(name, mangled_key(k).c_str()))
                g_fn[k] = f;
    }
    for (int k = 0; k < kCount; ++k)
        if (!g_fn[k]) {
            g_err = std::string("kernel not found: ") + mangled_key(k);
            return -1;
        }
    return 0;
}

// ---- stabilization launchers (flowconsistency.cu:288-374) -------------------
int rg_warp(Img in, Img flow, Img out)
{
    void* a[] = {&in, &flow, &out};
    if (launch(kWarp, grid_of(in.width, in.height), dim3(32, 32), a, 0))
        return -1;
    return sync();
}

int rg_adap_comb(Img ci, Img cp, Img pwi, Img pwp, Img nwi, Img nwp, Img ai, Img ap, Img lsw, float alpha)
{
    void* a[] = {&ci, &cp, &pwi, &pwp, &nwi, &nwp, &ai, &ap, &lsw, &alpha};
    if (launch(kAdap, grid_of(ci.width, ci.height), dim3(32, 32), a, 0))
        return -1;
    return sync();
}

// get_consist_wt(adapCmbIn, crntIn, consisWt, beta, gamma) launches
// kernel_consist_wt(crntIn, adapCmbIn, consisWt, beta, gamma)
int rg_consist_wt(Img ai, Img ci, Img wt, float beta, float gamma)
{
    void* a[] = {&ci, &ai, &wt, &beta, &gamma};
    if (launch(kWt, grid_of(ci.width, ci.height), dim3(32, 32), a, 0))
        return -1;
    return sync();
}

int rg_bilinear(Img in, Img out)
{
    void* a[] = {&in, &out};
    if (launch(kBil, grid_of(out.width, out.height), dim3(32, 32), a, 0))
        return -1;
    return sync();
}

int rg_consist_out(Img pr, Img stab, Img wt, int num_iter, float step, float mom, Img out)
{
    // GPUImage prevUpdt / prevConsis of the launcher: fresh, uninitialised allocations
    Img upd = out, prev = out;
    const size_t bytes = static_cast<size_t>(out.width) * out.height * 3 * sizeof(float);
    if (cudaMalloc(&upd.data, bytes) != cudaSuccess || cudaMalloc(&prev.data, bytes) != cudaSuccess)
        return (g_err = "cudaMalloc", -1);
    int rc = 0;
    for (int k = 0; k < num_iter && !rc; ++k) {
        void* a[] = {&out, &out, &upd, &pr, &stab, &wt, &step, &mom, &k};
        rc = launch(kOut, grid_of(out.width, out.height), dim3(32, 32), a, 0);
    }
    if (!rc)
        rc = sync();
    cudaFree(upd.data);
    cudaFree(prev.data);
    return rc;
}

int rg_to_float(const uint8_t* rgba, Img out)
{
    void* a[] = {&rgba, &out};
    if (launch(kToF, grid_of(out.width, out.height), dim3(32, 32), a, 0))
        return -1;
    return sync();
}

int rg_to_char(Img in, uint8_t* rgba)
{
    void* a[] = {&in, &rgba};
    if (launch(kToC, grid_of(in.width, in.height), dim3(32, 32), a, 0))
        return -1;
    return sync();
}

// ---- custom ops (correlation_cuda.cu:333-442, warp_cuda.cu:86-98) ----------
int rg_correlation(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md, void* stream)
{
    CUstream st = static_cast<CUstream>(stream);
    const int HW = H * W;
    float *r1 = nullptr, *r2 = nullptr;
    const size_t bytes = static_cast<size_t>(HW) * N * C * sizeof(float);
    if (cudaMalloc(&r1, bytes) != cudaSuccess || cudaMalloc(&r2, bytes) != cudaSuccess)
        return (g_err = "cudaMalloc", -1);
    int pad = 0;
    int rc = 0;
    const float* ins[2] = {f1, f2};
    float* outs[2] = {r1, r2};
    for (int i = 0; i < 2 && !rc; ++i) {
        void* a[] = {&ins[i], &outs[i], &N, &C, &W, &H, const_cast<int*>(&HW), &pad, const_cast<int*>(&HW)};
        rc = launch(kRearr, dim3((HW - 1) / 16 + 1, C, N), dim3(16), a, st);
    }
    int kH = 1, kW = 1, P = 2 * md + 1, one = 1, zero = 0;
    if (!rc) {
        void* a[] = {&r1, &r2, &out, &N, &C, &H, &W, &kH, &kW, &P, &P, &zero, &zero, &one, &one, &one, &one, &one,
            &one, &H, &W};
        rc = launch(kCorr, dim3(N, H, W), dim3(32), a, st);
    }
    cudaFree(r1);
    cudaFree(r2);
    return rc;
}

// legacy = 1: correlation_cuda_forward with spatial_corr_sampler = false
// (correlation_cuda.cu:350-400): both inputs rearranged to NHWC temporaries
// padded by 4 pixels on every side, then CorrelateData_old (:267-331) with
// kernel_size 1, strides 1, grid (W, H, N), 32 threads and C floats of
// dynamic shared memory.  The reference leaves the padding of its
// temporaries uninitialised (cudaMalloc, :366-370; the rearrange writes the
// interior only), so a border output reads whatever the allocation held;
// the harness clears the temporaries, which is the zero padding the op's
// CPU semantics define.  The kernel places the window centre at padded
// column x + max_displacement while the data sit at x + 4, so only
// max_displacement = 4 (PWC-Net's) is meaningful.
int rg_correlation_legacy(const float* f1, const float* f2, float* out, int N, int C, int H, int W, int md,
    void* stream)
{
    CUstream st = static_cast<CUstream>(stream);
    const int pad = 4;
    const int HW = H * W;
    int PW = W + 2 * pad, PH = H + 2 * pad;
    int pHW = PW * PH;
    float *r1 = nullptr, *r2 = nullptr;
    const size_t bytes = static_cast<size_t>(pHW) * N * C * sizeof(float);
    if (cudaMalloc(&r1, bytes) != cudaSuccess || cudaMalloc(&r2, bytes) != cudaSuccess)
        return (g_err = "cudaMalloc", -1);
    int rc = 0;
    if (cudaMemsetAsync(r1, 0, bytes, st) != cudaSuccess || cudaMemsetAsync(r2, 0, bytes, st) != cudaSuccess)
        rc = (g_err = "cudaMemset", -1);
    const float* ins[2] = {f1, f2};
    float* outs[2] = {r1, r2};
    int padv = pad;
    for (int i = 0; i < 2 && !rc; ++i) {
        void* a[] = {&ins[i], &outs[i], &N, &C, &W, &H, const_cast<int*>(&HW), &padv, &pHW};
        rc = launch(kRearr, dim3((HW - 1) / 16 + 1, C, N), dim3(16), a, st);
    }
    int P = 2 * md + 1;
    int planes = P * P, count = H * W * planes, radius = md, kradius = 0, ksize = 1, one = 1;
    if (!rc) {
        void* a[] = {&count, &N, &W, &H, &planes, &count, &md, &radius, &P, &kradius, &ksize, &one, &one, &PW, &PH,
            &C, &r1, &r2, &out};
        rc = launch(kCorrOld, dim3(W, H, N), dim3(32), a, st, static_cast<unsigned>(C * sizeof(float)));
    }
    if (!rc && cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess)
        rc = (g_err = "sync", -1);
    cudaFree(r1);
    cudaFree(r2);
    return rc;
}

int rg_warp_op(const float* in, const float* flow, float* out, int N, int C, int H, int W, void* stream)
{
    void* a[] = {&in, &flow, &out, &W, &H, &C};
    return launch(kWarpOp, dim3((H * W - 1) / 32 + 1, C, N), dim3(32), a, static_cast<CUstream>(stream));
}

// ---- one doOneStep stabilization pass (videostabilizer.cpp:178-247) ----------
// in: orig0..2, proc0..2, flow results fwd, bwd, lastStabilizedFrame (updated
// in place as the reference's feedback copy does, :247).  scratch: 11
// full-size images: prevWarpIn, prevWarpPr, nextWarpIn, nextWarpPr,
// lastStabWarp, adapCmbIn, adapCmbPr, consWt, consisOut, flowFwd, flowBwd.
// lvl0: pyrPr[0], pyrAdapCmbPr[0], pyrConsWt[0], pyrConsisOut[0]; lvl1: the
// same at half size.  host_rgba: the RGBA8 output (copyToQImage: device
// buffer allocated per call, kernel, synchronise, download, free).
int rg_stab_pass(const Img* in, const Img* scratch, const Img* lvl0, const Img* lvl1, int pyramid_levels,
    int num_iter, float alpha, float beta, float gamma, float step, float mom, uint8_t* host_rgba)
{
    const Img &o0 = in[0], &o1 = in[1], &o2 = in[2], &p0 = in[3], &p1 = in[4], &p2 = in[5];
    const Img &ffr = in[6], &fbr = in[7], &ls = in[8];
    const Img &pwi = scratch[0], &pwp = scratch[1], &nwi = scratch[2], &nwp = scratch[3], &lsw = scratch[4];
    const Img &ain = scratch[5], &apr = scratch[6], &cwt = scratch[7], &cout = scratch[8];
    const Img &ff = scratch[9], &fb = scratch[10];
    const size_t b3 = static_cast<size_t>(o1.width) * o1.height * 3 * sizeof(float);
    const size_t bf = static_cast<size_t>(o1.width) * o1.height * ff.channels * sizeof(float);
    auto cp = [](const Img& d, const Img& s, size_t n) {
        return cudaMemcpy(d.data, s.data, n, cudaMemcpyDeviceToDevice) == cudaSuccess;
    };
    if (!cp(ff, ffr, bf) || !cp(fb, fbr, bf))
        return (g_err = "copy", -1);
    if (rg_warp(o0, fb, pwi) || rg_warp(p0, fb, pwp) || rg_warp(o2, ff, nwi) || rg_warp(p2, ff, nwp) ||
        rg_warp(ls, fb, lsw))
        return -1;
    if (rg_adap_comb(o1, p1, pwi, pwp, nwi, nwp, ain, apr, lsw, alpha) || rg_consist_wt(ain, o1, cwt, beta, gamma))
        return -1;
    if (!cp(lvl0[0], p1, b3) || !cp(lvl0[1], apr, b3) || !cp(lvl0[2], cwt, b3) || !cp(lvl0[3], p1, b3))
        return (g_err = "copy", -1);
    if (pyramid_levels == 2) {
        for (int i = 0; i < 4; ++i)
            if (rg_bilinear(lvl0[i], lvl1[i]))
                return -1;
        if (rg_consist_out(lvl1[0], lvl1[1], lvl1[2], num_iter / 2, step, mom, lvl1[3]) ||
            rg_bilinear(lvl1[3], lvl0[3]))
            return -1;
    }
    if (rg_consist_out(lvl0[0], lvl0[1], lvl0[2], num_iter, step, mom, lvl0[3]))
        return -1;
    if (!cp(cout, lvl0[3], b3))
        return (g_err = "copy", -1);
    if (host_rgba) {
        uint8_t* dev = nullptr;
        const size_t nb = static_cast<size_t>(o1.width) * o1.height * 4;
        if (cudaMalloc(&dev, nb) != cudaSuccess)
            return (g_err = "cudaMalloc", -1);
        int rc = rg_to_char(cout, dev);
        if (!rc && cudaMemcpy(host_rgba, dev, nb, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = (g_err = "download", -1);
        cudaFree(dev);
        if (rc)
            return rc;
    }
    return cp(ls, cout, b3) ? 0 : (g_err = "copy", -1);
}

}  // extern "C"
