// ONNX Runtime custom-op library over the vsc C ABI: the drop-in replacement
// of the reference's op library (src/ort_custom_ops).
//
// Exports the same entry point, RegisterCustomOps (custom_ops.h:50,
// custom_ops.cpp:74-98), registers domain "custom" with the operators
// "Correlation" and "Warp", the same node attributes (legacy,
// max_displacement: correlation.h:19-31) and tensor signatures (two FLOAT
// inputs, one FLOAT output: correlation.h:71-80, warp.h:38-59).  Both
// execution providers are registered, as in custom_ops.cpp:18-52:
//   CUDAExecutionProvider : tensors are device memory; the kernels run on
//                           the context's compute stream (correlation_cuda.cc:80);
//   CPUExecutionProvider  : tensors are host memory; they are staged through
//                           device memory from the stream-ordered pool and the
//                           same CUDA kernels compute the result — the library
//                           has no CPU implementation.
// Errors are thrown as std::runtime_error with the library's message, as the
// reference kernels throw (correlation.h:23, correlation.cc:140-141).
//
// Build: only where ONNX Runtime headers exist (build.py: build_ort(<include dir>)).
#ifndef ORT_API_MANUAL_INIT
#define ORT_API_MANUAL_INIT
#endif
#include <onnxruntime_cxx_api.h>

#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "vsc.h"

namespace {

const char* const kCUDAProvider = "CUDAExecutionProvider";
const char* const kCPUProvider = "CPUExecutionProvider";

void check(vsc_status st, const char* what)
{
    if (st != VSC_OK)
        throw std::runtime_error(std::string(what) + ": " + vsc_last_error());
}

void check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess)
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

bool is_cuda(const char* provider) { return std::string(provider).find("CUDA") != std::string::npos; }

// Device staging of host tensors for the CPU provider (freed on scope exit,
// stream-ordered).
struct Staged {
    void* p = nullptr;
    cudaStream_t st = nullptr;
    Staged(size_t bytes, cudaStream_t s) : st(s) { check_cuda(cudaMallocAsync(&p, bytes, st), "staging"); }
    ~Staged()
    {
        if (p)
            cudaFreeAsync(p, st);
    }
};

struct KernelBase {
    KernelBase(const OrtApi& api, const char* provider) : api_(api), provider_(provider) { }
    const OrtApi& api_;
    const char* provider_;
};

std::vector<int64_t> shape_of(const Ort::ConstValue& v) { return v.GetTensorTypeAndShapeInfo().GetShape(); }

ONNXTensorElementDataType elem_type(const Ort::ConstValue& v) { return v.GetTensorTypeAndShapeInfo().GetElementType(); }

// CUDA provider: FLOAT only, as the reference's CUDA kernels (correlation_cuda.cc, warp_cuda.cc).
void require_float(const Ort::ConstValue& v)
{
    if (elem_type(v) != ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT)
        throw std::runtime_error("Unsupported input type. Must be float.");
}

// CPU provider: FLOAT or DOUBLE, as the reference's CPU kernels dispatch
// (correlation.cc:115-141, warp.cc:48-64); returns the element size.
size_t require_float_or_double(const Ort::ConstValue& a, const Ort::ConstValue& b)
{
    const auto t = elem_type(a);
    if ((t != ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT && t != ONNX_TENSOR_ELEMENT_DATA_TYPE_DOUBLE) || elem_type(b) != t)
        throw std::runtime_error("Unsupported input type. Must be float or double.");
    return t == ONNX_TENSOR_ELEMENT_DATA_TYPE_DOUBLE ? sizeof(double) : sizeof(float);
}

struct CorrelationKernel : KernelBase {
    CorrelationKernel(const OrtApi& api, const OrtKernelInfo* info, const char* provider) : KernelBase(api, provider)
    {
        // correlation.h:19-31: both attributes are required
        int64_t v = 0;
        OrtStatusPtr err = api.KernelInfoGetAttribute_int64(info, "legacy", &v);
        if (err)
            throw std::runtime_error(std::string("Error reading attribute 'legacy', with error: ") +
                                     api.GetErrorMessage(err));
        legacy_ = v;
        err = api.KernelInfoGetAttribute_int64(info, "max_displacement", &md_);
        if (err)
            throw std::runtime_error(std::string("Error reading attribute 'max_displacement', with error: ") +
                                     api.GetErrorMessage(err));
    }

    void Compute(OrtKernelContext* context)
    {
        Ort::KernelContext ctx{context};
        Ort::ConstValue in1 = ctx.GetInput(0);
        Ort::ConstValue in2 = ctx.GetInput(1);
        const bool cuda = is_cuda(provider_);
        if (cuda) {
            require_float(in1);
            require_float(in2);
        }
        const size_t es = cuda ? sizeof(float) : require_float_or_double(in1, in2);
        const std::vector<int64_t> d = shape_of(in1);
        if (d.size() != 4 || shape_of(in2) != d)
            throw std::runtime_error("Correlation: inputs must be two N x C x H x W tensors of the same shape");
        const int64_t N = d[0], C = d[1], H = d[2], W = d[3], P = 2 * md_ + 1;
        const std::vector<int64_t> od =
            legacy_ ? std::vector<int64_t>{N, P * P, H, W} : std::vector<int64_t>{N, P, P, H, W};
        auto out = ctx.GetOutput(0, od.data(), od.size());
        const size_t in_bytes = static_cast<size_t>(N * C * H * W) * es;
        const size_t out_bytes = static_cast<size_t>(N * P * P * H * W) * es;
        if (cuda) {
            auto st = static_cast<vsc_stream_t>(ctx.GetGPUComputeStream());
            check(vsc_correlation_fwd(in1.GetTensorData<float>(), in2.GetTensorData<float>(),
                      out.GetTensorMutableData<float>(), N, C, H, W, md_, legacy_, st),
                "Correlation");
            return;
        }
        if (legacy_)  // correlation.h:45-46
            throw std::runtime_error("Legacy correlation not supported in CPU mode (only cuda)");
        cudaStream_t st = cudaStreamPerThread;
        Staged a(in_bytes, st), b(in_bytes, st), o(out_bytes, st);
        check_cuda(cudaMemcpyAsync(a.p, in1.GetTensorRawData(), in_bytes, cudaMemcpyHostToDevice, st), "upload");
        check_cuda(cudaMemcpyAsync(b.p, in2.GetTensorRawData(), in_bytes, cudaMemcpyHostToDevice, st), "upload");
        if (es == sizeof(double))
            check(vsc_correlation_fwd_f64(static_cast<double*>(a.p), static_cast<double*>(b.p),
                      static_cast<double*>(o.p), N, C, H, W, md_, st),
                "Correlation");
        else
            check(vsc_correlation_fwd(static_cast<float*>(a.p), static_cast<float*>(b.p), static_cast<float*>(o.p), N,
                      C, H, W, md_, 0, st),
                "Correlation");
        check_cuda(cudaMemcpyAsync(out.GetTensorMutableRawData(), o.p, out_bytes, cudaMemcpyDeviceToHost, st),
            "download");
        check_cuda(cudaStreamSynchronize(st), "synchronize");
    }

    int64_t legacy_ = 0;
    int64_t md_ = 4;
};

struct WarpKernel : KernelBase {
    WarpKernel(const OrtApi& api, const OrtKernelInfo*, const char* provider) : KernelBase(api, provider) { }

    void Compute(OrtKernelContext* context)
    {
        Ort::KernelContext ctx{context};
        Ort::ConstValue x = ctx.GetInput(0);
        Ort::ConstValue flow = ctx.GetInput(1);
        const bool cuda = is_cuda(provider_);
        if (cuda) {
            require_float(x);
            require_float(flow);
        }
        const size_t es = cuda ? sizeof(float) : require_float_or_double(x, flow);
        const std::vector<int64_t> d = shape_of(x);
        const std::vector<int64_t> fd = shape_of(flow);
        // warp.cc reads the flow as N x 2 x H x W without checking; we do check
        if (d.size() != 4 || fd.size() != 4 || fd[0] != d[0] || fd[1] != 2 || fd[2] != d[2] || fd[3] != d[3])
            throw std::runtime_error("Warp: input N x C x H x W and flow N x 2 x H x W expected");
        const int64_t N = d[0], C = d[1], H = d[2], W = d[3];
        auto out = ctx.GetOutput(0, d.data(), d.size());
        if (cuda) {
            auto st = static_cast<vsc_stream_t>(ctx.GetGPUComputeStream());
            check(vsc_warp_fwd(x.GetTensorData<float>(), flow.GetTensorData<float>(), out.GetTensorMutableData<float>(),
                      N, C, H, W, st),
                "Warp");
            return;
        }
        cudaStream_t st = cudaStreamPerThread;
        const size_t xb = static_cast<size_t>(N * C * H * W) * es;
        const size_t fb = static_cast<size_t>(N * 2 * H * W) * es;
        Staged a(xb, st), f(fb, st), o(xb, st);
        check_cuda(cudaMemcpyAsync(a.p, x.GetTensorRawData(), xb, cudaMemcpyHostToDevice, st), "upload");
        check_cuda(cudaMemcpyAsync(f.p, flow.GetTensorRawData(), fb, cudaMemcpyHostToDevice, st), "upload");
        if (es == sizeof(double))
            check(vsc_warp_fwd_f64(static_cast<double*>(a.p), static_cast<double*>(f.p), static_cast<double*>(o.p), N,
                      C, H, W, st),
                "Warp");
        else
            check(vsc_warp_fwd(static_cast<float*>(a.p), static_cast<float*>(f.p), static_cast<float*>(o.p), N, C, H,
                      W, st),
                "Warp");
        check_cuda(cudaMemcpyAsync(out.GetTensorMutableRawData(), o.p, xb, cudaMemcpyDeviceToHost, st), "download");
        check_cuda(cudaStreamSynchronize(st), "synchronize");
    }
};

struct CorrelationOp : Ort::CustomOpBase<CorrelationOp, CorrelationKernel> {
    explicit CorrelationOp(const char* provider) : provider_(provider) { }
    void* CreateKernel(const OrtApi& api, const OrtKernelInfo* info) const
    {
        return new CorrelationKernel(api, info, provider_);
    }
    const char* GetName() const { return "Correlation"; }
    const char* GetExecutionProviderType() const { return provider_; }
    size_t GetInputTypeCount() const { return 2; }
    ONNXTensorElementDataType GetInputType(size_t) const { return ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT; }
    size_t GetOutputTypeCount() const { return 1; }
    ONNXTensorElementDataType GetOutputType(size_t) const { return ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT; }

private:
    const char* provider_;
};

struct WarpOp : Ort::CustomOpBase<WarpOp, WarpKernel> {
    explicit WarpOp(const char* provider) : provider_(provider) { }
    void* CreateKernel(const OrtApi& api, const OrtKernelInfo* info) const
    {
        return new WarpKernel(api, info, provider_);
    }
    const char* GetName() const { return "Warp"; }
    const char* GetExecutionProviderType() const { return provider_; }
    size_t GetInputTypeCount() const { return 2; }
    ONNXTensorElementDataType GetInputType(size_t) const { return ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT; }
    size_t GetOutputTypeCount() const { return 1; }
    ONNXTensorElementDataType GetOutputType(size_t) const { return ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT; }

private:
    const char* provider_;
};

// Op descriptors and domains live as long as the process (ORT keeps raw
// pointers to them), as in custom_ops.cpp:64-72.
struct Registry {
    std::mutex mu;
    std::vector<std::unique_ptr<CorrelationOp>> corr;
    std::vector<std::unique_ptr<WarpOp>> warp;
    std::vector<OrtCustomOpDomain*> domains;
};

Registry& registry()
{
    static Registry r;
    return r;
}

}  // namespace

extern "C" __attribute__((visibility("default"))) OrtStatus* ORT_API_CALL RegisterCustomOps(OrtSessionOptions* options,
    const OrtApiBase* api_base)
{
    const OrtApi* api = api_base->GetApi(ORT_API_VERSION);
    if (!api)
        return nullptr;  // custom_ops.cpp:79-84: version mismatch is reported by returning null
    Ort::InitApi(api);
    Registry& r = registry();
    std::lock_guard<std::mutex> lock(r.mu);
    OrtCustomOpDomain* domain = nullptr;
    if (OrtStatus* st = api->CreateCustomOpDomain("custom", &domain))
        return st;
    r.domains.push_back(domain);
    std::vector<OrtCustomOp*> ops;
    bool has_cuda = false;
    for (const std::string& p : Ort::GetAvailableProviders())
        has_cuda = has_cuda || p == kCUDAProvider;
    for (const char* p : {kCUDAProvider, kCPUProvider}) {
        if (p == kCUDAProvider && !has_cuda)
            continue;
        r.corr.emplace_back(new CorrelationOp(p));
        r.warp.emplace_back(new WarpOp(p));
        ops.push_back(r.corr.back().get());
        ops.push_back(r.warp.back().get());
    }
    for (OrtCustomOp* op : ops)
        if (OrtStatus* st = api->CustomOpDomain_Add(domain, op))
            return st;
    return api->AddCustomOpDomain(options, domain);
}
