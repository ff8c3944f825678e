/*
 * Minimal, project-written stand-in for the ONNX Runtime C++ API header.
 *
 * TEST INFRASTRUCTURE ONLY (see onnxruntime_c_api.h in this directory).  It
 * provides the C++ wrapper types the reference CPU custom ops use
 * (correlation.cc:47-93, warp.cc:25-66): Ort::KernelContext, Ort::ConstValue,
 * Ort::UnownedValue, Ort::TensorTypeAndShapeInfo, Ort::Status and the
 * Ort::CustomOpBase template their op descriptors derive from.  Semantics
 * follow the public ORT documentation: GetOutput(i, dims, n) hands back a
 * tensor of that shape owned by the runtime (here: a caller-provided buffer
 * of sufficient capacity).
 */
#pragma once

#include "onnxruntime_c_api.h"

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace Ort {

struct Status {
    explicit Status(OrtStatus* s = nullptr) : s_(s) { }
    bool IsOK() const { return s_ == nullptr; }
    std::string GetErrorMessage() const { return s_ ? std::string(s_->msg) : std::string(); }

private:
    OrtStatus* s_;
};

struct TensorTypeAndShapeInfo {
    explicit TensorTypeAndShapeInfo(const OrtStubTensor* t) : t_(t) { }
    ONNXTensorElementDataType GetElementType() const { return t_->type; }
    std::vector<int64_t> GetShape() const { return std::vector<int64_t>(t_->shape, t_->shape + t_->rank); }
    size_t GetElementCount() const
    {
        size_t n = 1;
        for (size_t i = 0; i < t_->rank; ++i)
            n *= static_cast<size_t>(t_->shape[i]);
        return n;
    }

private:
    const OrtStubTensor* t_;
};

struct ConstValue {
    explicit ConstValue(const OrtStubTensor* t) : t_(t) { }
    TensorTypeAndShapeInfo GetTensorTypeAndShapeInfo() const { return TensorTypeAndShapeInfo(t_); }
    template <typename T>
    const T* GetTensorData() const
    {
        return static_cast<const T*>(t_->data);
    }
    const void* GetTensorRawData() const { return t_->data; }

private:
    const OrtStubTensor* t_;
};

struct UnownedValue {
    explicit UnownedValue(OrtStubTensor* t) : t_(t) { }
    TensorTypeAndShapeInfo GetTensorTypeAndShapeInfo() const { return TensorTypeAndShapeInfo(t_); }
    template <typename T>
    T* GetTensorMutableData()
    {
        return static_cast<T*>(t_->data);
    }
    void* GetTensorMutableRawData() { return t_->data; }

private:
    OrtStubTensor* t_;
};

struct KernelContext {
    explicit KernelContext(OrtKernelContext* c) : c_(c) { }
    size_t GetInputCount() const { return c_->num_inputs; }
    size_t GetOutputCount() const { return c_->num_outputs; }
    ConstValue GetInput(size_t i) const
    {
        if (i >= c_->num_inputs)
            throw std::runtime_error("stub: input index out of range");
        return ConstValue(&c_->inputs[i]);
    }
    UnownedValue GetOutput(size_t i, const int64_t* dims, size_t n)
    {
        if (i >= c_->num_outputs || n > 8)
            throw std::runtime_error("stub: bad output request");
        OrtStubTensor& t = c_->outputs[i];
        size_t elems = 1;
        for (size_t k = 0; k < n; ++k) {
            t.shape[k] = dims[k];
            elems *= static_cast<size_t>(dims[k]);
        }
        t.rank = n;
        size_t esize = (t.type == ONNX_TENSOR_ELEMENT_DATA_TYPE_DOUBLE) ? 8 : 4;
        if (elems * esize > t.capacity) {
            c_->output_error = 1;
            throw std::runtime_error("stub: output buffer too small");
        }
        return UnownedValue(&t);
    }
    void* GetGPUComputeStream() const { return c_->gpu_stream; }

private:
    OrtKernelContext* c_;
};

/* Op descriptors derive from this.  As in ORT, the base fills the C
 * function table (OrtCustomOp) with thunks into the derived descriptor and
 * its kernel type; CreateKernel(api, info) and Compute(context) are the
 * derived classes' own. */
template <typename TOp, typename TKernel>
struct CustomOpBase : OrtCustomOp {
    CustomOpBase()
    {
        OrtCustomOp::version = ORT_API_VERSION;
        OrtCustomOp::CreateKernel = [](const OrtCustomOp* this_, const OrtApi* api, const OrtKernelInfo* info) {
            return static_cast<void*>(static_cast<const TOp*>(this_)->CreateKernel(*api, info));
        };
        OrtCustomOp::GetName = [](const OrtCustomOp* this_) { return static_cast<const TOp*>(this_)->GetName(); };
        OrtCustomOp::GetExecutionProviderType = [](const OrtCustomOp* this_) {
            return static_cast<const TOp*>(this_)->GetExecutionProviderType();
        };
        OrtCustomOp::GetInputType = [](const OrtCustomOp* this_, size_t i) {
            return static_cast<const TOp*>(this_)->GetInputType(i);
        };
        OrtCustomOp::GetInputTypeCount = [](const OrtCustomOp* this_) {
            return static_cast<const TOp*>(this_)->GetInputTypeCount();
        };
        OrtCustomOp::GetOutputType = [](const OrtCustomOp* this_, size_t i) {
            return static_cast<const TOp*>(this_)->GetOutputType(i);
        };
        OrtCustomOp::GetOutputTypeCount = [](const OrtCustomOp* this_) {
            return static_cast<const TOp*>(this_)->GetOutputTypeCount();
        };
        OrtCustomOp::KernelCompute = [](void* k, OrtKernelContext* ctx) { static_cast<TKernel*>(k)->Compute(ctx); };
        OrtCustomOp::KernelDestroy = [](void* k) { delete static_cast<TKernel*>(k); };
    }
};

/* Api access as in ORT's C++ wrapper under ORT_API_MANUAL_INIT. */
inline const OrtApi*& GlobalApi()
{
    static const OrtApi* api = nullptr;
    return api;
}
inline void InitApi(const OrtApi* api) { GlobalApi() = api; }
inline const OrtApi& GetApi() { return *GlobalApi(); }

inline std::vector<std::string> GetAvailableProviders()
{
    char** names = nullptr;
    int n = 0;
    std::vector<std::string> out;
    if (GetApi().GetAvailableProviders(&names, &n) == nullptr)
        for (int i = 0; i < n; ++i)
            out.emplace_back(names[i]);
    return out;
}

}  // namespace Ort
