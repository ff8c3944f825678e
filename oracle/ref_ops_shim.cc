/*
 * TEST INFRASTRUCTURE ONLY — builds oracle/_ref/libref_ops.so.
 *
 * Compiles the reference's own CPU custom ops IN PLACE (the .cc files are
 * #included from the reference tree given on the include path by
 * oracle/Makefile; nothing is copied) against the project-written ORT stub in
 * oracle/ort_stub, and exposes them through plain C entry points so tests can
 * compare this project's kernels and its C restatement against the reference:
 *
 *   CorrelationKernel::ComputeCPU  src/ort_custom_ops/src/opticalflow/correlation.cc:45-143
 *   WarpKernel::ComputeCPU         src/ort_custom_ops/src/opticalflow/warp.cc:25-66
 *
 * Each call builds an OrtKernelInfo with the node attributes
 * (correlation.h:19-31: "legacy", "max_displacement"), constructs the
 * reference kernel object with provider "CPUExecutionProvider" and calls its
 * Compute(), exactly as ONNX Runtime would through the custom-op table.
 * Errors (the reference throws std::runtime_error) come back as -1 with the
 * message available from ref_last_error().
 */
#include "correlation.cc"
#include "warp.cc"

#include <cstdint>
#include <cstring>
#include <string>

namespace {
thread_local std::string g_err;

const OrtApi& stub_api()
{
    static OrtApi api = {&OrtStubKernelInfoGetAttribute_int64};
    return api;
}

OrtStubTensor make_tensor(ONNXTensorElementDataType type, void* data, size_t capacity, const int64_t* shape,
    size_t rank)
{
    OrtStubTensor t;
    std::memset(&t, 0, sizeof(t));
    t.type = type;
    t.data = data;
    t.capacity = capacity;
    t.rank = rank;
    for (size_t i = 0; i < rank; ++i)
        t.shape[i] = shape[i];
    return t;
}

template <typename T>
int run_correlation(const T* f1, const T* f2, T* out, int64_t N, int64_t C, int64_t H, int64_t W, int64_t md,
    int64_t legacy, ONNXTensorElementDataType type)
{
    try {
        OrtKernelInfo info;
        std::memset(&info, 0, sizeof(info));
        info.names[0] = "legacy";
        info.values[0] = legacy;
        info.names[1] = "max_displacement";
        info.values[1] = md;
        info.count = 2;
        CorrelationKernel kernel(stub_api(), &info, "CPUExecutionProvider");
        const int64_t shp[4] = {N, C, H, W};
        OrtStubTensor in[2] = {make_tensor(type, const_cast<T*>(f1), 0, shp, 4),
            make_tensor(type, const_cast<T*>(f2), 0, shp, 4)};
        const int64_t P = 2 * md + 1;
        const size_t cap = static_cast<size_t>(N * P * P * H * W) * sizeof(T);
        OrtStubTensor o[1] = {make_tensor(type, out, cap, shp, 0)};
        OrtKernelContext ctx = {in, 2, o, 1, nullptr, 0};
        kernel.Compute(&ctx);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

template <typename T>
int run_warp(const T* input, const T* flow, T* out, int64_t N, int64_t C, int64_t H, int64_t W,
    ONNXTensorElementDataType type)
{
    try {
        OrtKernelInfo info;
        std::memset(&info, 0, sizeof(info));
        WarpKernel kernel(stub_api(), &info, "CPUExecutionProvider");
        const int64_t shp[4] = {N, C, H, W};
        const int64_t fshp[4] = {N, 2, H, W};
        OrtStubTensor in[2] = {make_tensor(type, const_cast<T*>(input), 0, shp, 4),
            make_tensor(type, const_cast<T*>(flow), 0, fshp, 4)};
        const size_t cap = static_cast<size_t>(N * C * H * W) * sizeof(T);
        OrtStubTensor o[1] = {make_tensor(type, out, cap, shp, 0)};
        OrtKernelContext ctx = {in, 2, o, 1, nullptr, 0};
        kernel.Compute(&ctx);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}
}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

int ref_correlation_f32(const float* f1, const float* f2, float* out, int64_t N, int64_t C, int64_t H, int64_t W,
    int64_t md, int64_t legacy)
{
    return run_correlation<float>(f1, f2, out, N, C, H, W, md, legacy, ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT);
}

int ref_correlation_f64(const double* f1, const double* f2, double* out, int64_t N, int64_t C, int64_t H,
    int64_t W, int64_t md, int64_t legacy)
{
    return run_correlation<double>(f1, f2, out, N, C, H, W, md, legacy, ONNX_TENSOR_ELEMENT_DATA_TYPE_DOUBLE);
}

int ref_warp_f32(const float* input, const float* flow, float* out, int64_t N, int64_t C, int64_t H, int64_t W)
{
    return run_warp<float>(input, flow, out, N, C, H, W, ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT);
}

int ref_warp_f64(const double* input, const double* flow, double* out, int64_t N, int64_t C, int64_t H, int64_t W)
{
    return run_warp<double>(input, flow, out, N, C, H, W, ONNX_TENSOR_ELEMENT_DATA_TYPE_DOUBLE);
}

}  // extern "C"
