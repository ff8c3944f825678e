/*
 * Minimal, project-written stand-in for the ONNX Runtime C API header.
 *
 * TEST INFRASTRUCTURE ONLY.  ONNX Runtime is not installed in this build
 * environment.  This header declares just the subset of the C API that the
 * reference's CPU custom ops (src/ort_custom_ops/src/opticalflow/correlation.cc,
 * warp.cc) and this project's ONNX Runtime adapter touch, so that both can be
 * compiled and driven from tests without the real runtime:
 *   - OrtKernelInfo attribute lookup (correlation.h:20-31 reads "legacy" and
 *     "max_displacement" through OrtApi::KernelInfoGetAttribute_int64),
 *   - a kernel context holding typed, shaped input/output tensors,
 *   - the CUDA compute stream of the context (correlation_cuda.cc:80).
 * The layout of these structs is NOT the real ORT ABI; nothing built against
 * this stub may be loaded into a real ONNX Runtime process.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#define ORT_API_VERSION 20
#define ORT_API_CALL

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ONNXTensorElementDataType {
    ONNX_TENSOR_ELEMENT_DATA_TYPE_UNDEFINED = 0,
    ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT = 1,
    ONNX_TENSOR_ELEMENT_DATA_TYPE_UINT8 = 2,
    ONNX_TENSOR_ELEMENT_DATA_TYPE_INT64 = 7,
    ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT16 = 10,
    ONNX_TENSOR_ELEMENT_DATA_TYPE_DOUBLE = 11,
    ONNX_TENSOR_ELEMENT_DATA_TYPE_BFLOAT16 = 16
} ONNXTensorElementDataType;

/* An error status: a heap-allocated message.  NULL means OK. */
typedef struct OrtStatus {
    char msg[256];
} OrtStatus;
typedef OrtStatus* OrtStatusPtr;

/* One tensor as the stub runtime sees it: caller-owned storage. */
typedef struct OrtStubTensor {
    ONNXTensorElementDataType type;
    int64_t shape[8];
    size_t rank;
    void* data;       /* element storage (host or device, as the provider expects) */
    size_t capacity;  /* bytes available at data (outputs) */
} OrtStubTensor;

/* Kernel attributes: int64 name/value pairs. */
typedef struct OrtKernelInfo {
    const char* names[8];
    int64_t values[8];
    size_t count;
} OrtKernelInfo;

/* A kernel invocation: inputs, outputs and the GPU stream ORT would hand out. */
typedef struct OrtKernelContext {
    OrtStubTensor* inputs;
    size_t num_inputs;
    OrtStubTensor* outputs;
    size_t num_outputs;
    void* gpu_stream;
    int output_error; /* set when an output was requested larger than its capacity */
} OrtKernelContext;

typedef struct OrtSessionOptions OrtSessionOptions;
typedef struct OrtCustomOpDomain OrtCustomOpDomain;
struct OrtApi;

/* The custom-op function table (the leading members of ORT's OrtCustomOp,
 * in its order). */
typedef struct OrtCustomOp {
    uint32_t version;
    void*(ORT_API_CALL* CreateKernel)(const struct OrtCustomOp* op, const struct OrtApi* api,
                                      const OrtKernelInfo* info);
    const char*(ORT_API_CALL* GetName)(const struct OrtCustomOp* op);
    const char*(ORT_API_CALL* GetExecutionProviderType)(const struct OrtCustomOp* op);
    ONNXTensorElementDataType(ORT_API_CALL* GetInputType)(const struct OrtCustomOp* op, size_t index);
    size_t(ORT_API_CALL* GetInputTypeCount)(const struct OrtCustomOp* op);
    ONNXTensorElementDataType(ORT_API_CALL* GetOutputType)(const struct OrtCustomOp* op, size_t index);
    size_t(ORT_API_CALL* GetOutputTypeCount)(const struct OrtCustomOp* op);
    void(ORT_API_CALL* KernelCompute)(void* op_kernel, OrtKernelContext* context);
    void(ORT_API_CALL* KernelDestroy)(void* op_kernel);
} OrtCustomOp;

typedef struct OrtApi {
    OrtStatusPtr(ORT_API_CALL* KernelInfoGetAttribute_int64)(const OrtKernelInfo* info, const char* name,
                                                            int64_t* out);
    OrtStatusPtr(ORT_API_CALL* CreateCustomOpDomain)(const char* domain, OrtCustomOpDomain** out);
    OrtStatusPtr(ORT_API_CALL* CustomOpDomain_Add)(OrtCustomOpDomain* domain, const OrtCustomOp* op);
    OrtStatusPtr(ORT_API_CALL* AddCustomOpDomain)(OrtSessionOptions* options, OrtCustomOpDomain* domain);
    void(ORT_API_CALL* ReleaseCustomOpDomain)(OrtCustomOpDomain* domain);
    const char*(ORT_API_CALL* GetErrorMessage)(const OrtStatus* status);
    OrtStatusPtr(ORT_API_CALL* CreateStatus)(int code, const char* msg);
    OrtStatusPtr(ORT_API_CALL* GetAvailableProviders)(char*** out_ptr, int* provider_length);
} OrtApi;

typedef struct OrtApiBase {
    const OrtApi*(ORT_API_CALL* GetApi)(uint32_t version);
    const char*(ORT_API_CALL* GetVersionString)(void);
} OrtApiBase;

/* The stub's implementation of OrtApi::KernelInfoGetAttribute_int64. */
static inline OrtStatusPtr OrtStubKernelInfoGetAttribute_int64(const OrtKernelInfo* info, const char* name,
                                                               int64_t* out)
{
    for (size_t i = 0; i < info->count; ++i) {
        const char* a = info->names[i];
        const char* b = name;
        while (*a && *a == *b) {
            ++a;
            ++b;
        }
        if (*a == 0 && *b == 0) {
            *out = info->values[i];
            return 0;
        }
    }
    static OrtStatus missing = {"attribute not found"};
    return &missing;
}

#ifdef __cplusplus
}
#endif
