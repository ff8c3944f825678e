/*
 * TEST INFRASTRUCTURE ONLY: a minimal stand-in ONNX Runtime that loads a
 * custom-op library's RegisterCustomOps through the stub headers of this
 * directory and drives the registered ops the way ORT's kernel dispatch
 * does (CreateKernel with node attributes, KernelCompute with a context of
 * shaped tensors, KernelDestroy).  Linked together with the op library under
 * test; exposes plain C entry points for the Python tests.
 */
#include "onnxruntime_cxx_api.h"

#include <cstring>
#include <exception>
#include <string>
#include <vector>

extern "C" OrtStatus* ORT_API_CALL RegisterCustomOps(OrtSessionOptions* options, const OrtApiBase* api);

struct OrtCustomOpDomain {
    std::string name;
    std::vector<const OrtCustomOp*> ops;
};

namespace {
std::vector<OrtCustomOpDomain*> g_session_domains;  // what AddCustomOpDomain received
bool g_with_cuda = true;
std::string g_err;
OrtStatus g_status;

OrtStatusPtr make_status(const char* msg)
{
    std::strncpy(g_status.msg, msg, sizeof(g_status.msg) - 1);
    return &g_status;
}

OrtStatusPtr ORT_API_CALL create_domain(const char* name, OrtCustomOpDomain** out)
{
    *out = new OrtCustomOpDomain{name, {}};
    return nullptr;
}
OrtStatusPtr ORT_API_CALL domain_add(OrtCustomOpDomain* d, const OrtCustomOp* op)
{
    d->ops.push_back(op);
    return nullptr;
}
OrtStatusPtr ORT_API_CALL add_domain(OrtSessionOptions*, OrtCustomOpDomain* d)
{
    g_session_domains.push_back(d);
    return nullptr;
}
void ORT_API_CALL release_domain(OrtCustomOpDomain* d) { delete d; }
const char* ORT_API_CALL error_message(const OrtStatus* s) { return s->msg; }
OrtStatusPtr ORT_API_CALL create_status(int, const char* msg) { return make_status(msg); }
OrtStatusPtr ORT_API_CALL providers(char*** out, int* n)
{
    static char cuda[] = "CUDAExecutionProvider";
    static char cpu[] = "CPUExecutionProvider";
    static char* both[] = {cuda, cpu};
    static char* only_cpu[] = {cpu};
    *out = g_with_cuda ? both : only_cpu;
    *n = g_with_cuda ? 2 : 1;
    return nullptr;
}

const OrtApi g_api = {&OrtStubKernelInfoGetAttribute_int64, &create_domain, &domain_add, &add_domain,
    &release_domain, &error_message, &create_status, &providers};
const OrtApi* ORT_API_CALL get_api(uint32_t version) { return version == ORT_API_VERSION ? &g_api : nullptr; }
const char* ORT_API_CALL version_string() { return "stub"; }
const OrtApiBase g_base = {&get_api, &version_string};

const OrtCustomOp* op_at(int i)
{
    int k = 0;
    for (auto* d : g_session_domains)
        for (auto* op : d->ops)
            if (k++ == i)
                return op;
    return nullptr;
}
}  // namespace

extern "C" {

const char* stub_last_error(void) { return g_err.c_str(); }

/* Registers the library's ops into a fresh stub session; returns the op count. */
int stub_register(int with_cuda)
{
    g_with_cuda = with_cuda != 0;
    g_session_domains.clear();
    OrtStatus* st = RegisterCustomOps(nullptr, &g_base);
    if (st) {
        g_err = st->msg;
        return -1;
    }
    int n = 0;
    for (auto* d : g_session_domains)
        n += static_cast<int>(d->ops.size());
    return n;
}

const char* stub_domain_name(void) { return g_session_domains.empty() ? "" : g_session_domains[0]->name.c_str(); }

/* name, provider, input/output counts and element types of op i */
int stub_op_info(int i, const char** name, const char** provider, int* n_in, int* n_out, int* in_type, int* out_type)
{
    const OrtCustomOp* op = op_at(i);
    if (!op)
        return -1;
    *name = op->GetName(op);
    *provider = op->GetExecutionProviderType(op);
    *n_in = static_cast<int>(op->GetInputTypeCount(op));
    *n_out = static_cast<int>(op->GetOutputTypeCount(op));
    *in_type = op->GetInputType(op, 0);
    *out_type = op->GetOutputType(op, 0);
    return 0;
}

/* Runs op i once.  attrs: n_attr (name, value) pairs.  Tensors: two float
 * inputs of rank 4 with the given shapes and one output buffer of capacity
 * out_bytes; the output shape the op requested comes back in out_shape. */
// element type of the tensors stub_run hands to Compute (FLOAT by default)
static ONNXTensorElementDataType g_run_type = ONNX_TENSOR_ELEMENT_DATA_TYPE_FLOAT;
void stub_set_tensor_type(int type) { g_run_type = static_cast<ONNXTensorElementDataType>(type); }

int stub_run(int i, int n_attr, const char** attr_names, const int64_t* attr_values, const void* in0,
    const int64_t* shape0, const void* in1, const int64_t* shape1, void* out, size_t out_bytes, int64_t* out_shape,
    int* out_rank, void* stream)
{
    const OrtCustomOp* op = op_at(i);
    if (!op)
        return -1;
    OrtKernelInfo info;
    std::memset(&info, 0, sizeof(info));
    for (int k = 0; k < n_attr && k < 8; ++k) {
        info.names[k] = attr_names[k];
        info.values[k] = attr_values[k];
    }
    info.count = static_cast<size_t>(n_attr);
    void* kernel = nullptr;
    try {
        kernel = op->CreateKernel(op, &g_api, &info);
        OrtStubTensor ins[2];
        std::memset(ins, 0, sizeof(ins));
        const void* data[2] = {in0, in1};
        const int64_t* shapes[2] = {shape0, shape1};
        for (int k = 0; k < 2; ++k) {
            ins[k].type = g_run_type;
            ins[k].rank = 4;
            for (int r = 0; r < 4; ++r)
                ins[k].shape[r] = shapes[k][r];
            ins[k].data = const_cast<void*>(data[k]);
        }
        OrtStubTensor o;
        std::memset(&o, 0, sizeof(o));
        o.type = g_run_type;
        o.data = out;
        o.capacity = out_bytes;
        OrtKernelContext ctx = {ins, 2, &o, 1, stream, 0};
        op->KernelCompute(kernel, &ctx);
        *out_rank = static_cast<int>(o.rank);
        for (size_t r = 0; r < o.rank; ++r)
            out_shape[r] = o.shape[r];
        op->KernelDestroy(kernel);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        if (kernel)
            op->KernelDestroy(kernel);
        return -1;
    }
}

}  // extern "C"
