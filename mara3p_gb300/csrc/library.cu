// Library-wide C ABI: error reporting and version.
#include <string>
#include "common.cuh"

namespace {
thread_local std::string g_last_error;
}

namespace mara {

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return MARA_ERR_CUDA;
}

} // namespace mara

extern "C" {

const char* mara_last_error(void) { return g_last_error.c_str(); }

const char* mara_version(void) { return "mara_gb300 0.1 (sm_103a)"; }

int mara_graph_upload(void* graph_exec, void* stream)
{
    if (graph_exec == nullptr) return mara::fail(MARA_ERR_ARGUMENT, "mara_graph_upload: graph_exec is null");
    const cudaError_t e = cudaGraphUpload(static_cast<cudaGraphExec_t>(graph_exec), static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? MARA_OK : mara::cuda_fail(e, "mara_graph_upload");
}

} // extern "C"
