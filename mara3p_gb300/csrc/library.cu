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

} // extern "C"
