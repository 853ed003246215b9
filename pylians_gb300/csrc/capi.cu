// Status strings, last-error detail and version of the C-ABI.
#include <string>

#include "common.cuh"

namespace pyl {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string &msg) { g_last_error = msg; }
}  // namespace pyl

extern "C" const char *pyl_strerror(int status)
{
    switch (status) {
        case PYL_OK: return "success";
        case PYL_ERR_INVALID: return "invalid argument";
        case PYL_ERR_CUDA: return "CUDA error";
        case PYL_ERR_CUFFT: return "cuFFT error";
        case PYL_ERR_WORKSPACE: return "workspace too small";
        case PYL_ERR_UNSUPPORTED: return "unsupported request";
        default: return "unknown status";
    }
}

extern "C" const char *pyl_last_error(void) { return pyl::g_last_error.c_str(); }

extern "C" int pyl_version(void) { return 100; }
