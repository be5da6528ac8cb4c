// core.cu -- error state and version of the C ABI.
#include <cstdarg>
#include <cstdio>

#include "ubs_common.cuh"

namespace ubs {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

// Reports a failed launch or runtime call (sticky or not) as UBS_ERR_CUDA.
int check_launch(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return UBS_OK;
    return set_error(UBS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

} // namespace ubs

extern "C" {

const char *ubs_last_error(void) { return ubs::g_last_error; }

int ubs_abi_version(void) { return 1; }

} // extern "C"
