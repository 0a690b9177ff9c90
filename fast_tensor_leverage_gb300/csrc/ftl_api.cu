// Status reporting of the C ABI: a thread-local message for the last error.
#include <cstdarg>
#include <cstdio>

#include "ftl_common.cuh"

namespace ftl {

static thread_local char g_last_error[1024] = {0};

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int fail(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

int check_launch(const char *what) {
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(FTL_E_CUDA, "%s: %s", what, cudaGetErrorString(err));
    return FTL_OK;
}

}  // namespace ftl

extern "C" const char *ftl_last_error(void) { return ftl::g_last_error; }

extern "C" int ftl_abi_version(void) { return 3; }
