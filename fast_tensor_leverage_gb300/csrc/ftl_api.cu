// Status reporting of the C ABI: a thread-local message for the last error.
#include <cstdarg>
#include <cstdio>

#include "attr_registry.h"
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

static AttrRegistry g_smem_attrs;

int ensure_smem(const void *func, size_t bytes, const char *name) {
    if (bytes <= 48 * 1024) return FTL_OK;
    if (bytes > 227 * 1024) return fail(FTL_E_UNSUPPORTED, "%s: %zu bytes of shared memory requested", name, bytes);
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return fail(FTL_E_CUDA, "%s: cudaGetDevice: %s", name, cudaGetErrorString(err));
    const int rc = g_smem_attrs.ensure(func, dev, (int)bytes, [func](int b) {
        return (int)cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    });
    if (rc != 0)
        return fail(FTL_E_CUDA, "%s: raising the shared-memory limit to %zu bytes: %s", name, bytes,
                    cudaGetErrorString((cudaError_t)rc));
    return FTL_OK;
}

constexpr int kMaxDevices = 64;
static int g_sm_count[kMaxDevices] = {0};

int num_sms() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = 0;
    int n = __atomic_load_n(&g_sm_count[dev], __ATOMIC_RELAXED);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        __atomic_store_n(&g_sm_count[dev], n, __ATOMIC_RELAXED);
    }
    return n;
}

}  // namespace ftl

extern "C" const char *ftl_last_error(void) { return ftl::g_last_error; }

extern "C" int ftl_abi_version(void) { return 4; }

extern "C" int ftl_host_register(void *ptr, size_t bytes, int *registered) {
    FTL_CHECK_ARG(ptr && bytes > 0 && registered, "ftl_host_register: bad arguments");
    *registered = 0;
    const cudaError_t err = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (err == cudaSuccess) {
        *registered = 1;
        return FTL_OK;
    }
    (void)cudaGetLastError();  // a refused registration must not surface in a later error check
    return FTL_OK;
}

extern "C" int ftl_host_unregister(void *ptr) {
    FTL_CHECK_ARG(ptr, "ftl_host_unregister: NULL pointer");
    const cudaError_t err = cudaHostUnregister(ptr);
    if (err != cudaSuccess) {
        (void)cudaGetLastError();
        return ftl::fail(FTL_E_CUDA, "ftl_host_unregister: %s", cudaGetErrorString(err));
    }
    return FTL_OK;
}
