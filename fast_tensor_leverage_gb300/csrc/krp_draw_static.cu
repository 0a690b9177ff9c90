// ftl_krp_draw_static: the exact KRP draw for callers that cannot allocate
// device memory.
//
// ftl_krp_draw needs per-draw scratch (the eigen-component trees, the FP64
// computeM matrices, eigenvalues and the FP32 pseudo-inverse) that the caller
// normally allocates and passes in the plan.  Some callers cannot call
// cudaMalloc at all: a host integration that reserves its whole device
// budget up front through another runtime (a cgo/JNI/FFI host whose memory
// is owned by a different allocator), or a request path that must not
// allocate because cudaMalloc can synchronise the device or fail under
// memory pressure in the middle of serving.  This entry point takes the same
// inputs and outputs but keeps that scratch in one file-scope device array of
// FTL_DRAW_STATIC_SCRATCH_BYTES (8 MiB), which every GPU that loads this
// library holds until the process exits.
//
// Rules of use:
//   * The first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.
//   * All calls share the one array and it keeps the last call's contents.
//     Each call clears the part it uses before computing.  Calls that overlap
//     on the GPU (different streams, or different host threads, without
//     ordering between them) race on the array: serialise them.
//   * Configurations whose scratch exceeds the array are rejected with
//     FTL_E_ARG before anything is launched.
//   * Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
#include <mutex>

#include "ftl_common.cuh"

static __device__ __align__(256) unsigned char g_draw_scratch[FTL_DRAW_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_draw_scratch on the current device, looked up once.
int scratch_address(void **out) {
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess)
        return ftl::fail(FTL_E_CUDA, "ftl_krp_draw_static: cudaGetDevice: %s", cudaGetErrorString(err));
    if (dev < 0 || dev >= kMaxDevices)
        return ftl::fail(FTL_E_UNSUPPORTED, "ftl_krp_draw_static: device ordinal %d not supported", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_ptr[dev] == nullptr) {
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_draw_scratch);
        if (err != cudaSuccess || p == nullptr)
            return ftl::fail(FTL_E_CUDA, "ftl_krp_draw_static: cudaGetSymbolAddress: %s",
                             cudaGetErrorString(err));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return FTL_OK;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

extern "C" int ftl_krp_draw_static(int N, int R, int64_t J, int prec, const int64_t *dims,
                                   const double *const *U_dev, void *const *gram_G_dev, uint32_t j,
                                   uint64_t *samples_dev, double *h_dev, double *weights_dev,
                                   const double *draws_dev, uint64_t seed, uint64_t ctr,
                                   void *stream) {
    FTL_CHECK_ARG(dims != nullptr && U_dev != nullptr && gram_G_dev != nullptr,
                  "ftl_krp_draw_static: null dims, factor or tree array");
    size_t eig_b = 0, M_b = 0, lam_b = 0, p32_b = 0;
    int rc = ftl_krp_plan_sizes(N, R, prec, &eig_b, &M_b, &lam_b, &p32_b);
    if (rc) return rc;
    const size_t off_M = align256(eig_b);
    const size_t off_lam = off_M + align256(M_b);
    const size_t off_p32 = off_lam + align256(lam_b);
    const size_t total = off_p32 + align256(p32_b);
    if (total > (size_t)FTL_DRAW_STATIC_SCRATCH_BYTES)
        return ftl::fail(FTL_E_ARG,
                         "ftl_krp_draw_static: N=%d, R=%d needs %zu bytes of scratch, more than the "
                         "%u-byte static array; use ftl_krp_draw with caller-allocated workspaces",
                         N, R, total, (unsigned)FTL_DRAW_STATIC_SCRATCH_BYTES);
    void *base = nullptr;
    rc = scratch_address(&base);
    if (rc) return rc;
    ftl_krp_plan plan = {};
    plan.N = N;
    plan.R = R;
    plan.J = J;
    plan.prec = prec;
    for (int k = 0; k < FTL_MAX_MODES; ++k) {
        plan.dims[k] = k < N ? dims[k] : 0;
        plan.U[k] = k < N ? U_dev[k] : nullptr;
        plan.gram_G[k] = k < N ? gram_G_dev[k] : nullptr;
    }
    unsigned char *b = (unsigned char *)base;
    plan.eig_G = b;
    plan.M = (double *)(b + off_M);
    plan.lambda = (double *)(b + off_lam);
    plan.pinv32 = (float *)(b + off_p32);
    cudaError_t err = cudaMemsetAsync(base, 0, total, (cudaStream_t)stream);
    if (err != cudaSuccess)
        return ftl::fail(FTL_E_CUDA, "ftl_krp_draw_static: clearing scratch: %s", cudaGetErrorString(err));
    return ftl_krp_draw(&plan, j, samples_dev, h_dev, weights_dev, draws_dev, seed, ctr, stream);
}
