// Handle form of the exact KRP sampler for hosts that are not Python: one
// opaque object owns the device factors, their Gram trees and the per-draw
// workspaces (the state of EfficientKRPSampler, efficient_krp_sampler.hpp:
// 32-75), so a caller needs four calls: create, set_factor per mode, draw,
// destroy.  Everything below is host code over the plan-based entry points
// (ftl_tree_build_ex, ftl_krp_draw); the device work is the
// same.  Unlike those entry points, create allocates (cudaMalloc) and destroy
// frees.
#include <cstring>
#include <vector>

#include "ftl_common.cuh"

struct ftl_sampler {
    ftl_krp_plan plan;
    int tree_prec;  // FTL_PREC_* the trees are built with (plan.prec is its node precision)
    int64_t F[FTL_MAX_MODES];
    std::vector<void *> owned;  // every cudaMalloc of this handle, freed by destroy
};

namespace {

void release(ftl_sampler *s) {
    for (void *p : s->owned) cudaFree(p);
    delete s;
}

int alloc(ftl_sampler *s, size_t bytes, void **out, bool zero) {
    void *p = nullptr;
    cudaError_t err = cudaMalloc(&p, bytes > 0 ? bytes : 16);
    if (err != cudaSuccess) {
        cudaGetLastError();
        return ftl::fail(FTL_E_OOM, "ftl_sampler_create: cudaMalloc of %zu bytes: %s", bytes,
                         cudaGetErrorString(err));
    }
    s->owned.push_back(p);
    if (zero) {
        err = cudaMemset(p, 0, bytes);
        if (err != cudaSuccess)
            return ftl::fail(FTL_E_CUDA, "ftl_sampler_create: cudaMemset: %s", cudaGetErrorString(err));
    }
    *out = p;
    return FTL_OK;
}

}  // namespace

extern "C" int ftl_sampler_create(int N, const int64_t *dims, int R, int64_t J, int prec, int factor_shadows,
                                  ftl_sampler **out) {
    FTL_CHECK_ARG(out && dims, "ftl_sampler_create: null pointer");
    *out = nullptr;
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES, "ftl_sampler_create: N=%d outside 1..%d", N, FTL_MAX_MODES);
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK, "ftl_sampler_create: R=%d outside 1..%d", R, FTL_MAX_RANK);
    FTL_CHECK_ARG(J >= 1, "ftl_sampler_create: J=%lld", (long long)J);
    FTL_CHECK_ARG(ftl::valid_prec(prec), "ftl_sampler_create: bad precision %d", prec);
    for (int k = 0; k < N; ++k)
        FTL_CHECK_ARG(dims[k] >= 1, "ftl_sampler_create: dims[%d]=%lld", k, (long long)dims[k]);
    ftl_sampler *s = new ftl_sampler();
    std::memset(&s->plan, 0, sizeof(s->plan));
    ftl_krp_plan &p = s->plan;
    p.N = N;
    p.R = R;
    p.J = J;
    p.prec = ftl::storage_prec(prec);  // the draws see FP64 or FP32 nodes
    s->tree_prec = prec;
    int rc = FTL_OK;
    for (int k = 0; k < N && rc == FTL_OK; ++k) {
        p.dims[k] = dims[k];
        s->F[k] = dims[k] < R ? dims[k] : R;  // F = min(R, I), efficient_krp_sampler.hpp:52-53
        void *u = nullptr, *g = nullptr;
        size_t tb = 0;
        rc = alloc(s, (size_t)dims[k] * R * sizeof(double), &u, true);
        if (rc == FTL_OK) rc = ftl_tree_bytes(dims[k], s->F[k], R, prec, &tb);
        if (rc == FTL_OK) rc = alloc(s, tb, &g, true);
        p.U[k] = (const double *)u;
        p.gram_G[k] = g;
        if (rc == FTL_OK && factor_shadows && prec != FTL_PREC_FP64) {
            void *u32 = nullptr;
            rc = alloc(s, (size_t)dims[k] * R * sizeof(float), &u32, true);
            p.U32[k] = (const float *)u32;
        }
    }
    size_t eb = 0, mb = 0, lb = 0, pb = 0;
    if (rc == FTL_OK) rc = ftl_krp_plan_sizes(N, R, prec, &eb, &mb, &lb, &pb);
    void *e = nullptr, *m = nullptr, *l = nullptr, *q = nullptr;
    if (rc == FTL_OK) rc = alloc(s, eb, &e, true);
    if (rc == FTL_OK) rc = alloc(s, mb, &m, true);
    if (rc == FTL_OK) rc = alloc(s, lb, &l, true);
    if (rc == FTL_OK) rc = alloc(s, pb, &q, true);
    if (rc != FTL_OK) {
        release(s);
        return rc;
    }
    p.eig_G = e;
    p.M = (double *)m;
    p.lambda = (double *)l;
    p.pinv32 = (float *)q;
    *out = s;
    return FTL_OK;
}

extern "C" int ftl_sampler_set_factor(ftl_sampler *s, int k, const double *U, int U_on_host, void *stream) {
    FTL_CHECK_ARG(s && U, "ftl_sampler_set_factor: null pointer");
    FTL_CHECK_ARG(k >= 0 && k < s->plan.N, "ftl_sampler_set_factor: k=%d outside 0..%d", k, s->plan.N - 1);
    ftl_krp_plan &p = s->plan;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = (size_t)p.dims[k] * p.R * sizeof(double);
    // a pageable host source makes this copy synchronous with the host
    cudaError_t err = cudaMemcpyAsync((void *)p.U[k], U, bytes,
                                      U_on_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st);
    if (err != cudaSuccess) return ftl::fail(FTL_E_CUDA, "ftl_sampler_set_factor: copy: %s", cudaGetErrorString(err));
    return ftl_sampler_update(s, k, stream);
}

extern "C" int ftl_sampler_update(ftl_sampler *s, int k, void *stream) {
    FTL_CHECK_ARG(s, "ftl_sampler_update: null pointer");
    FTL_CHECK_ARG(k >= 0 && k < s->plan.N, "ftl_sampler_update: k=%d outside 0..%d", k, s->plan.N - 1);
    ftl_krp_plan &p = s->plan;
    // the tree and the FP32 copy of the factor (when kept) in one pass
    return ftl_tree_build_ex(p.U[k], p.dims[k], p.R, s->F[k], s->tree_prec, p.gram_G[k], (float *)p.U32[k], stream);
}

extern "C" int ftl_sampler_factor(const ftl_sampler *s, int k, double **U_dev) {
    FTL_CHECK_ARG(s && U_dev, "ftl_sampler_factor: null pointer");
    FTL_CHECK_ARG(k >= 0 && k < s->plan.N, "ftl_sampler_factor: k=%d outside 0..%d", k, s->plan.N - 1);
    *U_dev = (double *)s->plan.U[k];
    return FTL_OK;
}

extern "C" int ftl_sampler_draw(ftl_sampler *s, uint32_t j, uint64_t *samples_dev, double *h_dev,
                                double *weights_dev, const double *draws_dev, uint64_t seed, uint64_t ctr,
                                void *stream) {
    FTL_CHECK_ARG(s, "ftl_sampler_draw: null pointer");
    return ftl_krp_draw(&s->plan, j, samples_dev, h_dev, weights_dev, draws_dev, seed, ctr, stream);
}

extern "C" int ftl_sampler_destroy(ftl_sampler *s) {
    if (!s) return FTL_OK;
    // the handle's buffers may still be read by queued work
    cudaError_t err = cudaDeviceSynchronize();
    release(s);
    if (err != cudaSuccess) return ftl::fail(FTL_E_CUDA, "ftl_sampler_destroy: %s", cudaGetErrorString(err));
    return FTL_OK;
}
