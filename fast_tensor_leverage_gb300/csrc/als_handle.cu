// Handle form of the sparse tensor and of the randomized CP-ALS (STS-CP) for
// hosts that are not Python: the objects behind the reference's
// SparseTensor(idx, vals, "sort") (sparse_tensor.hpp:46-77 with
// SortIdxLookup, sort_lookup.hpp:33-60) and ALS(LowRankTensor, SparseTensor)
// with initialize_ds_als / execute_ds_als_update (als.hpp:18-220), own their
// device state and run the same entry points the Python package calls
// (fiber keys, dedup, weighted Gram, pseudo-inverse, solve, row-grouped
// MTTKRP, renormalisation, tree rebuild).  Creating either allocates device
// memory (cudaMalloc); destroy frees it.
#include <cmath>
#include <cstring>
#include <vector>

#include <cub/cub.cuh>

#include "ftl_common.cuh"

namespace ftl {
}

struct ftl_sparse {
    int N = 0;
    int64_t nnz = 0;
    int64_t dims[FTL_MAX_MODES] = {};
    uint32_t *idx = nullptr;  // nnz x N, row-major
    double *vals = nullptr;
    // per mode: nonzeros sorted by their mode-j index (stable), with fiber keys
    int32_t *rows[FTL_MAX_MODES] = {};
    uint64_t *rkeys[FTL_MAX_MODES] = {};
    double *rvals[FTL_MAX_MODES] = {};
    double normsq = 0.0;
    std::vector<void *> owned;
};

struct ftl_als {
    const ftl_sparse *X = nullptr;
    ftl_sampler *S = nullptr;
    int N = 0, R = 0, prec = 0;
    int64_t J = 0;
    uint64_t seed = 0, counter = 0;
    double *U[FTL_MAX_MODES] = {};
    double *sigma = nullptr, *norms = nullptr;
    uint64_t *samples = nullptr, *keys = nullptr, *ukeys = nullptr;
    double *h = nullptr, *w = nullptr, *hp = nullptr;
    int32_t *urep = nullptr, *ucnt = nullptr;
    int64_t *nuniq = nullptr;
    double *gram = nullptr, *pinv = nullptr, *vscr = nullptr, *grams = nullptr, *terms = nullptr;
    void *ws_dedup = nullptr, *ws_mtt = nullptr, *ws_gram = nullptr, *ws_col = nullptr, *ws_fit = nullptr;
    size_t nb_dedup = 0, nb_mtt = 0, nb_gram = 0, nb_col = 0, nb_fit = 0;
    std::vector<void *> owned;
};

namespace {

template <typename H>
int dev_alloc(H *hd, size_t bytes, void **out, const char *who) {
    void *p = nullptr;
    cudaError_t err = cudaMalloc(&p, bytes > 0 ? bytes : 16);
    if (err != cudaSuccess) {
        cudaGetLastError();
        return ftl::fail(FTL_E_OOM, "%s: cudaMalloc of %zu bytes: %s", who, bytes, cudaGetErrorString(err));
    }
    hd->owned.push_back(p);
    *out = p;
    return FTL_OK;
}

template <typename H>
void release(H *hd) {
    for (void *p : hd->owned) cudaFree(p);
    delete hd;
}

int cuda_status(cudaError_t err, const char *who) {
    if (err == cudaSuccess) return FTL_OK;
    return ftl::fail(FTL_E_CUDA, "%s: %s", who, cudaGetErrorString(err));
}

__global__ void column_iota_kernel(const uint32_t *__restrict__ idx, int64_t nnz, int N, int j,
                                   uint32_t *__restrict__ col, int64_t *__restrict__ iota) {
    for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < nnz; z += (int64_t)gridDim.x * blockDim.x) {
        col[z] = idx[z * N + j];
        iota[z] = z;
    }
}

__global__ void rows_gather_kernel(const uint32_t *__restrict__ col_sorted, const int64_t *__restrict__ perm,
                                   const uint64_t *__restrict__ fkeys, const double *__restrict__ vals, int64_t nnz,
                                   int32_t *__restrict__ rows, uint64_t *__restrict__ rkeys,
                                   double *__restrict__ rvals) {
    for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < nnz; z += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = perm[z];
        rows[z] = (int32_t)col_sorted[z];
        rkeys[z] = fkeys[p];
        rvals[z] = vals[p];
    }
}

int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ftl::num_sms() * 16)); }

int key_bits(int64_t d) {
    int b = 1;
    while (b < 32 && (int64_t(1) << b) < d) ++b;
    return b;
}

}  // namespace

extern "C" int ftl_sparse_create(const uint32_t *idx, const double *vals, int64_t nnz, int N, const int64_t *dims,
                                 int on_host, void *stream, ftl_sparse **out) {
    FTL_CHECK_ARG(out && idx && vals && dims, "ftl_sparse_create: null pointer");
    *out = nullptr;
    FTL_CHECK_ARG(N >= 2 && N <= FTL_MAX_MODES, "ftl_sparse_create: N=%d outside 2..%d", N, FTL_MAX_MODES);
    FTL_CHECK_ARG(nnz >= 1 && nnz < (int64_t(1) << 40), "ftl_sparse_create: nnz=%lld", (long long)nnz);
    for (int k = 0; k < N; ++k)
        FTL_CHECK_ARG(dims[k] >= 1 && dims[k] <= (int64_t(1) << 31), "ftl_sparse_create: dims[%d]=%lld", k,
                      (long long)dims[k]);
    cudaStream_t st = (cudaStream_t)stream;
    ftl_sparse *X = new ftl_sparse();
    X->N = N;
    X->nnz = nnz;
    for (int k = 0; k < N; ++k) X->dims[k] = dims[k];
    int rc = FTL_OK;
    void *p = nullptr;
    if ((rc = dev_alloc(X, (size_t)nnz * N * sizeof(uint32_t), &p, "ftl_sparse_create"))) goto fail;
    X->idx = (uint32_t *)p;
    if ((rc = dev_alloc(X, (size_t)nnz * sizeof(double), &p, "ftl_sparse_create"))) goto fail;
    X->vals = (double *)p;
    if ((rc = cuda_status(cudaMemcpyAsync(X->idx, idx, (size_t)nnz * N * sizeof(uint32_t),
                                          on_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st),
                          "ftl_sparse_create: copy")))
        goto fail;
    if ((rc = cuda_status(cudaMemcpyAsync(X->vals, vals, (size_t)nnz * sizeof(double),
                                          on_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st),
                          "ftl_sparse_create: copy")))
        goto fail;
    {
        // scratch for the per-mode sorts, freed before returning
        uint64_t *fkeys = nullptr;
        uint32_t *col = nullptr, *col_s = nullptr;
        int64_t *iota = nullptr, *perm = nullptr;
        void *tmp = nullptr;
        size_t tmp_bytes = 0;
        std::vector<void *> scratch;
        auto salloc = [&](size_t bytes, void **q) -> int {
            cudaError_t e = cudaMalloc(q, bytes > 0 ? bytes : 16);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return ftl::fail(FTL_E_OOM, "ftl_sparse_create: scratch of %zu bytes: %s", bytes,
                                 cudaGetErrorString(e));
            }
            scratch.push_back(*q);
            return FTL_OK;
        };
        cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, col, col_s, iota, perm, (int64_t)nnz, 0, 32, st);
        rc = salloc((size_t)nnz * 8, (void **)&fkeys);
        if (!rc) rc = salloc((size_t)nnz * 4, (void **)&col);
        if (!rc) rc = salloc((size_t)nnz * 4, (void **)&col_s);
        if (!rc) rc = salloc((size_t)nnz * 8, (void **)&iota);
        if (!rc) rc = salloc((size_t)nnz * 8, (void **)&perm);
        if (!rc) rc = salloc(tmp_bytes, &tmp);
        for (int j = 0; j < N && rc == FTL_OK; ++j) {
            void *r = nullptr, *k = nullptr, *v = nullptr;
            if ((rc = dev_alloc(X, (size_t)nnz * 4, &r, "ftl_sparse_create"))) break;
            if ((rc = dev_alloc(X, (size_t)nnz * 8, &k, "ftl_sparse_create"))) break;
            if ((rc = dev_alloc(X, (size_t)nnz * 8, &v, "ftl_sparse_create"))) break;
            X->rows[j] = (int32_t *)r;
            X->rkeys[j] = (uint64_t *)k;
            X->rvals[j] = (double *)v;
            if ((rc = ftl_fiber_keys(X->idx, 0, nnz, N, 1, N, X->dims, j, fkeys, stream))) break;
            column_iota_kernel<<<grid_of(nnz), 256, 0, st>>>(X->idx, nnz, N, j, col, iota);
            size_t tb = tmp_bytes;
            if ((rc = cuda_status(cub::DeviceRadixSort::SortPairs(tmp, tb, col, col_s, iota, perm, (int64_t)nnz, 0,
                                                                  key_bits(X->dims[j]), st),
                                  "ftl_sparse_create: sort")))
                break;
            rows_gather_kernel<<<grid_of(nnz), 256, 0, st>>>(col_s, perm, fkeys, X->vals, nnz, X->rows[j],
                                                              X->rkeys[j], X->rvals[j]);
            if ((rc = cuda_status(cudaGetLastError(), "ftl_sparse_create: kernels"))) break;
        }
        if (rc == FTL_OK) {
            // SparseTensor's normsq (sparse_tensor.hpp:70-74), read once here
            size_t fb = 0;
            ftl_fit_workspace_bytes(&fb);
            void *ws = nullptr, *o = nullptr;
            rc = salloc(fb, &ws);
            if (!rc) rc = salloc(sizeof(double), &o);
            if (!rc) rc = ftl_sum_squares(X->vals, nnz, ws, fb, (double *)o, stream);
            if (!rc)
                rc = cuda_status(cudaMemcpyAsync(&X->normsq, o, sizeof(double), cudaMemcpyDeviceToHost, st),
                                 "ftl_sparse_create: normsq");
            if (!rc) rc = cuda_status(cudaStreamSynchronize(st), "ftl_sparse_create");
        } else {
            cudaStreamSynchronize(st);
        }
        for (void *q : scratch) cudaFree(q);
    }
    if (rc) goto fail;
    *out = X;
    return FTL_OK;
fail:
    cudaStreamSynchronize(st);
    release(X);
    return rc;
}

extern "C" int ftl_sparse_normsq(const ftl_sparse *X, double *out) {
    FTL_CHECK_ARG(X && out, "ftl_sparse_normsq: null pointer");
    *out = X->normsq;
    return FTL_OK;
}

extern "C" int ftl_sparse_destroy(ftl_sparse *X) {
    if (!X) return FTL_OK;
    cudaError_t err = cudaDeviceSynchronize();
    release(X);
    return cuda_status(err, "ftl_sparse_destroy");
}

extern "C" int ftl_als_create(const ftl_sparse *X, int R, int64_t J, int prec, uint64_t seed, ftl_als **out) {
    FTL_CHECK_ARG(X && out, "ftl_als_create: null pointer");
    *out = nullptr;
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && J >= 1 && J <= INT32_MAX / 4, "ftl_als_create: R=%d J=%lld", R,
                  (long long)J);
    FTL_CHECK_ARG(ftl::valid_prec(prec), "ftl_als_create: bad precision %d", prec);
    ftl_als *A = new ftl_als();
    A->X = X;
    A->N = X->N;
    A->R = R;
    A->J = J;
    A->prec = prec;
    A->seed = seed;
    const int N = A->N;
    int rc = ftl_sampler_create(N, X->dims, R, J, prec, 0, &A->S);
    auto get = [&](size_t bytes, void **q) -> int { return rc ? rc : (rc = dev_alloc(A, bytes, q, "ftl_als_create")); };
    for (int k = 0; k < N && rc == FTL_OK; ++k) rc = ftl_sampler_factor(A->S, k, &A->U[k]);
    if (!rc) rc = ftl_dedup_workspace_bytes(J, &A->nb_dedup);
    if (!rc) rc = ftl_mttkrp_rows_workspace_bytes(J, R, &A->nb_mtt);
    if (!rc) rc = ftl_gram_workspace_bytes(R, &A->nb_gram);
    if (!rc) rc = ftl_colnorm_workspace_bytes(R, &A->nb_col);
    if (!rc) rc = ftl_fit_workspace_bytes(&A->nb_fit);
    const size_t RR = (size_t)R * R * sizeof(double);
    get((size_t)R * sizeof(double), (void **)&A->sigma);
    get((size_t)N * R * sizeof(double), (void **)&A->norms);
    get((size_t)N * J * sizeof(uint64_t), (void **)&A->samples);
    get((size_t)J * R * sizeof(double), (void **)&A->h);
    get((size_t)J * sizeof(double), (void **)&A->w);
    get((size_t)J * R * sizeof(double), (void **)&A->hp);
    get((size_t)J * sizeof(uint64_t), (void **)&A->keys);
    get((size_t)J * sizeof(uint64_t), (void **)&A->ukeys);
    get((size_t)J * sizeof(int32_t), (void **)&A->urep);
    get((size_t)J * sizeof(int32_t), (void **)&A->ucnt);
    get(sizeof(int64_t), (void **)&A->nuniq);
    get(RR, (void **)&A->gram);
    get(RR, (void **)&A->pinv);
    get(RR, (void **)&A->vscr);
    get(RR * N, (void **)&A->grams);
    get(2 * sizeof(double), (void **)&A->terms);
    get(A->nb_dedup, &A->ws_dedup);
    get(A->nb_mtt, &A->ws_mtt);
    get(A->nb_gram, &A->ws_gram);
    get(A->nb_col, &A->ws_col);
    get(A->nb_fit, &A->ws_fit);
    if (!rc) {
        // sigma = 1 until set or renormalised
        std::vector<double> ones(R, 1.0);
        rc = cuda_status(cudaMemcpy(A->sigma, ones.data(), R * sizeof(double), cudaMemcpyHostToDevice),
                         "ftl_als_create: sigma");
    }
    if (rc) {
        ftl_sampler_destroy(A->S);
        release(A);
        return rc;
    }
    *out = A;
    return FTL_OK;
}

extern "C" int ftl_als_set_factor(ftl_als *A, int k, const double *U, int on_host, void *stream) {
    FTL_CHECK_ARG(A, "ftl_als_set_factor: null pointer");
    return ftl_sampler_set_factor(A->S, k, U, on_host, stream);
}

extern "C" int ftl_als_set_sigma(ftl_als *A, const double *sigma, int on_host, void *stream) {
    FTL_CHECK_ARG(A && sigma, "ftl_als_set_sigma: null pointer");
    return cuda_status(cudaMemcpyAsync(A->sigma, sigma, A->R * sizeof(double),
                                       on_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                       (cudaStream_t)stream),
                       "ftl_als_set_sigma");
}

extern "C" int ftl_als_factor(const ftl_als *A, int k, double **U_dev) {
    FTL_CHECK_ARG(A && U_dev && k >= 0 && k < A->N, "ftl_als_factor: bad arguments");
    *U_dev = A->U[k];
    return FTL_OK;
}

extern "C" int ftl_als_sigma(const ftl_als *A, double **sigma_dev) {
    FTL_CHECK_ARG(A && sigma_dev, "ftl_als_sigma: null pointer");
    *sigma_dev = A->sigma;
    return FTL_OK;
}

extern "C" int ftl_als_samples(const ftl_als *A, uint64_t **samples_dev) {
    FTL_CHECK_ARG(A && samples_dev, "ftl_als_samples: null pointer");
    *samples_dev = A->samples;
    return FTL_OK;
}

namespace {

// sigma = prod_k norms[k] (j < 0) or norms[j]; one thread per column
__global__ void sigma_kernel(const double *__restrict__ norms, int N, int R, int j, double *__restrict__ sigma) {
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        if (j >= 0) {
            sigma[r] = norms[j * R + r];
        } else {
            double s = 1.0;
            for (int k = 0; k < N; ++k) s *= norms[k * R + r];
            sigma[r] = s;
        }
    }
}

}  // namespace

extern "C" int ftl_als_renormalize(ftl_als *A, int j, void *stream) {
    FTL_CHECK_ARG(A && j >= -1 && j < A->N, "ftl_als_renormalize: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    int rc = FTL_OK;
    for (int k = 0; k < A->N && rc == FTL_OK; ++k) {
        if (j >= 0 && k != j) continue;
        rc = ftl_renormalize_columns(A->U[k], A->X->dims[k], A->R, A->norms + (size_t)k * A->R, A->ws_col, A->nb_col,
                                     1, stream);
        if (!rc) rc = ftl_sampler_update(A->S, k, stream);
    }
    if (rc) return rc;
    sigma_kernel<<<1, 128, 0, st>>>(A->norms, A->N, A->R, j, A->sigma);
    return cuda_status(cudaGetLastError(), "ftl_als_renormalize");
}

extern "C" int ftl_als_init_rrf(ftl_als *A, uint64_t seed, void *stream) {
    FTL_CHECK_ARG(A, "ftl_als_init_rrf: null pointer");
    const ftl_sparse *X = A->X;
    for (int j = 0; j < A->N; ++j) {
        int rc = ftl_sparse_rrf(X->rows[j], X->rkeys[j], X->rvals[j], X->nnz, A->R, seed, (uint32_t)j, A->U[j],
                                X->dims[j], stream);
        if (rc) return rc;
    }
    return ftl_als_renormalize(A, -1, stream);
}

extern "C" int ftl_als_update(ftl_als *A, int j, int renormalize, int update_sampler, const double *draws_dev,
                              void *stream) {
    FTL_CHECK_ARG(A && j >= 0 && j < A->N, "ftl_als_update: bad arguments");
    const ftl_sparse *X = A->X;
    const int N = A->N, R = A->R;
    const int64_t J = A->J;
    int rc = ftl_sampler_draw(A->S, (uint32_t)j, A->samples, A->h, A->w, draws_dev, A->seed, A->counter, stream);
    if (rc) return rc;
    if (!draws_dev) A->counter += 2 * (uint64_t)N * J;
    // fiber keys of the samples on the modes != j (samples are N x J)
    if ((rc = ftl_fiber_keys(A->samples, 1, J, 1, J, N, X->dims, j, A->keys, stream))) return rc;
    if ((rc = ftl_dedup(A->keys, J, A->ws_dedup, A->nb_dedup, A->ukeys, A->urep, A->ucnt, A->nuniq, stream)))
        return rc;
    if ((rc = ftl_weighted_gram(A->h, A->urep, A->w, A->ucnt, A->nuniq, J, R, A->ws_gram, A->nb_gram, A->gram,
                                stream)))
        return rc;
    if ((rc = ftl_pinv_square(A->gram, R, R, A->nuniq, 1e-11, A->pinv, A->vscr, stream))) return rc;
    // U_j = MTTKRP pinv, with the J sampled rows multiplied by pinv first
    if ((rc = ftl_solve_rows(A->h, A->pinv, J, R, A->hp, stream))) return rc;
    if ((rc = ftl_sparse_mttkrp_rows(X->rows[j], X->rkeys[j], X->rvals[j], X->nnz, A->ukeys, A->urep, A->ucnt,
                                     A->nuniq, J, J, A->w, A->hp, R, A->ws_mtt, A->nb_mtt, A->U[j], X->dims[j],
                                     stream)))
        return rc;
    if (renormalize) {
        if ((rc = ftl_renormalize_columns(A->U[j], X->dims[j], R, A->norms + (size_t)j * R, A->ws_col, A->nb_col, 1,
                                          stream)))
            return rc;
        sigma_kernel<<<1, 128, 0, (cudaStream_t)stream>>>(A->norms, N, R, j, A->sigma);
        if ((rc = cuda_status(cudaGetLastError(), "ftl_als_update"))) return rc;
    }
    if (update_sampler) rc = ftl_sampler_update(A->S, j, stream);
    return rc;
}

extern "C" int ftl_als_fit(ftl_als *A, double *fit, double *residual_normsq, void *stream) {
    FTL_CHECK_ARG(A, "ftl_als_fit: null pointer");
    const ftl_sparse *X = A->X;
    const int N = A->N, R = A->R;
    cudaStream_t st = (cudaStream_t)stream;
    const double *Uc[FTL_MAX_MODES];
    const double *Gc[FTL_MAX_MODES];
    for (int k = 0; k < N; ++k) Uc[k] = A->U[k];
    // ||X - M||^2 = sum over nonzeros of v^2 - 2 v m + ||M||^2 (sparse_tensor.hpp:117-119)
    int rc = ftl_sparse_residual_terms(X->idx, X->vals, X->nnz, N, Uc, A->sigma, R, A->ws_fit, A->nb_fit, A->terms,
                                       stream);
    for (int k = 0; k < N && rc == FTL_OK; ++k) {
        double *g = A->grams + (size_t)k * R * R;
        rc = ftl_weighted_gram(A->U[k], nullptr, nullptr, nullptr, nullptr, X->dims[k], R, A->ws_gram, A->nb_gram, g,
                               stream);
        Gc[k] = g;
    }
    if (!rc) rc = ftl_gram_hadamard(Gc, N, R, -1, A->sigma, A->sigma, nullptr, A->terms + 1, stream);
    double t[2] = {0.0, 0.0};
    if (!rc) rc = cuda_status(cudaMemcpyAsync(t, A->terms, sizeof(t), cudaMemcpyDeviceToHost, st), "ftl_als_fit");
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st), "ftl_als_fit");
    if (rc) return rc;
    const double resid = t[0] + t[1];
    if (residual_normsq) *residual_normsq = resid;
    // PyLowRank.compute_exact_fit, tensors.py:50-53
    if (fit) *fit = 1.0 - std::sqrt(resid) / std::sqrt(X->normsq);
    return FTL_OK;
}

extern "C" int ftl_als_destroy(ftl_als *A) {
    if (!A) return FTL_OK;
    int rc = ftl_sampler_destroy(A->S);
    release(A);
    return rc;
}
