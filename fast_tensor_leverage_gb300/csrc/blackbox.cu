// CP-ALS against black-box right-hand sides: a low-rank tensor [[s; V]] and a
// dense tensor, plus the low-rank algebra the fit needs.
//
// Reference semantics (vbharadwaj-bk/fast_tensor_leverage, cpp_ext/):
//   BlackBoxTensor::execute_downsampled_mttkrp  black_box_tensor.hpp:21-67
//     result (I_j x R) = sum over the (deduplicated) samples s of
//     fiber_s (I_j) (x) lhs_s (R), fiber_s = the tensor along mode j at the
//     sample's other indices; lhs_s = w_s count_s h_s (als.hpp:155-174).
//   LowRankTensor::materialize_rhs               low_rank_tensor.hpp:91-135
//     fiber_s = V_j (s o prod_{k != j} V_k[s_k, :])
//   LowRankTensor::compute_residual_normsq       low_rank_tensor.hpp:78-89
//   LowRankTensor::execute_exact_mttkrp          low_rank_tensor.hpp:147-180
//   LowRankTensor::evaluate_indices              low_rank_tensor.hpp:262-280
//   ATB_chain_prod / ATB_chain_prod_sum          common.h:152-226
//   DenseTensor::materialize_rhs                 dense_tensor.hpp:38-59
//
// Low-rank shortcut: the sum of fiber_s lhs_s^T over the samples is
// V_j (P^T L), P (samples x R_rhs) the rows s o prod V_k[s_k], L the lhs rows:
// an R_rhs x R reduction over the samples and one I_j x R_rhs x R product,
// instead of materialising samples x I_j fibers.
#include <algorithm>

#include "ftl_common.cuh"

namespace ftl {


struct BBFactors {
    const double *U[FTL_MAX_MODES];
};

// Rows of L: coef_u * h[rep_u], rep_u = urep ? urep[u] : u,
// coef_u = (w ? w[rep_u] : 1) * (cnt ? cnt[u] : 1).
__device__ __forceinline__ int64_t bb_rep(const int32_t *urep, int64_t u) { return urep ? (int64_t)urep[u] : u; }
__device__ __forceinline__ double bb_coef(const double *w, const int32_t *cnt, int64_t rep, int64_t u) {
    return (w ? w[rep] : 1.0) * (cnt ? (double)cnt[u] : 1.0);
}

// partial[b][a * R + c] = sum over block b's rows u of P[u][a] * L[u][c].
// Rows staged 32 at a time in shared memory; each thread keeps 4 entries of
// the Rr x R block per pass.  Fixed block ranges and a fixed-order reduction
// make the result deterministic.
__global__ void lr_pth_partial_kernel(BBFactors V, const double *__restrict__ srhs, int N, int Rr, int j,
                                      const uint64_t *__restrict__ samples, int64_t J,
                                      const int32_t *__restrict__ urep, const int32_t *__restrict__ cnt,
                                      const int64_t *__restrict__ n_dev, int64_t n_host,
                                      const double *__restrict__ w, const double *__restrict__ h, int R,
                                      double *__restrict__ partial) {
    extern __shared__ double sm[];
    double *Ps = sm;             // 32 x Rr
    double *Ls = sm + 32 * Rr;   // 32 x R
    const int64_t n = n_dev ? *n_dev : n_host;
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    const int E = Rr * R;
    for (int e0 = 0; e0 < E; e0 += 4 * blockDim.x) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int64_t u0 = r0; u0 < r1; u0 += 32) {
            const int m = (int)min((int64_t)32, r1 - u0);
            __syncthreads();
            for (int e = threadIdx.x; e < m * Rr; e += blockDim.x) {
                const int uu = e / Rr, a = e - uu * Rr;
                const int64_t rep = bb_rep(urep, u0 + uu);
                double p = srhs ? srhs[a] : 1.0;
                for (int k = 0; k < N; ++k)
                    if (k != j) p *= V.U[k][(int64_t)samples[(int64_t)k * J + rep] * Rr + a];
                Ps[e] = p;
            }
            for (int e = threadIdx.x; e < m * R; e += blockDim.x) {
                const int uu = e / R, c = e - uu * R;
                const int64_t u = u0 + uu, rep = bb_rep(urep, u);
                Ls[e] = bb_coef(w, cnt, rep, u) * h[rep * R + c];
            }
            __syncthreads();
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int e = e0 + threadIdx.x + t * blockDim.x;
                if (e < E) {
                    const int a = e / R, c = e - a * R;
                    for (int uu = 0; uu < m; ++uu) acc[t] = fma(Ps[uu * Rr + a], Ls[uu * R + c], acc[t]);
                }
            }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int e = e0 + threadIdx.x + t * blockDim.x;
            if (e < E) partial[(int64_t)blockIdx.x * E + e] = acc[t];
        }
    }
}

// partial[b][a * Rb + c] = sum over block b's rows i of A[i][a] * B[i][c]
// (A^T B, A: I x Ra, B: I x Rb, row-major).
__global__ void cross_partial_kernel(const double *__restrict__ A, int Ra, const double *__restrict__ B, int Rb,
                                     int64_t I, double *__restrict__ partial) {
    extern __shared__ double sm[];
    double *As = sm;             // 32 x Ra
    double *Bs = sm + 32 * Ra;   // 32 x Rb
    const int64_t per = (I + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = blockIdx.x * per, r1 = min(I, r0 + per);
    const int E = Ra * Rb;
    for (int e0 = 0; e0 < E; e0 += 4 * blockDim.x) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int64_t i0 = r0; i0 < r1; i0 += 32) {
            const int m = (int)min((int64_t)32, r1 - i0);
            __syncthreads();
            for (int e = threadIdx.x; e < m * Ra; e += blockDim.x) As[e] = A[i0 * Ra + e];
            for (int e = threadIdx.x; e < m * Rb; e += blockDim.x) Bs[e] = B[i0 * Rb + e];
            __syncthreads();
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int e = e0 + threadIdx.x + t * blockDim.x;
                if (e < E) {
                    const int a = e / Rb, c = e - a * Rb;
                    for (int ii = 0; ii < m; ++ii) acc[t] = fma(As[ii * Ra + a], Bs[ii * Rb + c], acc[t]);
                }
            }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int e = e0 + threadIdx.x + t * blockDim.x;
            if (e < E) partial[(int64_t)blockIdx.x * E + e] = acc[t];
        }
    }
}

__global__ void partial_sum_kernel(const double *__restrict__ partial, int nblk, int E, double *__restrict__ out) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += partial[(int64_t)b * E + e];
        out[e] = s;
    }
}

// out[i][c] = sum_a X[i][a] * M[a][c] for i < I (X: I x K, M: K x C in
// shared memory); rows I..out_rows-1 of out are zeroed.
__global__ void rows_times_small_kernel(const double *__restrict__ X, int64_t I, int K,
                                        const double *__restrict__ M, int C, double *__restrict__ out,
                                        int64_t out_rows) {
    extern __shared__ double Ms[];
    for (int e = threadIdx.x; e < K * C; e += blockDim.x) Ms[e] = M[e];
    __syncthreads();
    const int64_t total = out_rows * C;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / C;
        const int c = (int)(e - i * C);
        double s = 0.0;
        if (i < I) {
            const double *x = X + i * K;
            for (int a = 0; a < K; ++a) s = fma(x[a], Ms[a * C + c], s);
        }
        out[e] = s;
    }
}

struct BBGrams {
    const double *G[FTL_MAX_MODES];
};

// M = (sa sb^T) o prod_{k != exclude} G_k (each Ra x Rb), optionally its sum
// (ATB_chain_prod / ATB_chain_prod_sum, common.h:152-226).
__global__ void chain_prod_kernel(BBGrams gp, int N, int Ra, int Rb, int exclude, const double *__restrict__ sa,
                                  const double *__restrict__ sb, double *__restrict__ out_mat,
                                  double *__restrict__ out_sum) {
    __shared__ double red[1024];
    double acc = 0.0;
    for (int e = threadIdx.x; e < Ra * Rb; e += blockDim.x) {
        const int a = e / Rb, b = e - a * Rb;
        double m = (sa ? sa[a] : 1.0) * (sb ? sb[b] : 1.0);
        for (int k = 0; k < N; ++k)
            if (k != exclude) m *= gp.G[k][e];
        if (out_mat) out_mat[e] = m;
        acc += m;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0 && out_sum) {
        double s = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) s += red[t];
        *out_sum = s;
    }
}

// out[z] = sum_r s_r prod_k U_k[idx(z, k), r]; idx (n x N) row-major, uint32
// or uint64 (LowRankTensor::evaluate_indices).  One warp per index.
template <typename IT>
__global__ void lr_evaluate_kernel(BBFactors U, int N, int R, const double *__restrict__ s,
                                   const IT *__restrict__ idx, int64_t n, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t z = gw; z < n; z += nw) {
        double m = 0.0;
        for (int r = lane; r < R; r += 32) {
            double p = s ? s[r] : 1.0;
            for (int k = 0; k < N; ++k) p *= U.U[k][(int64_t)idx[z * N + k] * R + r];
            m += p;
        }
        m = warp_sum(m);
        if (lane == 0) out[z] = m;
    }
}

// Fibers of a low-rank tensor at n samples (n x N row-major uint64): j >= N:
// out (n x R) = s o prod_k U_k[s_k]; else out (n x I_j) = that row times U_j^T.
// One block per sample: the partial row in shared memory, threads over i.
__global__ void lr_materialize_kernel(BBFactors U, int N, int R, const double *__restrict__ s,
                                      const uint64_t *__restrict__ S, int64_t n, int j, int64_t I_j,
                                      double *__restrict__ out) {
    __shared__ double p[FTL_MAX_RANK];
    for (int64_t z = blockIdx.x; z < n; z += gridDim.x) {
        __syncthreads();
        for (int r = threadIdx.x; r < R; r += blockDim.x) {
            double v = s ? s[r] : 1.0;
            for (int k = 0; k < N; ++k)
                if (k != j) v *= U.U[k][(int64_t)S[z * N + k] * R + r];
            p[r] = v;
        }
        __syncthreads();
        if (j >= N) {
            for (int r = threadIdx.x; r < R; r += blockDim.x) out[z * R + r] = p[r];
        } else {
            const double *Uj = U.U[j];
            for (int64_t i = threadIdx.x; i < I_j; i += blockDim.x) {
                double v = 0.0;
                for (int r = 0; r < R; ++r) v = fma(p[r], Uj[i * R + r], v);
                out[z * I_j + i] = v;
            }
        }
    }
}

// ------------------------------------------------------------------ dense

struct DenseGeom {
    int N;
    int64_t dims[FTL_MAX_MODES];
    int64_t stride[FTL_MAX_MODES];  // row-major: stride[k] = prod_{l > k} dims[l]
};

// Dense sampled MTTKRP: out[i][c] = sum_u coef_u T[off_u + i ldt] h[rep_u][c]
// (off_u = sum_{k != j} s_k stride[k], ldt = stride[j]).  A block owns 32
// rows of out; the samples pass through shared memory 32 at a time with
// their 32 x 32 tile of tensor values and 32 scaled lhs rows.
template <typename VT>
__global__ void dense_mttkrp_kernel(const VT *__restrict__ T, DenseGeom dg, int j,
                                    const uint64_t *__restrict__ samples, int64_t J,
                                    const int32_t *__restrict__ urep, const int32_t *__restrict__ cnt,
                                    const int64_t *__restrict__ n_dev, int64_t n_host,
                                    const double *__restrict__ w, const double *__restrict__ h, int R,
                                    double *__restrict__ out, int64_t out_rows) {
    __shared__ double tv[32][33];
    __shared__ int64_t off[32];
    extern __shared__ double Ls[];  // 32 x R
    const int64_t n = n_dev ? *n_dev : n_host;
    const int64_t I_j = dg.dims[j], ldt = dg.stride[j];
    constexpr int OPT = 16;  // outputs per thread: 32 rows x R <= 4096 over 256 threads
    for (int64_t i0 = (int64_t)blockIdx.x * 32; i0 < out_rows; i0 += (int64_t)gridDim.x * 32) {
        double acc[OPT];
#pragma unroll
        for (int q = 0; q < OPT; ++q) acc[q] = 0.0;
        for (int64_t u0 = 0; u0 < n; u0 += 32) {
            const int m = (int)min((int64_t)32, n - u0);
            __syncthreads();
            if (threadIdx.x < m) {
                const int64_t rep = bb_rep(urep, u0 + threadIdx.x);
                int64_t o = 0;
                for (int k = 0; k < dg.N; ++k)
                    if (k != j) o += (int64_t)samples[(int64_t)k * J + rep] * dg.stride[k];
                off[threadIdx.x] = o;
            }
            for (int e = threadIdx.x; e < m * R; e += blockDim.x) {
                const int uu = e / R, c = e - uu * R;
                const int64_t u = u0 + uu, rep = bb_rep(urep, u);
                Ls[e] = bb_coef(w, cnt, rep, u) * h[rep * R + c];
            }
            __syncthreads();
            for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
                const int uu = e >> 5, ii = e & 31;
                const int64_t i = i0 + ii;
                tv[uu][ii] = (uu < m && i < I_j) ? (double)T[off[uu] + i * ldt] : 0.0;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < OPT; ++q) {
                const int e = threadIdx.x + q * blockDim.x;
                if (e < 32 * R) {
                    const int ii = e / R, c = e - ii * R;
                    double a = acc[q];
                    for (int uu = 0; uu < m; ++uu) a = fma(tv[uu][ii], Ls[uu * R + c], a);
                    acc[q] = a;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < OPT; ++q) {
            const int e = threadIdx.x + q * blockDim.x;
            if (e < 32 * R) {
                const int ii = e / R, c = e - ii * R;
                const int64_t i = i0 + ii;
                if (i < out_rows) out[i * R + c] = acc[q];
            }
        }
    }
}

// out (n x I_j) = fibers of T at n samples (n x N row-major uint64).
template <typename VT>
__global__ void dense_materialize_kernel(const VT *__restrict__ T, DenseGeom dg, int j,
                                         const uint64_t *__restrict__ S, int64_t n, double *__restrict__ out) {
    const int64_t I_j = dg.dims[j], ldt = dg.stride[j];
    const int64_t total = n * I_j;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t z = e / I_j, i = e - z * I_j;
        int64_t o = 0;
        for (int k = 0; k < dg.N; ++k)
            if (k != j) o += (int64_t)S[z * dg.N + k] * dg.stride[k];
        out[e] = (double)T[o + i * ldt];
    }
}

// partial[b] = (sum over block b's entries of (T - model)^2, of T^2), model =
// sum_r s_r prod_k U_k[i_k, r].  One thread per entry.
template <typename VT>
__global__ void dense_residual_kernel(const VT *__restrict__ T, DenseGeom dg, BBFactors U, const double *__restrict__ s,
                                      int R, int64_t total, double *__restrict__ partial) {
    __shared__ double red[2][256];
    double a0 = 0.0, a1 = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t rem = e;
        int64_t ik[FTL_MAX_MODES];
        for (int k = 0; k < dg.N; ++k) {
            ik[k] = rem / dg.stride[k];
            rem -= ik[k] * dg.stride[k];
        }
        double m = 0.0;
        if (U.U[0]) {
            for (int r = 0; r < R; ++r) {
                double p = s ? s[r] : 1.0;
                for (int k = 0; k < dg.N; ++k) p *= U.U[k][ik[k] * R + r];
                m += p;
            }
        }
        const double t = (double)T[e];
        a0 = fma(t - m, t - m, a0);
        a1 = fma(t, t, a1);
    }
    red[0][threadIdx.x] = a0;
    red[1][threadIdx.x] = a1;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int t = 0; t < (int)blockDim.x; ++t) {
            s0 += red[0][t];
            s1 += red[1][t];
        }
        partial[2 * blockIdx.x] = s0;
        partial[2 * blockIdx.x + 1] = s1;
    }
}

__global__ void pair_sum_kernel(const double *__restrict__ partial, int nblk, double *__restrict__ out) {
    // one warp, fixed order: lane-strided sums, then a shuffle tree
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    double s0 = 0.0, s1 = 0.0;
    for (int b = threadIdx.x; b < nblk; b += 32) {
        s0 += partial[2 * b];
        s1 += partial[2 * b + 1];
    }
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    if (threadIdx.x == 0) {
        out[0] = s0;
        out[1] = s1;
    }
}

static int bb_fill(BBFactors &f, const double *const *U, int N) {
    for (int k = 0; k < FTL_MAX_MODES; ++k) f.U[k] = k < N ? U[k] : nullptr;
    for (int k = 0; k < N; ++k) FTL_CHECK_ARG(U[k] != nullptr, "factor %d is NULL", k);
    return FTL_OK;
}

static int dense_geom(DenseGeom &dg, const int64_t *dims, int N) {
    FTL_CHECK_ARG(dims && N >= 1 && N <= FTL_MAX_MODES, "dense tensor: bad N=%d", N);
    dg.N = N;
    int64_t st = 1;
    for (int k = N - 1; k >= 0; --k) {
        FTL_CHECK_ARG(dims[k] >= 1, "dense tensor: dims[%d]=%lld", k, (long long)dims[k]);
        dg.dims[k] = dims[k];
        dg.stride[k] = st;
        st *= dims[k];
    }
    for (int k = N; k < FTL_MAX_MODES; ++k) dg.dims[k] = dg.stride[k] = 0;
    return FTL_OK;
}

static int smem_attr(const void *fn, size_t bytes) {
    FTL_CHECK_ARG(bytes <= 227 * 1024, "shared memory request of %zu bytes", bytes);
    return ensure_smem(fn, bytes, "black-box MTTKRP kernel");
}

}  // namespace ftl

using namespace ftl;

// ============================================================== C ABI

extern "C" int ftl_lowrank_mttkrp_workspace_bytes(int Rr, int R, size_t *out) {
    FTL_CHECK_ARG(out && Rr >= 1 && Rr <= FTL_MAX_RANK && R >= 1 && R <= FTL_MAX_RANK,
                  "ftl_lowrank_mttkrp_workspace_bytes: bad ranks %d, %d", Rr, R);
    *out = ((size_t)num_sms() + 1) * Rr * R * sizeof(double);
    return FTL_OK;
}

extern "C" int ftl_lowrank_sampled_mttkrp(const double *const *V, const double *sigma_rhs, int N, int Rr, int j,
                                          const uint64_t *samples, int64_t J, const int32_t *urep,
                                          const int32_t *ucnt, const int64_t *num_unique_dev, int64_t num_unique,
                                          const double *w, const double *h, int R, void *workspace,
                                          size_t ws_bytes, double *out, int64_t I_j, int64_t out_rows,
                                          void *stream) {
    FTL_CHECK_ARG(V && samples && h && workspace && out, "ftl_lowrank_sampled_mttkrp: null pointer");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && j >= 0 && j < N && Rr >= 1 && Rr <= FTL_MAX_RANK && R >= 1 &&
                      R <= FTL_MAX_RANK && I_j >= 1 && out_rows >= I_j && J >= 1,
                  "ftl_lowrank_sampled_mttkrp: bad shape");
    size_t need = 0;
    ftl_lowrank_mttkrp_workspace_bytes(Rr, R, &need);
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_lowrank_sampled_mttkrp: workspace %zu < %zu bytes", ws_bytes, need);
    BBFactors f;
    int rc = bb_fill(f, V, N);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int nblk = num_sms();
    double *partial = (double *)workspace, *M = partial + (size_t)nblk * Rr * R;
    const size_t sm1 = (size_t)32 * (Rr + R) * sizeof(double);
    rc = smem_attr((const void *)lr_pth_partial_kernel, sm1);
    if (rc) return rc;
    lr_pth_partial_kernel<<<nblk, 256, sm1, st>>>(f, sigma_rhs, N, Rr, j, samples, J, urep, ucnt, num_unique_dev,
                                                  num_unique, w, h, R, partial);
    partial_sum_kernel<<<std::max(1, (Rr * R + 255) / 256), 256, 0, st>>>(partial, nblk, Rr * R, M);
    const size_t sm2 = (size_t)Rr * R * sizeof(double);
    rc = smem_attr((const void *)rows_times_small_kernel, sm2);
    if (rc) return rc;
    int blocks = (int)std::min<int64_t>((out_rows * R + 255) / 256, (int64_t)nblk * 16);
    rows_times_small_kernel<<<std::max(blocks, 1), 256, sm2, st>>>(V[j], I_j, Rr, M, R, out, out_rows);
    return check_launch("low-rank sampled MTTKRP kernels");
}

extern "C" int ftl_cross_gram_workspace_bytes(int Ra, int Rb, size_t *out) {
    FTL_CHECK_ARG(out && Ra >= 1 && Ra <= FTL_MAX_RANK && Rb >= 1 && Rb <= FTL_MAX_RANK,
                  "ftl_cross_gram_workspace_bytes: bad ranks");
    *out = (size_t)num_sms() * Ra * Rb * sizeof(double);
    return FTL_OK;
}

extern "C" int ftl_cross_gram(const double *A, int Ra, const double *B, int Rb, int64_t I, void *workspace,
                              size_t ws_bytes, double *out, void *stream) {
    FTL_CHECK_ARG(A && B && workspace && out && I >= 1, "ftl_cross_gram: bad arguments");
    size_t need = 0;
    int rc = ftl_cross_gram_workspace_bytes(Ra, Rb, &need);
    if (rc) return rc;
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_cross_gram: workspace %zu < %zu bytes", ws_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    const int nblk = num_sms();
    const size_t sm = (size_t)32 * (Ra + Rb) * sizeof(double);
    rc = smem_attr((const void *)cross_partial_kernel, sm);
    if (rc) return rc;
    cross_partial_kernel<<<nblk, 256, sm, st>>>(A, Ra, B, Rb, I, (double *)workspace);
    partial_sum_kernel<<<std::max(1, (Ra * Rb + 255) / 256), 256, 0, st>>>((const double *)workspace, nblk, Ra * Rb,
                                                                          out);
    return check_launch("cross Gram kernels");
}

extern "C" int ftl_chain_prod(const double *const *grams, int N, int Ra, int Rb, int exclude, const double *sigma_a,
                              const double *sigma_b, double *out_mat, double *out_sum, void *stream) {
    FTL_CHECK_ARG(grams && (out_mat || out_sum), "ftl_chain_prod: null pointer");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && Ra >= 1 && Ra <= FTL_MAX_RANK && Rb >= 1 && Rb <= FTL_MAX_RANK,
                  "ftl_chain_prod: bad shape");
    BBGrams gp;
    for (int k = 0; k < FTL_MAX_MODES; ++k) gp.G[k] = k < N ? grams[k] : nullptr;
    chain_prod_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(gp, N, Ra, Rb, exclude, sigma_a, sigma_b, out_mat,
                                                            out_sum);
    return check_launch("chain_prod_kernel");
}

extern "C" int ftl_lowrank_evaluate(const double *const *U, int N, int R, const double *sigma, const void *idx,
                                    int idx_is_u64, int64_t n, double *out, void *stream) {
    FTL_CHECK_ARG(U && idx && out && n >= 0, "ftl_lowrank_evaluate: bad arguments");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && R >= 1 && R <= FTL_MAX_RANK, "ftl_lowrank_evaluate: bad shape");
    if (n == 0) return FTL_OK;
    BBFactors f;
    int rc = bb_fill(f, U, N);
    if (rc) return rc;
    int blocks = (int)std::min<int64_t>((n * 32 + 255) / 256, (int64_t)num_sms() * 16);
    if (idx_is_u64)
        lr_evaluate_kernel<uint64_t><<<blocks, 256, 0, (cudaStream_t)stream>>>(f, N, R, sigma, (const uint64_t *)idx,
                                                                             n, out);
    else
        lr_evaluate_kernel<uint32_t><<<blocks, 256, 0, (cudaStream_t)stream>>>(f, N, R, sigma, (const uint32_t *)idx,
                                                                             n, out);
    return check_launch("lr_evaluate_kernel");
}

extern "C" int ftl_lowrank_materialize(const double *const *U, int N, int R, const double *sigma,
                                       const uint64_t *samples, int64_t n, int j, int64_t I_j, double *out,
                                       void *stream) {
    FTL_CHECK_ARG(U && samples && out && n >= 0, "ftl_lowrank_materialize: bad arguments");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && R >= 1 && R <= FTL_MAX_RANK && j >= 0,
                  "ftl_lowrank_materialize: bad shape");
    if (n == 0) return FTL_OK;
    BBFactors f;
    int rc = bb_fill(f, U, N);
    if (rc) return rc;
    int blocks = (int)std::min<int64_t>(n, (int64_t)num_sms() * 16);
    lr_materialize_kernel<<<blocks, 128, 0, (cudaStream_t)stream>>>(f, N, R, sigma, samples, n, j, I_j, out);
    return check_launch("lr_materialize_kernel");
}

extern "C" int ftl_dense_sampled_mttkrp(const void *T, int is_f32, const int64_t *dims, int N, int j,
                                        const uint64_t *samples, int64_t J, const int32_t *urep,
                                        const int32_t *ucnt, const int64_t *num_unique_dev, int64_t num_unique,
                                        const double *w, const double *h, int R, double *out, int64_t out_rows,
                                        void *stream) {
    FTL_CHECK_ARG(T && samples && h && out, "ftl_dense_sampled_mttkrp: null pointer");
    FTL_CHECK_ARG(j >= 0 && j < N && R >= 1 && R <= FTL_MAX_RANK && J >= 1, "ftl_dense_sampled_mttkrp: bad shape");
    DenseGeom dg;
    int rc = dense_geom(dg, dims, N);
    if (rc) return rc;
    FTL_CHECK_ARG(out_rows >= dg.dims[j], "ftl_dense_sampled_mttkrp: out_rows %lld < dims[%d]",
                  (long long)out_rows, j);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t sm = (size_t)32 * R * sizeof(double);
    int blocks = (int)std::min<int64_t>((out_rows + 31) / 32, (int64_t)num_sms() * 8);
    if (is_f32)
        dense_mttkrp_kernel<float><<<blocks, 256, sm, st>>>((const float *)T, dg, j, samples, J, urep, ucnt,
                                                             num_unique_dev, num_unique, w, h, R, out, out_rows);
    else
        dense_mttkrp_kernel<double><<<blocks, 256, sm, st>>>((const double *)T, dg, j, samples, J, urep, ucnt,
                                                              num_unique_dev, num_unique, w, h, R, out, out_rows);
    return check_launch("dense_mttkrp_kernel");
}

extern "C" int ftl_dense_materialize(const void *T, int is_f32, const int64_t *dims, int N, int j,
                                     const uint64_t *samples, int64_t n, double *out, void *stream) {
    FTL_CHECK_ARG(T && samples && out && n >= 0 && j >= 0 && j < N, "ftl_dense_materialize: bad arguments");
    DenseGeom dg;
    int rc = dense_geom(dg, dims, N);
    if (rc) return rc;
    if (n == 0) return FTL_OK;
    int blocks = (int)std::min<int64_t>((n * dg.dims[j] + 255) / 256, (int64_t)num_sms() * 16);
    if (is_f32)
        dense_materialize_kernel<float><<<blocks, 256, 0, (cudaStream_t)stream>>>((const float *)T, dg, j, samples, n,
                                                                                 out);
    else
        dense_materialize_kernel<double><<<blocks, 256, 0, (cudaStream_t)stream>>>((const double *)T, dg, j, samples,
                                                                                  n, out);
    return check_launch("dense_materialize_kernel");
}

extern "C" int ftl_dense_residual_workspace_bytes(size_t *out) {
    FTL_CHECK_ARG(out, "ftl_dense_residual_workspace_bytes: null");
    *out = (size_t)num_sms() * 8 * 2 * sizeof(double);
    return FTL_OK;
}

extern "C" int ftl_dense_residual_terms(const void *T, int is_f32, const int64_t *dims, int N,
                                        const double *const *U, const double *sigma, int R, void *workspace,
                                        size_t ws_bytes, double *out, void *stream) {
    FTL_CHECK_ARG(T && workspace && out, "ftl_dense_residual_terms: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK, "ftl_dense_residual_terms: bad R=%d", R);
    size_t need = 0;
    ftl_dense_residual_workspace_bytes(&need);
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_dense_residual_terms: workspace too small");
    DenseGeom dg;
    int rc = dense_geom(dg, dims, N);
    if (rc) return rc;
    BBFactors f;
    if (U) {
        rc = bb_fill(f, U, N);
        if (rc) return rc;
    } else {
        for (int k = 0; k < FTL_MAX_MODES; ++k) f.U[k] = nullptr;
    }
    const int64_t total = dg.dims[0] * dg.stride[0];
    const int nblk = num_sms() * 8;
    cudaStream_t st = (cudaStream_t)stream;
    if (is_f32)
        dense_residual_kernel<float><<<nblk, 256, 0, st>>>((const float *)T, dg, f, sigma, R, total,
                                                           (double *)workspace);
    else
        dense_residual_kernel<double><<<nblk, 256, 0, st>>>((const double *)T, dg, f, sigma, R, total,
                                                            (double *)workspace);
    pair_sum_kernel<<<1, 32, 0, st>>>((const double *)workspace, nblk, out);
    return check_launch("dense residual kernels");
}

extern "C" int ftl_rows_times(const double *X, int64_t I, int K, const double *M, int C, double *out,
                              int64_t out_rows, void *stream) {
    FTL_CHECK_ARG(X && M && out && I >= 0 && out_rows >= I, "ftl_rows_times: bad arguments");
    FTL_CHECK_ARG(K >= 1 && K <= FTL_MAX_RANK && C >= 1 && C <= FTL_MAX_RANK, "ftl_rows_times: bad K=%d C=%d", K, C);
    if (out_rows == 0) return FTL_OK;
    const size_t sm = (size_t)K * C * sizeof(double);
    int rc = smem_attr((const void *)rows_times_small_kernel, sm);
    if (rc) return rc;
    int blocks = (int)std::min<int64_t>((out_rows * C + 255) / 256, (int64_t)num_sms() * 16);
    rows_times_small_kernel<<<std::max(blocks, 1), 256, sm, (cudaStream_t)stream>>>(X, I, K, M, C, out, out_rows);
    return check_launch("rows_times_small_kernel");
}
