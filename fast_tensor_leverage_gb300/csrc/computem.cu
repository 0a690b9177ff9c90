// Per-draw set-up of the exact KRP sampler (EfficientKRPSampler::computeM,
// cpp_ext/efficient_krp_sampler.hpp:90-194), on device, in FP64:
//
//   M[k]   = G_k(root) o M[next included mode]      suffix Hadamard products
//   M[0]   = full product over the included modes   (M[1] when j == 0)
//   pinv   = sum_{lambda_v > 1e-8} v v^T / lambda_v  (eigendecomposition of M[0])
//   M[N]   = rows lambda_v^{-1/2} v^T, descending lambda (the reference's
//            reversed, transposed V Lambda^{-1/2})
//   M[k]  o= pinv, then rows sqrt(lambda_v) v^T of its eigendecomposition,
//            ascending lambda (k = 1..N-1, k != j)
//   eigen tree k: leaves w_u w_u^T over the rows w_u of M[offset(k)],
//            internal nodes = child sums, every node then o G_k(root).
//
// The eigensolver is a cyclic parallel-order (round-robin) two-sided Jacobi
// method on a dense symmetric matrix in shared memory, one CTA per matrix,
// rotations skipped when |a_pq| <= 2^-53 sqrt(|a_pp a_qq|) (the relative
// criterion of Demmel and Veselic), eigenpairs sorted ascending as LAPACK's
// dsyev returns them.  Eigenvector signs are irrelevant downstream (only
// outer products v v^T are used).
#include <algorithm>

#include "eig.cuh"

// Mixed precision runs the per-mode eigensolvers in FP32 (1: in FP64, the
// reference's precision; an accuracy diagnostic, slower on GB300's FP64 pipe).
#ifndef FTL_CM_MIXED_EIG_FP64
#define FTL_CM_MIXED_EIG_FP64 0
#endif
// Mixed precision, R <= 32: the per-mode eigensolvers run in one warp
// (one-sided Jacobi in registers) instead of the block-wide two-sided one.
#ifndef FTL_CM_WARP_JACOBI
#define FTL_CM_WARP_JACOBI 1
#endif

namespace ftl {

struct CMParams {
    int N, R, P, prec;
    uint32_t j;               // normalised: j < N excluded, j == N+1 none
    const void *root[FTL_MAX_MODES];  // packed root Gram of each tree (tree precision)
    double *M;                // (N+2) x R x R, then (N+1) x R x R Jacobi scratch
    bool v_global;            // eigenvectors kept in the scratch slots (large R)
    double *lambda;           // (N+1) x R
    float *pinv32;            // P
    void *eig_G;              // N x (2R-1) x P
    DGeom eig;                // geometry of an eigen tree (n = R, F = 1)
};

// Element (a, b) of mode k's root Gram, in the tree's layout and precision.
__device__ __forceinline__ double root_ab(const CMParams &p, int k, int a, int b) {
    if (p.prec == FTL_PREC_FP64) return ((const double *)p.root[k])[node_pos(a, b, p.R, 8)];
    return (double)((const float *)p.root[k])[node_pos(a, b, p.R, 4)];
}

// Shared memory: A (R*R), V (R*R unless kept in global scratch), cs (R+2),
// pq (R+2 ints), order (R ints), flag.
static size_t cm_smem_bytes(int R, bool v_global) {
    return (size_t)((v_global ? 1 : 2) * R * R + R + 2) * sizeof(double) +
           (size_t)(2 * R + 4) * sizeof(int) + 16;
}

__global__ void computem_pinv_kernel(CMParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int R = p.R, RR = R * R, N = p.N, tid = threadIdx.x, nth = blockDim.x;
    double *A = (double *)smem_raw;
    double *V = p.v_global ? p.M + (size_t)(N + 2) * RR : A + RR;
    double *cs = A + (p.v_global ? 1 : 2) * RR;
    int *pq = (int *)(cs + R + 2);
    int *order = pq + R + 2;
    int *flag = order + R;

    // Suffix Hadamard products (full symmetric storage).
    int last = N;  // slot N holds all ones in the reference
    for (int k = N - 1; k >= 0; --k) {
        if ((uint32_t)k == p.j) continue;
        for (int e = tid; e < RR; e += nth) {
            int a = e / R, b = e - a * R;
            double g = root_ab(p, k, a, b);
            double prev = (last == N) ? 1.0 : p.M[(size_t)last * RR + e];
            p.M[(size_t)k * RR + e] = g * prev;
        }
        last = k;
        __syncthreads();
    }
    if (p.j == 0) {
        for (int e = tid; e < RR; e += nth) p.M[e] = p.M[(size_t)RR + e];
        __syncthreads();
    }
    double *status = p.M + cm_status_offset(N, R);  // 1.0: Cholesky path taken
    bool chol = false;
    bool gj = false;  // A holds the swept matrix (sweep-operator path)
    if (p.prec == FTL_PREC_FP32 && !FTL_CM_MIXED_EIG_FP64) {
        // Mixed mode: when every eigenvalue of M[0] exceeds the reference's
        // 1e-8 cut, its pseudo-inverse is the inverse, computed in FP64 by
        // the sweep operator (R <= 32) or from the Cholesky factor, pinv
        // = L^-T L^-1 (larger R).  The cut is certified by ||pinv||_F < 1 /
        // (2e-8): lambda_min = 1 / ||M^-1||_2 >= 1 / ||M^-1||_F > 2e-8.
        // Otherwise (or when a pivot is not positive) the Jacobi path below
        // runs.
        for (int e = tid; e < RR; e += nth) A[e] = p.M[e];
        __syncthreads();
        double *rdiag = cs + 2;  // R doubles of the cs scratch (R + 2 long), cs[0] is used below
        if (R <= 32 && nth * 2 >= R * (R + 1) / 2) {
            // small R: the inverse itself by the sweep operator (upper
            // triangle, -M^-1 on return; no triangular solve)
            gj = true;
            chol = sweep_inverse_spd(A, R, cs + 1, flag);
        } else {
            chol = cholesky_lower(A, R, 0.0, flag, cs + 1);
            if (chol) {
                // V = L^-1 (lower), one column per thread, forward substitution;
                // the diagonal reciprocals first, in parallel, so each column's
                // dependent chain holds multiplications only (an FP64 division is
                // a long dependent sequence on GB300's narrow FP64 pipe)
                for (int i = tid; i < R; i += nth) rdiag[i] = 1.0 / A[i * R + i];
                __syncthreads();
                for (int jc = tid; jc < R; jc += nth) {
                    for (int i = 0; i < R; ++i) {
                        double y = 0.0;
                        if (i >= jc) {
                            double acc = (i == jc) ? 1.0 : 0.0;
                            for (int kk = jc; kk < i; ++kk) acc -= A[i * R + kk] * V[kk * R + jc];
                            y = acc * rdiag[i];
                        }
                        V[i * R + jc] = y;
                    }
                }
                __syncthreads();
            }
        }
        if (chol) {
            if (tid == 0) cs[0] = 0.0;
            __syncthreads();
            double fro = 0.0;
            if (gj) {
                // M^-1 = minus the swept upper triangle, mirrored
                double v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int e = tid + q * nth;
                    v[q] = 0.0;
                    if (e < RR) {
                        const int a = e / R, b = e - a * R;
                        v[q] = -A[min(a, b) * R + max(a, b)];
                        fro += v[q] * v[q];
                    }
                }
                __syncthreads();
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (tid + q * nth < RR) A[tid + q * nth] = v[q];
            } else {
                for (int e = tid; e < RR; e += nth) {
                    int a = e / R, b = e - a * R;
                    int lo = max(a, b);
                    double acc = 0.0;
                    for (int kk = lo; kk < R; ++kk) acc += V[kk * R + a] * V[kk * R + b];
                    A[e] = acc;  // A is free again: the factor is no longer needed after this pass
                    fro += acc * acc;
                }
            }
            for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
            if ((tid & 31) == 0) atomicAdd(cs, fro);
            __syncthreads();
            chol = cs[0] == cs[0] && 4e-16 * cs[0] < 1.0;
            __syncthreads();
        }
    }
    if (tid == 0) *status = chol ? 1.0 : 0.0;
    if (!chol) {
    for (int e = tid; e < RR; e += nth) A[e] = p.M[e];
    __syncthreads();
    jacobi_eigen<double>(A, V, R, cs, pq, flag);
    sort_ascending<double>(A, R, order);
    // W = M[N]: row (R-1-r) = v_r / sqrt(lambda_r) for lambda_r > 1e-8, else 0,
    // r the ascending rank (column R-1-r of the reference's V Lambda^{-1/2}).
    double *W = p.M + (size_t)N * RR;
    for (int e = tid; e < RR; e += nth) {
        int row = e / R, a = e - row * R;
        int r = R - 1 - row;
        int v = order[r];
        double lam = A[v * R + v];
        W[e] = lam > 1e-8 ? V[a * R + v] / sqrt(lam) : 0.0;
    }
    for (int r = tid; r < R; r += nth) p.lambda[r] = A[order[r] * R + order[r]];
    __syncthreads();
    // pinv = W^T W summed over W's rows in order (the reference's dsyrk over
    // the columns of V Lambda^{-1/2}); full symmetric into slot 0, packed FP64
    // into slot N+1, packed FP32 into pinv32.
    for (int e = tid; e < RR; e += nth) {
        int a = e / R, b = e - a * R;
        int lo = min(a, b), hi = max(a, b);
        double acc = 0.0;
        for (int row = 0; row < R; ++row) acc += W[row * R + lo] * W[row * R + hi];
        A[e] = acc;
    }
    __syncthreads();
    }
    double *pinv_packed = p.M + cm_pinv64_offset(N, R);
    for (int e = tid; e < RR; e += nth) {
        p.M[e] = A[e];
        int a = e / R, b = e - a * R;
        if (a <= b) pinv_packed[packed_index(a, b, R)] = A[e];
    }
    // zero padding up to the node stride, read by the vectorised forms
    for (int e = p.P + tid; e < node_stride(R, 8); e += nth) pinv_packed[e] = 0.0;
    // FP32 copy in the FP32 node layout (the weights of FP32 draws)
    if (node_layout(R, 4) == FTL_LAYOUT_DIAG32) {
        for (int e = tid; e < kDiag32Stride; e += nth) {
            int a, b;
            diag32_entry(e, a, b);
            p.pinv32[e] = (a < R && b < R) ? (float)A[a * R + b] : 0.0f;
        }
    } else {
        for (int e = tid; e < node_stride(R, 4); e += nth) {
            float v = 0.0f;
            if (e < p.P) {
                int a = 0, rem = e;
                while (rem >= R - a) {
                    rem -= R - a;
                    ++a;
                }
                v = (float)A[a * R + a + rem];
            }
            p.pinv32[e] = v;
        }
    }
    // M[k] o= pinv for k = N-1 .. 1, k != j
    for (int k = N - 1; k >= 1; --k) {
        if ((uint32_t)k == p.j) continue;
        for (int e = tid; e < RR; e += nth) p.M[(size_t)k * RR + e] *= A[e];
    }
}

#ifndef FTL_CM_THREADS
#define FTL_CM_THREADS 512
#endif

template <typename T>
__global__ void __launch_bounds__(FTL_CM_THREADS) computem_eig_kernel(CMParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int R = p.R, RR = R * R, N = p.N, P = p.P, tid = threadIdx.x, nth = blockDim.x;
    const int k = blockIdx.x;
    if ((uint32_t)k == p.j || k >= N) return;
    double *A = (double *)smem_raw;
    double *V = p.v_global ? p.M + (size_t)(N + 3 + k) * RR : A + RR;
    double *cs = A + (p.v_global ? 1 : 2) * RR;
    int *pq = (int *)(cs + R + 2);
    int *order = pq + R + 2;
    int *flag = order + R;
    const int offset = ((uint32_t)(k + 1) == p.j) ? k + 2 : k + 1;
    double *W = p.M + (size_t)offset * RR;
    const bool chol = p.M[cm_status_offset(N, R)] == 1.0;
    if (p.prec == FTL_PREC_FP32 && !FTL_CM_MIXED_EIG_FP64 && (offset < N || chol)) {
        // Mixed mode: FP32 Jacobi of M[offset] (offset < N), or of the FP64
        // pseudo-inverse when it came from the Cholesky path (offset == N;
        // its eigenvectors are those of M[0], its eigenvalues 1/lambda, so
        // ascending order here is the reference's descending-lambda order of
        // the rows lambda^-1/2 v^T).  Rows sqrt(mu_r) v_r, ascending mu_r.
        float *A32 = (float *)smem_raw;
        float *V32 = A32 + RR;
        float *cs32 = V32 + RR;
        int *pq32 = (int *)(cs32 + R + 2);
        int *order32 = pq32 + R + 2;
        int *flag32 = order32 + R;
        const double *src = offset < N ? W : p.M;  // M[0] holds the full pseudo-inverse
        // scale by 2^k (k even, exact) so the largest entry is near 1: the
        // FP32 copy and its squares stay inside the FP32 range whatever the
        // scale of the Grams (products of N Grams of 10^9-sized entries)
        if (tid == 0) *flag32 = 0;
        __syncthreads();
        int emax = 0;
        for (int e = tid; e < RR; e += nth) emax = max(emax, (int)(((unsigned)__double2hiint(src[e]) >> 20) & 0x7ffu));
        atomicMax(flag32, emax);
        __syncthreads();
        const int eb = *flag32;
        int k = (eb >= 1 && eb <= 2045) ? 1023 - eb : 0;
        k -= (k & 1);  // even: the square roots scale back exactly
        __syncthreads();
        const double sc = ldexp(1.0, k);
        for (int e = tid; e < RR; e += nth) A32[e] = (float)(src[e] * sc);
        __syncthreads();
        if (R <= 32 && FTL_CM_WARP_JACOBI) {
            // the PSD matrix by one warp (one-sided Jacobi in registers)
            if (tid < 32) warp_jacobi_psd32(A32, R, k, W, p.lambda + (size_t)offset * R, tid);
        } else {
            jacobi_eigen<float>(A32, V32, R, cs32, pq32, flag32);
            sort_ascending<float>(A32, R, order32);
            const double wsc = ldexp(1.0, -k / 2), lsc = ldexp(1.0, -k);
            for (int e = tid; e < RR; e += nth) {
                int r = e / R, a = e - r * R;
                int v = order32[r];
                float lam = A32[v * R + v];
                W[e] = (double)(sqrtf(fmaxf(lam, 0.0f)) * V32[a * R + v]) * wsc;
            }
            for (int r = tid; r < R; r += nth)
                p.lambda[(size_t)offset * R + r] = (double)A32[order32[r] * R + order32[r]] * lsc;
        }
        __syncthreads();
    } else if (offset < N) {
        for (int e = tid; e < RR; e += nth) A[e] = W[e];
        __syncthreads();
        jacobi_eigen<double>(A, V, R, cs, pq, flag);
        sort_ascending<double>(A, R, order);
        // row r = sqrt(lambda_r) v_r, ascending (negative rounding noise -> 0)
        for (int e = tid; e < RR; e += nth) {
            int r = e / R, a = e - r * R;
            int v = order[r];
            double lam = A[v * R + v];
            W[e] = sqrt(fmax(lam, 0.0)) * V[a * R + v];
        }
        for (int r = tid; r < R; r += nth) p.lambda[(size_t)offset * R + r] = A[order[r] * R + order[r]];
        __syncthreads();
    }
    // Eigen tree over the R rows of W (F = 1): leaves, child sums, then o root.
    const int S = node_stride(R, sizeof(T));
    T *G = (T *)p.eig_G + (size_t)k * (2 * R - 1) * S;
    const DGeom g = p.eig;
    if constexpr (sizeof(T) == 4) {
        if (R <= 32) {
            // FP32 trees, R <= 32: each thread owns node positions e and builds
            // the whole tree at e in registers -- leaves (nodes R-1 .. 2R-2),
            // then every internal node c = R-2 .. 0 as left + right (the same
            // sums as level by level), then o root -- with no barrier and no
            // re-reads of the tree.  Register indices are compile-time: the
            // loops run over the 63 heap positions of R = 32 with predicates.
            const T *root = (const T *)p.root[k];
            // the eigenvector rows rounded to FP32 once, in shared memory (free
            // again after the eigensolve): a conversion per use would run on
            // the FP64 pipe
            float *W32 = (float *)smem_raw;
            __syncthreads();
            for (int e = tid; e < RR; e += nth) W32[e] = (float)W[e];
            __syncthreads();
            for (int e = tid; e < S; e += nth) {
                int a = 0, b = 0;
                bool valid;
                if (node_layout(R, 4) == FTL_LAYOUT_DIAG32) {
                    diag32_entry(e, a, b);
                    valid = a < R && b < R;
                } else {
                    valid = e < P;
                    int rem = e;
                    while (valid && rem >= R - a) {
                        rem -= R - a;
                        ++a;
                    }
                    b = a + rem;
                }
                T v[63];
#pragma unroll
                for (int c = 62; c >= 0; --c) {
                    if (c >= 2 * R - 1) {
                        v[c] = T(0);
                    } else if (c >= R - 1) {
                        const int u = (int)leaf_index(g, c);
                        v[c] = valid ? W32[u * R + a] * W32[u * R + b] : T(0);
                    } else {
                        v[c] = v[c <= 30 ? 2 * c + 1 : 62] + v[c <= 30 ? 2 * c + 2 : 62];
                    }
                }
                const T rt = root[e];
#pragma unroll
                for (int c = 0; c < 63; ++c)
                    if (c < 2 * R - 1) G[c * S + e] = v[c] * rt;
            }
            return;
        }
    }
    // (an eigen tree has 2R - 1 <= 255 nodes of S <= 8256 values: 32-bit indexing)
    const int leaf_count = R;
    if (node_layout(R, sizeof(T)) == FTL_LAYOUT_DIAG32) {
        // leaves: one work item per (leaf u, node position e)
        for (int w = tid; w < leaf_count * S; w += nth) {
            const int u = w / S, e = w - u * S;
            int a, b;
            diag32_entry(e, a, b);
            G[(int)leaf_node(g, u) * S + e] = (a < R && b < R) ? (T)W[u * R + a] * (T)W[u * R + b] : T(0);
        }
    } else {
        // leaves: one work item per (leaf u, packed row a), the row's entries
        // b = a..R-1 contiguous in the packed layout; then the node padding
        for (int w = tid; w < leaf_count * R; w += nth) {
            const int u = w / R, a = w - u * R;
            T *row = G + (int)leaf_node(g, u) * S + packed_row_offset(a, R);
            const T wa = (T)W[u * R + a];
            for (int b = a; b < R; ++b) row[b - a] = wa * (T)W[u * R + b];
        }
        for (int w = tid; w < leaf_count * (S - P); w += nth) {
            const int u = w / (S - P);
            G[(int)leaf_node(g, u) * S + P + (w - u * (S - P))] = T(0);
        }
    }
    __syncthreads();
    int start = (int)(g.nodes_upto_lfill - ((g.nodes_upto_lfill + 1) / 2));  // nodes_before_lfill
    int end = (int)(g.node_count - leaf_count);
    while (true) {
        for (int e = tid; e < (end - start) * S; e += nth) {
            const int cc = e / S;
            const int c = start + cc, pe = e - cc * S;
            G[c * S + pe] = G[(2 * c + 1) * S + pe] + G[(2 * c + 2) * S + pe];
        }
        __syncthreads();
        if (start <= 0) break;
        end = start;
        start = (start + 1) / 2 - 1;
    }
    // o root, position by position (the root Gram is stored in the same
    // layout and precision; padding is zero in both)
    const T *root = (const T *)p.root[k];
    for (int e = tid; e < (2 * R - 1) * S; e += nth) G[e] = G[e] * root[e % S];
}

#ifndef FTL_CM_THREADS
#define FTL_CM_THREADS 512
#endif

int computem_launch(const ftl_krp_plan *plan, uint32_t j_norm, cudaStream_t st) {
    CMParams p;
    p.N = plan->N;
    p.R = plan->R;
    p.P = packed_size(plan->R);
    p.prec = plan->prec;
    p.j = j_norm;
    for (int k = 0; k < FTL_MAX_MODES; ++k) p.root[k] = k < plan->N ? plan->gram_G[k] : nullptr;
    p.M = plan->M;
    p.lambda = plan->lambda;
    p.pinv32 = plan->pinv32;
    p.eig_G = plan->eig_G;
    p.eig = to_dgeom(make_geom(plan->R, 1));
    p.v_global = cm_smem_bytes(plan->R, false) > 200 * 1024;
    size_t smem = cm_smem_bytes(plan->R, p.v_global);
    if (smem > 227 * 1024) return fail(FTL_E_UNSUPPORTED, "computeM: R=%d too large", plan->R);
    int rc = ensure_smem((const void *)computem_pinv_kernel, smem, "computem_pinv_kernel");
    if (!rc)
        rc = plan->prec == FTL_PREC_FP64
                 ? ensure_smem((const void *)computem_eig_kernel<double>, smem, "computem_eig_kernel")
                 : ensure_smem((const void *)computem_eig_kernel<float>, smem, "computem_eig_kernel");
    if (rc) return rc;
    computem_pinv_kernel<<<1, FTL_CM_THREADS, smem, st>>>(p);
    rc = check_launch("computem_pinv_kernel");
    if (rc) return rc;
    if (plan->prec == FTL_PREC_FP64)
        computem_eig_kernel<double><<<plan->N, FTL_CM_THREADS, smem, st>>>(p);
    else
        computem_eig_kernel<float><<<plan->N, FTL_CM_THREADS, smem, st>>>(p);
    return check_launch("computem_eig_kernel");
}

}  // namespace ftl
