/*
 * ftl.h -- C ABI of libftl_gb300.so: exact leverage-score sampling from
 * Khatri-Rao products (STS-CP) and the randomized CP-ALS built on it, as
 * sm_103a CUDA kernels.
 *
 * Conventions
 *   - Every entry point returns an int status (FTL_OK == 0).  On failure,
 *     ftl_last_error() returns a thread-local message for the last error.
 *   - Pointers named *_dev are device pointers owned by the caller; nothing
 *     here frees caller memory.  `stream` is a cudaStream_t passed as void*
 *     (NULL = legacy default stream).  Calls are asynchronous on `stream`
 *     unless stated otherwise.
 *   - Matrices are row-major, contiguous.  Node Gram matrices are stored in
 *     one of two layouts (ftl_node_layout tells which, with the position of
 *     every element):
 *       PACKED (FTL_LAYOUT_PACKED; FP64 nodes, FP32 nodes with R <= 16 or
 *       R > 32): the upper triangle, element (a,b), a <= b, at
 *       a*R - a*(a-1)/2 + (b-a); P = R*(R+1)/2 values, zero padded to 16 bytes.
 *       DIAG32 (FTL_LAYOUT_DIAG32; FP32 nodes with 16 < R <= 32): the Gram
 *       zero padded to 32 x 32, stored by wrapped diagonals so that lane a
 *       of a warp reads row a with coalesced loads: G[a][(a+d) mod 32] at
 *       ((d/4)*32 + a)*4 + d%4 for d = 0..15, and G[a][(a+16) mod 32] at
 *       512 + a (those entries twice, once from each end); 544 values.
 *   - Tree node numbering, leaf numbering and the descent arithmetic follow
 *     the reference's PartitionTree exactly (heap order, children 2c+1 and
 *     2c+2, partial deepest level first).
 *
 * Reference interfaces replaced (paths are within vbharadwaj-bk/fast_tensor_leverage):
 *   cpp_ext/partition_tree.hpp, cpp_ext/efficient_krp_sampler.hpp,
 *   cpp_ext/sampler.hpp, cpp_ext/als.hpp, cpp_ext/sort_lookup.hpp,
 *   cpp_ext/sparse_tensor.hpp, cpp_ext/low_rank_tensor.hpp,
 *   exposed to Python by cpp_ext/als_module.cpp and cpp_ext/partition_tree.cpp.
 */
#ifndef FTL_GB300_H
#define FTL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FTL_OK 0
#define FTL_E_ARG 1         /* invalid argument (shape, range, alignment, null) */
#define FTL_E_OOM 2         /* allocation failed */
#define FTL_E_CUDA 3        /* CUDA runtime error (launch or execution) */
#define FTL_E_TIMEOUT 4     /* a bounded device wait ran out */
#define FTL_E_CANCELLED 5   /* request cancelled by the host */
#define FTL_E_UNSUPPORTED 6 /* configuration not compiled in (e.g. R > 128) */

/* Node-Gram precision.  FP64 reproduces the reference's arithmetic (sample
 * indices match it given the same uniforms, up to ties within rounding);
 * FP32 stores node Grams in FP32 and evaluates quadratic forms in FP32 with
 * the running draw offset kept in double-float. */
#define FTL_PREC_FP64 0
#define FTL_PREC_FP32 1
/* Tree-build precisions with FP32 nodes (plans and draws treat these trees
 * as FTL_PREC_FP32).  For F <= R <= 32 the leaf Grams run on the tensor
 * cores (tcgen05, TMA-fed) with FP32 accumulation, from the factor rows split
 * as 3xTF32 (hi*hi + hi*lo + lo*hi, about FP32 accuracy) or rounded to BF16;
 * for larger R they fall back to the FP32 CUDA-core build. */
#define FTL_PREC_TF32X3 2
#define FTL_PREC_BF16 3

#define FTL_MAX_MODES 16
#define FTL_MAX_RANK 128
#define FTL_MAX_PACK 16  /* requests per packed draw launch */

/* Last error message of the calling thread ("" if none). */
const char *ftl_last_error(void);
/* ABI version, bumped on any signature change. */
int ftl_abi_version(void);

/* Page-lock a caller-owned host buffer (cudaHostRegister) so device results
 * can be copied into it by DMA; *registered = 0 (and FTL_OK) when the runtime
 * refuses (e.g. the pages are already registered), which callers treat as
 * "stay pageable".  ftl_host_unregister must run before the buffer is
 * freed.  No counterpart in the reference (its results are written by the
 * CPU). */
int ftl_host_register(void *ptr, size_t bytes, int *registered);
int ftl_host_unregister(void *ptr);

/* ---------------------------------------------------------------- trees */

typedef struct ftl_tree_geom {
    int64_t n;                     /* rows of the matrix the tree covers */
    int64_t F;                     /* rows per leaf block */
    int64_t leaf_count;            /* ceil(n / F) */
    int64_t node_count;            /* 2 * leaf_count - 1 */
    int64_t lfill_level;           /* floor(log2(leaf_count)) */
    int64_t lfill_count;           /* 2^lfill_level */
    int64_t total_levels;
    int64_t nodes_upto_lfill;      /* 2 * lfill_count - 1 */
    int64_t nodes_before_lfill;    /* lfill_count - 1 */
    int64_t complete_level_offset;
} ftl_tree_geom;

/* Tree geometry.  Replaces the PartitionTree constructor,
 * cpp_ext/partition_tree.hpp:83-105 (log2_round_down: cpp_ext/common.h:21-33). */
int ftl_tree_geometry(int64_t n, int64_t F, ftl_tree_geom *out);

/* Node layout of an R-column Gram in precision prec: *layout_out =
 * FTL_LAYOUT_PACKED or FTL_LAYOUT_DIAG32, *stride_out = values per node, and
 * (pos_out, P = R*(R+1)/2 entries, may be NULL) the position inside a node of
 * upper-triangle element number e (row-major order over a <= b).  No
 * counterpart in the reference (it stores full R x R matrices). */
#define FTL_LAYOUT_PACKED 0
#define FTL_LAYOUT_DIAG32 1
int ftl_node_layout(int R, int prec, int *layout_out, int *stride_out, int32_t *pos_out);

/* Bytes of one tree's node array: node_count * node_stride * (8 for FP64, 4 for FP32). */
int ftl_tree_bytes(int64_t n, int64_t F, int R, int prec, size_t *out_bytes);

/* Node arrays (trees, eigen trees) and the computeM workspaces must be
 * 16-byte aligned: nodes are read with 16-byte loads.  Each node occupies
 * node_stride values (ftl_node_layout), zero padded. */

/* Build the node Grams of the tree over U_dev (n x R, FP64): each leaf holds
 * U_blk^T U_blk of its <= F rows, each internal node the sum of its children.
 * G_dev receives node_count * P values of the requested precision.
 * Replaces PartitionTree::build_tree, cpp_ext/partition_tree.hpp:120-170. */
int ftl_tree_build(const double *U_dev, int64_t n, int R, int64_t F, int prec,
                   void *G_dev, void *stream);

/* ftl_tree_build that also writes U32_dev (n x R FP32, may be NULL; not for
 * FP64 trees) = U rounded to FP32, the copy FP32 draws read their leaf blocks
 * from, in the same pass over U.  No counterpart in the reference. */
int ftl_tree_build_ex(const double *U_dev, int64_t n, int R, int64_t F, int prec,
                      void *G_dev, float *U32_dev, void *stream);

/* Device-side status bits of bounded waits that ran out since the last call
 * (bit 0: the tensor-core tree build stopped on a wait), cleared on read.
 * Waits for the device.  No counterpart in the reference. */
int ftl_device_status(uint32_t *status_out);

/* G_dst[node] = G_src[node] o mat (elementwise on the packed upper triangle);
 * mat_dev holds P FP64 values.  G_src may equal G_dst.
 * Replaces PartitionTree::multiply_matrices_against_provided,
 * cpp_ext/partition_tree.hpp:183-194. */
int ftl_tree_scale(const void *G_src_dev, void *G_dst_dev, int64_t node_count, int R,
                   int prec, const double *mat_dev, void *stream);

/* One descent per row of scaled_h_dev (J x R): sample a row of U with
 * probability proportional to (u_row . x)^2, x = scaled_h[i]; write the row
 * index to samples_dev[i] and multiply h_dev[i] by U[row] elementwise.
 * draws_dev holds J uniforms in [0,1).
 * Replaces PartitionTree::PTSample_internal, cpp_ext/partition_tree.hpp:232-405. */
int ftl_tree_sample(const void *G_dev, int prec, const double *U_dev, int64_t n, int R,
                    int64_t F, double *h_dev, const double *scaled_h_dev,
                    uint64_t *samples_dev, const double *draws_dev, int64_t J,
                    void *stream);

/* ------------------------------------------------------ KRP sampler (STS-CP) */

/* Device state of one exact KRP leverage sampler.  The caller allocates every
 * buffer (ftl_krp_plan_sizes gives the sizes) and fills this struct. */
typedef struct ftl_krp_plan {
    int N;                               /* number of factor matrices */
    int R;                               /* columns (rank), 1..FTL_MAX_RANK */
    int64_t J;                           /* samples per draw */
    int prec;                            /* FTL_PREC_* of gram_G and eig_G */
    int64_t dims[FTL_MAX_MODES];         /* rows of each factor */
    const double *U[FTL_MAX_MODES];      /* device factors, dims[k] x R */
    void *gram_G[FTL_MAX_MODES];         /* device Gram trees, F = min(R, dims[k]) */
    void *eig_G;                         /* device, N x (2R-1) x P, prec */
    double *M;                           /* device workspace, (2N+3) x R x R FP64 */
    double *lambda;                      /* device workspace, (N+1) x R FP64 */
    float *pinv32;                       /* device workspace, one FP32 node (FP32 weights) */
    const float *U32[FTL_MAX_MODES];     /* optional, FP32 plans: FP32 copies of U (ftl_factor_shadow);
                                            leaf scans then read these rows; NULL: they read U */
} ftl_krp_plan;

/* FP32 copy of a factor, out[i] = (float)U[i] for i < count.  FP32 draws whose
 * plans carry these copies read the leaf blocks at half the bytes; results
 * are unchanged (the leaf scan rounds the FP64 rows to FP32 anyway).  No
 * counterpart in the reference (its sampler is FP64 only). */
int ftl_factor_shadow(const double *U, int64_t count, float *out, void *stream);

/* Sizes in bytes of the plan's workspaces. */
int ftl_krp_plan_sizes(int N, int R, int prec, size_t *eig_bytes, size_t *M_bytes,
                       size_t *lambda_bytes, size_t *pinv32_bytes);

/* Per-draw set-up for excluded mode j (j >= N: no mode excluded): Hadamard
 * products of the root Grams, FP64 pseudo-inverse and eigendecompositions
 * (Jacobi, on device), eigen-component trees.
 * Replaces EfficientKRPSampler::computeM, cpp_ext/efficient_krp_sampler.hpp:90-194. */
int ftl_krp_compute_m(const ftl_krp_plan *plan, uint32_t j, void *stream);

/* Draw J samples from the KRP of all factors except j: computeM followed by
 * one fused eigen-then-Gram descent per included mode and the weight
 * epilogue w_i = R / (J * h_i^T pinv h_i).
 *   samples_dev : N x J uint64 (row j is left untouched when j < N)
 *   h_dev       : J x R FP64 (sampled KRP rows), may be NULL
 *   weights_dev : J FP64, may be NULL
 *   draws_dev   : 2N x J uniforms (eigen draws of mode k at k*J, Gram draws
 *                 at N*J + k*J, the reference's layout), or NULL to generate
 *                 them in-kernel: uniform #idx = Philox4x32-10(key=seed,
 *                 counter=ctr+idx), idx the same flat index.
 * Replaces EfficientKRPSampler::KRPDrawSamples,
 * cpp_ext/efficient_krp_sampler.hpp:209-268, and compute_DAGAT,
 * cpp_ext/sampler.hpp:94-123. */
int ftl_krp_draw(const ftl_krp_plan *plan, uint32_t j, uint64_t *samples_dev,
                 double *h_dev, double *weights_dev, const double *draws_dev,
                 uint64_t seed, uint64_t ctr, void *stream);

/* The descent part of ftl_krp_draw alone: uses the computeM state left in
 * the plan's workspaces by the last ftl_krp_compute_m for the same j (and
 * unchanged trees).  Lets callers amortise computeM over several batches of
 * J samples. */
int ftl_krp_sample(const ftl_krp_plan *plan, uint32_t j, uint64_t *samples_dev,
                   double *h_dev, double *weights_dev, const double *draws_dev,
                   uint64_t seed, uint64_t ctr, void *stream);

/* Handle form of the sampler (EfficientKRPSampler, efficient_krp_sampler.hpp:
 * 32-75 for the state, :209-268 for KRPDrawSamples) for hosts that are not
 * Python: the handle owns the device factors, Gram trees and workspaces.
 * Unlike the plan-based entry points, create allocates device memory
 * (cudaMalloc) and destroy frees it.
 *   create     : factors zeroed; factor_shadows (FP32 only) keeps FP32 copies
 *                of the factors for the leaf scans (same results).
 *   set_factor : copy factor k (dims[k] x R FP64, row-major, host or device)
 *                and rebuild its tree (Sampler ctor / update_sampler).
 *   update     : rebuild tree k after the caller wrote the device factor
 *                returned by ftl_sampler_factor (EfficientKRPSampler::
 *                update_sampler, :73-75).
 *   draw       : ftl_krp_draw on the handle's plan (KRPDrawSamples).
 *   destroy    : waits for the device, frees everything. */
typedef struct ftl_sampler ftl_sampler;
int ftl_sampler_create(int N, const int64_t *dims, int R, int64_t J, int prec, int factor_shadows,
                       ftl_sampler **out);
int ftl_sampler_set_factor(ftl_sampler *s, int k, const double *U, int U_on_host, void *stream);
int ftl_sampler_update(ftl_sampler *s, int k, void *stream);
int ftl_sampler_factor(const ftl_sampler *s, int k, double **U_dev);
int ftl_sampler_draw(ftl_sampler *s, uint32_t j, uint64_t *samples_dev, double *h_dev,
                     double *weights_dev, const double *draws_dev, uint64_t seed, uint64_t ctr,
                     void *stream);
int ftl_sampler_destroy(ftl_sampler *s);

/* ------------------------------------------------ sparse tensors and CP-ALS */

/* Fiber keys: keys_out[i] = mixed-radix number of the indices of every mode
 * except j (first mode most significant; the product of the other modes'
 * sizes must stay below 2^63), indices cast to uint32 first.  idx element
 * (i, k) is at idx[i*stride_item + k*stride_mode], of type uint64 when
 * idx_is_u64 else uint32 (nnz x N tensor indices: strides N, 1; an N x J
 * sample array: strides 1, J).  The order of the keys is the lexicographic
 * order of the reference's comparators on modes != j.
 * Replaces the comparators of SortIdxLookup, cpp_ext/sort_lookup.hpp:49-59,
 * and of the ALS dedup, cpp_ext/als.hpp:92-117. */
int ftl_fiber_keys(const void *idx_dev, int idx_is_u64, int64_t n, int64_t stride_item,
                   int64_t stride_mode, int N, const int64_t *dims, int j, uint64_t *keys_dev,
                   void *stream);

/* After sorting mode j's keys (perm = the sorting permutation): idxj_out[i] =
 * idx[perm[i]*N + j], vals_out[i] = vals[perm[i]].  Replaces the sorted
 * pointer array of SortIdxLookup, cpp_ext/sort_lookup.hpp:33-60. */
int ftl_sparse_gather(const int64_t *perm_dev, const uint32_t *idx_dev, const double *vals_dev,
                      int64_t nnz, int N, int j, uint32_t *idxj_out, double *vals_out, void *stream);

/* Dedup of J sample keys: unique keys (slot order of a device hash table),
 * the first sample index carrying each (rep) and its multiplicity (cnt);
 * *num_unique_dev receives the count.  Replaces the sort / unique_copy /
 * equal_range dedup of ALS::execute_ds_als_update, cpp_ext/als.hpp:83-153. */
int ftl_dedup_workspace_bytes(int64_t J, size_t *out);
int ftl_dedup(const uint64_t *keys_dev, int64_t J, void *workspace, size_t ws_bytes,
              uint64_t *ukeys_dev, int32_t *urep_dev, int32_t *ucnt_dev,
              int64_t *num_unique_dev, void *stream);

/* gram_out (R x R, FP64) = sum over rows u of s_u lhs[row(u)] lhs[row(u)]^T,
 * row(u) = rowidx ? rowidx[u] : u, s_u = (w ? w[row(u)] : 1) * (cnt ? cnt[u] : 1),
 * u < (n_rows_dev ? *n_rows_dev : n_rows).  Deterministic (fixed-order
 * reduction).  Replaces compute_pinv's Gram, cpp_ext/common.h:271-306, with
 * the sqrt(w) row scaling of cpp_ext/als.hpp:155-160 folded in. */
int ftl_gram_workspace_bytes(int R, size_t *out);
int ftl_weighted_gram(const double *lhs_dev, const int32_t *rowidx_dev, const double *w_dev,
                      const int32_t *cnt_dev, const int64_t *n_rows_dev, int64_t n_rows, int R,
                      void *workspace, size_t ws_bytes, double *gram_out, void *stream);

/* Pseudo-inverse of a symmetric R x R matrix (upper triangle read): keep
 * eigenpair v (ascending) when v >= R - target and lambda_v > tol, target =
 * min(*rank_cap_dev, R) when rank_cap_dev is given, else target_rank.
 * vscratch (R*R FP64) is needed when R > 90.  Replaces compute_pinv_square,
 * cpp_ext/common.h:228-269. */
int ftl_pinv_square(const double *M_dev, int R, int target_rank, const int64_t *rank_cap_dev,
                    double tol, double *out_dev, double *vscratch_dev, void *stream);

/* Sparse MTTKRP through fiber lookup: out (I_j x R) is zeroed, then for every
 * query q < (num_queries_dev ? *num_queries_dev : num_queries): the fiber of
 * nonzeros whose mode-j-excluded key equals query_keys[q] is found by binary
 * search in sorted_keys, and each of its nonzeros adds value * s_q *
 * lhs[row(q)] to out[idx_j], row(q) = query_row ? query_row[q] : q,
 * s_q = (w ? w[row(q)] : 1) * (cnt ? cnt[q] : 1).  Replaces
 * SortIdxLookup::execute_spmm, cpp_ext/sort_lookup.hpp:69-132. */
int ftl_sparse_mttkrp(const uint64_t *sorted_keys, const uint32_t *sorted_idxj,
                      const double *sorted_vals, int64_t nnz, const uint64_t *query_keys,
                      const int32_t *query_row, const double *w, const int32_t *cnt,
                      const int64_t *num_queries_dev, int64_t num_queries, const double *lhs,
                      int R, double *out, int64_t I_j, void *stream);

/* The same MTTKRP grouped by output row: nonzeros sorted by their mode-j
 * index, given as row_idx (that index), row_keys (fiber keys) and row_vals;
 * the queries are the unique fibers ukeys[u] with rows urep[u] and
 * multiplicities ucnt[u], u < (num_unique_dev ? *num_unique_dev :
 * num_unique), as ftl_dedup returns them; each query's nonzeros add
 * value * s_u * lhs[urep[u]] to out[idx_j], s_u = (w ? w[urep[u]] : 1) *
 * (ucnt ? ucnt[u] : 1).  One pass over the nonzeros in fixed chunks
 * (balanced under any row skew), probing a device table of the queries,
 * per-row accumulation, one atomic add per row segment; out (I_j x R) is
 * zeroed first.  Workspace: ftl_mttkrp_rows_workspace_bytes(J, R). */
int ftl_mttkrp_rows_workspace_bytes(int64_t J, int R, size_t *out);
int ftl_sparse_mttkrp_rows(const int32_t *row_idx, const uint64_t *row_keys,
                           const double *row_vals, int64_t nnz, const uint64_t *ukeys,
                           const int32_t *urep, const int32_t *ucnt,
                           const int64_t *num_unique_dev, int64_t num_unique, int64_t J,
                           const double *w, const double *h, int R, void *workspace,
                           size_t ws_bytes, double *out, int64_t I_j, void *stream);

/* U = B pinv row by row (pinv R x R symmetric); all-zero rows of B give zero
 * rows without arithmetic.  Replaces the cblas_dsymm of
 * cpp_ext/als.hpp:189-203. */
int ftl_solve_rows(const double *B_dev, const double *pinv_dev, int64_t I, int R, double *U_dev,
                   void *stream);

/* Handle form of the sparse tensor and of the randomized CP-ALS for hosts
 * that are not Python (SparseTensor + SortIdxLookup, sparse_tensor.hpp:46-77,
 * sort_lookup.hpp:33-60; ALS initialize_ds_als / execute_ds_als_update,
 * als.hpp:39-220; execute_rrf, sparse_tensor.hpp:84-92; the exact fit,
 * sparse_tensor.hpp:117-119 and tensors.py:41-53).  Creating allocates device
 * memory; destroy frees it.
 *   ftl_sparse_create : copies idx (nnz x N uint32, row-major) and vals
 *                       (host or device), sorts the nonzeros by each mode's
 *                       index (stable) with their fiber keys, and computes
 *                       the squared norm (the call waits for the device).
 *   ftl_als_create    : an ALS over the tensor's dims with rank R and J samples
 *                       per update; owns a sampler handle (the factors) and
 *                       every buffer an update needs; sigma starts at ones.
 *   ftl_als_set_factor / set_sigma : initial factors (tree rebuilt) and sigma.
 *   ftl_als_init_rrf  : range-finder factors (execute_rrf), then
 *                       ftl_als_renormalize(-1).
 *   ftl_als_renormalize : column norms of factor j (-1: all), sigma = the
 *                       norms (product over modes for -1), trees rebuilt.
 *   ftl_als_update    : one sampled update of mode j; draws_dev (2N x J
 *                       uniforms) or NULL for the handle's Philox stream.
 *   ftl_als_fit       : 1 - ||X - model|| / ||X|| and ||X - model||^2 (waits). */
typedef struct ftl_sparse ftl_sparse;
typedef struct ftl_als ftl_als;
int ftl_sparse_create(const uint32_t *idx, const double *vals, int64_t nnz, int N, const int64_t *dims,
                      int on_host, void *stream, ftl_sparse **out);
int ftl_sparse_normsq(const ftl_sparse *X, double *out);
int ftl_sparse_destroy(ftl_sparse *X);
int ftl_als_create(const ftl_sparse *X, int R, int64_t J, int prec, uint64_t seed, ftl_als **out);
int ftl_als_set_factor(ftl_als *A, int k, const double *U, int on_host, void *stream);
int ftl_als_set_sigma(ftl_als *A, const double *sigma, int on_host, void *stream);
int ftl_als_factor(const ftl_als *A, int k, double **U_dev);
int ftl_als_sigma(const ftl_als *A, double **sigma_dev);
int ftl_als_samples(const ftl_als *A, uint64_t **samples_dev);
int ftl_als_renormalize(ftl_als *A, int j, void *stream);
int ftl_als_init_rrf(ftl_als *A, uint64_t seed, void *stream);
int ftl_als_update(ftl_als *A, int j, int renormalize, int update_sampler, const double *draws_dev,
                   void *stream);
int ftl_als_fit(ftl_als *A, double *fit, double *residual_normsq, void *stream);
int ftl_als_destroy(ftl_als *A);

/* Column norms of U (I x R) with norms <= 1e-7 replaced by 1, and (apply != 0)
 * U *= 1/norms (the reference divides; this differs by at most one rounding).  Replaces LowRankTensor::renormalize_columns for one factor,
 * cpp_ext/low_rank_tensor.hpp:203-247. */
int ftl_colnorm_workspace_bytes(int R, size_t *out);
int ftl_renormalize_columns(double *U_dev, int64_t I, int R, double *norms_out, void *workspace,
                            size_t ws_bytes, int apply, void *stream);

/* *out = sum over nonzeros of v^2 - 2 v model(idx), model = sum_r sigma_r
 * prod_k U_k[idx_k, r] (the nonzero part of
 * SortIdxLookup::compute_residual_normsq, cpp_ext/sort_lookup.hpp:134-193);
 * U_dev is a host array of N device pointers. */
int ftl_fit_workspace_bytes(size_t *out);
int ftl_sparse_residual_terms(const uint32_t *idx_dev, const double *vals_dev, int64_t nnz, int N,
                              const double *const *U_dev, const double *sigma_dev, int R,
                              void *workspace, size_t ws_bytes, double *out_dev, void *stream);
/* *out = sum of v_i^2 (SparseTensor's normsq, cpp_ext/sparse_tensor.hpp:70-74). */
int ftl_sum_squares(const double *v_dev, int64_t n, void *workspace, size_t ws_bytes,
                    double *out_dev, void *stream);

/* Exact MTTKRP over all nonzeros: out[idx_j] += v prod_{k != j} U_k[idx_k]
 * (out zeroed first).  Replaces SortIdxLookup::execute_exact_mttkrp,
 * cpp_ext/sort_lookup.hpp:199-254. */
int ftl_sparse_exact_mttkrp(const uint32_t *idx_dev, const double *vals_dev, int64_t nnz, int N,
                            int j, const double *const *U_dev, int R, double *out_dev,
                            int64_t I_j, void *stream);

/* Randomized range finder of mode j (SortIdxLookup::execute_rrf,
 * cpp_ext/sort_lookup.hpp:262-353): out (I_j x R, zeroed first) = X_(j) Omega,
 * Omega holding one N(0,1) R-vector per fiber (modes != j).  Inputs are the
 * nonzeros sorted by their mode-j index (row index, fiber key, value, as for
 * ftl_sparse_mttkrp_rows).  The reference draws from unseeded per-thread
 * generators; here fiber f's vector is Philox4x32-10 (counter (f lo, f hi,
 * column pair p, mode), key seed) through Box-Muller in FP32: u1 = ((x0 >> 8)
 * + 1) 2^-24, u2 = (x1 >> 8) 2^-24, columns 2p, 2p+1 = sqrt(-2 ln u1)
 * (cos, sin)(2 pi u2).  Reproducible and independent of the launch shape. */
int ftl_sparse_rrf(const int32_t *row_idx, const uint64_t *row_keys, const double *row_vals, int64_t nnz,
                   int R, uint64_t seed, uint32_t mode, double *out, int64_t I_j, void *stream);

/* ---- black-box right-hand sides (low-rank and dense tensors) --------------
 * The sampled MTTKRP of ALS against a tensor that is not sparse
 * (BlackBoxTensor::execute_downsampled_mttkrp, cpp_ext/black_box_tensor.hpp:21-67):
 * out (rows 0..I_j-1) = sum over unique samples u of fiber_u (x) coef_u h[rep_u],
 * coef_u = w[rep_u] * ucnt[u] (urep/ucnt/w NULL: u itself, 1, 1); rows
 * I_j..out_rows-1 are zeroed.  samples is N x J (mode-major, as ftl_krp_draw
 * writes them); num_unique comes from num_unique_dev when that is not NULL. */

/* Low-rank tensor [[sigma_rhs; V]] (rank Rr): fiber = V_j (sigma o prod V_k[s_k])
 * (LowRankTensor::materialize_rhs, cpp_ext/low_rank_tensor.hpp:91-135), computed
 * as V_j (P^T L) without materialising fibers.  Deterministic. */
int ftl_lowrank_mttkrp_workspace_bytes(int Rr, int R, size_t *out);
int ftl_lowrank_sampled_mttkrp(const double *const *V, const double *sigma_rhs, int N, int Rr, int j,
                               const uint64_t *samples, int64_t J, const int32_t *urep, const int32_t *ucnt,
                               const int64_t *num_unique_dev, int64_t num_unique, const double *w,
                               const double *h, int R, void *workspace, size_t ws_bytes, double *out,
                               int64_t I_j, int64_t out_rows, void *stream);
/* Dense row-major tensor (FP64 or FP32, dims[N]): fiber = T[s_0, .., :, .., s_N-1]
 * (DenseTensor::materialize_rhs, cpp_ext/dense_tensor.hpp:38-59). */
int ftl_dense_sampled_mttkrp(const void *T, int is_f32, const int64_t *dims, int N, int j,
                             const uint64_t *samples, int64_t J, const int32_t *urep, const int32_t *ucnt,
                             const int64_t *num_unique_dev, int64_t num_unique, const double *w,
                             const double *h, int R, double *out, int64_t out_rows, void *stream);
/* out (n x I_j) = the dense tensor's fibers at n samples (n x N, row-major). */
int ftl_dense_materialize(const void *T, int is_f32, const int64_t *dims, int N, int j,
                          const uint64_t *samples, int64_t n, double *out, void *stream);
/* out[0] = sum over all entries of (T - [[sigma; U]])^2 (U NULL: model 0),
 * out[1] = sum of T^2.  The reference's DenseTensor has no residual (its base
 * class returns -1); this is an addition. */
int ftl_dense_residual_workspace_bytes(size_t *out);
int ftl_dense_residual_terms(const void *T, int is_f32, const int64_t *dims, int N, const double *const *U,
                             const double *sigma, int R, void *workspace, size_t ws_bytes, double *out,
                             void *stream);
/* Low-rank tensor at n index tuples (n x N, uint32 or uint64, row-major):
 * out[z] = sum_r sigma_r prod_k U_k[idx(z,k), r]
 * (LowRankTensor::evaluate_indices, cpp_ext/low_rank_tensor.hpp:262-280). */
int ftl_lowrank_evaluate(const double *const *U, int N, int R, const double *sigma, const void *idx,
                         int idx_is_u64, int64_t n, double *out, void *stream);
/* Fibers of a low-rank tensor at n samples (n x N uint64, row-major): j >= N:
 * out (n x R) = sigma o prod_k U_k[s_k]; else out (n x I_j) = that row times
 * U_j^T (LowRankTensor::materialize_rhs, cpp_ext/low_rank_tensor.hpp:91-135). */
int ftl_lowrank_materialize(const double *const *U, int N, int R, const double *sigma, const uint64_t *samples,
                            int64_t n, int j, int64_t I_j, double *out, void *stream);
/* Counter-hash Gaussian noise on a black-box tensor of dims[N] (no
 * counterpart in the reference): Z at the entry with linear (row-major) index
 * L (mod 2^64) is the SplitMix64 finaliser of L * 0x9E3779B97F4A7C15 + seed,
 * z, through Box-Muller in FP32: u1 = ((z >> 40) + 1) 2^-24, u2 = ((z >> 16)
 * mod 2^24) 2^-24, Z = sqrt(-2 ln u1) cos(2 pi u2).  The noisy tensor is
 * X + sigma Z; nothing is stored.
 *   ftl_noise_sampled_mttkrp: out (rows 0..dims[j]-1, R columns) += sigma
 *     sum_u coef_u Z(i, s_u) h[rep_u] over the unique samples, with the
 *     arguments and coefficients of ftl_lowrank_sampled_mttkrp (FP32
 *     accumulation over 512 samples, folded in FP64; deterministic)
 *   ftl_noise_add_at: out[z] += sigma Z(idx_z) at n index tuples (n x N)
 *   ftl_noise_add_fibers: out (n x dims[j]) += the noise fibers at n samples
 *     (n x N uint64 row-major), mode j varying */
int ftl_noise_sampled_mttkrp(const int64_t *dims, int N, int j, uint64_t seed, double sigma,
                             const uint64_t *samples, int64_t J, const int32_t *urep, const int32_t *ucnt,
                             const int64_t *num_unique_dev, int64_t num_unique, const double *w,
                             const double *h, int R, double *out, int64_t out_rows, void *stream);
int ftl_noise_add_at(const int64_t *dims, int N, uint64_t seed, double sigma, const void *idx, int idx_is_u64,
                     int64_t n, double *out, void *stream);
int ftl_noise_add_fibers(const int64_t *dims, int N, uint64_t seed, double sigma, const uint64_t *samples,
                         int64_t n, int j, double *out, void *stream);
/* out (out_rows x C) = X (I x K) M (K x C) in rows 0..I-1, zeros below
 * (the final product of LowRankTensor::execute_exact_mttkrp,
 * cpp_ext/low_rank_tensor.hpp:147-180). */
int ftl_rows_times(const double *X, int64_t I, int K, const double *M, int C, double *out, int64_t out_rows,
                   void *stream);
/* out (Ra x Rb) = A^T B over I rows (FP64, fixed-order two-stage reduction). */
int ftl_cross_gram_workspace_bytes(int Ra, int Rb, size_t *out);
int ftl_cross_gram(const double *A, int Ra, const double *B, int Rb, int64_t I, void *workspace,
                   size_t ws_bytes, double *out, void *stream);
/* M = (sigma_a sigma_b^T) o prod_{k != exclude} grams[k] (each Ra x Rb), and/or
 * the sum of M's entries (ATB_chain_prod / ATB_chain_prod_sum,
 * cpp_ext/common.h:152-226, rectangular). */
int ftl_chain_prod(const double *const *grams, int N, int Ra, int Rb, int exclude, const double *sigma_a,
                   const double *sigma_b, double *out_mat, double *out_sum, void *stream);

/* out_mat (R x R) = (sigma_a sigma_b^T) o prod_{k != exclude} G_k over N full
 * R x R FP64 Grams (host array of device pointers; exclude = -1 for none; a
 * NULL sigma means all ones); out_sum = sum of its entries.  Either output
 * may be NULL.  Replaces ATB_chain_prod / ATB_chain_prod_sum with A = B,
 * cpp_ext/common.h:152-226. */
int ftl_gram_hadamard(const double *const *grams_dev, int N, int R, int exclude,
                      const double *sigma_a, const double *sigma_b, double *out_mat,
                      double *out_sum, void *stream);

/* Size of the device array that ftl_krp_draw_static uses for scratch. */
#define FTL_DRAW_STATIC_SCRATCH_BYTES (8u << 20)

/* ftl_krp_draw for callers that cannot allocate device memory.  No
 * counterpart in the reference (its sampler allocates host buffers freely).
 * Some callers cannot call cudaMalloc: hosts that reserve their whole device
 * budget up front through another runtime (cgo/JNI/FFI integrations), or a
 * request path that must not allocate because cudaMalloc can synchronise the
 * device or fail under memory pressure.  Same inputs and outputs as
 * ftl_krp_draw, without workspaces: the eigen trees, computeM matrices,
 * eigenvalues and FP32 pseudo-inverse live in one static device array of
 * FTL_DRAW_STATIC_SCRATCH_BYTES that every GPU loading the library holds
 * until exit.  Configurations needing more (N x (2R-1) eigen-tree nodes plus
 * (2N+3) x R x R FP64, e.g. beyond N=16 at R=32) return FTL_E_ARG.  The
 * first call on a device looks up the array's address with that device
 * current; make it before any stream capture.  All calls share the array
 * (each clears the part it uses): calls that overlap on the GPU race and
 * must be serialised by the caller.  FP32 draws here read their leaf blocks
 * from the FP64 factors (there is no argument for FP32 factor copies), with
 * the same results as ftl_krp_draw and a slower leaf scan.  Allocates
 * nothing. */
int ftl_krp_draw_static(int N, int R, int64_t J, int prec, const int64_t *dims,
                        const double *const *U_dev, void *const *gram_G_dev, uint32_t j,
                        uint64_t *samples_dev, double *h_dev, double *weights_dev,
                        const double *draws_dev, uint64_t seed, uint64_t ctr, void *stream);

/* The descent of n <= FTL_MAX_PACK draws in ONE launch (continuous batching
 * of concurrent sampling requests).  All plans share R and precision; plan i
 * must have had ftl_krp_compute_m for js[i] ordered before this call on
 * `stream`.  Per request the arguments of ftl_krp_sample (draws[i] may be
 * NULL for the in-kernel Philox stream); each request's results are
 * identical to its own ftl_krp_sample. */
int ftl_krp_sample_packed(const ftl_krp_plan *const *plans, int n, const uint32_t *js,
                          uint64_t *const *samples_dev, double *const *h_dev,
                          double *const *weights_dev, const double *const *draws_dev,
                          const uint64_t *seeds, const uint64_t *ctrs, void *stream);

/* ------------------------------------------------------------ tuning */

/* Kernel variants: some kernels are compiled in several variants with the
 * same results and different launch shapes.  The autotuner times them and
 * records its choice for the current device; launches then use it.  No
 * counterpart in the reference (its tuning knobs are compile flags).
 *   ftl_tune_variants : number of variants of (family, R, prec) and the default
 *   ftl_tune_set      : choose variant v (-1: the default) on the current device
 *   ftl_tune_get      : the variant launches use now
 * FTL_TUNE_DRAW: the FP32 draw on DIAG32 trees (16 < R <= 32); variants 0, 1,
 * 2 descend 1, 2, 3 samples per warp in lockstep with the query weights in
 * registers, variants 3, 4, 5 descend 3, 4, 6 with the weights in shared
 * memory (default 2). */
#define FTL_TUNE_DRAW 0
int ftl_tune_variants(int family, int R, int prec, int *count, int *default_variant);
int ftl_tune_set(int family, int R, int prec, int variant);
int ftl_tune_get(int family, int R, int prec, int *variant);

/* Status block of a controlled packed draw (device memory or host memory the
 * device can access, 8-byte aligned); ftl_krp_sample_packed_ctl clears it on
 * the stream before the launch.  No counterpart in the reference (it has no
 * serving loop). */
typedef struct ftl_pack_status {
    uint64_t start_ns;               /* set by the launch (device global timer) */
    uint32_t status[FTL_MAX_PACK];   /* per request: FTL_OK, FTL_E_CANCELLED or FTL_E_TIMEOUT */
} ftl_pack_status;

/* ftl_krp_sample_packed with serving controls.  cancel[i] (n pointers, the
 * array or any entry may be NULL) points to a flag the host may set while
 * the launch runs (pinned host memory or device memory): request i's
 * remaining samples are then skipped and its status becomes
 * FTL_E_CANCELLED.  budget_ns > 0: once the launch has run that long
 * (device global timer), the remaining samples of every request are skipped
 * and those requests get FTL_E_TIMEOUT.  A request with a non-zero status
 * has incomplete results; the others are identical to ftl_krp_sample_packed.
 * The kernel never waits on the flags: it reads them as it goes (the cancel
 * flag on a warp's first sample of the request and then every 8th) and
 * finishes early; a flag set before the launch stops every sample of its
 * request.  Read the
 * statuses after the stream reaches the end of the launch. */
int ftl_krp_sample_packed_ctl(const ftl_krp_plan *const *plans, int n, const uint32_t *js,
                              uint64_t *const *samples_dev, double *const *h_dev,
                              double *const *weights_dev, const double *const *draws_dev,
                              const uint64_t *seeds, const uint64_t *ctrs,
                              const uint32_t *const *cancel, uint64_t budget_ns,
                              ftl_pack_status *status, void *stream);

/* Fill out_dev[0..n) with the uniforms the in-kernel generator uses
 * (Philox4x32-10, key=seed, counter=ctr+i). */
int ftl_philox_uniforms(double *out_dev, int64_t n, uint64_t seed, uint64_t ctr,
                        void *stream);

/* The same uniforms with the counter read from device memory, which is then
 * advanced by n: out[i] = Philox4x32-10(seed, *ctr_dev + i); *ctr_dev += n.
 * Stream-ordered and free of host arguments that change between calls, so a
 * captured CUDA graph replays with fresh uniforms each time. */
int ftl_philox_uniforms_dev(double *out_dev, int64_t n, uint64_t seed, uint64_t *ctr_dev,
                            void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FTL_GB300_H */
