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
 *   - Matrices are row-major, contiguous.  Node Gram matrices are stored as
 *     packed upper triangles: element (a,b), a <= b, of an R x R Gram lives
 *     at a*R - a*(a-1)/2 + (b-a); P = R*(R+1)/2 values per node.
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

#define FTL_MAX_MODES 16
#define FTL_MAX_RANK 128

/* Last error message of the calling thread ("" if none). */
const char *ftl_last_error(void);
/* ABI version, bumped on any signature change. */
int ftl_abi_version(void);

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

/* Bytes of one tree's node array: node_count * P * (8 for FP64, 4 for FP32). */
int ftl_tree_bytes(int64_t n, int64_t F, int R, int prec, size_t *out_bytes);

/* Build the node Grams of the tree over U_dev (n x R, FP64): each leaf holds
 * U_blk^T U_blk of its <= F rows, each internal node the sum of its children.
 * G_dev receives node_count * P values of the requested precision.
 * Replaces PartitionTree::build_tree, cpp_ext/partition_tree.hpp:120-170. */
int ftl_tree_build(const double *U_dev, int64_t n, int R, int64_t F, int prec,
                   void *G_dev, void *stream);

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
    float *pinv32;                       /* device workspace, P FP32 (FP32 weights) */
} ftl_krp_plan;

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
 * until exit.  Configurations needing more (N x (2R-1) x P tree values plus
 * (2N+3) x R x R FP64, e.g. beyond N=16 at R=32) return FTL_E_ARG.  The
 * first call on a device looks up the array's address with that device
 * current; make it before any stream capture.  All calls share the array
 * (each clears the part it uses): calls that overlap on the GPU race and
 * must be serialised by the caller.  Allocates nothing. */
int ftl_krp_draw_static(int N, int R, int64_t J, int prec, const int64_t *dims,
                        const double *const *U_dev, void *const *gram_G_dev, uint32_t j,
                        uint64_t *samples_dev, double *h_dev, double *weights_dev,
                        const double *draws_dev, uint64_t seed, uint64_t ctr, void *stream);

/* Fill out_dev[0..n) with the uniforms the in-kernel generator uses
 * (Philox4x32-10, key=seed, counter=ctr+i). */
int ftl_philox_uniforms(double *out_dev, int64_t n, uint64_t seed, uint64_t ctr,
                        void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FTL_GB300_H */
