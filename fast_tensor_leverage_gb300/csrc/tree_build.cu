// Partition-tree construction: leaf block Grams U_blk^T U_blk and the
// level-by-level child sums, stored as packed upper triangles in heap order.
//
// Semantics follow PartitionTree::build_tree (cpp_ext/partition_tree.hpp:120-170):
// leaf block `b` covers rows [b*F, min((b+1)*F, n)), sits at heap position
// leaf_node(b), and every internal node is the elementwise sum of its two
// children (parent = left + right, the reference's association).
//
// Work layout: one CTA loads LB leaf blocks into shared memory (converted to
// the tree precision, columns zero-padded to a multiple of 4), then each
// thread accumulates one 4x4 tile of the upper triangle of one block's Gram
// over the block's rows (2 vector shared loads per 16 FMAs) and writes its
// packed elements.  The HBM traffic is the read of U plus the write of the
// leaf Grams; the internal levels are a second, purely elementwise pass.
#include <algorithm>
#include <cstdio>
#include <type_traits>

#include "ftl_common.cuh"

namespace ftl {

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
    using type = float4;
};
template <>
struct Vec4<double> {
    using type = double4_32a;
};

template <typename T>
__device__ __forceinline__ T to_tree(double x) {
    if constexpr (sizeof(T) == 4) return d2f_rn(x);
    else return x;
}

template <typename T>
__global__ void __launch_bounds__(256) leaf_gram_kernel(const double *__restrict__ U, int64_t n,
                                                        int R, int RP, DGeom g, int LB,
                                                        T *__restrict__ G, float *__restrict__ U32) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    T *Us = reinterpret_cast<T *>(smem_raw);  // LB x F x RP
    const int64_t F = g.F;
    const int P = packed_size(R);
    const int S = node_stride(R, sizeof(T));
    const int nt = RP / 4;
    const int tiles = nt * (nt + 1) / 2;
    const int64_t leaf_count = (n + F - 1) / F;
    const int64_t nbatch = (leaf_count + LB - 1) / LB;
    const int64_t blk_elems = F * RP;

    for (int64_t batch = blockIdx.x; batch < nbatch; batch += gridDim.x) {
        const int64_t leaf0 = batch * LB;
        // Stage LB blocks (rows past n and columns past R are zero).  The LB
        // blocks are LB * F consecutive rows of U, copied one row per warp.
        const int64_t row0 = leaf0 * F;
        const int nrows = LB * (int)F;
        const int lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
        if (R == 32 && RP == 32 && ((uintptr_t)U & 15u) == 0 && ((uintptr_t)U32 & 7u) == 0) {
            // 32 columns: a half warp per row, two columns per lane (16-byte
            // loads, 8-byte copy stores): half the instructions per value
            const int col = 2 * (lane & 15);
#pragma unroll 4
            for (int rr = 2 * (threadIdx.x >> 5) + (lane >> 4); rr < nrows; rr += 2 * nwarps) {
                const int64_t row = row0 + rr;
                T v0 = T(0), v1 = T(0);
                if (row < n) {
                    const double2 x = *reinterpret_cast<const double2 *>(U + row * 32 + col);
                    v0 = to_tree<T>(x.x);
                    v1 = to_tree<T>(x.y);
                    if (sizeof(T) == 4 && U32)
                        *reinterpret_cast<float2 *>(U32 + row * 32 + col) = make_float2((float)v0, (float)v1);
                }
                Us[rr * 32 + col] = v0;
                Us[rr * 32 + col + 1] = v1;
            }
        } else {
#pragma unroll 4
            for (int rr = threadIdx.x >> 5; rr < nrows; rr += nwarps) {
                const int64_t row = row0 + rr;
                for (int col = lane; col < RP; col += 32) {
                    T v = T(0);
                    if (row < n && col < R) {
                        v = to_tree<T>(U[row * R + col]);
                        if (sizeof(T) == 4 && U32) U32[row * R + col] = (float)v;  // the FP32 copy, same pass
                    }
                    Us[rr * RP + col] = v;
                }
            }
        }
        __syncthreads();
        const int lay = node_layout(R, sizeof(T));
        if (lay == FTL_LAYOUT_DIAG32 && R < 32) {
            // entries of the 32 x 32 padding outside the R x R Gram are zero
            for (int w = threadIdx.x; w < LB * S; w += blockDim.x) {
                const int lb = w / S, e = w - lb * S;
                const int64_t leaf = leaf0 + lb;
                int a, b;
                diag32_entry(e, a, b);
                if (leaf < leaf_count && (a >= R || b >= R)) G[leaf_node(g, leaf) * (int64_t)S + e] = T(0);
            }
        }
        const int work = LB * tiles;
        for (int w = threadIdx.x; w < work; w += blockDim.x) {
            int lb = w / tiles;
            int tile = w - lb * tiles;
            int64_t leaf = leaf0 + lb;
            if (leaf >= leaf_count) continue;
            // tile -> (ta, tb), ta <= tb, row-major over the upper triangle
            int ta = 0, rem = tile;
            while (rem >= nt - ta) {
                rem -= nt - ta;
                ++ta;
            }
            int tb = ta + rem;
            T acc[4][4];
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) acc[x][y] = T(0);
            const T *base = Us + (int64_t)lb * blk_elems;
            for (int64_t r = 0; r < F; ++r) {
                typename Vec4<T>::type va =
                    *reinterpret_cast<const typename Vec4<T>::type *>(base + r * RP + 4 * ta);
                typename Vec4<T>::type vb =
                    *reinterpret_cast<const typename Vec4<T>::type *>(base + r * RP + 4 * tb);
                T a4[4] = {va.x, va.y, va.z, va.w};
                T b4[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
                for (int x = 0; x < 4; ++x)
#pragma unroll
                    for (int y = 0; y < 4; ++y) acc[x][y] = fma(a4[x], b4[y], acc[x][y]);
            }
            T *Gn = G + leaf_node(g, leaf) * (int64_t)S;
            if (tile == 0 && lay == FTL_LAYOUT_PACKED)
                for (int e = P; e < S; ++e) Gn[e] = T(0);
#pragma unroll
            for (int x = 0; x < 4; ++x) {
                int a = 4 * ta + x;
                if (a >= R) continue;
#pragma unroll
                for (int y = 0; y < 4; ++y) {
                    int b = 4 * tb + y;
                    if (b < a || b >= R) continue;
                    if (lay == FTL_LAYOUT_DIAG32) {
                        Gn[diag32_pos(a, b)] = acc[x][y];
                        if (((b - a) & 31) == 16) Gn[512 + b] = acc[x][y];  // the second copy
                    } else {
                        Gn[packed_index(a, b, R)] = acc[x][y];
                    }
                }
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ float4 vadd(float4 a, float4 b) {
    return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ double2 vadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// G[c] = G[2c+1] + G[2c+2] for c in [start, end) (S = node stride; the
// zero padding sums to zero), in 16-byte vectors (a node stride is a whole
// number of them); V = the vector type, S16 = vectors per node, I = the
// index type (32-bit when the level fits).
template <typename V, typename I>
__global__ void level_sum_kernel(V *__restrict__ G, int64_t start, int64_t end, int S16) {
    const I total = (I)((end - start) * S16);
    for (I e = (I)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (I)gridDim.x * blockDim.x) {
        const I cc = e / (I)S16;
        const int k = (int)(e - cc * (I)S16);
        const int64_t c = start + (int64_t)cc;
        const V a = G[(2 * c + 1) * S16 + k], b = G[(2 * c + 2) * S16 + k];
        G[c * S16 + k] = vadd(a, b);
    }
}

// H complete levels in one pass: for each node a of the top level (heap
// indices [top_start, top_start + top_count)) and vector component k, the
// 2^H descendants of a at depth H (already built) are loaded, then summed
// pairwise bottom-up, writing every node of a's subtree above them (the same
// parent = left + right association as level_sum_kernel).
template <typename V, int H>
__global__ void __launch_bounds__(256) levels_fused_kernel(V *__restrict__ G, int64_t top_start, int64_t top_count,
                                                           int S16) {
    const int64_t total = top_count * S16;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = top_start + e / S16;
        const int k = (int)(e % S16);
        V x[1 << H];
        const int64_t base = ((a + 1) << H) - 1;  // first descendant at depth H
#pragma unroll
        for (int i = 0; i < (1 << H); ++i) x[i] = G[(base + i) * S16 + k];
#pragma unroll
        for (int m = 1; m <= H; ++m) {
            // nodes at height m above depth H: 2^(H-m) of them
            const int64_t first = ((a + 1) << (H - m)) - 1;
#pragma unroll
            for (int i = 0; i < (1 << (H - m)); ++i) {
                x[i] = vadd(x[2 * i], x[2 * i + 1]);
                G[(first + i) * S16 + k] = x[i];
            }
        }
    }
}

template <typename V, int H>
static void launch_fused(V *G, int64_t top_start, int64_t top_count, int S16, cudaStream_t st) {
    const int64_t total = top_count * S16;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
    levels_fused_kernel<V, H><<<std::max(blocks, 1), 256, 0, st>>>(G, top_start, top_count, S16);
}

template <typename T>
__global__ void tree_scale_kernel(const T *__restrict__ src, T *__restrict__ dst, int64_t total,
                                  int R, int P, int S, const double *__restrict__ mat) {
    const bool diag = node_layout(R, sizeof(T)) == FTL_LAYOUT_DIAG32;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int k = (int)(e % S);
        if (diag) {
            int a, b;
            diag32_entry(k, a, b);
            dst[e] = (a < R && b < R) ? (T)((double)src[e] * mat[packed_index(min(a, b), max(a, b), R)]) : T(0);
        } else {
            dst[e] = k < P ? (T)((double)src[e] * mat[k]) : T(0);
        }
    }
}


int tc_leaf_grams(const double *U, int64_t n, int R, int64_t F, int mode, float *G, float *U32, cudaStream_t st);

template <typename T>
static int build_internal(const Geom &geom, int R, T *G, cudaStream_t st);

// prec: FTL_PREC_FP64 (T = double) or one of the FP32-node precisions.
template <typename T>
static int build_impl(const double *U, int64_t n, int R, int64_t F, int prec, T *G, float *U32, cudaStream_t st) {
    Geom geom = make_geom(n, F);
    DGeom g = to_dgeom(geom);
    int rc = FTL_OK;
    if (sizeof(T) == 4 && (prec == FTL_PREC_TF32X3 || prec == FTL_PREC_BF16) && F <= R && R <= 32 &&
        n < ((int64_t)1 << 31)) {
        rc = tc_leaf_grams(U, n, R, F, prec == FTL_PREC_TF32X3 ? 0 : 1, (float *)G, U32, st);
        if (rc) return rc;
        return build_internal<T>(geom, R, G, st);
    }
    const int P = packed_size(R);
    const int RP = (R + 3) / 4 * 4;
    const size_t blk_bytes = (size_t)F * RP * sizeof(T);
    const int nt = RP / 4;
    const int tiles = nt * (nt + 1) / 2;
    // Leaves per CTA: fill the 256 threads with 4x4 tiles, bounded by shared memory.
    int LB = std::max(1, 256 / tiles);
    while (LB > 1 && (size_t)LB * blk_bytes > 112u * 1024u) --LB;
    size_t smem = (size_t)LB * blk_bytes;
    if (smem > 227 * 1024)
        return fail(FTL_E_UNSUPPORTED, "tree_build: leaf block of %lld x %d needs %zu B of shared memory",
                    (long long)F, R, smem);
    rc = ensure_smem((const void *)leaf_gram_kernel<T>, smem, "leaf_gram_kernel");
    if (rc) return rc;
    int64_t nbatch = (geom.leaf_count + LB - 1) / LB;
    // one wave of resident CTAs, each looping over batches: a grid larger
    // than what fits at once leaves a partial second wave
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, leaf_gram_kernel<T>, 256, smem) != cudaSuccess || occ < 1)
        occ = 1;
    int grid = (int)std::min<int64_t>(nbatch, (int64_t)num_sms() * occ);
    leaf_gram_kernel<T><<<grid, 256, smem, st>>>(U, n, R, RP, g, LB, G, U32);
    rc = check_launch("leaf_gram_kernel");
    if (rc) return rc;
    return build_internal<T>(geom, R, G, st);
}

// Internal nodes of a tree whose leaves are built: parent = left + right.
template <typename T>
static int build_internal(const Geom &geom, int R, T *G, cudaStream_t st) {
    int rc = FTL_OK;
    using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    const int S16 = node_stride(R, sizeof(T)) * (int)sizeof(T) / 16;
    // internal nodes of the partial level (children: leaves of the last level)
    const int64_t start = geom.nodes_before_lfill;
    const int64_t end = geom.node_count - geom.leaf_count;
    if (end > start) {
        const int64_t total = (end - start) * (int64_t)S16;
        const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
        if (total < (int64_t)INT32_MAX)
            level_sum_kernel<V, uint32_t><<<blocks, 256, 0, st>>>((V *)G, start, end, S16);
        else
            level_sum_kernel<V, int64_t><<<blocks, 256, 0, st>>>((V *)G, start, end, S16);
        rc = check_launch("level_sum_kernel");
        if (rc) return rc;
    }
    // the complete levels lfill_level - 1 .. 0 (level d = heap [2^d - 1,
    // 2^(d+1) - 1)), four at a time from the bottom
    for (int64_t d = geom.lfill_level - 1; d >= 0;) {
        const int h = (int)std::min<int64_t>(4, d + 1);
        const int64_t top = d - h + 1;
        const int64_t top_start = (int64_t(1) << top) - 1, top_count = int64_t(1) << top;
        if (h == 4)
            launch_fused<V, 4>((V *)G, top_start, top_count, S16, st);
        else if (h == 3)
            launch_fused<V, 3>((V *)G, top_start, top_count, S16, st);
        else if (h == 2)
            launch_fused<V, 2>((V *)G, top_start, top_count, S16, st);
        else
            launch_fused<V, 1>((V *)G, top_start, top_count, S16, st);
        rc = check_launch("levels_fused_kernel");
        if (rc) return rc;
        d = top - 1;
    }
    return FTL_OK;
}

}  // namespace ftl

using namespace ftl;

extern "C" int ftl_tree_geometry(int64_t n, int64_t F, ftl_tree_geom *out) {
    FTL_CHECK_ARG(out != nullptr, "ftl_tree_geometry: out is NULL");
    FTL_CHECK_ARG(n >= 1 && F >= 1, "ftl_tree_geometry: need n >= 1 and F >= 1 (got n=%lld F=%lld)",
                  (long long)n, (long long)F);
    Geom g = make_geom(n, F);
    out->n = g.n;
    out->F = g.F;
    out->leaf_count = g.leaf_count;
    out->node_count = g.node_count;
    out->lfill_level = g.lfill_level;
    out->lfill_count = g.lfill_count;
    out->total_levels = g.total_levels;
    out->nodes_upto_lfill = g.nodes_upto_lfill;
    out->nodes_before_lfill = g.nodes_before_lfill;
    out->complete_level_offset = g.complete_level_offset;
    return FTL_OK;
}

extern "C" int ftl_node_layout(int R, int prec, int *layout_out, int *stride_out, int32_t *pos_out) {
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK, "ftl_node_layout: R=%d outside [1, %d]", R, FTL_MAX_RANK);
    FTL_CHECK_ARG(valid_prec(prec), "ftl_node_layout: bad precision %d", prec);
    const int esize = prec_bytes(prec);
    if (layout_out) *layout_out = node_layout(R, esize);
    if (stride_out) *stride_out = node_stride(R, esize);
    if (pos_out) {
        int e = 0;
        for (int a = 0; a < R; ++a)
            for (int b = a; b < R; ++b) pos_out[e++] = node_pos(a, b, R, esize);
    }
    return FTL_OK;
}

extern "C" int ftl_tree_bytes(int64_t n, int64_t F, int R, int prec, size_t *out_bytes) {
    FTL_CHECK_ARG(out_bytes != nullptr, "ftl_tree_bytes: out_bytes is NULL");
    FTL_CHECK_ARG(n >= 1 && F >= 1 && R >= 1 && R <= FTL_MAX_RANK,
                  "ftl_tree_bytes: bad shape n=%lld F=%lld R=%d", (long long)n, (long long)F, R);
    FTL_CHECK_ARG(valid_prec(prec), "ftl_tree_bytes: bad precision %d", prec);
    Geom g = make_geom(n, F);
    const int esize = prec_bytes(prec);
    *out_bytes = (size_t)g.node_count * node_stride(R, esize) * esize;
    return FTL_OK;
}

extern "C" int ftl_tree_build_ex(const double *U, int64_t n, int R, int64_t F, int prec, void *G, float *U32,
                                 void *stream) {
    FTL_CHECK_ARG(U != nullptr && G != nullptr, "ftl_tree_build: null pointer");
    FTL_CHECK_ARG(n >= 1 && F >= 1 && R >= 1 && R <= FTL_MAX_RANK,
                  "ftl_tree_build: bad shape n=%lld F=%lld R=%d", (long long)n, (long long)F, R);
    FTL_CHECK_ARG(F <= FTL_MAX_RANK, "ftl_tree_build: F=%lld exceeds %d", (long long)F, FTL_MAX_RANK);
    FTL_CHECK_ARG(aligned16(G), "ftl_tree_build: the tree must be 16-byte aligned");
    FTL_CHECK_ARG(valid_prec(prec), "ftl_tree_build: bad precision %d", prec);
    FTL_CHECK_ARG(U32 == nullptr || prec != FTL_PREC_FP64, "ftl_tree_build: FP32 factor copies need an FP32 tree");
    cudaStream_t st = (cudaStream_t)stream;
    if (prec == FTL_PREC_FP64) return build_impl<double>(U, n, R, F, prec, (double *)G, nullptr, st);
    return build_impl<float>(U, n, R, F, prec, (float *)G, U32, st);
}

extern "C" int ftl_tree_build(const double *U, int64_t n, int R, int64_t F, int prec, void *G,
                              void *stream) {
    return ftl_tree_build_ex(U, n, R, F, prec, G, nullptr, stream);
}

extern "C" int ftl_tree_scale(const void *G_src, void *G_dst, int64_t node_count, int R, int prec,
                              const double *mat, void *stream) {
    FTL_CHECK_ARG(G_src && G_dst && mat, "ftl_tree_scale: null pointer");
    FTL_CHECK_ARG(node_count >= 1 && R >= 1 && R <= FTL_MAX_RANK, "ftl_tree_scale: bad shape");
    FTL_CHECK_ARG(valid_prec(prec), "ftl_tree_scale: bad precision %d", prec);
    prec = storage_prec(prec);
    const int P = packed_size(R);
    const int S = node_stride(R, prec_bytes(prec));
    int64_t total = node_count * (int64_t)S;
    int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)num_sms() * 16);
    cudaStream_t st = (cudaStream_t)stream;
    if (prec == FTL_PREC_FP64)
        tree_scale_kernel<double><<<blocks, 256, 0, st>>>((const double *)G_src, (double *)G_dst, total, R, P, S, mat);
    else
        tree_scale_kernel<float><<<blocks, 256, 0, st>>>((const float *)G_src, (float *)G_dst, total, R, P, S, mat);
    return check_launch("tree_scale_kernel");
}
