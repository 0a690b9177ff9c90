// Shared device/host helpers of libftl_gb300: status reporting, tree
// geometry, packed-triangle indexing, warp reductions, Philox4x32-10.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/ftl.h"

namespace ftl {

// ------------------------------------------------------------ error state

void set_error(const char *fmt, ...);
int fail(int status, const char *fmt, ...);
int check_launch(const char *what);

// Raise `func`'s dynamic shared-memory limit to at least `bytes` on the
// current device (a no-op below the 48 KB default, and once per kernel,
// device and size); FTL_E_CUDA with `name` in the message when the runtime
// refuses.
int ensure_smem(const void *func, size_t bytes, const char *name);

// SM count of the current device (cached per device).
int num_sms();

#define FTL_CHECK_ARG(cond, ...)                                  \
    do {                                                          \
        if (!(cond)) return ::ftl::fail(FTL_E_ARG, __VA_ARGS__);  \
    } while (0)

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// ---------------------------------------------------------- tree geometry

// Geometry of a PartitionTree over n rows with F rows per leaf.  Mirrors the
// constructor in cpp_ext/partition_tree.hpp:83-105: leaf_count = ceil(n/F),
// node_count = 2*leaf_count-1, lfill_level = floor(log2(leaf_count)), the
// partial deepest level holding leaves 0 .. (node_count-nodes_upto_lfill)-1.
struct Geom {
    int64_t n, F, leaf_count, node_count, lfill_level, lfill_count, total_levels,
        nodes_upto_lfill, nodes_before_lfill, complete_level_offset;
};

inline Geom make_geom(int64_t n, int64_t F) {
    Geom g;
    g.n = n;
    g.F = F;
    g.leaf_count = (n + F - 1) / F;
    g.node_count = 2 * g.leaf_count - 1;
    g.lfill_level = 0;
    g.lfill_count = 1;
    while (g.lfill_count * 2 <= g.leaf_count) {
        g.lfill_level++;
        g.lfill_count *= 2;
    }
    g.total_levels = g.node_count > g.lfill_count ? g.lfill_level + 1 : g.lfill_level;
    g.nodes_upto_lfill = g.lfill_count * 2 - 1;
    g.nodes_before_lfill = g.lfill_count - 1;
    int64_t half_partial = (g.node_count - g.nodes_upto_lfill) / 2;
    g.complete_level_offset = g.nodes_before_lfill - half_partial;
    return g;
}

// Compact copy used inside kernels.
struct DGeom {
    int64_t n, F, node_count, lfill_level, nodes_upto_lfill, complete_level_offset;
};

inline DGeom to_dgeom(const Geom &g) {
    DGeom d;
    d.n = g.n;
    d.F = g.F;
    d.node_count = g.node_count;
    d.lfill_level = g.lfill_level;
    d.nodes_upto_lfill = g.nodes_upto_lfill;
    d.complete_level_offset = g.complete_level_offset;
    return d;
}

__host__ __device__ inline bool is_leaf(const DGeom &g, int64_t c) {
    return 2 * c + 1 >= g.node_count;
}

__host__ __device__ inline int64_t leaf_index(const DGeom &g, int64_t c) {
    return c >= g.nodes_upto_lfill ? c - g.nodes_upto_lfill : c - g.complete_level_offset;
}

// Heap position of leaf block `leaf` (inverse of leaf_index).
__host__ __device__ inline int64_t leaf_node(const DGeom &g, int64_t leaf) {
    int64_t partial = g.node_count - g.nodes_upto_lfill;  // leaves on deepest level
    return leaf < partial ? g.nodes_upto_lfill + leaf : leaf + g.complete_level_offset;
}

// ------------------------------------------------------ packed triangles

__host__ __device__ inline int packed_size(int R) { return R * (R + 1) / 2; }
__host__ __device__ inline int packed_row_offset(int a, int R) { return a * R - a * (a - 1) / 2; }

// Node layouts.
//   PACKED: the upper triangle in row-major order, element (a,b), a <= b, at
//     a*R - a*(a-1)/2 + b - a, zero padded to a multiple of 16 bytes.
//   DIAG32 (FP32 nodes with 16 < R <= 32): the Gram zero padded to 32 x 32
//     and stored by wrapped diagonals, so that lane a of a warp reads row a:
//     G[a][(a+d) mod 32] for d = 0..15 at ((d/4)*32 + a)*4 + d%4 (four
//     128-bit vectors per lane, each warp load 512 contiguous bytes), and
//     G[a][(a+16) mod 32] at 512 + a.  The distance-16 entries are stored
//     twice (once from each end); 544 values per node.
// x^T G x over a DIAG32 node is sum_a sum_d c_d x_a x_{(a+d) mod 32} G_pos(a,d)
// with c_0 = 1, c_1..15 = 2 and c_16 = 1 (each stored copy counted once).
// (FTL_LAYOUT_PACKED and FTL_LAYOUT_DIAG32 are defined in ftl.h)
constexpr int kDiag32Stride = 544;

__host__ __device__ inline int node_layout(int R, int elem_bytes) {
    return (elem_bytes == 4 && R > 16 && R <= 32) ? FTL_LAYOUT_DIAG32 : FTL_LAYOUT_PACKED;
}

// Node stride in elements: every node starts 16-byte aligned and is read
// with 128-bit loads.
__host__ __device__ inline int node_stride(int R, int elem_bytes) {
    if (node_layout(R, elem_bytes) == FTL_LAYOUT_DIAG32) return kDiag32Stride;
    const int w = 16 / elem_bytes;
    return (packed_size(R) + w - 1) / w * w;
}

// Position of element (a, b) (either order) of a DIAG32 node; for d = 16
// the copy stored from row a.
__host__ __device__ inline int diag32_pos(int a, int b) {
    int d = (b - a) & 31;
    if (d > 16) {
        const int t = a;
        a = b;
        b = t;
        d = 32 - d;
    }
    return d < 16 ? (((d >> 2) * 32 + a) << 2) + (d & 3) : 512 + a;
}

// Element (a, b) stored at position e of a DIAG32 node (e < 544).
__host__ __device__ inline void diag32_entry(int e, int &a, int &b) {
    if (e < 512) {
        const int d = ((e >> 7) << 2) + (e & 3);
        a = (e >> 2) & 31;
        b = (a + d) & 31;
    } else {
        a = e - 512;
        b = (a + 16) & 31;
    }
}

// computeM workspace layout (doubles): 2N+3 dense R x R slots, one status
// word, then the packed FP64 pseudo-inverse at a 16-byte aligned offset
// (it is read with 16-byte vector loads), padded to its node stride.
__host__ __device__ inline size_t cm_status_offset(int N, int R) { return (size_t)(2 * N + 3) * R * R; }
__host__ __device__ inline size_t cm_pinv64_offset(int N, int R) {
    return (cm_status_offset(N, R) + 1 + 1) / 2 * 2;
}
__host__ __device__ inline int packed_index(int a, int b, int R) {
    return packed_row_offset(a, R) + (b - a);
}
// Position of element (a, b) (either order) in a node of the layout that
// R and the element size select.
__host__ __device__ inline int node_pos(int a, int b, int R, int elem_bytes) {
    if (node_layout(R, elem_bytes) == FTL_LAYOUT_DIAG32) return diag32_pos(a, b);
    return a <= b ? packed_index(a, b, R) : packed_index(b, a, R);
}

// ------------------------------------------------------------ precisions

// Tree precisions: FP64 stores FP64 nodes; FP32, TF32X3 and BF16 store FP32
// nodes (TF32X3 and BF16 name how the leaf Grams are formed).
inline bool valid_prec(int prec) { return prec >= FTL_PREC_FP64 && prec <= FTL_PREC_BF16; }
inline int storage_prec(int prec) { return prec == FTL_PREC_FP64 ? FTL_PREC_FP64 : FTL_PREC_FP32; }
inline int prec_bytes(int prec) { return prec == FTL_PREC_FP64 ? 8 : 4; }

// FP64 -> FP32, round to nearest even, by integer operations for results in
// the normal FP32 range (FP64 exponents 897..1150); zeros and FP64
// subnormals give signed zero; the rest (FP32 subnormal results, overflow,
// infinities, NaN) take the hardware conversion.  Same results as
// __double2float_rn; avoids GB300's narrow FP64 pipe for the common case.
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu);
    if (e >= 897 && e <= 1150) {
        unsigned r = ((unsigned)(e - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned rest = lo & 0x1fffffffu;
        r += (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ? 1u : 0u;
        return __uint_as_float((hi & 0x80000000u) | r);
    }
    if (e == 0) return __uint_as_float(hi & 0x80000000u);
    return __double2float_rn(x);
}

// ------------------------------------------------------------------ warps

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// --------------------------------------------------------- Philox4x32-10
// Counter-based generator of Salmon, Moraes, Dror and Shaw, "Parallel random
// numbers: as easy as 1, 2, 3" (SC'11), 10 rounds, 4x32-bit counter and
// 2x32-bit key.  Uniform #idx of a stream = the first two output words of
// block (counter = ctr + idx) combined into a 53-bit double in [0, 1).

__host__ __device__ inline void philox_round(uint32_t c[4], uint32_t k[2]) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    uint64_t p0 = (uint64_t)M0 * c[0];
    uint64_t p1 = (uint64_t)M1 * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k[0];
    uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
}

// The 53 random bits of uniform #counter: the uniform is bits * 2^-53.
__host__ __device__ inline uint64_t philox_bits53(uint64_t seed, uint64_t counter) {
    uint32_t c[4] = {(uint32_t)counter, (uint32_t)(counter >> 32), 0u, 0u};
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        philox_round(c, k);
        k[0] += W0;
        k[1] += W1;
    }
    return ((uint64_t)(c[0] >> 5) << 26) | (uint64_t)(c[1] >> 6);
}

__host__ __device__ inline double philox_uniform(uint64_t seed, uint64_t counter) {
    return (double)philox_bits53(seed, counter) * (1.0 / 9007199254740992.0);  // 2^-53
}

}  // namespace ftl
