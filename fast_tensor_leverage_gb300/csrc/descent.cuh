// Warp-per-sample partition-tree descent shared by the standalone tree
// sampler and the fused KRP draw.
//
// A descent for query x evaluates x^T G x against node Grams.  With the
// packed upper triangle of G and the packed weighted outer product
// xx_e = (2 - [a==b]) x_a x_b, the form is a plain dot product over
// P = R(R+1)/2 values, so a warp holds xx in registers (R <= 32: 17 values
// per lane) or in its shared-memory slot (R > 32) for the whole descent and
// every level costs P coalesced loads, P FMAs and one warp reduction.
//
// Two arithmetics:
//   * FP64 (parity mode): exactly the reference's decisions,
//     cpp_ext/partition_tree.hpp:253-332 -- root mass m, cutoff = low + mL/m,
//     go left iff draw <= cutoff, then the leaf fraction (draw-low)/(high-low)
//     and the leaf row scan of :370-398 (exclusive prefix of q_r^2 divided by
//     the total, first j <= F-2 with frac < q[j+1], else F-1).
//   * FP32 (mixed mode): FP32 node Grams and forms; the draw is carried as an
//     absolute mass offset t = (draw - low) * m in double-float (two floats),
//     so "draw <= low + mL/m" becomes "t <= mL" and a right turn is t -= mL.
//     Identical decisions in exact arithmetic, no FP64 instructions per level.
#pragma once

#include "ftl_common.cuh"

// Compile-time tuning knobs (defaults are the measured best on GB300).
#ifndef FTL_DESC_PREFETCH
#define FTL_DESC_PREFETCH 0        // L2 prefetch of next-level candidates (measured slower)
#endif
#ifndef FTL_DESC_XX_SMEM32
#define FTL_DESC_XX_SMEM32 1       // keep the outer product in shared memory also for R <= 32
#endif
#ifndef FTL_DESC_EVAL2
#define FTL_DESC_EVAL2 1           // root and first-level forms in one round trip
#endif
#ifndef FTL_DESC_LEAF_CHUNK
#define FTL_DESC_LEAF_CHUNK 16     // leaf rows loaded per round trip (8, 16 or 32)
#endif
#ifndef FTL_DESC_WARPS32
#define FTL_DESC_WARPS32 8         // warps per block for R <= 32
#endif
#ifndef FTL_DESC_WARPS128_F32
#define FTL_DESC_WARPS128_F32 6    // FP32, R > 64: one block of 6 warps fills the shared memory
#endif
#ifndef FTL_DESC_REDO
#define FTL_DESC_REDO 1            // FP32: flag samples that met a zero-mass block for the careful redo
#endif
#ifndef FTL_DESC_RESIDENT_F32
#define FTL_DESC_RESIDENT_F32 1536 // threads per SM the FP32 kernels are register-budgeted for
#endif
#ifndef FTL_DESC_RESIDENT_F64
#define FTL_DESC_RESIDENT_F64 512
#endif
#ifndef FTL_DESC_WARPS_D32
#define FTL_DESC_WARPS_D32 4       // FP32 DIAG32 packed (multi-request) draws and tree sampler: warps per block
#endif
#ifndef FTL_DESC_RESIDENT_D32
#define FTL_DESC_RESIDENT_D32 512  // the same kernels: threads per SM the register budget is set for (128)
#endif

namespace ftl {

template <int RMAX>
struct Shape {
    static constexpr int PMAX = RMAX * (RMAX + 1) / 2;
    static constexpr int XPL = (RMAX + 31) / 32;  // vector entries per lane
    static constexpr int FQ = (RMAX + 31) / 32;   // leaf rows per lane (F <= R)
    static constexpr bool XX_SMEM = RMAX > 32 || FTL_DESC_XX_SMEM32;
    static constexpr int WARPS = RMAX <= 32 ? FTL_DESC_WARPS32 : (RMAX <= 64 ? 4 : 2);
};

// Warps per block of the draw kernels.  R > 64: each warp's slot holds the
// 8256-entry packed outer product (33 KB in FP32, 66 KB in FP64) next to the
// block's pair table (16.5 KB): 6 FP32 warps fit one block per SM (224 KB),
// where blocks of 2 gave 2 blocks per SM (4 warps).
template <int RMAX, typename T, bool DIAG = false>
struct Blk {
    static constexpr int WARPS =
        (DIAG && sizeof(T) == 4)
            ? FTL_DESC_WARPS_D32
            : (RMAX <= 64 ? Shape<RMAX>::WARPS : (sizeof(T) == 4 ? FTL_DESC_WARPS128_F32 : Shape<RMAX>::WARPS));
};

// 16-byte vector of the tree precision.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int W = 4;
    static __device__ __forceinline__ void get(const type &v, float (&o)[4]) {
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
        o[3] = v.w;
    }
};
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int W = 2;
    static __device__ __forceinline__ void get(const type &v, double (&o)[2]) {
        o[0] = v.x;
        o[1] = v.y;
    }
};

// Node geometry of one precision: S = node stride (packed triangle padded to
// 16 bytes), NV = 16-byte vectors per lane to cover the largest node.
template <int RMAX, typename T>
struct NodeShape {
    static constexpr int W = Vec16<T>::W;
    static constexpr int SMAX = (Shape<RMAX>::PMAX + W - 1) / W * W;
    static constexpr int NV = (SMAX / W + 31) / 32;
};

// Per-warp shared-memory slot: the query in FP64 and in the compute type,
// plus the packed outer product when it does not fit in registers.
template <int RMAX, typename T, bool DIAG = false>
struct WarpSlot {
    static constexpr size_t xx_elems = (Shape<RMAX>::XX_SMEM && !DIAG) ? NodeShape<RMAX, T>::SMAX : 0;
    static constexpr size_t bytes =
        ((RMAX * sizeof(double) + RMAX * sizeof(T) + xx_elems * sizeof(T)) + 15) / 16 * 16;
};

// x^T G x for one query x against any node G (packed, node stride S): the
// node is read as 16-byte vectors, vector v of lane l is v = l + 32 t, and
// the matching weighted outer-product values live in registers (R <= 32) or
// in the warp's shared-memory slot.
template <int RMAX, typename T>
struct QForm {
    using S_ = Shape<RMAX>;
    using NS = NodeShape<RMAX, T>;
    using V = typename Vec16<T>::type;
    static constexpr int W = NS::W;
    T r[S_::XX_SMEM ? 1 : NS::NV * W];
    T *s;
    int P, S;

    __device__ __forceinline__ void setup(const T *x, const uint16_t *pairs, int lane) {
        if (S_::XX_SMEM) {
            for (int e = lane; e < S; e += 32) {
                T v = T(0);
                if (e < P) {
                    unsigned pr = pairs[e];
                    int a = pr >> 8, b = pr & 0xff;
                    v = x[a] * x[b];
                    if (a != b) v += v;
                }
                s[e] = v;
            }
            __syncwarp();
        } else {
#pragma unroll
            for (int t = 0; t < NS::NV; ++t) {
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    int e = (lane + 32 * t) * W + w;
                    T v = T(0);
                    if (e < P) {
                        unsigned pr = pairs[e];
                        int a = pr >> 8, b = pr & 0xff;
                        v = x[a] * x[b];
                        if (a != b) v += v;
                    }
                    r[t * W + w] = v;
                }
            }
        }
    }

    __device__ __forceinline__ T eval(const T *__restrict__ node, int lane) const {
        T acc = T(0);
        if (S_::XX_SMEM) {
#pragma unroll(NS::NV <= 8 ? NS::NV : 2)
            for (int t = 0; t < NS::NV; ++t) {
                int e = (lane + 32 * t) * W;
                if (e < S) {
                    V g = __ldg(reinterpret_cast<const V *>(node + e));
                    V x = *reinterpret_cast<const V *>(s + e);
                    T gv[W], xv[W];
                    Vec16<T>::get(g, gv);
                    Vec16<T>::get(x, xv);
#pragma unroll
                    for (int w = 0; w < W; ++w) acc = fma(gv[w], xv[w], acc);
                }
            }
        } else {
#pragma unroll
            for (int t = 0; t < NS::NV; ++t) {
                int e = (lane + 32 * t) * W;
                if (e < S) {
                    V g = __ldg(reinterpret_cast<const V *>(node + e));
                    T gv[W];
                    Vec16<T>::get(g, gv);
#pragma unroll
                    for (int w = 0; w < W; ++w) acc = fma(gv[w], r[t * W + w], acc);
                }
            }
        }
        return warp_sum(acc);
    }

    // Two independent forms with interleaved loads (one memory round trip).
    __device__ __forceinline__ void eval2(const T *__restrict__ na, const T *__restrict__ nb,
                                          int lane, T &ra, T &rb) const {
        T acc_a = T(0), acc_b = T(0);
        if (S_::XX_SMEM) {
#pragma unroll 2
            for (int e = lane * W; e < S; e += 32 * W) {
                V ga = __ldg(reinterpret_cast<const V *>(na + e));
                V gb = __ldg(reinterpret_cast<const V *>(nb + e));
                V x = *reinterpret_cast<const V *>(s + e);
                T av[W], bv[W], xv[W];
                Vec16<T>::get(ga, av);
                Vec16<T>::get(gb, bv);
                Vec16<T>::get(x, xv);
#pragma unroll
                for (int w = 0; w < W; ++w) {
                    acc_a = fma(av[w], xv[w], acc_a);
                    acc_b = fma(bv[w], xv[w], acc_b);
                }
            }
        } else {
#pragma unroll
            for (int t = 0; t < NS::NV; ++t) {
                int e = (lane + 32 * t) * W;
                if (e < S) {
                    V ga = __ldg(reinterpret_cast<const V *>(na + e));
                    V gb = __ldg(reinterpret_cast<const V *>(nb + e));
                    T av[W], bv[W];
                    Vec16<T>::get(ga, av);
                    Vec16<T>::get(gb, bv);
#pragma unroll
                    for (int w = 0; w < W; ++w) {
                        acc_a = fma(av[w], r[t * W + w], acc_a);
                        acc_b = fma(bv[w], r[t * W + w], acc_b);
                    }
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            acc_a += __shfl_xor_sync(0xffffffffu, acc_a, o);
            acc_b += __shfl_xor_sync(0xffffffffu, acc_b, o);
        }
        ra = acc_a;
        rb = acc_b;
    }
};

// x^T G x against DIAG32 nodes (FP32, 16 < R <= 32; layout in
// ftl_common.cuh): lane a keeps the 17 weights c_d x_a x_{(a+d) mod 32} of
// its node row in registers, so a level costs four 128-bit loads and one
// 32-bit load per lane (each a contiguous 512- or 128-byte warp access), 17
// FMAs and one warp reduction, with no shared-memory traffic.  The query x
// comes zero padded to 32 entries (entries R..31 zero).
struct QFormD32 {
    float xx[17];
    float *s;  // unused (interface of QForm)
    int P, S;

    __device__ __forceinline__ void setup(const float *x, const uint16_t *, int lane) { setup_reg(x[lane], lane); }

    // lane a passes x_a (zero for a >= R)
    __device__ __forceinline__ void setup_reg(float xa, int lane) {
        xx[0] = xa * xa;
#pragma unroll
        for (int d = 1; d < 16; ++d) xx[d] = (xa + xa) * __shfl_sync(0xffffffffu, xa, (lane + d) & 31);
        xx[16] = xa * __shfl_sync(0xffffffffu, xa, (lane + 16) & 31);
    }

    __device__ __forceinline__ float partial(const float *__restrict__ node, int lane) const {
        const float4 *v = reinterpret_cast<const float4 *>(node);
        const float4 g[4] = {__ldg(v + lane), __ldg(v + 32 + lane), __ldg(v + 64 + lane), __ldg(v + 96 + lane)};
        return dot(g, __ldg(node + 512 + lane));
    }

    // this lane's part of the form from its row of a node (already loaded):
    // two independent FMA chains (half the dependent latency)
    __device__ __forceinline__ float dot(const float4 (&g)[4], float g16) const {
        float a0 = g[0].x * xx[0], a1 = g[0].y * xx[1];
        a0 = fmaf(g[0].z, xx[2], a0);
        a1 = fmaf(g[0].w, xx[3], a1);
        a0 = fmaf(g[1].x, xx[4], a0);
        a1 = fmaf(g[1].y, xx[5], a1);
        a0 = fmaf(g[1].z, xx[6], a0);
        a1 = fmaf(g[1].w, xx[7], a1);
        a0 = fmaf(g[2].x, xx[8], a0);
        a1 = fmaf(g[2].y, xx[9], a1);
        a0 = fmaf(g[2].z, xx[10], a0);
        a1 = fmaf(g[2].w, xx[11], a1);
        a0 = fmaf(g[3].x, xx[12], a0);
        a1 = fmaf(g[3].y, xx[13], a1);
        a0 = fmaf(g[3].z, xx[14], a0);
        a1 = fmaf(g[3].w, xx[15], a1);
        a0 = fmaf(g16, xx[16], a0);
        return a0 + a1;
    }

    __device__ __forceinline__ float eval(const float *__restrict__ node, int lane) const {
        return warp_sum(partial(node, lane));
    }

    __device__ __forceinline__ void eval2(const float *__restrict__ na, const float *__restrict__ nb, int lane,
                                          float &ra, float &rb) const {
        float a = partial(na, lane), b = partial(nb, lane);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        ra = a;
        rb = b;
    }
};

// QFormD32 with the 17 query weights of each lane kept in shared memory
// instead of registers (a per-sample slot of 544 floats: four [lane] rows of
// float4 for d = 0..15, then one [lane] row for d = 16; every lane reads and
// writes only its own entries, so no synchronisation is needed).  Frees 17
// registers per sample in flight; the same products in the same order as
// QFormD32, so the same results bit for bit.
struct QFormD32S {
    float4 *w4;
    float *w16;

    __device__ __forceinline__ void bind(float *slot) {
        w4 = reinterpret_cast<float4 *>(slot);
        w16 = slot + 512;
    }

    __device__ __forceinline__ void setup_reg(float xa, int lane) {
        float xx[17];
        xx[0] = xa * xa;
#pragma unroll
        for (int d = 1; d < 16; ++d) xx[d] = (xa + xa) * __shfl_sync(0xffffffffu, xa, (lane + d) & 31);
        xx[16] = xa * __shfl_sync(0xffffffffu, xa, (lane + 16) & 31);
#pragma unroll
        for (int q = 0; q < 4; ++q) w4[32 * q + lane] = make_float4(xx[4 * q], xx[4 * q + 1], xx[4 * q + 2], xx[4 * q + 3]);
        w16[lane] = xx[16];
    }

    __device__ __forceinline__ float dot(const float4 (&g)[4], float g16) const {
        const int lane = threadIdx.x & 31;
        float4 x = w4[lane];
        float a0 = g[0].x * x.x, a1 = g[0].y * x.y;
        a0 = fmaf(g[0].z, x.z, a0);
        a1 = fmaf(g[0].w, x.w, a1);
        x = w4[32 + lane];
        a0 = fmaf(g[1].x, x.x, a0);
        a1 = fmaf(g[1].y, x.y, a1);
        a0 = fmaf(g[1].z, x.z, a0);
        a1 = fmaf(g[1].w, x.w, a1);
        x = w4[64 + lane];
        a0 = fmaf(g[2].x, x.x, a0);
        a1 = fmaf(g[2].y, x.y, a1);
        a0 = fmaf(g[2].z, x.z, a0);
        a1 = fmaf(g[2].w, x.w, a1);
        x = w4[96 + lane];
        a0 = fmaf(g[3].x, x.x, a0);
        a1 = fmaf(g[3].y, x.y, a1);
        a0 = fmaf(g[3].z, x.z, a0);
        a1 = fmaf(g[3].w, x.w, a1);
        a0 = fmaf(g16, w16[lane], a0);
        return a0 + a1;
    }

    __device__ __forceinline__ float partial(const float *__restrict__ node, int lane) const {
        const float4 *v = reinterpret_cast<const float4 *>(node);
        const float4 g[4] = {__ldg(v + lane), __ldg(v + 32 + lane), __ldg(v + 64 + lane), __ldg(v + 96 + lane)};
        return dot(g, __ldg(node + 512 + lane));
    }

    __device__ __forceinline__ float eval(const float *__restrict__ node, int lane) const {
        return warp_sum(partial(node, lane));
    }
};

// The form type of a (rank bound, precision, layout).
template <int RMAX, typename T, bool DIAG>
struct QSel {
    using type = QForm<RMAX, T>;
};
template <>
struct QSel<32, float, true> {
    using type = QFormD32;
};

// L2 prefetch of the 128-byte lines covering [p, p + bytes), one line per
// lane per pass.  Every address issued is the start of a line that holds at
// least one byte of the range, so it lies inside the range's allocation.
__device__ __forceinline__ void prefetch_lines(const void *p, int64_t bytes, int lane) {
    const uintptr_t a0 = (uintptr_t)p & ~(uintptr_t)127;
    const uintptr_t a1 = ((uintptr_t)p + (uintptr_t)bytes - 1) & ~(uintptr_t)127;
    for (uintptr_t a = a0 + 128 * (uintptr_t)lane; a <= a1; a += 32 * 128)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

// Before evaluating level `c` -> child 2c+1, fetch into L2 what the next step
// can need: for each child c' of c, its left child's node (next level), or,
// when c' is a leaf of a tree with a leaf scan, its factor block.
template <typename T>
__device__ __forceinline__ void prefetch_next(const T *G, int S, const DGeom &g, int64_t c,
                                              const double *U, int R, int lane) {
    if (!FTL_DESC_PREFETCH) return;
    const int64_t c1 = 2 * c + 1;
    if (!is_leaf(g, c1 + 1)) {
        // both children internal: their left children are adjacent pairs
        // 2c1+1 and 2c1+3 -> two node ranges
        prefetch_lines(G + (2 * c1 + 1) * (int64_t)S, (int64_t)S * sizeof(T), lane);
        prefetch_lines(G + (2 * c1 + 3) * (int64_t)S, (int64_t)S * sizeof(T), lane);
        return;
    }
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const int64_t cc = c1 + side;
        if (cc >= g.node_count) continue;
        if (!is_leaf(g, cc)) {
            prefetch_lines(G + (2 * cc + 1) * (int64_t)S, (int64_t)S * sizeof(T), lane);
        } else if (U != nullptr) {
            const int64_t row0 = leaf_index(g, cc) * g.F;
            const int64_t rows = min(g.F, g.n - row0);
            prefetch_lines(U + row0 * R, rows * R * (int64_t)sizeof(double), lane);
        }
    }
}

// ----------------------------------------------------------------- FP64

template <int RMAX>
__device__ __forceinline__ int64_t descend(const double *__restrict__ G, int S, const DGeom &g,
                                           double draw, const QForm<RMAX, double> &qf, int lane,
                                           double &frac, const double *U = nullptr, int R = 0,
                                           double *mroot = nullptr) {
    int64_t c = 0;
    double low = 0.0, high = 1.0;
    if (is_leaf(g, 0)) {  // single-leaf tree: the leaf fraction is the draw
        frac = draw;
        if (mroot) *mroot = 1.0;  // not evaluated; the leaf scan sees the block
        return 0;
    }
    // the root mass and the first left-child mass need no decision between
    // them: one round trip for both
    prefetch_next(G, S, g, 0, U, R, lane);
    double m, mL0;
    if (FTL_DESC_EVAL2) {
        qf.eval2(G, G + S, lane, m, mL0);
    } else {
        m = qf.eval(G, lane);
        mL0 = qf.eval(G + S, lane);
    }
    if (mroot) *mroot = m;
    for (int64_t lvl = 0; lvl < g.lfill_level; ++lvl) {
        double mL;
        if (lvl == 0) {
            mL = mL0;
        } else {
            prefetch_next(G, S, g, c, U, R, lane);
            mL = qf.eval(G + (2 * c + 1) * (int64_t)S, lane);
        }
        double cutoff = low + mL / m;
        if (draw <= cutoff) {
            c = 2 * c + 1;
            high = cutoff;
        } else {
            c = 2 * c + 2;
            low = cutoff;
        }
    }
    if (!is_leaf(g, c)) {
        prefetch_next(G, S, g, c, U, R, lane);
        double mL = qf.eval(G + (2 * c + 1) * (int64_t)S, lane);
        double cutoff = low + mL / m;
        if (draw <= cutoff) {
            c = 2 * c + 1;
            high = cutoff;
        } else {
            c = 2 * c + 2;
            low = cutoff;
        }
    }
    frac = (draw - low) / (high - low);
    return c;
}

// ----------------------------------------------------------------- FP32

// t -= m for a double-float t = (th, tl) (Knuth TwoSum, then renormalise).
__device__ __forceinline__ void df_sub(float &th, float &tl, float m) {
    float s = th - m;
    float bb = s - th;
    float err = (th - (s - bb)) + (-m - bb);
    tl += err;
    float nh = s + tl;
    tl = tl - (nh - s);
    th = nh;
}

// A uniform in [0, 1) as a double-float dh + dl (dh its FP32 rounding, dl
// the FP32 rounding of the rest): exact to about 2^-48.
__device__ __forceinline__ void split_df(double d, float &dh, float &dl) {
    dh = d2f_rn(d);
    dl = (float)(d - (double)dh);
}

// The same for a Philox uniform given by its 53 bits B (uniform = B 2^-53):
// dh = (B >> 29) 2^-24 exactly, dl = the low 29 bits 2^-53 -- integer
// conversions only.
__device__ __forceinline__ void split_bits53(uint64_t B, float &dh, float &dl) {
    dh = (float)(uint32_t)(B >> 29) * 5.9604644775390625e-08f;         // 2^-24
    dl = (float)(uint32_t)(B & 0x1fffffffu) * 1.1102230246251565e-16f;  // 2^-53
}

template <int RMAX, class QF>
__device__ __forceinline__ int64_t descend_df(const float *__restrict__ G, int S, const DGeom &g, float dh,
                                              float dl, const QF &qf, int lane, float &frac,
                                              const double *U = nullptr, int R = 0, float *mroot = nullptr) {
    int64_t c = 0;
    if (is_leaf(g, 0)) {  // single-leaf tree: the leaf fraction is the draw
        frac = fminf(dh + dl, 1.0f);
        if (mroot) *mroot = 1.0f;  // not evaluated; the leaf scan sees the block
        return 0;
    }
    prefetch_next(G, S, g, 0, U, R, lane);
    float mP, mL0;
    if (FTL_DESC_EVAL2) {
        qf.eval2(G, G + S, lane, mP, mL0);
    } else {
        mP = qf.eval(G, lane);
        mL0 = qf.eval(G + S, lane);
    }
    if (mroot) *mroot = mP;
    // t = draw * mP in double-float (exact product of dh and mP, plus dl mP)
    float th = dh * mP;
    float tl = fmaf(dl, mP, fmaf(dh, mP, -th));
    {
        const float s = th + tl;
        tl = tl - (s - th);
        th = s;
    }
    // 32-bit node index and level counter (node counts are far below 2^31:
    // a tree is at most 2 I / F nodes)
    const uint32_t ncount = (uint32_t)g.node_count;
    const int lf = (int)g.lfill_level;
    uint32_t cu = 0;
    for (int lvl = 0; lvl <= lf; ++lvl) {
        if (lvl == lf && 2u * cu + 1u >= ncount) break;
        float mL;
        if (lvl == 0) {
            mL = mL0;
        } else {
            prefetch_next(G, S, g, (int64_t)cu, U, R, lane);
            mL = qf.eval(G + (size_t)(2u * cu + 1u) * (size_t)S, lane);
        }
        bool left = ((th - mL) + tl) <= 0.0f;
        if (left) {
            cu = 2u * cu + 1u;
            mP = mL;
        } else {
            cu = 2u * cu + 2u;
            df_sub(th, tl, mL);
            mP = fmaxf(mP - mL, 0.0f);
        }
    }
    c = (int64_t)cu;
    float f = mP > 0.0f ? (th + tl) / mP : 0.0f;
    frac = fminf(fmaxf(f, 0.0f), 1.0f);
    return c;
}

template <int RMAX, class QF>
__device__ __forceinline__ int64_t descend(const float *__restrict__ G, int S, const DGeom &g,
                                           double draw, const QF &qf, int lane,
                                           float &frac, const double *U = nullptr, int R = 0,
                                           float *mroot = nullptr) {
    float dh, dl;
    split_df(draw, dh, dl);
    return descend_df<RMAX, QF>(G, S, g, dh, dl, qf, lane, frac, U, R, mroot);
}

// The FP32 descent above carries the mass of a right child as parent - left
// instead of evaluating it, so where a right subtree has exactly zero mass
// (a block of all-zero factor rows: rows of an ALS factor that no sampled
// fiber touched) rounding can send t into it.  This variant, run only when
// the first descent ended in a block whose forms are all zero, evaluates both
// children at every level, never enters a child with a non-positive form
// while its sibling's is positive, and rescales t onto the evaluated child
// masses (t in FP64).  In exact arithmetic it samples the same distribution.
template <int RMAX, class QF>
__device__ __forceinline__ int64_t descend_careful(const float *__restrict__ G, int S, const DGeom &g,
                                                   double draw, const QF &qf, int lane,
                                                   float &frac) {
    int64_t c = 0;
    if (is_leaf(g, 0)) {
        frac = (float)draw;
        return 0;
    }
    float mL, mR;
    qf.eval2(G + S, G + 2 * (int64_t)S, lane, mL, mR);
    double t = draw * ((double)fmaxf(mL, 0.0f) + (double)fmaxf(mR, 0.0f));
    double m;
    while (true) {
        bool left;
        if (!(mR > 0.0f))
            left = true;
        else if (!(mL > 0.0f))
            left = false;
        else
            left = t <= (double)mL;
        if (left) {
            c = 2 * c + 1;
            m = fmax((double)mL, 0.0);
        } else {
            c = 2 * c + 2;
            t -= (double)fmaxf(mL, 0.0f);
            m = (double)mR;
        }
        t = fmin(fmax(t, 0.0), m);
        if (is_leaf(g, c)) break;
        qf.eval2(G + (2 * c + 1) * (int64_t)S, G + (2 * c + 2) * (int64_t)S, lane, mL, mR);
        const double mc = (double)fmaxf(mL, 0.0f) + (double)fmaxf(mR, 0.0f);
        t = m > 0.0 ? t * (mc / m) : 0.0;
    }
    frac = m > 0.0 ? (float)fmin(fmax(t / m, 0.0), 1.0) : 0.0f;
    return c;
}

// Lockstep descents of NC independent queries through one DIAG32 FP32 tree
// (one warp, lane a = row a): each level issues every chain's node loads
// before any form is computed, so NC dependent read chains are in flight at
// once; the root and its left child, common to all chains, are read once.
// The decisions are descend_df's: t = draw * m_root in double-float, left
// iff t <= m_left, a right turn subtracts m_left.  cu[c] receives the leaf,
// frac[c] the leaf fraction, mroot[c] the root form.
template <int NC, class QF>
__device__ __forceinline__ void descend_d32_multi(const float *__restrict__ G, const DGeom &g, const float (&dh)[NC],
                                                  const float (&dl)[NC], const QF (&qf)[NC], int lane,
                                                  uint32_t (&cu)[NC], float (&frac)[NC], float (&mroot)[NC]) {
    constexpr int S = kDiag32Stride;
    if (is_leaf(g, 0)) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            cu[c] = 0;
            frac[c] = fminf(dh[c] + dl[c], 1.0f);
            mroot[c] = 1.0f;
        }
        return;
    }
    float th[NC], tl[NC], mP[NC], mL[NC];
    {
        const float4 *r4 = reinterpret_cast<const float4 *>(G), *l4 = reinterpret_cast<const float4 *>(G + S);
        const float4 rv[4] = {__ldg(r4 + lane), __ldg(r4 + 32 + lane), __ldg(r4 + 64 + lane), __ldg(r4 + 96 + lane)};
        const float4 lv[4] = {__ldg(l4 + lane), __ldg(l4 + 32 + lane), __ldg(l4 + 64 + lane), __ldg(l4 + 96 + lane)};
        const float r16 = __ldg(G + 512 + lane), l16 = __ldg(G + S + 512 + lane);
        float a[NC], b[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            a[c] = qf[c].dot(rv, r16);
            b[c] = qf[c].dot(lv, l16);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                a[c] += __shfl_xor_sync(0xffffffffu, a[c], o);
                b[c] += __shfl_xor_sync(0xffffffffu, b[c], o);
            }
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            mroot[c] = mP[c] = a[c];
            mL[c] = b[c];
            th[c] = dh[c] * mP[c];
            tl[c] = fmaf(dl[c], mP[c], fmaf(dh[c], mP[c], -th[c]));
            const float s = th[c] + tl[c];
            tl[c] = tl[c] - (s - th[c]);
            th[c] = s;
            cu[c] = 0;
        }
    }
    const uint32_t ncount = (uint32_t)g.node_count;
    const int lf = (int)g.lfill_level;
    for (int lvl = 0; lvl <= lf; ++lvl) {
        bool go[NC];
        bool any = false;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            go[c] = !(lvl == lf && 2u * cu[c] + 1u >= ncount);
            any |= go[c];
        }
        if (!any) break;
        if (lvl > 0) {
            float4 v[NC][4];
            float v16[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const float *node = G + (size_t)(go[c] ? 2u * cu[c] + 1u : 0u) * (size_t)S;
                const float4 *n4 = reinterpret_cast<const float4 *>(node);
#pragma unroll
                for (int q = 0; q < 4; ++q) v[c][q] = __ldg(n4 + 32 * q + lane);
                v16[c] = __ldg(node + 512 + lane);
            }
            float part[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) part[c] = qf[c].dot(v[c], v16[c]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int c = 0; c < NC; ++c) part[c] += __shfl_xor_sync(0xffffffffu, part[c], o);
#pragma unroll
            for (int c = 0; c < NC; ++c) mL[c] = part[c];
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            if (!go[c]) continue;
            if (((th[c] - mL[c]) + tl[c]) <= 0.0f) {
                cu[c] = 2u * cu[c] + 1u;
                mP[c] = mL[c];
            } else {
                cu[c] = 2u * cu[c] + 2u;
                df_sub(th[c], tl[c], mL[c]);
                mP[c] = fmaxf(mP[c] - mL[c], 0.0f);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const float f = mP[c] > 0.0f ? (th[c] + tl[c]) / mP[c] : 0.0f;
        frac[c] = fminf(fmaxf(f, 0.0f), 1.0f);
    }
}

// ------------------------------------------------------------- leaf scan

// The warp's staged query as per-lane registers (entry lane + 32q in [q]).
template <int RMAX, typename T>
struct LaneQuery {
    T v[Shape<RMAX>::XPL];
};

template <int RMAX, typename T>
__device__ __forceinline__ LaneQuery<RMAX, T> lane_query(const T *x, int R, int lane) {
    LaneQuery<RMAX, T> q;
#pragma unroll
    for (int i = 0; i < Shape<RMAX>::XPL; ++i) {
        int col = lane + 32 * i;
        q.v[i] = col < R ? x[col] : T(0);
    }
    return q;
}

// Sum over lanes of K per-lane values at once (K = 8, 16 or 32): a butterfly
// that halves the live values per stage, then plain adds.  Afterwards lane l
// holds in v[0] the warp-wide sum of value index (l >> (5 - log2 K)).
template <int K, typename T>
__device__ __forceinline__ T transpose_reduce(T (&v)[K], int lane) {
    static_assert(K == 8 || K == 16 || K == 32, "K must be 8, 16 or 32");
    int live = K;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        if (live > 1) {
            const int h = live / 2;
            const bool upper = (lane & off) != 0;
#pragma unroll
            for (int i = 0; i < K / 2; ++i) {
                if (i < h) {
                    T send = upper ? v[i] : v[i + h];
                    T keep = upper ? v[i + h] : v[i];
                    v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
                }
            }
            live = h;
        } else {
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], off);
        }
    }
    return v[0];
}

// Row selection inside leaf block c (F > 1): q_r = U[row0+r] . x for the
// block's rows, inclusive prefix of q_r^2 in row order, first r <= F-2 with
// frac < prefix_r / total, else F-1.  The block is read in chunks of K rows
// with coalesced loads (lane = column), all loads of a chunk issued before
// any use, and each chunk's K row dot products are finished by one
// transpose-reduce.  xq holds the warp's query in the compute type.  A
// selection past the last row of a partial block (only reachable when frac
// rounds to >= 1) is clamped to that last row.
template <int RMAX, typename T, typename UT = double>
__device__ __forceinline__ int64_t leaf_scan(const UT *__restrict__ U, int R, const DGeom &g,
                                             int64_t c, T frac, const LaneQuery<RMAX, T> &xq,
                                             int lane, bool &empty) {
    constexpr int XPL = Shape<RMAX>::XPL;
    constexpr int K = FTL_DESC_LEAF_CHUNK;
    constexpr int LOGK = K == 8 ? 3 : (K == 16 ? 4 : 5);
    constexpr int NCH = (RMAX + K - 1) / K;  // chunks covering F <= RMAX rows
    const int64_t leaf = leaf_index(g, c);
    const int F = (int)g.F;
    const int64_t row0 = leaf * g.F;
    const int rows = (int)min((int64_t)F, g.n - row0);
    T q2[NCH];
#pragma unroll
    for (int ch = 0; ch < NCH; ++ch) {
        T v[K];
#pragma unroll
        for (int rr = 0; rr < K; ++rr) {
            const int r = K * ch + rr;
            T acc = T(0);
            if (r < rows) {
                const UT *u = U + (row0 + r) * (int64_t)R;
#pragma unroll
                for (int q = 0; q < XPL; ++q) {
                    const int col = lane + 32 * q;
                    if (col < R) acc = fma((T)__ldg(u + col), xq.v[q], acc);
                }
            }
            v[rr] = acc;
        }
        T q = transpose_reduce<K, T>(v, lane);
        q2[ch] = q * q;
    }
    // Sequential prefix in row order (same association as the reference's
    // running sum); every lane walks the same sequence, lane r keeps row r's
    // prefix (rows >= 32 in the further slots).
    constexpr int FQ = Shape<RMAX>::FQ;
    T incl[FQ];
    T tot;
    if (sizeof(T) == 8) {
        // FP64: the reference's sequential running sum (same association)
#pragma unroll
        for (int qi = 0; qi < FQ; ++qi) incl[qi] = T(0);
        T run = T(0);
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) {
            for (int rr = 0; rr < K; ++rr) {
                const int r = K * ch + rr;
                if (r >= F) break;
                T v = __shfl_sync(0xffffffffu, q2[ch], rr << (5 - LOGK));
                run += v;
                if (lane == (r & 31)) incl[(K * ch) >> 5] = run;
            }
        }
        tot = run;
    } else {
        // FP32: lane l gathers the form of row l + 32 qi, then a warp
        // inclusive scan per 32 rows with the carry of the previous ones
        // (5 steps instead of F sequential ones; the FP32 mode is not tied
        // to the reference's association)
        constexpr int CPW = 32 / K;   // chunks per 32 rows
        T carry = T(0);
#pragma unroll
        for (int qi = 0; qi < FQ; ++qi) {
            T v = T(0);
#pragma unroll
            for (int cc = 0; cc < CPW; ++cc) {
                if (qi * CPW + cc < NCH) {
                    const T t = __shfl_sync(0xffffffffu, q2[qi * CPW + cc], (lane % K) << (5 - LOGK));
                    if (lane / K == cc) v = t;
                }
            }
            if (lane + 32 * qi >= F) v = T(0);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const T u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            incl[qi] = v + carry;
            carry += __shfl_sync(0xffffffffu, v, 31);
        }
        tot = carry;
    }
    int res = F - 1;
    bool found = false;
#pragma unroll
    for (int qi = FQ - 1; qi >= 0; --qi) {
        int r = lane + 32 * qi;
        bool pred;
        if (sizeof(T) == 8)
            pred = (r <= F - 2) && (frac < incl[qi] / tot);
        else
            pred = (r <= F - 2) && (frac * tot < incl[qi]);
        unsigned bal = __ballot_sync(0xffffffffu, pred);
        if (bal) {
            res = 32 * qi + (__ffs(bal) - 1);
            found = true;
        }
    }
    empty = false;
    if (sizeof(T) == 4 && !found) {
        // FP32: a row found above has a positive form (its inclusive prefix
        // exceeds the previous one); when none is, take the last row with a
        // positive form rather than the last row, and report a block whose
        // forms are all zero, so the caller can redo the descent.  (FP64
        // keeps the reference's rule: the last row.)
        // q2[ch] of lane l is the form of row K ch + (l >> (5 - LOGK))
        int lastpos = -1;
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) {
            const int r = K * ch + (lane >> (5 - LOGK));
            const unsigned bal = __ballot_sync(0xffffffffu, r < rows && q2[ch] > T(0));
            if (bal) lastpos = K * ch + ((31 - __clz((int)bal)) >> (5 - LOGK));
        }
        if (lastpos >= 0) res = lastpos;
        else empty = true;
    }
    if (res >= rows) res = rows - 1;
    return row0 + res;
}

// Leaf row selection for R = F = 32 from the FP32 factor copy (the same
// rule as leaf_scan's FP32 branch): the 32 x 32 block is read as eight
// 512-byte warp loads of 16-byte vectors (lane l, step t: row 4t + l/8,
// columns 4(l%8)..+3), each lane forms four-column partial dot products
// with the query xa (lane a holds x_a), a three-step transpose-reduce
// within groups of eight lanes leaves row 4(l%8) + l/8's form in lane l, a
// shuffle puts row r's square in lane r, and a warp inclusive scan gives the
// prefix.  Rows past a partial last block read as zero and are never chosen.
__device__ __forceinline__ int64_t leaf_scan_d32(const float *__restrict__ U32, const DGeom &g, int64_t c,
                                                 float frac, float xa, int lane, bool &empty) {
    const int64_t leaf = leaf_index(g, c);
    const int64_t row0 = leaf * 32;
    const int rows = (int)min((int64_t)32, g.n - row0);
    const float4 *blk = reinterpret_cast<const float4 *>(U32 + row0 * 32);
    const int cg = lane & 7, rg = lane >> 3;
    float xq[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) xq[w] = __shfl_sync(0xffffffffu, xa, 4 * cg + w);
    float v[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
        if (4 * t + rg < rows) u = __ldg(blk + 32 * t + lane);
        v[t] = fmaf(u.w, xq[3], fmaf(u.z, xq[2], fmaf(u.y, xq[1], u.x * xq[0])));
    }
    // transpose-reduce over the 8 lanes of a group (offsets 4, 2, 1)
#pragma unroll
    for (int off = 4, live = 8; off >= 1; off >>= 1, live >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (i < live / 2) {
                const float send = upper ? v[i] : v[i + live / 2];
                const float keep = upper ? v[i + live / 2] : v[i];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
            }
        }
    }
    const float q = v[0];  // form of row 4 cg + rg
    float q2 = __shfl_sync(0xffffffffu, q * q, 8 * (lane & 3) + (lane >> 2));  // row `lane`
    if (lane >= rows) q2 = 0.0f;
    float incl = q2;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    const float tot = __shfl_sync(0xffffffffu, incl, 31);
    const unsigned bal = __ballot_sync(0xffffffffu, lane <= 30 && frac * tot < incl);
    int res = 31;
    empty = false;
    if (bal) {
        res = __ffs(bal) - 1;
    } else {
        // the last row with a positive form, or an all-zero block (redone)
        const unsigned pos = __ballot_sync(0xffffffffu, q2 > 0.0f);
        if (pos) res = 31 - __clz((int)pos);
        else empty = true;
    }
    if (res >= rows) res = rows - 1;
    return row0 + res;
}

// x * 2^sh rounded to FP32 by integer operations (x * 2^sh below 2^-126 is
// flushed to zero; the caller's shift keeps the largest |x| in [1, 2)).
__device__ __forceinline__ float scaled_f32(double x, int sh) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const int es = e + sh;
    if (e == 0 || es < 897) return __uint_as_float(hi & 0x80000000u);
    unsigned r = ((unsigned)(es - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    r += (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ? 1u : 0u;
    return __uint_as_float((hi & 0x80000000u) | r);
}

// The shift that puts the largest |x| of the warp's vector (lane a holds x_a,
// zero past R) in [1, 2): 1023 - (largest biased FP64 exponent).
__device__ __forceinline__ int query_shift(double x) {
    const int e = (int)(((unsigned)__double2hiint(x) >> 20) & 0x7ffu);
    const int emax = (int)__reduce_max_sync(0xffffffffu, (unsigned)e);
    return (emax >= 1 && emax <= 2045) ? 1023 - emax : 0;
}

// Packed (a << 8 | b) table of the upper triangle in row-major order.
__device__ __forceinline__ void build_pairs(uint16_t *pairs, int R) {
    const int P = packed_size(R);
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        int a = 0, rem = e;
        while (rem >= R - a) {
            rem -= R - a;
            ++a;
        }
        pairs[e] = (uint16_t)((a << 8) | (a + rem));
    }
}

// Stage an FP64 vector held as XPL entries per lane into the warp's slot:
// xd gets it verbatim; for FP32 mode xf gets it times a power of two that
// puts max|x| in [0.5, 1) (exact, so quadratic-form ratios are unchanged).
// Returns that power of two (1.0 in FP64 mode).
template <int RMAX, typename T>
__device__ __forceinline__ double stage_query(const double (&v)[Shape<RMAX>::XPL], int R, double *xd,
                                              T *xT, int lane) {
    constexpr int XPL = Shape<RMAX>::XPL;
#pragma unroll
    for (int q = 0; q < XPL; ++q) {
        int col = lane + 32 * q;
        if (col < R) xd[col] = v[q];
    }
    double scale = 1.0;
    if (sizeof(T) == 4) {
        unsigned emax = 0;
#pragma unroll
        for (int q = 0; q < XPL; ++q) {
            int col = lane + 32 * q;
            unsigned e = col < R ? ((unsigned)__double2hiint(v[q]) >> 20) & 0x7ffu : 0u;
            emax = max(emax, e);
        }
        emax = __reduce_max_sync(0xffffffffu, emax);
        if (emax >= 1 && emax <= 2045) scale = __hiloint2double((int)((2046u - emax) << 20), 0);
#pragma unroll
        for (int q = 0; q < XPL; ++q) {
            int col = lane + 32 * q;
            xT[col] = col < R ? (T)(v[q] * scale) : T(0);  // zero padded to RMAX
        }
    }
    __syncwarp();
    return scale;
}

}  // namespace ftl
