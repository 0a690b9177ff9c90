// Dense symmetric eigensolver and Cholesky factorisation for one CTA,
// R x R matrices in shared (or global scratch) memory.  Used by computeM and
// by the ALS pseudo-inverse.
//
// jacobi_eigen: cyclic parallel-order (round-robin) two-sided Jacobi; each
// round rotates R/2 disjoint pairs (p, q) with the classical rotation that
// zeroes a_pq (tau = (a_qq - a_pp) / (2 a_pq), t = sign(tau) / (|tau| +
// sqrt(1 + tau^2)), c = 1 / sqrt(1 + t^2), s = t c), skipping pairs with
// |a_pq| <= eps sqrt(|a_pp a_qq|) (Demmel and Veselic's relative criterion);
// stops after a sweep without rotations (at most 40 sweeps).
#pragma once

#include "ftl_common.cuh"

// Stopping rule of the warp Jacobi: a pair is rotated while |a_p . a_q| >
// FTL_CM_JACOBI_TOL 2^-24 |a_p| |a_q|.
#ifndef FTL_CM_JACOBI_TOL
#define FTL_CM_JACOBI_TOL 1.0f
#endif

namespace ftl {

// In-place Jacobi on A (R x R, symmetric, row-major, element type T); V
// receives the eigenvectors as columns.  All threads of the block must call it.
template <typename T>
__device__ void jacobi_eigen(T *A, T *V, int R, T *csbuf, int *pqbuf, int *flag) {
    const int tid = threadIdx.x, nth = blockDim.x;
    const int n = R + (R & 1);
    const int half = n / 2;
    const T eps = sizeof(T) == 8 ? T(1.1102230246251565e-16) : T(5.9604645e-08);
    for (int e = tid; e < R * R; e += nth) V[e] = (e / R == e % R) ? T(1) : T(0);
    __syncthreads();
    for (int sweep = 0; sweep < 40; ++sweep) {
        if (tid == 0) *flag = 0;
        __syncthreads();
        for (int round = 0; round < n - 1; ++round) {
            if (tid < half) {
                int p, q;
                if (tid == 0) {
                    p = round;
                    q = n - 1;
                } else {
                    p = (round + tid) % (n - 1);
                    q = (round - tid + (n - 1)) % (n - 1);
                }
                if (p > q) {
                    int t = p;
                    p = q;
                    q = t;
                }
                T c = T(1), s = T(0);
                if (q < R) {
                    T apq = A[p * R + q];
                    T app = A[p * R + p];
                    T aqq = A[q * R + q];
                    if (apq != T(0) && fabs(apq) > eps * sqrt(fabs(app * aqq))) {
                        T theta = (aqq - app) / (T(2) * apq);
                        T t;
                        if (fabs(theta) > T(sizeof(T) == 8 ? 1e150 : 1e18))
                            t = T(0.5) / theta;
                        else
                            t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(T(1) + theta * theta));
                        c = T(1) / sqrt(T(1) + t * t);
                        s = t * c;
                        *flag = 1;
                    }
                }
                csbuf[2 * tid] = c;
                csbuf[2 * tid + 1] = s;
                pqbuf[2 * tid] = p;
                pqbuf[2 * tid + 1] = q;
            }
            __syncthreads();
            // A <- J^T A J and V <- V J in one pass: every entry of A lies in
            // exactly one 2 x 2 block (row pair i, column pair k), rotated by
            // columns (A J) and then by rows (J^T A), the order of the two
            // separate passes; the rotated pairs' off-diagonal entries are
            // then exact zeros.  Indices >= R (the padding pair of odd R,
            // whose rotation is the identity) have no storage.
            const int nblk = half * half;
            for (int w = tid; w < nblk + half * R; w += nth) {
                if (w < nblk) {
                    const int i = w / half, k = w - i * half;
                    const T si = csbuf[2 * i + 1], sk = csbuf[2 * k + 1];
                    if (si == T(0) && sk == T(0)) continue;
                    const T ci = csbuf[2 * i], ck = csbuf[2 * k];
                    const int pi = pqbuf[2 * i], qi = pqbuf[2 * i + 1];
                    const int pk = pqbuf[2 * k], qk = pqbuf[2 * k + 1];
                    const bool rq = qi < R, cq = qk < R;
                    T x00 = A[pi * R + pk];
                    T x01 = cq ? A[pi * R + qk] : T(0);
                    T x10 = rq ? A[qi * R + pk] : T(0);
                    T x11 = (rq && cq) ? A[qi * R + qk] : T(0);
                    if (sk != T(0)) {
                        const T t00 = ck * x00 - sk * x01, t01 = sk * x00 + ck * x01;
                        const T t10 = ck * x10 - sk * x11, t11 = sk * x10 + ck * x11;
                        x00 = t00;
                        x01 = t01;
                        x10 = t10;
                        x11 = t11;
                    }
                    if (si != T(0)) {
                        const T u00 = ci * x00 - si * x10, u10 = si * x00 + ci * x10;
                        const T u01 = ci * x01 - si * x11, u11 = si * x01 + ci * x11;
                        x00 = u00;
                        x10 = u10;
                        x01 = u01;
                        x11 = u11;
                    }
                    if (i == k) {
                        x01 = T(0);
                        x10 = T(0);
                    }
                    A[pi * R + pk] = x00;
                    if (cq) A[pi * R + qk] = x01;
                    if (rq) A[qi * R + pk] = x10;
                    if (rq && cq) A[qi * R + qk] = x11;
                } else {
                    const int w2 = w - nblk;
                    const int k = w2 / R, r = w2 - k * R;
                    const T sk = csbuf[2 * k + 1];
                    if (sk == T(0)) continue;
                    const T ck = csbuf[2 * k];
                    const int pk = pqbuf[2 * k], qk = pqbuf[2 * k + 1];
                    const T vrp = V[r * R + pk], vrq = V[r * R + qk];
                    V[r * R + pk] = ck * vrp - sk * vrq;
                    V[r * R + qk] = sk * vrp + ck * vrq;
                }
            }
            __syncthreads();
        }
        if (*flag == 0) break;
        __syncthreads();
    }
    __syncthreads();
}

// order[r] = index of the r-th smallest eigenvalue (ties by index).
template <typename T>
__device__ void sort_ascending(const T *A, int R, int *order) {
    // A NaN on the diagonal (from a NaN input) ranks as +infinity, so the
    // ranks are always a permutation of 0..R-1 and every order[] slot is
    // written: plain < and == on NaN would give colliding ranks and leave
    // slots holding stale shared memory that callers use as indexes.
    for (int v = threadIdx.x; v < R; v += blockDim.x) {
        T lv = A[v * R + v];
        if (lv != lv) lv = T(INFINITY);
        int rank = 0;
        for (int u = 0; u < R; ++u) {
            T lu = A[u * R + u];
            if (lu != lu) lu = T(INFINITY);
            if (lu < lv || (lu == lv && u < v)) ++rank;
        }
        order[rank] = v;
    }
    __syncthreads();
}

// Eigendecomposition of a symmetric positive semidefinite R x R matrix
// (R <= 32) by one warp, in FP32: the one-sided Jacobi method of Hestenes
// ("Inversion of matrices by biorthogonalization", J. SIAM 6, 1958) on the
// columns of A.  Lane j keeps column j of A (and of V, starting at the
// identity) in registers; a round pairs the 32 columns by the round-robin
// (circle) schedule -- lane 31 meets lane r in round r, lane l meets
// (2r - l) mod 31 otherwise -- and each pair exchanges its columns with
// shuffles, forms alpha = |a_p|^2, beta = |a_q|^2, gamma = a_p . a_q (both
// lanes the same sums in the same order) and, unless |gamma| <= tol
// sqrt(alpha beta), rotates [a_p a_q] (and [v_p v_q]) by the angle that
// makes them orthogonal.  A sweep is 31 rounds; sweeps stop when one rotates
// nothing.  Then A V has orthogonal columns A v_j = lambda_j v_j (A is PSD),
// so lambda_j = |column j| and v_j = column j of V.  No block barrier: the
// warp works alone.  Lanes past R hold zero columns and never rotate.
//
// Outputs (lane j < R writes its own entries): W[rank_j * R + a] =
// sqrt(lambda_j) v_j[a] for a < R, rank_j the ascending rank of lambda_j
// (a NaN ranks last, ties by index), and lam[rank_j] = lambda_j.
//
// A holds the matrix times 2^k (k even, chosen by the caller so that its
// largest entry is near 1: the squared column norms stay inside the FP32
// range); the outputs are scaled back: lambda 2^-k, W rows 2^(-k/2).
__device__ inline void warp_jacobi_psd32(const float *A, int R, int k, double *W, double *lam, int lane) {
    float a[32], v[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
        a[i] = (i < R && lane < R) ? A[i * R + lane] : 0.0f;
        v[i] = i == lane ? 1.0f : 0.0f;
    }
    const float tol = FTL_CM_JACOBI_TOL * 5.9604645e-08f;  // units of FP32 rounding
    for (int sweep = 0; sweep < 30; ++sweep) {
        bool rotated = false;
        for (int r = 0; r < 31; ++r) {
            const int partner = lane == 31 ? r : (lane == r ? 31 : (2 * r - lane + 31) % 31);
            float b[32];
            float own = 0.0f, g = 0.0f;
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                b[i] = __shfl_sync(0xffffffffu, a[i], partner);
                own = fmaf(a[i], a[i], own);
            }
            const bool lo = lane < partner;
            // gamma summed in the same order by both lanes: p's entry first
#pragma unroll
            for (int i = 0; i < 32; ++i) g = lo ? fmaf(a[i], b[i], g) : fmaf(b[i], a[i], g);
            const float oth = __shfl_sync(0xffffffffu, own, partner);
            const float ap = lo ? own : oth, aq = lo ? oth : own;
            bool rot = g != 0.0f && fabsf(g) > tol * sqrtf(ap * aq);
            float c = 1.0f, s = 0.0f;
            if (rot) {
                const float zeta = (aq - ap) / (2.0f * g);
                const float t = (zeta >= 0.0f ? 1.0f : -1.0f) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                c = 1.0f / sqrtf(1.0f + t * t);
                s = c * t;
            }
            rotated |= rot;
            // p: c a_p - s a_q;  q: s a_p + c a_q  (both lanes of a pair
            // rotate or neither: rot is computed from the same values)
            const float cs_own = c, cs_oth = lo ? -s : s;
            if (__any_sync(0xffffffffu, rot)) {
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float vb = __shfl_sync(0xffffffffu, v[i], partner);
                    if (rot) {
                        a[i] = fmaf(cs_own, a[i], cs_oth * b[i]);
                        v[i] = fmaf(cs_own, v[i], cs_oth * vb);
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, rotated)) break;
    }
    float nrm = 0.0f;
#pragma unroll
    for (int i = 0; i < 32; ++i) nrm = fmaf(a[i], a[i], nrm);
    float lv = sqrtf(nrm);
    if (lv != lv) lv = INFINITY;
    int rank = 0;
    for (int u = 0; u < R; ++u) {
        const float lu = __shfl_sync(0xffffffffu, lv, u);
        if (lu < lv || (lu == lv && u < lane)) ++rank;
    }
    if (lane < R) {
        const double sq = (double)sqrtf(fmaxf(lv, 0.0f)) * ldexp(1.0, -k / 2);
#pragma unroll
        for (int i = 0; i < 32; ++i)
            if (i < R) W[rank * R + i] = sq * (double)v[i];
        lam[rank] = (double)sqrtf(nrm) * ldexp(1.0, -k);
    }
}

// 1/d for a positive normal FP64 d below 2^1023, by the Newton-Raphson
// iteration for the reciprocal: the mantissa m in [1, 2) is inverted in FP32
// (24 correct bits) and refined by two steps x <- x + x (1 - m x) in FP64
// (each step doubles the correct bits: 48, then past 53), and the exponent is
// restored by an exact power of two.  Other inputs take the IEEE division.
// Its dependent path is a few FP64 operations, shorter than the division's
// on GB300's long-latency FP64 pipe.
__device__ __forceinline__ double rcp_newton(double d) {
    const int hi = __double2hiint(d), lo = __double2loint(d);
    const int ef = (hi >> 20) & 0x7ff;
    if (hi < 0 || ef == 0 || ef >= 2046) return 1.0 / d;
    const double m = __hiloint2double((hi & 0x000fffff) | (1023 << 20), lo);
    double x = (double)(1.0f / (float)m);
    double e = fma(-m, x, 1.0);
    x = fma(x, e, x);
    e = fma(-m, x, 1.0);
    x = fma(x, e, x);
    return x * __hiloint2double((2046 - ef) << 20, 0);
}

// Inverse of a symmetric positive definite A (dense R x R FP64 in shared
// memory, upper triangle used, R <= 32) by the sweep operator (Goodnight,
// "A tutorial on the SWEEP operator", The American Statistician 33, 1979):
// sweeping pivot k with d = a_kk and r = 1/d sets
//   a_kk <- -r,  a_kj <- a_kj r,  a_ik <- a_ik r,  a_ij <- a_ij - (a_ik r) a_kj,
// keeps the matrix symmetric, and after all R pivots leaves -A^-1.  The
// pivots of an SPD matrix are its Schur complements, all positive.  Only the
// R(R+1)/2 upper entries are stored and updated, at most two per thread
// (blockDim.x * 2 >= R(R+1)/2), with two FP64 operations per entry and step
// (GB300's FP64 pipe retires two lanes per cycle per SM: every FP64
// instruction a warp issues holds it for 16 cycles).  At each step warp 0
// copies row k (a_kj = a_jk, half of it a strided column of the upper
// triangle) into a contiguous buffer, so the bulk update reads its operands
// without shared-memory bank conflicts, and lane 0 forms the pivot's
// reciprocal (rcp_newton).  On return (true) the upper triangle holds -A^-1;
// false (block-uniformly) when a pivot is not positive.  scratch: R + 1
// doubles; flag: one int.
__device__ inline bool sweep_inverse_spd(double *A, int R, double *scratch, int *flag) {
    const int tid = threadIdx.x, nth = blockDim.x, nup = R * (R + 1) / 2;
    double *row = scratch + 1;
    int oi[2], oj[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        int w = tid + q * nth;
        oi[q] = -1;
        oj[q] = -1;
        if (w < nup) {
            int i = 0;
            while (w >= R - i) {
                w -= R - i;
                ++i;
            }
            oi[q] = i;
            oj[q] = i + w;
        }
    }
    for (int k = 0; k < R; ++k) {
        if (tid < 32) {
            if (tid < R) row[tid] = A[min(k, tid) * R + max(k, tid)];
            if (tid == 0) {
                const double d = A[k * R + k];
                *flag = d > 0.0 ? 1 : 0;
                scratch[0] = d > 0.0 ? rcp_newton(d) : 0.0;
            }
        }
        __syncthreads();
        if (*flag == 0) return false;
        const double r = scratch[0];
        double nv[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            nv[q] = 0.0;
            const int i = oi[q], j = oj[q];
            if (i < 0) continue;
            if (i == k) {
                nv[q] = (j == k) ? -r : row[j] * r;
            } else if (j == k) {
                nv[q] = row[i] * r;
            } else {
                nv[q] = fma(-(row[i] * r), row[j], A[i * R + j]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 2; ++q)
            if (oi[q] >= 0) A[oi[q] * R + oj[q]] = nv[q];
        __syncthreads();
    }
    return true;
}

// Block Cholesky pivots through rsqrt (one library call: l = d rsqrt(d), 1/l
// = rsqrt(d)) instead of a square root and a division: a shorter dependent
// FP64 path per step (measured 146k -> 129k cycles for the R = 32 factor and
// inverse in one CTA).
#ifndef FTL_CHOL_RSQRT
#define FTL_CHOL_RSQRT 1
#endif

// In-place lower Cholesky factor of (A - shift I), A dense R x R FP64 in
// shared memory (lower triangle used).  Returns true (block-uniformly) when
// every pivot is positive, i.e. A - shift I is positive definite.  The column
// below a pivot is scaled by the pivot's reciprocal (one FP64 division per
// step instead of one per entry); rinv is one shared-memory double of scratch
// (no static shared memory here: the callers' kernels opt in to the whole
// 227 KB as dynamic shared memory).
__device__ inline bool cholesky_lower(double *A, int R, double shift, int *flag, double *rinv) {
    const int tid = threadIdx.x, nth = blockDim.x;
    if (tid == 0) *flag = 1;
    for (int e = tid; e < R; e += nth) A[e * R + e] -= shift;
    __syncthreads();
    for (int k = 0; k < R; ++k) {
        if (tid == 0) {
            double d = A[k * R + k];
            if (!(d > 0.0)) *flag = 0;
#if FTL_CHOL_RSQRT
            const double r = d > 0.0 ? rsqrt(d) : 1.0;
            A[k * R + k] = d > 0.0 ? d * r : 1.0;
            *rinv = r;
#else
            const double l = d > 0.0 ? sqrt(d) : 1.0;
            A[k * R + k] = l;
            *rinv = 1.0 / l;
#endif
        }
        __syncthreads();
        if (*flag == 0) break;
        const double r = *rinv;
        for (int i = k + 1 + tid; i < R; i += nth) A[i * R + k] *= r;
        __syncthreads();
        const int m = R - k - 1;
        for (int w = tid; w < m * m; w += nth) {
            int i = k + 1 + w / m, jj = k + 1 + w % m;
            if (jj <= i) A[i * R + jj] -= A[i * R + k] * A[jj * R + k];
        }
        __syncthreads();
    }
    __syncthreads();
    return *flag != 0;
}

}  // namespace ftl
