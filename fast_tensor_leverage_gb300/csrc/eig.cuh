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
            // A <- A J and V <- V J (columns p, q of each rotated pair)
            for (int w = tid; w < half * R; w += nth) {
                int i = w / R, r = w - i * R;
                T s = csbuf[2 * i + 1];
                if (s == T(0)) continue;
                T c = csbuf[2 * i];
                int p = pqbuf[2 * i], q = pqbuf[2 * i + 1];
                T arp = A[r * R + p], arq = A[r * R + q];
                A[r * R + p] = c * arp - s * arq;
                A[r * R + q] = s * arp + c * arq;
                T vrp = V[r * R + p], vrq = V[r * R + q];
                V[r * R + p] = c * vrp - s * vrq;
                V[r * R + q] = s * vrp + c * vrq;
            }
            __syncthreads();
            // A <- J^T A (rows p, q)
            for (int w = tid; w < half * R; w += nth) {
                int i = w / R, col = w - i * R;
                T s = csbuf[2 * i + 1];
                if (s == T(0)) continue;
                T c = csbuf[2 * i];
                int p = pqbuf[2 * i], q = pqbuf[2 * i + 1];
                T apc = A[p * R + col], aqc = A[q * R + col];
                A[p * R + col] = c * apc - s * aqc;
                A[q * R + col] = s * apc + c * aqc;
            }
            __syncthreads();
            if (tid < half) {
                T s = csbuf[2 * tid + 1];
                if (s != T(0)) {
                    int p = pqbuf[2 * tid], q = pqbuf[2 * tid + 1];
                    A[p * R + q] = T(0);
                    A[q * R + p] = T(0);
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
            const double l = d > 0.0 ? sqrt(d) : 1.0;
            A[k * R + k] = l;
            *rinv = 1.0 / l;
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
