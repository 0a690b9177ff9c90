// Randomized CP-ALS on a sparse tensor: sampled-fiber dedup, weighted Gram
// and FP64 pseudo-inverse, sparse MTTKRP through sorted fiber keys, the
// normal-equation solve, column renormalisation and the fit.
//
// Reference semantics (vbharadwaj-bk/fast_tensor_leverage, cpp_ext/):
//   ALS::execute_ds_als_update        als.hpp:57-220
//   compute_pinv / compute_pinv_square common.h:228-323
//   SortIdxLookup ctor / execute_spmm  sort_lookup.hpp:33-132
//   SortIdxLookup::compute_residual_normsq, ATB_chain_prod_sum
//                                      sort_lookup.hpp:134-197, common.h:152-226
//   LowRankTensor::renormalize_columns low_rank_tensor.hpp:203-260
//   SortIdxLookup::execute_exact_mttkrp sort_lookup.hpp:199-254
//
// A fiber key is the mixed-radix number formed by the indices of every mode
// except j, first mode most significant -- exactly the lexicographic order
// of the reference's comparators on modes != j.  Sample indices are cast to
// uint32 first, as the reference does (als.hpp:79, sparse_tensor.hpp:106-109).
#include <algorithm>
#include <cstring>

#include "eig.cuh"

namespace ftl {


struct KeyRadix {
    int N, j;
    uint64_t mult[FTL_MAX_MODES];  // place value of mode k (0 for k == j)
};

static int make_radix(int N, const int64_t *dims, int j, KeyRadix &kr) {
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES, "fiber keys: N=%d outside [1, %d]", N, FTL_MAX_MODES);
    FTL_CHECK_ARG(dims != nullptr, "fiber keys: dims is NULL");
    kr.N = N;
    kr.j = j;
    // place values from the last mode upwards; the product of the dims of
    // the modes != j must stay below 2^63
    unsigned __int128 place = 1;
    for (int k = N - 1; k >= 0; --k) {
        FTL_CHECK_ARG(dims[k] >= 1, "fiber keys: dims[%d]=%lld", k, (long long)dims[k]);
        if (k == j) {
            kr.mult[k] = 0;
            continue;
        }
        kr.mult[k] = (uint64_t)place;
        place *= (unsigned __int128)dims[k];
        if (place > ((unsigned __int128)1 << 63))
            return fail(FTL_E_UNSUPPORTED,
                        "fiber keys: the product of the mode sizes other than mode %d exceeds 2^63", j);
    }
    for (int k = N; k < FTL_MAX_MODES; ++k) kr.mult[k] = 0;
    return FTL_OK;
}

// keys[i] = sum_k (uint32)idx(i, k) * mult[k]; idx element (i, k) at
// idx[i * si + k * sk] (row-major nnz x N tensors: si = N, sk = 1; the N x J
// sample layout: si = 1, sk = J).
template <typename I>
__global__ void keys_kernel(const I *__restrict__ idx, int64_t n, int64_t si, int64_t sk, KeyRadix kr,
                            uint64_t *__restrict__ keys) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t key = 0;
        for (int k = 0; k < kr.N; ++k)
            if (k != kr.j) key += (uint64_t)(uint32_t)idx[i * si + k * sk] * kr.mult[k];
        keys[i] = key;
    }
}

__global__ void gather_mode_kernel(const int64_t *__restrict__ perm, const uint32_t *__restrict__ idx,
                                   const double *__restrict__ vals, int64_t nnz, int N, int j,
                                   uint32_t *__restrict__ idxj, double *__restrict__ vout) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = perm[i];
        idxj[i] = idx[p * N + j];
        vout[i] = vals[p];
    }
}

static int grid_for(int64_t n, int threads = 256) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, (int64_t)num_sms() * 16));
}

// ------------------------------------------------------------------ dedup

constexpr uint64_t kEmpty = ~0ull;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    // splitmix64 finaliser
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__global__ void table_clear_kernel(uint64_t *keys, int32_t *first, int32_t *count, int64_t T) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < T; s += (int64_t)gridDim.x * blockDim.x) {
        keys[s] = kEmpty;
        first[s] = INT32_MAX;
        count[s] = 0;
    }
}

// Open addressing with linear probing; at most T probes (T >= 2 J, so a slot
// is always found).
__global__ void table_insert_kernel(const uint64_t *__restrict__ skeys, int64_t J, uint64_t *keys,
                                    int32_t *first, int32_t *count, int64_t T) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < J; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = skeys[i];
        uint64_t s = mix64(key) & (uint64_t)(T - 1);
        for (int64_t probe = 0; probe < T; ++probe) {
            unsigned long long prev = atomicCAS((unsigned long long *)&keys[s], (unsigned long long)kEmpty,
                                                (unsigned long long)key);
            if (prev == kEmpty || prev == key) {
                atomicAdd(&count[s], 1);
                atomicMin(&first[s], (int32_t)i);
                break;
            }
            s = (s + 1) & (uint64_t)(T - 1);
        }
    }
}

// Deterministic compaction in slot order, in two launches: the table is cut
// into slices of `slice` slots, one CTA each; table_count_kernel counts each
// slice's occupied slots, table_write_kernel offsets its slice by the counts
// of the slices before it and writes the unique keys in slot order.
__global__ void table_count_kernel(const uint64_t *__restrict__ keys, int64_t T, int64_t slice,
                                   int32_t *__restrict__ bcount) {
    __shared__ int warp_tot[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t b0 = blockIdx.x * slice, b1 = min(T, b0 + slice);
    int c = 0;
    for (int64_t s = b0 + tid; s < b1; s += blockDim.x) c += keys[s] != kEmpty ? 1 : 0;
    c = __reduce_add_sync(0xffffffffu, (unsigned)c);
    if (lane == 0) warp_tot[warp] = c;
    __syncthreads();
    if (tid == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_tot[w];
        bcount[blockIdx.x] = t;
    }
}

__global__ void table_write_kernel(const uint64_t *__restrict__ keys, const int32_t *__restrict__ first,
                                   const int32_t *__restrict__ count, int64_t T, int64_t slice,
                                   const int32_t *__restrict__ bcount, uint64_t *__restrict__ ukeys,
                                   int32_t *__restrict__ urep, int32_t *__restrict__ ucnt,
                                   int64_t *__restrict__ num_unique) {
    __shared__ int warp_tot[32];
    __shared__ int64_t base_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (warp == 0) {
        int64_t t = 0;
        for (int b = lane; b < (int)blockIdx.x; b += 32) t += bcount[b];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) base_s = t;
    }
    __syncthreads();
    const int64_t b0 = blockIdx.x * slice, b1 = min(T, b0 + slice);
    for (int64_t off = b0; off < b1; off += blockDim.x) {
        const int64_t s = off + tid;
        const int occ = (s < b1 && keys[s] != kEmpty) ? 1 : 0;
        const unsigned bal = __ballot_sync(0xffffffffu, occ);
        const int pre = __popc(bal & ((1u << lane) - 1));
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        int wbase = 0, total = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            if (w < warp) wbase += warp_tot[w];
            total += warp_tot[w];
        }
        if (occ) {
            const int64_t o = base_s + wbase + pre;
            ukeys[o] = keys[s];
            urep[o] = first[s];
            ucnt[o] = count[s];
        }
        __syncthreads();
        if (tid == 0) base_s += total;
        __syncthreads();
    }
    if (tid == 0 && blockIdx.x == gridDim.x - 1) *num_unique = base_s;
}

// Slice of the compaction: 2048 slots, doubled until there are at most 1024
// slices (T is a power of two >= 1024).
static int64_t compact_slice(int64_t T) {
    int64_t sl = 2048;
    while (T / sl > 1024) sl <<= 1;
    return sl;
}

static int64_t table_size_for(int64_t J) {
    int64_t T = 1024;
    while (T < 2 * J) T <<= 1;
    return T;
}

// -------------------------------------------------------- weighted Gram

// partial[b][e] = sum over this block's rows u of s_u * h_a h_b, e = packed
// (a, b); rows u < *n_rows (or n_rows_host), h row = lhs[row(u)], s_u =
// (w ? w[row(u)] : 1) * (cnt ? cnt[u] : 1).  Rows are staged 32 at a time
// with their scaled copy s_u h; each thread owns up to GRAM_EPT packed
// entries (thread t: entries t, t + blockDim, ...; up to 9 covers R = 128,
// 8256 entries, on 1024 threads) and adds one FMA per
// entry and row.  All-zero rows are skipped (they add exact zeros): most
// rows of a sampled-ALS factor are zero, and this is FP64 arithmetic at a
// low issue rate.
static int gram_threads(int R) {
    const int P = packed_size(R);
    return std::min(1024, (P + 31) / 32 * 32);
}

template <int GRAM_EPT>
__global__ void gram_partial_kernel(const double *__restrict__ lhs, const int32_t *__restrict__ rowidx,
                                    const double *__restrict__ w, const int32_t *__restrict__ cnt,
                                    const int64_t *__restrict__ n_rows_dev, int64_t n_rows_host, int R,
                                    double *__restrict__ partial) {
    extern __shared__ double hs[];  // 32 rows x R, 32 scaled rows x R
    __shared__ int nz[32];          // row has a nonzero entry
    const int P = packed_size(R);
    const int64_t n = n_rows_dev ? *n_rows_dev : n_rows_host;
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = blockIdx.x * per, r1 = min(n, r0 + per);
    double *hsc = hs + 32 * R;
    double acc[GRAM_EPT];
    int ea[GRAM_EPT], eb[GRAM_EPT];
#pragma unroll
    for (int t = 0; t < GRAM_EPT; ++t) {
        acc[t] = 0.0;
        const int e = threadIdx.x + t * blockDim.x;
        ea[t] = eb[t] = -1;
        if (e < P) {
            int a = 0, rem = e;
            while (rem >= R - a) {
                rem -= R - a;
                ++a;
            }
            ea[t] = a;
            eb[t] = a + rem;
        }
    }
    for (int64_t u0 = r0; u0 < r1; u0 += 32) {
        const int m = (int)min((int64_t)32, r1 - u0);
        __syncthreads();
        if (threadIdx.x < 32) nz[threadIdx.x] = 0;
        __syncthreads();
        for (int e = threadIdx.x; e < m * R; e += blockDim.x) {
            const int uu = e / R;
            const int64_t u = u0 + uu;
            const int64_t row = rowidx ? rowidx[u] : u;
            const double v = lhs[row * R + (e - uu * R)];
            const double su = (w ? w[row] : 1.0) * (cnt ? (double)cnt[u] : 1.0);
            hs[e] = v;
            hsc[e] = su * v;
            if (v != 0.0) nz[uu] = 1;
        }
        __syncthreads();
        for (int uu = 0; uu < m; ++uu) {
            if (!nz[uu]) continue;
            const double *hr = hs + uu * R;
            const double *hq = hsc + uu * R;
#pragma unroll
            for (int t = 0; t < GRAM_EPT; ++t)
                if (ea[t] >= 0) acc[t] = fma(hq[ea[t]], hr[eb[t]], acc[t]);
        }
    }
#pragma unroll
    for (int t = 0; t < GRAM_EPT; ++t)
        if (ea[t] >= 0) partial[(int64_t)blockIdx.x * P + threadIdx.x + t * blockDim.x] = acc[t];
}

// out (R x R, full symmetric) = sum of the partials; one warp per packed
// entry, lanes over the blocks.
__global__ void gram_reduce_kernel(const double *__restrict__ partial, int nblk, int R, double *__restrict__ out) {
    const int P = packed_size(R);
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int pe = wg; pe < P; pe += nw) {
        double s = 0.0;
        for (int k = lane; k < nblk; k += 32) s += partial[(int64_t)k * P + pe];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            int a = 0, rem = pe;
            while (rem >= R - a) {
                rem -= R - a;
                ++a;
            }
            const int b = a + rem;
            out[a * R + b] = s;
            out[b * R + a] = s;
        }
    }
}

// --------------------------------------------------------- pseudo-inverse

// compute_pinv_square (common.h:228-269): eigendecomposition of M (upper
// triangle), keep eigenpair v (ascending rank r) when r >= R - target and
// lambda > tol, out = sum_kept v v^T / lambda.  target = min(cap, R) with cap
// read from *rank_cap when given.
//
// When every eigenpair is kept (target = R) and M is safely positive
// definite, that sum is M^-1, computed here from the Cholesky factor M = L L^T
// as L^-T L^-1 (R sequential steps instead of Jacobi sweeps).  The fast path
// is taken when the factorisation succeeds and ||M^-1||_F < 1 / (2 tol): then
// lambda_min(M) = 1 / ||M^-1||_2 >= 1 / ||M^-1||_F > 2 tol, so the reference
// keeps every eigenpair too.  Otherwise M is reloaded and the Jacobi path
// runs.
__global__ void pinv_square_kernel(const double *__restrict__ M, int R, int target, const int64_t *rank_cap,
                                   double tol, double *__restrict__ out, double *vscratch) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int RR = R * R, tid = threadIdx.x, nth = blockDim.x;
    double *A = (double *)smem_raw;
    double *V = vscratch ? vscratch : A + RR;
    double *cs = A + (vscratch ? 1 : 2) * RR;
    int *pq = (int *)(cs + R + 2);
    int *order = pq + R + 2;
    int *flag = order + R;
    int tr = target;
    if (rank_cap) tr = (int)min((int64_t)R, *rank_cap);
    if (tr >= R) {
        for (int e = tid; e < RR; e += nth) {
            int a = e / R, b = e - a * R;
            A[e] = a <= b ? M[e] : M[b * R + a];
        }
        __syncthreads();
        // small R: the inverse itself by the sweep operator (-M^-1 in the
        // upper triangle); larger R: block-wide Cholesky factor, then column c
        // of X = L^-1 by forward substitution, into V
        const bool small = R <= 32 && nth * 2 >= R * (R + 1) / 2;
        bool chol;
        if (small) {
            chol = sweep_inverse_spd(A, R, cs + 1, flag);
        } else {
            chol = cholesky_lower(A, R, 0.0, flag, cs + 1);
            if (chol) {
                for (int c = tid; c < R; c += nth) {
                    for (int i = 0; i < c; ++i) V[i * R + c] = 0.0;
                    for (int i = c; i < R; ++i) {
                        double t = (i == c) ? 1.0 : 0.0;
                        for (int k = c; k < i; ++k) t -= A[i * R + k] * V[k * R + c];
                        V[i * R + c] = t / A[i * R + i];
                    }
                }
            }
            __syncthreads();
        }
        if (chol) {
            // out = X^T X (or the swept inverse); cs[0] accumulates ||out||_F^2
            if (tid == 0) cs[0] = 0.0;
            __syncthreads();
            double fro = 0.0;
            for (int e = tid; e < RR; e += nth) {
                int a = e / R, b = e - a * R;
                double t = 0.0;
                if (small) {
                    t = -A[min(a, b) * R + max(a, b)];  // the swept upper triangle, mirrored
                } else {
                    const int k0 = a > b ? a : b;
                    for (int k = k0; k < R; ++k) t += V[k * R + a] * V[k * R + b];
                }
                out[e] = t;
                fro += t * t;
            }
            for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
            if ((tid & 31) == 0) atomicAdd(cs, fro);
            __syncthreads();
            const bool ok = cs[0] == cs[0] && 4.0 * tol * tol * cs[0] < 1.0;
            __syncthreads();
            if (ok) return;
        }
        __syncthreads();
    }
    for (int e = tid; e < RR; e += nth) {
        int a = e / R, b = e - a * R;
        A[e] = a <= b ? M[e] : M[b * R + a];
    }
    __syncthreads();
    jacobi_eigen<double>(A, V, R, cs, pq, flag);
    sort_ascending<double>(A, R, order);
    for (int e = tid; e < RR; e += nth) {
        int a = e / R, b = e - a * R;
        double s = 0.0;
        for (int r = 0; r < R; ++r) {
            const int v = order[r];
            const double lam = A[v * R + v];
            if (r >= R - tr && lam > tol) s += (V[a * R + v] / sqrt(lam)) * (V[b * R + v] / sqrt(lam));
        }
        out[e] = s;
    }
}

// ------------------------------------------------------------- MTTKRP

// One warp per query: lower_bound of the query's fiber key in the sorted
// keys, then out[idx_j, :] += value * scale * lhs[row, :] for every nonzero
// of the fiber (SortIdxLookup::execute_spmm, sort_lookup.hpp:69-132).
__global__ void mttkrp_kernel(const uint64_t *__restrict__ skeys, const uint32_t *__restrict__ sidx,
                              const double *__restrict__ svals, int64_t nnz, const uint64_t *__restrict__ qkeys,
                              const int32_t *__restrict__ qrow, const double *__restrict__ w,
                              const int32_t *__restrict__ cnt, const int64_t *__restrict__ nq_dev, int64_t nq_host,
                              const double *__restrict__ lhs, int R, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nq = nq_dev ? *nq_dev : nq_host;
    for (int64_t q = warp; q < nq; q += nwarps) {
        const uint64_t key = qkeys[q];
        int64_t lo = 0, hi = nnz;
        while (lo < hi) {
            int64_t mid = lo + (hi - lo) / 2;
            if (skeys[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        if (lo >= nnz || skeys[lo] != key) continue;
        const int64_t row = qrow ? qrow[q] : q;
        const double scale = (w ? w[row] : 1.0) * (cnt ? (double)cnt[q] : 1.0);
        for (int64_t z = lo; z < nnz && skeys[z] == key; ++z) {
            const double v = svals[z] * scale;
            double *o = out + (int64_t)sidx[z] * R;
            for (int col = lane; col < R; col += 32) atomicAdd(o + col, v * lhs[row * R + col]);
        }
    }
}

// Row-grouped MTTKRP (the same sum as mttkrp_kernel): nonzeros sorted by
// their mode-j index, each carrying its row and fiber key.  The sorted
// nonzeros are cut into fixed chunks of MTT_CHUNK, one warp per chunk, so
// work is balanced however skewed the rows are.  Lanes probe a table of the
// unique fibers for 32 nonzeros at a time; hits are applied in nonzero order
// to a per-row accumulator (lane = column) that is flushed with one atomic
// add per column whenever the row changes -- a handful of atomics per chunk
// instead of R per touched nonzero.
constexpr int MTT_CHUNK = 512;
#ifndef FTL_MTT_MINB
#define FTL_MTT_MINB 4
#endif
#ifndef FTL_MTT_G
#define FTL_MTT_G 4
#endif

// Probe table of the unique fibers: 16-byte slots {fiber key, unique index},
// open addressing with linear probing, at most 1/4 full (slots = power of two
// >= 4 J), Fibonacci hashing (key * 2^64/phi, top bits).
constexpr uint64_t kFib = 0x9E3779B97F4A7C15ull;

static int64_t probe_slots_for(int64_t J) {
    int64_t T = 1024;
    while (T < 4 * J) T <<= 1;
    return T;
}

static int log2_exact(int64_t T) {
    int l = 0;
    while ((int64_t(1) << l) < T) ++l;
    return l;
}

static int padded_rank(int R) { return (R + 3) & ~3; }

__global__ void probe_insert_kernel(const uint64_t *__restrict__ ukeys, const int64_t *__restrict__ nq_dev,
                                    int64_t nq_host, ulonglong2 *__restrict__ pt, int64_t T, int shift) {
    const int64_t nq = nq_dev ? *nq_dev : nq_host;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nq; u += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = ukeys[u];
        uint64_t s = (key * kFib) >> shift;
        // the keys are distinct, so a slot is either free or holds another key
        for (int64_t probe = 0; probe < T; ++probe) {
            const unsigned long long prev =
                atomicCAS((unsigned long long *)&pt[s].x, (unsigned long long)kEmpty, (unsigned long long)key);
            if (prev == kEmpty) {
                pt[s].y = (unsigned long long)u;
                break;
            }
            s = (s + 1) & (uint64_t)(T - 1);
        }
    }
}

// hs[u, c] = s_u lhs[rep(u), c] with s_u = (w ? w[rep(u)] : 1) (cnt ? cnt[u] : 1),
// row stride Rp (columns R..Rp-1 zero).
__global__ void scaled_unique_rows_kernel(const int32_t *__restrict__ urep, const int32_t *__restrict__ ucnt,
                                          const double *__restrict__ w, const int64_t *__restrict__ nq_dev,
                                          int64_t nq_host, const double *__restrict__ lhs, int R, int Rp,
                                          double *__restrict__ hs) {
    const int64_t nq = nq_dev ? *nq_dev : nq_host;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nq * Rp;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = e / Rp;
        const int c = (int)(e - u * Rp);
        double v = 0.0;
        if (c < R) {
            const int64_t rep = urep[u];
            const double sc = (w ? w[rep] : 1.0) * (ucnt ? (double)ucnt[u] : 1.0);
            v = sc * lhs[rep * R + c];
        }
        hs[e] = v;
    }
}

// One warp per chunk.  The key, row and value of the next 32 nonzeros are
// loaded before the current 32 are probed, so the streaming loads overlap
// the probes and the hit processing (a deeper pipeline that also issued the
// next batch's first probe early measured no faster).  Hits are applied G at a time: their
// scaled rows (lane = column, CPL columns per lane) are loaded together before
// the ordered accumulation.
template <int CPL, int G>
__global__ void __launch_bounds__(256, FTL_MTT_MINB)
    mttkrp_rows_kernel(const int32_t *__restrict__ rrows, const uint64_t *__restrict__ rkeys,
                       const double *__restrict__ rvals, int64_t nnz, const ulonglong2 *__restrict__ pt, int64_t T,
                       int shift, const double *__restrict__ hs, int R, int Rp, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = (nnz + MTT_CHUNK - 1) / MTT_CHUNK;
    const uint64_t mask = (uint64_t)(T - 1);
    for (int64_t ch = gw; ch < nchunks; ch += nw) {
        const int64_t z0 = ch * MTT_CHUNK, z1 = min(nnz, z0 + MTT_CHUNK);
        double acc[CPL];
#pragma unroll
        for (int c = 0; c < CPL; ++c) acc[c] = 0.0;
        int32_t cur = -1;  // row held in acc (warp-uniform)
        uint64_t nkey = kEmpty;
        int32_t nrow = 0;
        double nval = 0.0;
        if (z0 + lane < z1) {
            nkey = rkeys[z0 + lane];
            nrow = rrows[z0 + lane];
            nval = rvals[z0 + lane];
        }
        for (int64_t zb = z0; zb < z1; zb += 32) {
            const uint64_t key = nkey;
            const int32_t row = nrow;
            const double val = nval;
            const int64_t zn = zb + 32 + lane;
            nkey = kEmpty;
            if (zn < z1) {
                nkey = rkeys[zn];
                nrow = rrows[zn];
                nval = rvals[zn];
            }
            int32_t u = -1;
            if (key != kEmpty) {
                uint64_t s = (key * kFib) >> shift;
                for (int64_t probe = 0; probe < T; ++probe) {
                    const ulonglong2 e = pt[s];
                    if (e.x == key) {
                        u = (int32_t)e.y;
                        break;
                    }
                    if (e.x == kEmpty) break;
                    s = (s + 1) & mask;
                }
            }
            unsigned hits = __ballot_sync(0xffffffffu, u >= 0);
            while (hits) {
                int32_t hu[G], hrow[G];
                double hval[G], hv[G][CPL];
                int nh = 0;
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    int src = 0;
                    if (hits) {
                        src = __ffs(hits) - 1;
                        hits &= hits - 1;
                        nh = g + 1;
                    }
                    hu[g] = __shfl_sync(0xffffffffu, u, src);
                    hrow[g] = __shfl_sync(0xffffffffu, row, src);
                    hval[g] = __shfl_sync(0xffffffffu, val, src);
                }
#pragma unroll
                for (int g = 0; g < G; ++g) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        const int col = lane + 32 * c;
                        hv[g][c] = (g < nh && col < Rp) ? hs[(int64_t)hu[g] * Rp + col] : 0.0;
                    }
                }
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (g < nh) {
                        if (hrow[g] != cur) {
                            if (cur >= 0) {
#pragma unroll
                                for (int c = 0; c < CPL; ++c) {
                                    const int col = lane + 32 * c;
                                    if (col < R) atomicAdd(out + (int64_t)cur * R + col, acc[c]);
                                    acc[c] = 0.0;
                                }
                            }
                            cur = hrow[g];
                        }
#pragma unroll
                        for (int c = 0; c < CPL; ++c) acc[c] = fma(hval[g], hv[g][c], acc[c]);
                    }
                }
            }
        }
        if (cur >= 0) {
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                const int col = lane + 32 * c;
                if (col < R) atomicAdd(out + (int64_t)cur * R + col, acc[c]);
            }
        }
    }
}

// Two-phase form of mttkrp_rows_kernel (the same sums in the same order): a
// warp first probes the whole chunk, UNR batches of 32 nonzeros at a time
// (their keys, rows, values and first probes all in flight together), and
// appends the hits (unique index, row, value) to its shared-memory list in
// nonzero order; it then applies the hits G at a time, loading the G scaled
// rows together.  The probes and the row loads of a chunk overlap instead of
// alternating batch by batch.
constexpr int MTT2_CHUNK = 256;
#ifndef FTL_MTT2_UNR
#define FTL_MTT2_UNR 4
#endif
#ifndef FTL_MTT2_G
#define FTL_MTT2_G 8
#endif

struct HitEntry {
    int32_t u, row;
    double val;
};

#ifndef FTL_MTT2_MINB
#define FTL_MTT2_MINB 4
#endif
template <int CPL, int G, int UNR>
__global__ void __launch_bounds__(256, FTL_MTT2_MINB)
    mttkrp_rows2_kernel(const int32_t *__restrict__ rrows, const uint64_t *__restrict__ rkeys,
                        const double *__restrict__ rvals, int64_t nnz, const ulonglong2 *__restrict__ pt, int64_t T,
                        int shift, const double *__restrict__ hs, int R, int Rp, double *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    HitEntry *hits = reinterpret_cast<HitEntry *>(smem_raw) + (threadIdx.x >> 5) * MTT2_CHUNK;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t nchunks = (nnz + MTT2_CHUNK - 1) / MTT2_CHUNK;
    const uint64_t mask = (uint64_t)(T - 1);
    const unsigned lt = (1u << lane) - 1u;
    for (int64_t ch = gw; ch < nchunks; ch += nw) {
        const int64_t z0 = ch * MTT2_CHUNK, z1 = min(nnz, z0 + MTT2_CHUNK);
        int nh = 0;
        for (int64_t zb = z0; zb < z1; zb += 32 * UNR) {
            uint64_t key[UNR], slot[UNR];
            int32_t row[UNR];
            double val[UNR];
            ulonglong2 e[UNR];
#pragma unroll
            for (int q = 0; q < UNR; ++q) {
                const int64_t z = zb + 32 * q + lane;
                key[q] = kEmpty;
                row[q] = 0;
                val[q] = 0.0;
                if (z < z1) {
                    key[q] = rkeys[z];
                    row[q] = rrows[z];
                    val[q] = rvals[z];
                }
            }
#pragma unroll
            for (int q = 0; q < UNR; ++q) {
                slot[q] = (key[q] * kFib) >> shift;
                e[q] = make_ulonglong2(kEmpty, 0);
                if (key[q] != kEmpty) e[q] = pt[slot[q]];
            }
#pragma unroll
            for (int q = 0; q < UNR; ++q) {
                int32_t u = -1;
                if (key[q] != kEmpty) {
                    uint64_t sl = slot[q];
                    ulonglong2 x = e[q];
                    for (int64_t probe = 0; probe < T; ++probe) {
                        if (x.x == key[q]) {
                            u = (int32_t)x.y;
                            break;
                        }
                        if (x.x == kEmpty) break;
                        sl = (sl + 1) & mask;
                        x = pt[sl];
                    }
                }
                const unsigned b = __ballot_sync(0xffffffffu, u >= 0);
                if (u >= 0) {
                    HitEntry &h = hits[nh + __popc(b & lt)];
                    h.u = u;
                    h.row = row[q];
                    h.val = val[q];
                }
                nh += __popc(b);
            }
        }
        __syncwarp();
        double acc[CPL];
#pragma unroll
        for (int c = 0; c < CPL; ++c) acc[c] = 0.0;
        int32_t cur = -1;  // row held in acc (warp-uniform)
        for (int g0 = 0; g0 < nh; g0 += G) {
            int32_t hu[G], hrow[G];
            double hval[G], hv[G][CPL];
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const bool ok = g0 + g < nh;
                hu[g] = ok ? hits[g0 + g].u : 0;
                hrow[g] = ok ? hits[g0 + g].row : -1;
                hval[g] = ok ? hits[g0 + g].val : 0.0;
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
#pragma unroll
                for (int c = 0; c < CPL; ++c) {
                    const int col = lane + 32 * c;
                    hv[g][c] = (g0 + g < nh && col < Rp) ? hs[(int64_t)hu[g] * Rp + col] : 0.0;
                }
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (g0 + g < nh) {
                    if (hrow[g] != cur) {
                        if (cur >= 0) {
#pragma unroll
                            for (int c = 0; c < CPL; ++c) {
                                const int col = lane + 32 * c;
                                if (col < R) atomicAdd(out + (int64_t)cur * R + col, acc[c]);
                                acc[c] = 0.0;
                            }
                        }
                        cur = hrow[g];
                    }
#pragma unroll
                    for (int c = 0; c < CPL; ++c) acc[c] = fma(hval[g], hv[g][c], acc[c]);
                }
            }
        }
        if (cur >= 0) {
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                const int col = lane + 32 * c;
                if (col < R) atomicAdd(out + (int64_t)cur * R + col, acc[c]);
            }
        }
        __syncwarp();  // the list is rewritten by the next chunk
    }
}

// ---------------------------------------------------- range finder (rrf)

// Standard normals of one fiber, two columns per Philox4x32-10 block:
// block p of fiber key f in mode j = Philox(counter (f lo, f hi, p, j), key
// seed); u1 = ((x0 >> 8) + 1) 2^-24 in (0, 1], u2 = (x1 >> 8) 2^-24 in [0, 1)
// (exact in FP32), r = sqrt(-2 ln u1), columns 2p and 2p+1 = r cos(2 pi u2),
// r sin(2 pi u2) (Box-Muller, FP32).
__device__ __forceinline__ void fiber_normals(uint64_t seed, uint32_t mode, uint64_t key, uint32_t p, float &z0,
                                              float &z1) {
    uint32_t c[4] = {(uint32_t)key, (uint32_t)(key >> 32), p, mode};
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        philox_round(c, k);
        k[0] += 0x9E3779B9u;
        k[1] += 0xBB67AE85u;
    }
    const float u1 = (float)((c[0] >> 8) + 1u) * (1.0f / 16777216.0f);
    const float u2 = (float)(c[1] >> 8) * (1.0f / 16777216.0f);
    const float r = sqrtf(-2.0f * logf(u1));
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    z0 = r * cs;
    z1 = r * sn;
}

// out[idx_j(z), :] += val(z) * g(fiber(z)) over the nonzeros sorted by their
// mode-j index (SortIdxLookup::execute_rrf, sort_lookup.hpp:262-353: one
// Gaussian R-vector per fiber).  Chunks of MTT_CHUNK nonzeros per warp, lane
// l owns column pairs l, l + 32, ...; per-row accumulation, one atomic add
// per column when the row changes.
constexpr int RRF_CHUNK = 512;

__global__ void rrf_rows_kernel(const int32_t *__restrict__ rrows, const uint64_t *__restrict__ rkeys,
                                const double *__restrict__ rvals, int64_t nnz, int R, uint64_t seed, uint32_t mode,
                                double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    constexpr int PPL = (FTL_MAX_RANK / 2 + 31) / 32;  // column pairs per lane
    const int npairs = (R + 1) / 2;
    const int64_t nchunks = (nnz + RRF_CHUNK - 1) / RRF_CHUNK;
    for (int64_t ch = gw; ch < nchunks; ch += nw) {
        const int64_t z0 = ch * RRF_CHUNK, z1 = min(nnz, z0 + RRF_CHUNK);
        double acc[2 * PPL];
#pragma unroll
        for (int c = 0; c < 2 * PPL; ++c) acc[c] = 0.0;
        int32_t cur = -1;
        for (int64_t z = z0; z < z1; ++z) {
            const int32_t row = rrows[z];
            const uint64_t key = rkeys[z];
            const double v = rvals[z];
            if (row != cur) {
                if (cur >= 0) {
#pragma unroll
                    for (int q = 0; q < PPL; ++q) {
                        const int pp = lane + 32 * q;
                        if (2 * pp < R) atomicAdd(out + (int64_t)cur * R + 2 * pp, acc[2 * q]);
                        if (2 * pp + 1 < R) atomicAdd(out + (int64_t)cur * R + 2 * pp + 1, acc[2 * q + 1]);
                        acc[2 * q] = acc[2 * q + 1] = 0.0;
                    }
                }
                cur = row;
            }
#pragma unroll
            for (int q = 0; q < PPL; ++q) {
                const int pp = lane + 32 * q;
                if (pp < npairs) {
                    float g0, g1;
                    fiber_normals(seed, mode, key, (uint32_t)pp, g0, g1);
                    acc[2 * q] = fma(v, (double)g0, acc[2 * q]);
                    acc[2 * q + 1] = fma(v, (double)g1, acc[2 * q + 1]);
                }
            }
        }
        if (cur >= 0) {
#pragma unroll
            for (int q = 0; q < PPL; ++q) {
                const int pp = lane + 32 * q;
                if (2 * pp < R) atomicAdd(out + (int64_t)cur * R + 2 * pp, acc[2 * q]);
                if (2 * pp + 1 < R) atomicAdd(out + (int64_t)cur * R + 2 * pp + 1, acc[2 * q + 1]);
            }
        }
    }
}

// ------------------------------------------------------ solve / renorm

// U = B pinv (pinv R x R symmetric) row by row; an all-zero row of B (a row
// no sampled fiber touched) is written as zeros without arithmetic.
__global__ void solve_rows_kernel(const double *__restrict__ B, const double *__restrict__ pinv, int64_t I, int R,
                                  double *__restrict__ U) {
    extern __shared__ double sm[];
    double *ps = sm;               // R x R
    double *bs = sm + R * R;       // blockDim.x rows x R (row-major)
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) ps[e] = pinv[e];
    for (int64_t r0 = (int64_t)blockIdx.x * blockDim.x; r0 < I; r0 += (int64_t)gridDim.x * blockDim.x) {
        const int m = (int)min((int64_t)blockDim.x, I - r0);
        __syncthreads();
        for (int e = threadIdx.x; e < m * R; e += blockDim.x) bs[e] = B[r0 * R + e];
        __syncthreads();
        if (threadIdx.x < m) {
            const double *b = bs + threadIdx.x * R;
            bool any = false;
            for (int c = 0; c < R; ++c) any |= (b[c] != 0.0);
            double *o = bs + threadIdx.x * R;
            if (any) {
                double tmp[FTL_MAX_RANK];
                for (int c = 0; c < R; ++c) tmp[c] = b[c];
                for (int c = 0; c < R; ++c) {
                    double s = 0.0;
                    for (int k = 0; k < R; ++k) s = fma(tmp[k], ps[k * R + c], s);
                    o[c] = s;
                }
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < m * R; e += blockDim.x) U[r0 * R + e] = bs[e];
    }
}

// Thread t owns column t % R of rows t / R, t / R + rows_per_pass, ... (a
// block covers rows_per_pass whole rows per step, so loads are contiguous).
__global__ void colsq_partial_kernel(const double *__restrict__ U, int64_t I, int R, double *__restrict__ partial) {
    const int tid = threadIdx.x;
    const int rows_per_pass = blockDim.x / R;
    double acc = 0.0;
    const int col = tid % R, r_in = tid / R;
    if (r_in < rows_per_pass) {
        const int64_t step = (int64_t)gridDim.x * rows_per_pass;
#pragma unroll 4
        for (int64_t r = (int64_t)blockIdx.x * rows_per_pass + r_in; r < I; r += step) {
            double x = U[r * R + col];
            acc = fma(x, x, acc);
        }
    }
    __shared__ double red[1024];
    red[tid] = (r_in < rows_per_pass) ? acc : 0.0;
    __syncthreads();
    if (tid < R) {
        double s = 0.0;
        for (int k = 0; k < rows_per_pass; ++k) s += red[k * R + tid];
        partial[(int64_t)blockIdx.x * R + tid] = s;
    }
}

// norms: sqrt of the column sums, <= 1e-7 -> 1 (low_rank_tensor.hpp:229-238);
// one warp per column, lanes over the block partials.
__global__ void colnorm_finish_kernel(const double *__restrict__ partial, int nblk, int R, double *__restrict__ norms) {
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int c = threadIdx.x >> 5; c < R; c += nw) {
        double s = 0.0;
        for (int k = lane; k < nblk; k += 32) s += partial[(int64_t)k * R + c];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            const double n = sqrt(s);
            norms[c] = n <= 1e-7 ? 1.0 : n;
        }
    }
}

// U /= norms per column, as a multiplication by the reciprocal (one rounding
// more than the reference's division; an FP64 division per entry would cost
// ~10x the FP64 issue of the multiply on this GPU).
__global__ void colscale_kernel(double *__restrict__ U, int64_t I, int R, const double *__restrict__ norms) {
    __shared__ double inv[FTL_MAX_RANK];
    for (int c = threadIdx.x; c < R; c += blockDim.x) inv[c] = 1.0 / norms[c];
    __syncthreads();
    // same row ownership as colsq_partial_kernel: no per-element index division
    const int rows_per_pass = blockDim.x / R;
    const int col = threadIdx.x % R, r_in = threadIdx.x / R;
    if (r_in >= rows_per_pass) return;
    const double f = inv[col];
    const int64_t step = (int64_t)gridDim.x * rows_per_pass;
#pragma unroll 4
    for (int64_t r = (int64_t)blockIdx.x * rows_per_pass + r_in; r < I; r += step) U[r * R + col] *= f;
}

// ------------------------------------------------------------ fit terms

struct FactorPtrs {
    const double *U[FTL_MAX_MODES];
};

// partial[b] = sum over this block's nonzeros of v^2 - 2 v model(idx), model
// = sum_r sigma_r prod_k U_k[idx_k, r] (sort_lookup.hpp:183-191); one warp
// per nonzero, lanes over r.
__global__ void residual_partial_kernel(const uint32_t *__restrict__ idx, const double *__restrict__ vals,
                                        int64_t nnz, int N, FactorPtrs fp, const double *__restrict__ sigma,
                                        int R, double *__restrict__ partial) {
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double acc = 0.0;
    for (int64_t z = gw; z < nnz; z += nw) {
        double m = 0.0;
        for (int r = lane; r < R; r += 32) {
            double p = sigma[r];
            for (int k = 0; k < N; ++k) p *= fp.U[k][(int64_t)idx[z * N + k] * R + r];
            m += p;
        }
        m = warp_sum(m);
        const double v = vals[z];
        if (lane == 0) acc += v * v - 2.0 * m * v;
    }
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        partial[blockIdx.x] = s;
    }
}

// The same sum with one thread per nonzero (N a template constant, so the N
// row pointers stay in registers): R x N FP64 products per nonzero as lane
// operations.  The warp-per-nonzero form above spends most of its FP64 issue
// on the warp reduction of each nonzero, and the FP64 pipe (one warp
// instruction per 16 cycles per SM) is what bounds this pass.
template <int N>
__global__ void residual_thread_kernel(const uint32_t *__restrict__ idx, const double *__restrict__ vals,
                                       int64_t nnz, FactorPtrs fp, const double *__restrict__ sigma, int R,
                                       double *__restrict__ partial) {
    __shared__ double sig[FTL_MAX_RANK];
    __shared__ double red[32];
    for (int r = threadIdx.x; r < R; r += blockDim.x) sig[r] = sigma[r];
    __syncthreads();
    double acc = 0.0;
    for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < nnz; z += (int64_t)gridDim.x * blockDim.x) {
        const double *row[N];
#pragma unroll
        for (int k = 0; k < N; ++k) row[k] = fp.U[k] + (int64_t)idx[z * N + k] * R;
        double m = 0.0;
        for (int r = 0; r < R; ++r) {
            double p = sig[r];
#pragma unroll
            for (int k = 0; k < N; ++k) p *= row[k][r];
            m += p;
        }
        const double v = vals[z];
        acc += v * v - 2.0 * m * v;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        partial[blockIdx.x] = t;
    }
}

// *out = sum of the n partials in a fixed order (lane-strided sums, then a
// fixed shuffle tree): one warp, so the result does not depend on timing.
__global__ void sum_kernel(const double *__restrict__ partial, int n, double *__restrict__ out) {
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    double s = 0.0;
    for (int k = threadIdx.x; k < n; k += 32) s += partial[k];
    s = warp_sum(s);
    if (threadIdx.x == 0) *out = s;
}

__global__ void sumsq_partial_kernel(const double *__restrict__ v, int64_t n, double *__restrict__ partial) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc = fma(v[i], v[i], acc);
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        partial[blockIdx.x] = s;
    }
}

// Exact MTTKRP (sort_lookup.hpp:199-254): out[idx_j] += v * prod_{k != j} U_k[idx_k]
__global__ void exact_mttkrp_kernel(const uint32_t *__restrict__ idx, const double *__restrict__ vals, int64_t nnz,
                                    int N, int j, FactorPtrs fp, int R, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t z = gw; z < nnz; z += nw) {
        const double v = vals[z];
        double *o = out + (int64_t)idx[z * N + j] * R;
        for (int r = lane; r < R; r += 32) {
            double p = 1.0;
            for (int k = 0; k < N; ++k)
                if (k != j) p *= fp.U[k][(int64_t)idx[z * N + k] * R + r];
            atomicAdd(o + r, v * p);
        }
    }
}

struct GramPtrs {
    const double *G[FTL_MAX_MODES];
};

// M = (sa sb^T) o prod_{k != exclude} G_k (ATB_chain_prod, common.h:152-213);
// optionally out_sum = sum of M's entries (ATB_chain_prod_sum, :215-226).
__global__ void gram_hadamard_kernel(GramPtrs gp, int N, int R, int exclude, const double *__restrict__ sa,
                                     const double *__restrict__ sb, double *__restrict__ out_mat,
                                     double *__restrict__ out_sum) {
    __shared__ double red[1024];
    double acc = 0.0;
    for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        int a = e / R, b = e - a * R;
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

}  // namespace ftl

using namespace ftl;

// ============================================================== C ABI

extern "C" int ftl_gram_hadamard(const double *const *grams_dev, int N, int R, int exclude, const double *sigma_a,
                                 const double *sigma_b, double *out_mat, double *out_sum, void *stream) {
    FTL_CHECK_ARG(grams_dev && (out_mat || out_sum), "ftl_gram_hadamard: null pointer");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && R >= 1 && R <= FTL_MAX_RANK, "ftl_gram_hadamard: bad shape");
    GramPtrs gp;
    for (int k = 0; k < FTL_MAX_MODES; ++k) gp.G[k] = k < N ? grams_dev[k] : nullptr;
    gram_hadamard_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(gp, N, R, exclude, sigma_a, sigma_b, out_mat, out_sum);
    return check_launch("gram_hadamard_kernel");
}

extern "C" int ftl_fiber_keys(const void *idx, int idx_is_u64, int64_t n, int64_t stride_item, int64_t stride_mode,
                              int N, const int64_t *dims, int j, uint64_t *keys_out, void *stream) {
    FTL_CHECK_ARG(idx && keys_out, "ftl_fiber_keys: null pointer");
    FTL_CHECK_ARG(n >= 0, "ftl_fiber_keys: n=%lld", (long long)n);
    KeyRadix kr;
    int rc = make_radix(N, dims, j, kr);
    if (rc) return rc;
    if (n == 0) return FTL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (idx_is_u64)
        keys_kernel<uint64_t><<<grid_for(n), 256, 0, st>>>((const uint64_t *)idx, n, stride_item, stride_mode, kr, keys_out);
    else
        keys_kernel<uint32_t><<<grid_for(n), 256, 0, st>>>((const uint32_t *)idx, n, stride_item, stride_mode, kr, keys_out);
    return check_launch("keys_kernel");
}

extern "C" int ftl_sparse_gather(const int64_t *perm, const uint32_t *idx, const double *vals, int64_t nnz, int N,
                                 int j, uint32_t *idxj_out, double *vals_out, void *stream) {
    FTL_CHECK_ARG(perm && idx && vals && idxj_out && vals_out, "ftl_sparse_gather: null pointer");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && j >= 0 && j < N, "ftl_sparse_gather: bad N=%d j=%d", N, j);
    if (nnz == 0) return FTL_OK;
    gather_mode_kernel<<<grid_for(nnz), 256, 0, (cudaStream_t)stream>>>(perm, idx, vals, nnz, N, j, idxj_out, vals_out);
    return check_launch("gather_mode_kernel");
}

extern "C" int ftl_dedup_workspace_bytes(int64_t J, size_t *out) {
    FTL_CHECK_ARG(out && J >= 1 && J <= INT32_MAX / 2, "ftl_dedup_workspace_bytes: bad J=%lld", (long long)J);
    // slot keys, first, count; then one count per compaction slice
    const size_t T = (size_t)table_size_for(J);
    *out = T * (sizeof(uint64_t) + 2 * sizeof(int32_t)) + (size_t)(T / compact_slice(T) + 1) * sizeof(int32_t);
    return FTL_OK;
}

extern "C" int ftl_dedup(const uint64_t *keys, int64_t J, void *workspace, size_t ws_bytes, uint64_t *ukeys,
                         int32_t *urep, int32_t *ucnt, int64_t *num_unique, void *stream) {
    FTL_CHECK_ARG(keys && workspace && ukeys && urep && ucnt && num_unique, "ftl_dedup: null pointer");
    size_t need = 0;
    int rc = ftl_dedup_workspace_bytes(J, &need);
    if (rc) return rc;
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_dedup: workspace %zu < %zu bytes", ws_bytes, need);
    const int64_t T = table_size_for(J);
    uint64_t *tk = (uint64_t *)workspace;
    int32_t *tf = (int32_t *)(tk + T);
    int32_t *tc = tf + T;
    int32_t *bc = tc + T;
    const int64_t slice = compact_slice(T);
    const int nsl = (int)((T + slice - 1) / slice);
    cudaStream_t st = (cudaStream_t)stream;
    table_clear_kernel<<<grid_for(T), 256, 0, st>>>(tk, tf, tc, T);
    table_insert_kernel<<<grid_for(J), 256, 0, st>>>(keys, J, tk, tf, tc, T);
    table_count_kernel<<<nsl, 256, 0, st>>>(tk, T, slice, bc);
    table_write_kernel<<<nsl, 256, 0, st>>>(tk, tf, tc, T, slice, bc, ukeys, urep, ucnt, num_unique);
    return check_launch("dedup kernels");
}

extern "C" int ftl_mttkrp_rows_workspace_bytes(int64_t J, int R, size_t *out) {
    FTL_CHECK_ARG(out && J >= 1 && J <= INT32_MAX / 4 && R >= 1 && R <= FTL_MAX_RANK,
                  "ftl_mttkrp_rows_workspace_bytes: bad J=%lld or R=%d", (long long)J, R);
    // probe table, then the scaled unique rows (16-byte aligned: slots are 16 B)
    *out = (size_t)probe_slots_for(J) * sizeof(ulonglong2) + (size_t)J * padded_rank(R) * sizeof(double);
    return FTL_OK;
}

extern "C" int ftl_sparse_mttkrp_rows(const int32_t *row_idx, const uint64_t *row_keys, const double *row_vals,
                                      int64_t nnz, const uint64_t *ukeys, const int32_t *urep, const int32_t *ucnt,
                                      const int64_t *num_unique_dev, int64_t num_unique, int64_t J, const double *w,
                                      const double *h, int R, void *workspace, size_t ws_bytes, double *out,
                                      int64_t I_j, void *stream) {
    FTL_CHECK_ARG(row_idx && row_keys && row_vals && ukeys && urep && h && workspace && out,
                  "ftl_sparse_mttkrp_rows: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && I_j >= 1 && J >= 1 && nnz >= 0 && num_unique >= 0 &&
                      num_unique <= J,
                  "ftl_sparse_mttkrp_rows: bad shape");
    size_t need = 0;
    int rc = ftl_mttkrp_rows_workspace_bytes(J, R, &need);
    if (rc) return rc;
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_sparse_mttkrp_rows: workspace %zu < %zu bytes", ws_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t err = cudaMemsetAsync(out, 0, (size_t)I_j * R * sizeof(double), st);
    if (err != cudaSuccess) return fail(FTL_E_CUDA, "ftl_sparse_mttkrp_rows: memset: %s", cudaGetErrorString(err));
    if (nnz == 0) return FTL_OK;
    const int64_t T = probe_slots_for(J);
    const int shift = 64 - log2_exact(T);
    const int Rp = padded_rank(R);
    ulonglong2 *pt = (ulonglong2 *)workspace;
    double *hs = (double *)(pt + T);
    err = cudaMemsetAsync(pt, 0xFF, (size_t)T * sizeof(ulonglong2), st);
    if (err != cudaSuccess) return fail(FTL_E_CUDA, "ftl_sparse_mttkrp_rows: memset: %s", cudaGetErrorString(err));
    probe_insert_kernel<<<grid_for(J), 256, 0, st>>>(ukeys, num_unique_dev, num_unique, pt, T, shift);
    scaled_unique_rows_kernel<<<grid_for(J * Rp), 256, 0, st>>>(urep, ucnt, w, num_unique_dev, num_unique, h, R, Rp,
                                                                 hs);
#ifndef FTL_MTT_TWO_PHASE
#define FTL_MTT_TWO_PHASE 1
#endif
    if (FTL_MTT_TWO_PHASE && R <= 32) {
        const int64_t nch2 = (nnz + MTT2_CHUNK - 1) / MTT2_CHUNK;
        int blocks2 = (int)std::min<int64_t>((nch2 * 32 + 255) / 256, (int64_t)num_sms() * 32);
        blocks2 = std::max(blocks2, 1);
        const size_t smem2 = (size_t)8 * MTT2_CHUNK * sizeof(HitEntry);
        mttkrp_rows2_kernel<1, FTL_MTT2_G, FTL_MTT2_UNR><<<blocks2, 256, smem2, st>>>(
            row_idx, row_keys, row_vals, nnz, pt, T, shift, hs, R, Rp, out);
        return check_launch("mttkrp_rows2_kernel");
    }
    const int64_t nchunks = (nnz + MTT_CHUNK - 1) / MTT_CHUNK;
    int blocks = (int)std::min<int64_t>((nchunks * 32 + 255) / 256, (int64_t)num_sms() * 32);
    blocks = std::max(blocks, 1);
    if (R <= 32)
        mttkrp_rows_kernel<1, FTL_MTT_G><<<blocks, 256, 0, st>>>(row_idx, row_keys, row_vals, nnz, pt, T, shift, hs,
                                                                 R, Rp, out);
    else if (R <= 64)
        mttkrp_rows_kernel<2, 4><<<blocks, 256, 0, st>>>(row_idx, row_keys, row_vals, nnz, pt, T, shift, hs, R, Rp,
                                                         out);
    else
        mttkrp_rows_kernel<4, 2><<<blocks, 256, 0, st>>>(row_idx, row_keys, row_vals, nnz, pt, T, shift, hs, R, Rp,
                                                         out);
    return check_launch("mttkrp_rows_kernel");
}

extern "C" int ftl_gram_workspace_bytes(int R, size_t *out) {
    FTL_CHECK_ARG(out && R >= 1 && R <= FTL_MAX_RANK, "ftl_gram_workspace_bytes: bad R=%d", R);
    *out = (size_t)num_sms() * packed_size(R) * sizeof(double);
    return FTL_OK;
}

extern "C" int ftl_weighted_gram(const double *lhs, const int32_t *rowidx, const double *w, const int32_t *cnt,
                                 const int64_t *n_rows_dev, int64_t n_rows, int R, void *workspace, size_t ws_bytes,
                                 double *gram_out, void *stream) {
    FTL_CHECK_ARG(lhs && workspace && gram_out, "ftl_weighted_gram: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK, "ftl_weighted_gram: bad R=%d", R);
    size_t need = 0;
    ftl_gram_workspace_bytes(R, &need);
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_weighted_gram: workspace %zu < %zu bytes", ws_bytes, need);
    const int nblk = num_sms();
    cudaStream_t st = (cudaStream_t)stream;
    const size_t smem = (size_t)(64 * R) * sizeof(double);
    const int P = packed_size(R);
    const int threads = gram_threads(R);
    const int ept = (P + threads - 1) / threads;
    {
        const void *fn = ept <= 1   ? (const void *)gram_partial_kernel<1>
                         : ept <= 2 ? (const void *)gram_partial_kernel<2>
                         : ept <= 4 ? (const void *)gram_partial_kernel<4>
                                    : (const void *)gram_partial_kernel<9>;
        const int arc = ensure_smem(fn, smem, "gram_partial_kernel");
        if (arc) return arc;
    }
    double *part = (double *)workspace;
    if (ept <= 1)
        gram_partial_kernel<1><<<nblk, threads, smem, st>>>(lhs, rowidx, w, cnt, n_rows_dev, n_rows, R, part);
    else if (ept <= 2)
        gram_partial_kernel<2><<<nblk, threads, smem, st>>>(lhs, rowidx, w, cnt, n_rows_dev, n_rows, R, part);
    else if (ept <= 4)
        gram_partial_kernel<4><<<nblk, threads, smem, st>>>(lhs, rowidx, w, cnt, n_rows_dev, n_rows, R, part);
    else
        gram_partial_kernel<9><<<nblk, threads, smem, st>>>(lhs, rowidx, w, cnt, n_rows_dev, n_rows, R, part);
    gram_reduce_kernel<<<std::max(1, (P * 32 + 255) / 256), 256, 0, st>>>((const double *)workspace, nblk, R,
                                                                          gram_out);
    return check_launch("weighted gram kernels");
}

extern "C" int ftl_pinv_square(const double *M, int R, int target_rank, const int64_t *rank_cap_dev, double tol,
                               double *out, double *vscratch, void *stream) {
    FTL_CHECK_ARG(M && out, "ftl_pinv_square: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK, "ftl_pinv_square: bad R=%d", R);
    const bool vglob = (size_t)(2 * R * R + R + 2) * sizeof(double) > 200 * 1024;
    FTL_CHECK_ARG(!vglob || vscratch, "ftl_pinv_square: R=%d needs an R*R FP64 scratch buffer", R);
    const size_t smem = (size_t)((vglob ? 1 : 2) * R * R + R + 2) * sizeof(double) + (2 * R + 4) * sizeof(int) + 16;
    {
        const int arc = ensure_smem((const void *)pinv_square_kernel, smem, "pinv_square_kernel");
        if (arc) return arc;
    }
    pinv_square_kernel<<<1, 512, smem, (cudaStream_t)stream>>>(M, R, target_rank, rank_cap_dev, tol, out,
                                                                vglob ? vscratch : nullptr);
    return check_launch("pinv_square_kernel");
}

extern "C" int ftl_sparse_mttkrp(const uint64_t *sorted_keys, const uint32_t *sorted_idxj, const double *sorted_vals,
                                 int64_t nnz, const uint64_t *query_keys, const int32_t *query_row, const double *w,
                                 const int32_t *cnt, const int64_t *num_queries_dev, int64_t num_queries,
                                 const double *lhs, int R, double *out, int64_t I_j, void *stream) {
    FTL_CHECK_ARG(sorted_keys && sorted_idxj && sorted_vals && query_keys && lhs && out,
                  "ftl_sparse_mttkrp: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && I_j >= 1, "ftl_sparse_mttkrp: bad R=%d or I_j", R);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t err = cudaMemsetAsync(out, 0, (size_t)I_j * R * sizeof(double), st);
    if (err != cudaSuccess) return fail(FTL_E_CUDA, "ftl_sparse_mttkrp: memset: %s", cudaGetErrorString(err));
    if (nnz == 0) return FTL_OK;
    const int64_t nq = std::max<int64_t>(num_queries, 1);
    int blocks = (int)std::min<int64_t>((nq * 32 + 255) / 256, (int64_t)num_sms() * 16);
    mttkrp_kernel<<<std::max(blocks, 1), 256, 0, st>>>(sorted_keys, sorted_idxj, sorted_vals, nnz, query_keys,
                                                        query_row, w, cnt, num_queries_dev, num_queries, lhs, R, out);
    return check_launch("mttkrp_kernel");
}

extern "C" int ftl_solve_rows(const double *B, const double *pinv, int64_t I, int R, double *U, void *stream) {
    FTL_CHECK_ARG(B && pinv && U, "ftl_solve_rows: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && I >= 1, "ftl_solve_rows: bad shape");
    // R x R pinv plus one staged row per thread: 128 threads up to R = 64
    // (96 KB), 64 threads above (196 KB at R = 128)
    const int threads = R > 64 ? 64 : 128;
    const size_t smem = (size_t)(R * R + threads * R) * sizeof(double);
    FTL_CHECK_ARG(smem <= 227 * 1024, "ftl_solve_rows: R=%d too large", R);
    {
        const int arc = ensure_smem((const void *)solve_rows_kernel, smem, "solve_rows_kernel");
        if (arc) return arc;
    }
    int blocks = (int)std::min<int64_t>((I + threads - 1) / threads, (int64_t)num_sms() * 8);
    solve_rows_kernel<<<blocks, threads, smem, (cudaStream_t)stream>>>(B, pinv, I, R, U);
    return check_launch("solve_rows_kernel");
}

extern "C" int ftl_colnorm_workspace_bytes(int R, size_t *out) {
    FTL_CHECK_ARG(out && R >= 1 && R <= FTL_MAX_RANK, "ftl_colnorm_workspace_bytes: bad R");
    *out = (size_t)num_sms() * 4 * R * sizeof(double);
    return FTL_OK;
}

extern "C" int ftl_renormalize_columns(double *U, int64_t I, int R, double *norms_out, void *workspace,
                                       size_t ws_bytes, int apply, void *stream) {
    FTL_CHECK_ARG(U && norms_out && workspace, "ftl_renormalize_columns: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && I >= 1, "ftl_renormalize_columns: bad shape");
    size_t need = 0;
    ftl_colnorm_workspace_bytes(R, &need);
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_renormalize_columns: workspace too small");
    const int nblk = num_sms() * 4;
    const int threads = std::max(R, 1024 / R * R);
    cudaStream_t st = (cudaStream_t)stream;
    colsq_partial_kernel<<<nblk, threads, 0, st>>>(U, I, R, (double *)workspace);
    colnorm_finish_kernel<<<1, 1024, 0, st>>>((const double *)workspace, nblk, R, norms_out);
    if (apply) colscale_kernel<<<nblk * 2, threads, 0, st>>>(U, I, R, norms_out);
    return check_launch("renormalize kernels");
}

extern "C" int ftl_fit_workspace_bytes(size_t *out) {
    FTL_CHECK_ARG(out, "ftl_fit_workspace_bytes: null");
    *out = (size_t)num_sms() * 16 * sizeof(double);
    return FTL_OK;
}

extern "C" int ftl_sparse_residual_terms(const uint32_t *idx, const double *vals, int64_t nnz, int N,
                                         const double *const *U_dev, const double *sigma, int R, void *workspace,
                                         size_t ws_bytes, double *out, void *stream) {
    FTL_CHECK_ARG(idx && vals && U_dev && sigma && workspace && out, "ftl_sparse_residual_terms: null pointer");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && R >= 1 && R <= FTL_MAX_RANK, "ftl_sparse_residual_terms: bad shape");
    size_t need = 0;
    ftl_fit_workspace_bytes(&need);
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_sparse_residual_terms: workspace too small");
    FactorPtrs fp;
    for (int k = 0; k < FTL_MAX_MODES; ++k) fp.U[k] = k < N ? U_dev[k] : nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    double *part = (double *)workspace;
    // one wave of resident CTAs for the thread-per-nonzero forms (equal work
    // per CTA: a grid of a few waves plus a fraction leaves SMs idle at the end)
    int nblk = num_sms() * 16;
    if (N >= 2 && N <= 6) {
        const void *fn = N == 2 ? (const void *)residual_thread_kernel<2> : N == 3 ? (const void *)residual_thread_kernel<3>
                       : N == 4 ? (const void *)residual_thread_kernel<4> : N == 5 ? (const void *)residual_thread_kernel<5>
                                                                           : (const void *)residual_thread_kernel<6>;
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 256, 0) == cudaSuccess && occ >= 1)
            nblk = num_sms() * std::min(occ, 16);
    }
    switch (N) {
        case 2: residual_thread_kernel<2><<<nblk, 256, 0, st>>>(idx, vals, nnz, fp, sigma, R, part); break;
        case 3: residual_thread_kernel<3><<<nblk, 256, 0, st>>>(idx, vals, nnz, fp, sigma, R, part); break;
        case 4: residual_thread_kernel<4><<<nblk, 256, 0, st>>>(idx, vals, nnz, fp, sigma, R, part); break;
        case 5: residual_thread_kernel<5><<<nblk, 256, 0, st>>>(idx, vals, nnz, fp, sigma, R, part); break;
        case 6: residual_thread_kernel<6><<<nblk, 256, 0, st>>>(idx, vals, nnz, fp, sigma, R, part); break;
        default: residual_partial_kernel<<<nblk, 256, 0, st>>>(idx, vals, nnz, N, fp, sigma, R, part);
    }
    sum_kernel<<<1, 32, 0, st>>>((const double *)workspace, nblk, out);
    return check_launch("residual kernels");
}

extern "C" int ftl_sum_squares(const double *v, int64_t n, void *workspace, size_t ws_bytes, double *out,
                               void *stream) {
    FTL_CHECK_ARG(v && workspace && out, "ftl_sum_squares: null pointer");
    size_t need = 0;
    ftl_fit_workspace_bytes(&need);
    FTL_CHECK_ARG(ws_bytes >= need, "ftl_sum_squares: workspace too small");
    const int nblk = num_sms() * 16;
    cudaStream_t st = (cudaStream_t)stream;
    sumsq_partial_kernel<<<nblk, 256, 0, st>>>(v, n, (double *)workspace);
    sum_kernel<<<1, 32, 0, st>>>((const double *)workspace, nblk, out);
    return check_launch("sum of squares kernels");
}

extern "C" int ftl_sparse_exact_mttkrp(const uint32_t *idx, const double *vals, int64_t nnz, int N, int j,
                                       const double *const *U_dev, int R, double *out, int64_t I_j, void *stream) {
    FTL_CHECK_ARG(idx && vals && U_dev && out, "ftl_sparse_exact_mttkrp: null pointer");
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && j >= 0 && j < N && R >= 1 && R <= FTL_MAX_RANK,
                  "ftl_sparse_exact_mttkrp: bad shape");
    FactorPtrs fp;
    for (int k = 0; k < FTL_MAX_MODES; ++k) fp.U[k] = k < N ? U_dev[k] : nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t err = cudaMemsetAsync(out, 0, (size_t)I_j * R * sizeof(double), st);
    if (err != cudaSuccess) return fail(FTL_E_CUDA, "ftl_sparse_exact_mttkrp: memset: %s", cudaGetErrorString(err));
    if (nnz == 0) return FTL_OK;
    exact_mttkrp_kernel<<<num_sms() * 16, 256, 0, st>>>(idx, vals, nnz, N, j, fp, R, out);
    return check_launch("exact_mttkrp_kernel");
}

extern "C" int ftl_sparse_rrf(const int32_t *row_idx, const uint64_t *row_keys, const double *row_vals, int64_t nnz,
                              int R, uint64_t seed, uint32_t mode, double *out, int64_t I_j, void *stream) {
    FTL_CHECK_ARG(row_idx && row_keys && row_vals && out, "ftl_sparse_rrf: null pointer");
    FTL_CHECK_ARG(R >= 1 && R <= FTL_MAX_RANK && I_j >= 1 && nnz >= 0, "ftl_sparse_rrf: bad shape R=%d I_j=%lld",
                  R, (long long)I_j);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t err = cudaMemsetAsync(out, 0, (size_t)I_j * R * sizeof(double), st);
    if (err != cudaSuccess) return fail(FTL_E_CUDA, "ftl_sparse_rrf: memset: %s", cudaGetErrorString(err));
    if (nnz == 0) return FTL_OK;
    const int64_t nchunks = (nnz + RRF_CHUNK - 1) / RRF_CHUNK;
    int blocks = (int)std::min<int64_t>((nchunks * 32 + 255) / 256, (int64_t)num_sms() * 32);
    rrf_rows_kernel<<<std::max(blocks, 1), 256, 0, st>>>(row_idx, row_keys, row_vals, nnz, R, seed, mode, out);
    return check_launch("rrf_rows_kernel");
}
