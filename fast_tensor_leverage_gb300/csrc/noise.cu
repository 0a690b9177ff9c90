// Counter-hash Gaussian noise on a black-box tensor: X = [[s; V]] + sigma Z,
// Z(i_1, .., i_N) one standard normal per entry, a pure function of the
// entry's linear index and a seed, so the noise is never stored and any
// entry, fiber or sampled MTTKRP can be formed on the fly (the noisy
// low-rank ground truth of the precision study; the reference builds its
// tensors in memory, low_rank_tensor.hpp / dense_tensor.hpp, and has no
// noise model of its own).
//
// Z at linear index L (row-major over dims, L < prod dims <= 2^64): the
// SplitMix64 finaliser (Steele, Lea and Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014) of x = L * 0x9E3779B97F4A7C15 + seed gives
// 64 bits z; u1 = ((z >> 40) + 1) 2^-24 in (0, 1], u2 = ((z >> 16) & (2^24 -
// 1)) 2^-24 in [0, 1) (exact in FP32); Z = sqrt(-2 ln u1) cos(2 pi u2)
// (Box-Muller, FP32).
//
// Sampled MTTKRP term (BlackBoxTensor::execute_downsampled_mttkrp semantics,
// black_box_tensor.hpp:21-67, for the noise part of the right-hand side):
//   out[i, c] += sigma sum_u coef_u Z(L(i, s_u)) h[rep_u, c]
// over the unique samples u (coef_u = w[rep_u] cnt[u] as in the low-rank
// shortcut).  Every (i, u) pair needs a fresh Z, so the kernel is bound by
// the hash and Box-Muller arithmetic (one per pair): blocks own 64 rows i,
// walk the samples 64 at a time (noise tile and coefficient rows staged in
// shared memory), accumulate in FP32 registers and fold into FP64 every 512
// samples; fixed order throughout, so the result is deterministic.
#include <algorithm>

#include "ftl_common.cuh"

namespace ftl {

namespace {

constexpr int kNoiseRows = 64;     // rows i per block
constexpr int kNoiseChunk = 64;    // samples per shared-memory chunk
constexpr int kNoiseFold = 8;      // chunks per FP64 fold
constexpr int kNoiseThreads = 256;

struct NoiseDims {
    uint64_t stride[FTL_MAX_MODES];  // row-major strides (wrapping uint64 arithmetic)
    int64_t dims[FTL_MAX_MODES];
    int N;
};

__device__ __forceinline__ float noise_value(uint64_t L, uint64_t seed) {
    uint64_t z = L * 0x9E3779B97F4A7C15ull + seed;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const float u1 = (float)((uint32_t)(z >> 40) + 1u) * (1.0f / 16777216.0f);
    const float u2 = (float)((uint32_t)(z >> 16) & 0xFFFFFFu) * (1.0f / 16777216.0f);
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

int fill_dims(NoiseDims &d, const int64_t *dims, int N) {
    FTL_CHECK_ARG(dims && N >= 1 && N <= FTL_MAX_MODES, "noise: bad mode count %d", N);
    d.N = N;
    uint64_t s = 1;
    for (int k = N - 1; k >= 0; --k) {
        FTL_CHECK_ARG(dims[k] >= 1, "noise: dims[%d] = %lld", k, (long long)dims[k]);
        d.dims[k] = dims[k];
        d.stride[k] = s;
        s *= (uint64_t)dims[k];
    }
    return FTL_OK;
}

template <int PER>
__global__ void __launch_bounds__(kNoiseThreads) noise_mttkrp_kernel(
    NoiseDims nd, int j, uint64_t seed, double sigma, const uint64_t *__restrict__ samples, int64_t J,
    const int32_t *__restrict__ urep, const int32_t *__restrict__ cnt, const int64_t *__restrict__ n_dev,
    int64_t n_host, const double *__restrict__ w, const double *__restrict__ h, int R, double *__restrict__ out,
    int64_t I_j) {
    extern __shared__ __align__(16) unsigned char noise_smem[];
    float *Zs = (float *)noise_smem;                       // kNoiseRows x kNoiseChunk
    float *Ls = Zs + kNoiseRows * kNoiseChunk;             // kNoiseChunk x R
    uint64_t *base = (uint64_t *)(Ls + kNoiseChunk * R);   // kNoiseChunk (offset 256 (16 + R) bytes: aligned)
    const int tid = threadIdx.x;
    const int64_t n = n_dev ? *n_dev : n_host;
    // each thread owns PER entries of the block's kNoiseRows x R output tile
    // (PER >= kNoiseRows * R / kNoiseThreads, chosen by R at launch)
    for (int64_t i0 = (int64_t)blockIdx.x * kNoiseRows; i0 < I_j; i0 += (int64_t)gridDim.x * kNoiseRows) {
        double acc64[PER];
        float acc[PER];
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            acc64[q] = 0.0;
            acc[q] = 0.0f;
        }
        int chunks = 0;
        for (int64_t u0 = 0; u0 < n; u0 += kNoiseChunk) {
            const int m = (int)min((int64_t)kNoiseChunk, n - u0);
            __syncthreads();
            // chunk metadata: the other modes' part of each sample's linear
            // index, and the coefficient rows sigma coef_u h[rep_u] in FP32
            for (int uu = tid; uu < kNoiseChunk; uu += kNoiseThreads) {
                uint64_t b = 0;
                if (uu < m) {
                    const int64_t rep = urep ? (int64_t)urep[u0 + uu] : u0 + uu;
                    for (int k = 0; k < nd.N; ++k)
                        if (k != j) b += samples[(int64_t)k * J + rep] * nd.stride[k];
                }
                base[uu] = b;
            }
            for (int e = tid; e < kNoiseChunk * R; e += kNoiseThreads) {
                const int uu = e / R, c = e - uu * R;
                float v = 0.0f;
                if (uu < m) {
                    const int64_t u = u0 + uu;
                    const int64_t rep = urep ? (int64_t)urep[u] : u;
                    const double coef = (w ? w[rep] : 1.0) * (cnt ? (double)cnt[u] : 1.0);
                    v = (float)(sigma * coef * h[rep * R + c]);
                }
                Ls[e] = v;
            }
            __syncthreads();
            for (int e = tid; e < kNoiseRows * kNoiseChunk; e += kNoiseThreads) {
                const int r = e / kNoiseChunk, uu = e - r * kNoiseChunk;
                const int64_t i = i0 + r;
                Zs[e] = (uu < m && i < I_j) ? noise_value(base[uu] + (uint64_t)i * nd.stride[j], seed) : 0.0f;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < PER; ++q) {
                const int e = tid + q * kNoiseThreads;
                if (e >= kNoiseRows * R) break;
                const int r = e / R, c = e - r * R;
                float a = acc[q];
                for (int uu = 0; uu < m; ++uu) a = fmaf(Zs[r * kNoiseChunk + uu], Ls[uu * R + c], a);
                acc[q] = a;
            }
            if (++chunks == kNoiseFold) {
                chunks = 0;
#pragma unroll
                for (int q = 0; q < PER; ++q) {
                    acc64[q] += (double)acc[q];
                    acc[q] = 0.0f;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int e = tid + q * kNoiseThreads;
            if (e >= kNoiseRows * R) break;
            const int r = e / R, c = e - r * R;
            const int64_t i = i0 + r;
            if (i < I_j) out[i * R + c] += acc64[q] + (double)acc[q];
        }
    }
}

template <typename IT>
__global__ void noise_add_at_kernel(NoiseDims nd, uint64_t seed, double sigma, const IT *__restrict__ idx, int64_t n,
                                    double *__restrict__ out) {
    for (int64_t z = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; z < n; z += (int64_t)gridDim.x * blockDim.x) {
        uint64_t L = 0;
        for (int k = 0; k < nd.N; ++k) L += (uint64_t)idx[z * nd.N + k] * nd.stride[k];
        out[z] += sigma * (double)noise_value(L, seed);
    }
}

__global__ void noise_add_fibers_kernel(NoiseDims nd, uint64_t seed, double sigma, const uint64_t *__restrict__ S,
                                        int64_t n, int j, double *__restrict__ out) {
    const int64_t I_j = nd.dims[j];
    for (int64_t z = blockIdx.x; z < n; z += gridDim.x) {
        uint64_t b = 0;
        for (int k = 0; k < nd.N; ++k)
            if (k != j) b += S[z * nd.N + k] * nd.stride[k];
        for (int64_t i = threadIdx.x; i < I_j; i += blockDim.x)
            out[z * I_j + i] += sigma * (double)noise_value(b + (uint64_t)i * nd.stride[j], seed);
    }
}

}  // namespace

}  // namespace ftl

using namespace ftl;

extern "C" int ftl_noise_sampled_mttkrp(const int64_t *dims, int N, int j, uint64_t seed, double sigma,
                                        const uint64_t *samples, int64_t J, const int32_t *urep, const int32_t *ucnt,
                                        const int64_t *num_unique_dev, int64_t num_unique, const double *w,
                                        const double *h, int R, double *out, int64_t out_rows, void *stream) {
    NoiseDims nd;
    int rc = fill_dims(nd, dims, N);
    if (rc) return rc;
    FTL_CHECK_ARG(j >= 0 && j < N, "ftl_noise_sampled_mttkrp: j=%d outside [0, %d)", j, N);
    FTL_CHECK_ARG(samples && h && out && J >= 1 && R >= 1 && R <= FTL_MAX_RANK && out_rows >= dims[j],
                  "ftl_noise_sampled_mttkrp: bad arguments (J=%lld R=%d out_rows=%lld)", (long long)J, R,
                  (long long)out_rows);
    FTL_CHECK_ARG(num_unique_dev || (num_unique >= 0 && num_unique <= J), "ftl_noise_sampled_mttkrp: bad count");
    if (sigma == 0.0) return FTL_OK;
    const int64_t I_j = dims[j];
    const size_t smem = (size_t)kNoiseRows * kNoiseChunk * sizeof(float) +
                        (size_t)kNoiseChunk * R * sizeof(float) + kNoiseChunk * sizeof(uint64_t);
    const int blocks = (int)std::max<int64_t>(1, (I_j + kNoiseRows - 1) / kNoiseRows);
    const int per = (kNoiseRows * R + kNoiseThreads - 1) / kNoiseThreads;
    cudaStream_t st = (cudaStream_t)stream;
#define FTL_NOISE_LAUNCH(P)                                                                                   \
    do {                                                                                                      \
        rc = ensure_smem((const void *)noise_mttkrp_kernel<P>, smem, "noise_mttkrp_kernel");                  \
        if (rc) return rc;                                                                                    \
        noise_mttkrp_kernel<P><<<blocks, kNoiseThreads, smem, st>>>(nd, j, seed, sigma, samples, J, urep,     \
                                                                    ucnt, num_unique_dev, num_unique, w, h, R, \
                                                                    out, I_j);                                \
    } while (0)
    if (per <= 4)
        FTL_NOISE_LAUNCH(4);
    else if (per <= 8)
        FTL_NOISE_LAUNCH(8);
    else if (per <= 16)
        FTL_NOISE_LAUNCH(16);
    else
        FTL_NOISE_LAUNCH(32);
#undef FTL_NOISE_LAUNCH
    return check_launch("noise_mttkrp_kernel");
}

extern "C" int ftl_noise_add_at(const int64_t *dims, int N, uint64_t seed, double sigma, const void *idx,
                                int idx_is_u64, int64_t n, double *out, void *stream) {
    NoiseDims nd;
    int rc = fill_dims(nd, dims, N);
    if (rc) return rc;
    FTL_CHECK_ARG(idx && out && n >= 0, "ftl_noise_add_at: bad arguments");
    if (n == 0) return FTL_OK;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 16);
    if (idx_is_u64)
        noise_add_at_kernel<uint64_t><<<blocks, 256, 0, (cudaStream_t)stream>>>(nd, seed, sigma,
                                                                              (const uint64_t *)idx, n, out);
    else
        noise_add_at_kernel<uint32_t><<<blocks, 256, 0, (cudaStream_t)stream>>>(nd, seed, sigma,
                                                                              (const uint32_t *)idx, n, out);
    return check_launch("noise_add_at_kernel");
}

extern "C" int ftl_noise_add_fibers(const int64_t *dims, int N, uint64_t seed, double sigma,
                                    const uint64_t *samples, int64_t n, int j, double *out, void *stream) {
    NoiseDims nd;
    int rc = fill_dims(nd, dims, N);
    if (rc) return rc;
    FTL_CHECK_ARG(samples && out && n >= 0 && j >= 0 && j < N, "ftl_noise_add_fibers: bad arguments");
    if (n == 0) return FTL_OK;
    const int blocks = (int)std::min<int64_t>(n, (int64_t)num_sms() * 16);
    noise_add_fibers_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(nd, seed, sigma, samples, n, j, out);
    return check_launch("noise_add_fibers_kernel");
}
