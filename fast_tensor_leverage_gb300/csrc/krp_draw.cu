// Fused KRP leverage-score draw and the standalone tree sampler.
//
// krp_draw_kernel: one warp per sample runs, for every included mode k in
// increasing order, the eigen-component descent (query h) and the Gram-tree
// descent (query h o W[u]) of EfficientKRPSampler::KRPDrawSamples
// (cpp_ext/efficient_krp_sampler.hpp:209-254), keeping the running KRP row h
// in registers across modes, then the weight epilogue w = R / (J h^T pinv h)
// (compute_DAGAT, cpp_ext/sampler.hpp:94-123; :257-267).  Uniforms come from
// the caller (2N x J, the reference's layout) or from Philox4x32-10 keyed by
// (seed, ctr + flat index) -- the same flat index, so both sources are
// interchangeable.
#include <algorithm>

#include <type_traits>

#include "descent.cuh"

namespace ftl {

int computem_launch(const ftl_krp_plan *plan, uint32_t j_norm, cudaStream_t st);
int tuned_variant(int family, int R, int prec);

struct DrawParams {
    int N, R, P, S;
    uint32_t j;
    int64_t J;
    DGeom gram[FTL_MAX_MODES];
    DGeom eig;
    const double *U[FTL_MAX_MODES];
    const float *U32[FTL_MAX_MODES];  // FP32 copies of U for the leaf scans (S32 kernels)
    const void *gram_G[FTL_MAX_MODES];
    const void *eig_G;
    const double *M;
    const float *pinv32;
    int offset[FTL_MAX_MODES];
    uint64_t *samples;
    double *h;
    double *weights;
    const double *draws;
    uint64_t seed, ctr;
};

__device__ __forceinline__ double get_draw(const DrawParams &p, int64_t idx) {
    return p.draws ? p.draws[idx] : philox_uniform(p.seed, p.ctr + (uint64_t)idx);
}

// Per-warp state of the draw kernels: the block's pair table and the warp's
// shared-memory slot.
template <int RMAX, typename T, bool DIAG = false>
struct DrawWarp {
    const uint16_t *pairs;
    double *xd;
    T *xT;
    typename QSel<RMAX, T, DIAG>::type qf;
    int lane;
};

template <int RMAX, typename T, bool DIAG>
__device__ __forceinline__ void setup_draw_warp(DrawWarp<RMAX, T, DIAG> &dw, unsigned char *smem_raw, int R, int P,
                                                int S) {
    uint16_t *pairs = (uint16_t *)smem_raw;
    build_pairs(pairs, R);
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    unsigned char *slot = smem_raw + ((NodeShape<RMAX, T>::SMAX * sizeof(uint16_t) + 15) / 16 * 16) +
                          warp * WarpSlot<RMAX, T, DIAG>::bytes;
    dw.pairs = pairs;
    dw.xd = (double *)slot;
    dw.xT = sizeof(T) == 8 ? (T *)dw.xd : (T *)(dw.xd + RMAX);
    dw.qf.P = P;
    dw.qf.S = S;
    dw.qf.s = (T *)(slot + RMAX * sizeof(double) + RMAX * sizeof(T));
    dw.lane = threadIdx.x & 31;
}

// Row index written by an FP32 draw for a mode whose Gram-tree descent met a
// zero query (the eigen component chosen has zero mass under h) or ended in a
// block whose forms are all zero -- possible because the FP32 descent carries
// right-child masses as parent - left, and blocks of exactly-zero factor rows
// (rows of an ALS factor that no sampled fiber touched) have zero mass.  The
// fix-up kernel redoes every such sample with descend_careful.
constexpr uint64_t kRedoSample = ~0ull;

// Sample i of one draw: for every included mode the eigen-component descent
// and the Gram-tree descent, then the weight and the row of h.  CAREFUL (FP32
// fix-up pass only): both descents evaluate both children at every level.
template <int RMAX, typename T, bool CAREFUL = false, bool S32 = false, bool DIAG = false>
__device__ __forceinline__ void draw_sample(const DrawParams &p, int64_t i, DrawWarp<RMAX, T, DIAG> &dw) {
    using S = Shape<RMAX>;
    constexpr int XPL = S::XPL;
    const int R = p.R;
    const int lane = dw.lane;
    const uint16_t *pairs = dw.pairs;
    double *xd = dw.xd;
    T *xT = dw.xT;
    auto &qf = dw.qf;
    const size_t RR = (size_t)R * R;
    const size_t eig_stride = (size_t)(2 * R - 1) * p.S;
    const float RJ = (float)((double)R / (double)p.J);
    double h[XPL];
#pragma unroll
    for (int q = 0; q < XPL; ++q) h[q] = 1.0;
#pragma unroll 1
    for (int k = 0; k < p.N; ++k) {
        if ((uint32_t)k == p.j) continue;
        // phase 0: eigen-component descent, query h;
        // phase 1: Gram-tree descent, query h o W[u], leaf scan, h o= U_k[t]
        double x[XPL];
#pragma unroll
        for (int q = 0; q < XPL; ++q) x[q] = h[q];
#pragma unroll 1
        for (int phase = 0; phase < 2; ++phase) {
            const T *G = phase == 0 ? (const T *)p.eig_G + k * eig_stride : (const T *)p.gram_G[k];
            const DGeom &g = phase == 0 ? p.eig : p.gram[k];
            const double *Uk = p.U[k];
            __syncwarp();
            stage_query<RMAX, T>(x, R, xd, xT, lane);
            qf.setup(xT, pairs, lane);
            T frac, mroot = T(1);
            const double u = get_draw(p, (int64_t)(phase * p.N + k) * p.J + i);
            int64_t c;
            if constexpr (CAREFUL && sizeof(T) == 4)
                c = descend_careful<RMAX>(G, p.S, g, u, qf, lane, frac);
            else
                c = descend<RMAX>(G, p.S, g, u, qf, lane, frac, (phase == 1 && g.F > 1) ? Uk : nullptr, R, &mroot);
            if (phase == 0) {
                const double *Wr = p.M + (size_t)p.offset[k] * RR + (size_t)leaf_index(g, c) * R;
#pragma unroll
                for (int q = 0; q < XPL; ++q) {
                    int col = lane + 32 * q;
                    x[q] = col < R ? h[q] * Wr[col] : 0.0;
                }
            } else {
                bool empty = false;
                int64_t t = 0;
                if (FTL_DESC_REDO && sizeof(T) == 4 && !CAREFUL && !(mroot > T(0))) {
                    empty = true;  // zero query: the eigen component has no mass under h
                    t = leaf_index(g, c) * g.F;  // any valid row; the sample is redone
                } else if (g.F > 1)
                    t = S32 ? leaf_scan<RMAX, T, float>(p.U32[k], R, g, c, frac, lane_query<RMAX, T>(xT, R, lane),
                                                        lane, empty)
                            : leaf_scan<RMAX, T, double>(Uk, R, g, c, frac, lane_query<RMAX, T>(xT, R, lane), lane,
                                                         empty);
                else
                    t = leaf_index(g, c);
                // the careful pass (and FP64) keep what they found
                if (!FTL_DESC_REDO || sizeof(T) == 8 || CAREFUL) empty = false;
                const double *Ur = Uk + t * R;
#pragma unroll
                for (int q = 0; q < XPL; ++q) {
                    int col = lane + 32 * q;
                    if (col < R) h[q] *= Ur[col];
                }
                if (lane == 0) p.samples[(int64_t)k * p.J + i] = empty ? kRedoSample : (uint64_t)t;
            }
        }
        __syncwarp();
    }
    if (p.weights) {
        double scale = stage_query<RMAX, T>(h, R, xd, xT, lane);
        qf.setup(xT, pairs, lane);
        if (sizeof(T) == 8) {
            double lev = (double)qf.eval((const T *)(p.M + cm_pinv64_offset(p.N, R)), lane);
            if (lane == 0) p.weights[i] = (double)R / (lev * (double)p.J);
        } else {
            // w = R / (J lev), lev = lev_scaled / scale^2: the quotient in
            // FP32, the power-of-two rescale as one exact FP64 product
            float lev_s = (float)qf.eval((const T *)p.pinv32, lane);
            if (lane == 0) p.weights[i] = (double)(RJ / lev_s) * (scale * scale);
        }
    }
    if (p.h) {
#pragma unroll
        for (int q = 0; q < XPL; ++q) {
            int col = lane + 32 * q;
            if (col < R) p.h[i * R + col] = h[q];
        }
    }
    __syncwarp();
}

// Threads per SM the register budget of a draw kernel is set for.
template <typename T, bool DIAG>
struct Resident {
    static constexpr int value =
        sizeof(T) == 8 ? FTL_DESC_RESIDENT_F64 : (DIAG ? FTL_DESC_RESIDENT_D32 : FTL_DESC_RESIDENT_F32);
};

// Samples i0 + c (c < NC, those below J) of one draw for FP32 trees in the
// DIAG32 layout (16 < R <= 32): the descents of draw_sample with registers
// only, the NC samples' descents in lockstep (descend_d32_multi) so that
// their dependent node reads overlap.  Lane l < 2N draws uniform l of each
// sample (phase l / N, mode l % N: the reference's 2N x J layout) once, as
// an FP32 pair; the queries are the FP64 vectors h and h o W[u] scaled by a
// power of two and rounded to FP32 with integer operations; lane a keeps
// x_a, its 17 outer-product weights and h_a; R = F = 32 leaf blocks are
// scanned with vector loads from the FP32 factor copy.  FP64 work per mode:
// h o W[u] and the h update.  Samples that meet a zero-mass block are
// flagged for the careful redo as in draw_sample.  Each sample's arithmetic
// does not depend on NC.
template <bool S32, int NC, bool SW = false>
__device__ __forceinline__ void draw_samples_d32(const DrawParams &p, int64_t i0, int lane, float *slots = nullptr) {
    const int R = p.R, N = p.N;
    const size_t RR = (size_t)R * R;
    const float RJ = (float)((double)R / (double)p.J);
    const bool col = lane < R;
    float uh[NC], ul[NC];
    double h[NC];
    typename std::conditional<SW, QFormD32S, QFormD32>::type qf[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        if constexpr (SW) qf[c].bind(slots + c * kDiag32Stride);
        uh[c] = ul[c] = 0.0f;
        const int64_t i = i0 + c;
        if (lane < 2 * N && i < p.J) {
            const int64_t idx = (int64_t)lane * p.J + i;
            if (p.draws)
                split_df(p.draws[idx], uh[c], ul[c]);
            else
                split_bits53(philox_bits53(p.seed, p.ctr + (uint64_t)idx), uh[c], ul[c]);
        }
        h[c] = col ? 1.0 : 0.0;
    }
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
        if ((uint32_t)k == p.j) continue;
        float dh[NC], dl[NC], frac[NC], mroot[NC], xf[NC];
        uint32_t cu[NC];
        // eigen-component descents, query h
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            qf[c].setup_reg(scaled_f32(h[c], query_shift(h[c])), lane);
            dh[c] = __shfl_sync(0xffffffffu, uh[c], k);
            dl[c] = __shfl_sync(0xffffffffu, ul[c], k);
        }
        const float *Ge = (const float *)p.eig_G + (size_t)k * (size_t)(2 * R - 1) * kDiag32Stride;
        descend_d32_multi<NC>(Ge, p.eig, dh, dl, qf, lane, cu, frac, mroot);
        // Gram-tree descents, query h o W[u]
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const double *Wr = p.M + (size_t)p.offset[k] * RR + (size_t)leaf_index(p.eig, cu[c]) * R;
            const double x = col ? h[c] * Wr[lane] : 0.0;
            xf[c] = scaled_f32(x, query_shift(x));
            qf[c].setup_reg(xf[c], lane);
            dh[c] = __shfl_sync(0xffffffffu, uh[c], N + k);
            dl[c] = __shfl_sync(0xffffffffu, ul[c], N + k);
        }
        const DGeom &g = p.gram[k];
        descend_d32_multi<NC>((const float *)p.gram_G[k], g, dh, dl, qf, lane, cu, frac, mroot);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            bool empty = false;
            int64_t t;
            if (FTL_DESC_REDO && !(mroot[c] > 0.0f)) {
                empty = true;  // zero query: the eigen component has no mass under h
                t = leaf_index(g, cu[c]) * g.F;
            } else if (g.F > 1) {
                if (S32 && R == 32 && g.F == 32) {
                    t = leaf_scan_d32(p.U32[k], g, cu[c], frac[c], xf[c], lane, empty);
                } else {
                    LaneQuery<32, float> lq;
                    lq.v[0] = xf[c];
                    t = S32 ? leaf_scan<32, float, float>(p.U32[k], R, g, cu[c], frac[c], lq, lane, empty)
                            : leaf_scan<32, float, double>(p.U[k], R, g, cu[c], frac[c], lq, lane, empty);
                }
            } else {
                t = leaf_index(g, cu[c]);
            }
            if (!FTL_DESC_REDO) empty = false;
            if (col) h[c] *= p.U[k][t * R + lane];
            if (lane == 0 && i0 + c < p.J) p.samples[(int64_t)k * p.J + i0 + c] = empty ? kRedoSample : (uint64_t)t;
        }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const int64_t i = i0 + c;
        if (p.weights) {
            // w = R / (J lev), lev = h^T pinv h = lev_s 2^(-2 sh)
            const int sh = query_shift(h[c]);
            qf[c].setup_reg(scaled_f32(h[c], sh), lane);
            const float lev_s = qf[c].eval(p.pinv32, lane);
            if (lane == 0 && i < p.J) {
                const double sc = (sh >= -1022 && sh <= 1023) ? __hiloint2double((1023 + sh) << 20, 0) : 0.0;
                p.weights[i] = (double)(RJ / lev_s) * sc * sc;
            }
        }
        if (p.h && col && i < p.J) p.h[i * R + lane] = h[c];
    }
}

template <int RMAX, typename T, bool S32, bool DIAG>
__global__ void __launch_bounds__(Blk<RMAX, T>::WARPS * 32, Resident<T, DIAG>::value / (Blk<RMAX, T>::WARPS * 32)) krp_draw_kernel(DrawParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DrawWarp<RMAX, T, DIAG> dw;
    setup_draw_warp<RMAX, T, DIAG>(dw, smem_raw, p.R, p.P, p.S);
    const int warp = threadIdx.x >> 5;
    for (int64_t i = (int64_t)blockIdx.x * Blk<RMAX, T>::WARPS + warp; i < p.J;
         i += (int64_t)gridDim.x * Blk<RMAX, T>::WARPS)
        draw_sample<RMAX, T, false, S32, DIAG>(p, i, dw);
}

// Block shape of the FP32 DIAG32 draw kernel per variant NC (samples a warp
// descends in lockstep): warps per block and threads per SM its register
// budget is set for.  NC = 1: 8 warps, 768 threads (85 registers); NC = 2
// and 3: 4 warps, 512 threads (128 registers).  Which variant runs is the
// autotuner's choice (ftl_tune_set), default NC = 3.
template <int NC, bool SW = false>
struct D32Shape {
    static constexpr int WARPS = NC == 1 ? 8 : 4;
    static constexpr int RESIDENT = SW ? (NC <= 3 ? 640 : NC == 4 ? 512 : 384) : (NC == 1 ? 768 : 512);
    static constexpr size_t SMEM = SW ? (size_t)WARPS * NC * kDiag32Stride * sizeof(float) : 0;
};

template <bool S32, int NC, bool SW>
__global__ void __launch_bounds__(D32Shape<NC, SW>::WARPS * 32, D32Shape<NC, SW>::RESIDENT / (D32Shape<NC, SW>::WARPS * 32))
    krp_draw_d32_kernel(DrawParams p) {
    constexpr int WARPS = D32Shape<NC, SW>::WARPS;
    extern __shared__ __align__(16) float d32_slots[];
    const int warp = threadIdx.x >> 5;
    for (int64_t i0 = ((int64_t)blockIdx.x * WARPS + warp) * NC; i0 < p.J; i0 += (int64_t)gridDim.x * WARPS * NC)
        draw_samples_d32<S32, NC, SW>(p, i0, threadIdx.x & 31, SW ? d32_slots + warp * NC * kDiag32Stride : nullptr);
}

// Packed draw: the samples of up to FTL_MAX_PACK requests of the same rank
// and precision in one launch; warp w takes global sample w, which belongs to
// the request r with cum[r] <= w < cum[r+1].  Each sample runs exactly the
// code of krp_draw_kernel, so results equal the per-request launches.
struct MultiDrawParams {
    int n;
    int64_t cum[FTL_MAX_PACK + 1];
    DrawParams req[FTL_MAX_PACK];
    // serving controls (ftl_krp_sample_packed_ctl); ctl == nullptr: none
    ftl_pack_status *ctl;
    const volatile uint32_t *cancel[FTL_MAX_PACK];  // per request, may be null
    uint64_t budget_ns;                             // 0: no time budget
};

// Serving controls of a packed draw, checked by a warp before each sample:
// a request whose cancel flag is set, or any request once the launch has run
// longer than its budget (%globaltimer since the first warp started), has
// its remaining samples skipped and its status set (first reason wins).  The
// cancel flag (host-writable memory) is read on a warp's first sample of a
// request and then every 8th sample, so a flag set before the launch stops
// every sample of its request; the timer is read every sample.  `stopped`
// caches the requests this warp stopped.  Nothing waits: a stopped launch
// just finishes early.
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool pack_stop(const MultiDrawParams &mp, int r, int &iter, int &last_r,
                                          unsigned &stopped, int lane) {
    if (mp.ctl == nullptr) return false;
    if (stopped & (1u << r)) return true;
    if (r != last_r) {
        last_r = r;
        iter = 0;
    }
    uint32_t code = 0;
    if (lane == 0) {
        if (mp.cancel[r] && (iter & 7) == 0 && *mp.cancel[r] != 0u) code = FTL_E_CANCELLED;
        if (!code && mp.budget_ns) {
            unsigned long long *t0p = (unsigned long long *)&mp.ctl->start_ns;
            const uint64_t now = global_ns();
            unsigned long long t0 = *(volatile unsigned long long *)t0p;
            if (t0 == 0ull) {
                const unsigned long long prev = atomicCAS(t0p, 0ull, (unsigned long long)now);
                t0 = prev == 0ull ? (unsigned long long)now : prev;
            }
            // another warp may have set t0 after this warp read `now`
            if (now > (uint64_t)t0 && now - (uint64_t)t0 > mp.budget_ns) code = FTL_E_TIMEOUT;
        }
        if (code) atomicCAS((unsigned int *)&mp.ctl->status[r], 0u, code);
    }
    ++iter;
    code = __shfl_sync(0xffffffffu, code, 0);
    if (code) stopped |= 1u << r;
    return code != 0;
}

template <int RMAX, typename T, bool S32, bool DIAG>
__global__ void __launch_bounds__(Blk<RMAX, T, DIAG>::WARPS * 32, Resident<T, DIAG>::value / (Blk<RMAX, T, DIAG>::WARPS * 32)) krp_draw_multi_kernel(MultiDrawParams mp) {
    constexpr int WARPS = Blk<RMAX, T, DIAG>::WARPS;
    const int warp = threadIdx.x >> 5;
    const int64_t total = mp.cum[mp.n];
    if constexpr (DIAG && sizeof(T) == 4) {
        // one sample per warp (neighbouring samples may belong to different
        // requests, i.e. different trees); the same per-sample arithmetic as
        // krp_draw_kernel
        int iter = 0, last_r = -1;
        unsigned stopped = 0u;
        for (int64_t g = (int64_t)blockIdx.x * WARPS + warp; g < total; g += (int64_t)gridDim.x * WARPS) {
            int r = 0;
            while (r + 1 < mp.n && mp.cum[r + 1] <= g) ++r;
            if (pack_stop(mp, r, iter, last_r, stopped, threadIdx.x & 31)) continue;
            draw_samples_d32<S32, 1>(mp.req[r], g - mp.cum[r], threadIdx.x & 31);
        }
    } else {
        extern __shared__ __align__(16) unsigned char smem_raw[];
        DrawWarp<RMAX, T, DIAG> dw;
        setup_draw_warp<RMAX, T, DIAG>(dw, smem_raw, mp.req[0].R, mp.req[0].P, mp.req[0].S);
        int iter = 0, last_r = -1;
        unsigned stopped = 0u;
        for (int64_t g = (int64_t)blockIdx.x * WARPS + warp; g < total; g += (int64_t)gridDim.x * WARPS) {
            int r = 0;
            while (r + 1 < mp.n && mp.cum[r + 1] <= g) ++r;
            if (pack_stop(mp, r, iter, last_r, stopped, dw.lane)) continue;
            draw_sample<RMAX, T, false, S32, DIAG>(mp.req[r], g - mp.cum[r], dw);
        }
    }
}

// FP32 fix-up pass: every sample of the draw with a kRedoSample row is drawn
// again with careful descents (same uniforms, all modes), overwriting its
// samples, h and weight.  Lanes test 32 samples at once; a warp then redoes
// its flagged samples one by one.  Samples are almost never flagged, so the
// pass costs one read of the N x J sample rows.
template <int RMAX>
__device__ __forceinline__ bool needs_redo(const DrawParams &p, int64_t i) {
    bool bad = false;
    if (i < p.J)
        for (int k = 0; k < p.N; ++k)
            if ((uint32_t)k != p.j) bad |= p.samples[(int64_t)k * p.J + i] == kRedoSample;
    return bad;
}

template <int RMAX, bool S32, bool DIAG>
__global__ void __launch_bounds__(Blk<RMAX, float>::WARPS * 32) krp_fixup_kernel(DrawParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DrawWarp<RMAX, float, DIAG> dw;
    setup_draw_warp<RMAX, float, DIAG>(dw, smem_raw, p.R, p.P, p.S);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * Blk<RMAX, float>::WARPS;
    for (int64_t b = ((int64_t)blockIdx.x * Blk<RMAX, float>::WARPS + warp) * 32; b < p.J; b += nw * 32) {
        unsigned bal = __ballot_sync(0xffffffffu, needs_redo<RMAX>(p, b + lane));
        while (bal) {
            const int src = __ffs(bal) - 1;
            bal &= bal - 1;
            draw_sample<RMAX, float, true, S32, DIAG>(p, b + src, dw);
        }
    }
}

template <int RMAX, bool S32, bool DIAG>
__global__ void __launch_bounds__(Blk<RMAX, float>::WARPS * 32) krp_fixup_multi_kernel(MultiDrawParams mp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DrawWarp<RMAX, float, DIAG> dw;
    setup_draw_warp<RMAX, float, DIAG>(dw, smem_raw, mp.req[0].R, mp.req[0].P, mp.req[0].S);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = mp.cum[mp.n];
    const int64_t nw = (int64_t)gridDim.x * Blk<RMAX, float>::WARPS;
    for (int64_t b = ((int64_t)blockIdx.x * Blk<RMAX, float>::WARPS + warp) * 32; b < total; b += nw * 32) {
        const int64_t g = b + lane;
        int r = 0;
        while (r + 1 < mp.n && mp.cum[r + 1] <= g) ++r;
        // requests stopped by their controls are left as they are
        const bool live = mp.ctl == nullptr || *(volatile uint32_t *)&mp.ctl->status[r] == 0u;
        const bool bad = g < total && live && needs_redo<RMAX>(mp.req[r], g - mp.cum[r]);
        unsigned bal = __ballot_sync(0xffffffffu, bad);
        while (bal) {
            const int src = __ffs(bal) - 1;
            bal &= bal - 1;
            const int rs = __shfl_sync(0xffffffffu, r, src);
            draw_sample<RMAX, float, true, S32, DIAG>(mp.req[rs], b + src - mp.cum[rs], dw);
        }
    }
}

struct TreeSampleParams {
    const void *G;
    const double *U;
    int R, P, S;
    DGeom g;
    double *h;
    const double *scaled_h;
    uint64_t *samples;
    const double *draws;
    int64_t J;
};

// PartitionTree::PTSample_internal (cpp_ext/partition_tree.hpp:232-405):
// x = scaled_h[i]; samples[i] = selected row; h[i] o= U[row].
template <int RMAX, typename T, bool DIAG>
__global__ void __launch_bounds__(Blk<RMAX, T>::WARPS * 32, Resident<T, DIAG>::value / (Blk<RMAX, T>::WARPS * 32)) tree_sample_kernel(TreeSampleParams p) {
    using S = Shape<RMAX>;
    constexpr int XPL = S::XPL;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint16_t *pairs = (uint16_t *)smem_raw;
    const int R = p.R, P = p.P;
    build_pairs(pairs, R);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *slot = smem_raw + ((NodeShape<RMAX, T>::SMAX * sizeof(uint16_t) + 15) / 16 * 16) +
                          warp * WarpSlot<RMAX, T, DIAG>::bytes;
    double *xd = (double *)slot;
    T *xT = sizeof(T) == 8 ? (T *)xd : (T *)(xd + RMAX);
    typename QSel<RMAX, T, DIAG>::type qf;
    qf.P = P;
    qf.S = p.S;
    qf.s = (T *)(slot + RMAX * sizeof(double) + RMAX * sizeof(T));
    for (int64_t i = (int64_t)blockIdx.x * Blk<RMAX, T>::WARPS + warp; i < p.J;
         i += (int64_t)gridDim.x * Blk<RMAX, T>::WARPS) {
        double x[XPL];
#pragma unroll
        for (int q = 0; q < XPL; ++q) {
            int col = lane + 32 * q;
            x[q] = col < R ? p.scaled_h[i * R + col] : 0.0;
        }
        stage_query<RMAX, T>(x, R, xd, xT, lane);
        qf.setup(xT, pairs, lane);
        T frac;
        int64_t c = descend<RMAX>((const T *)p.G, p.S, p.g, p.draws[i], qf, lane, frac,
                                  p.g.F > 1 ? p.U : nullptr, R);
        bool empty = false;
        int64_t t = p.g.F > 1 ? leaf_scan<RMAX, T>(p.U, R, p.g, c, frac, lane_query<RMAX, T>(xT, R, lane), lane, empty)
                              : leaf_index(p.g, c);
        if constexpr (sizeof(T) == 4) {
            if (empty) {  // FP32 descent ended in an all-zero block: redo it evaluating both children
                c = descend_careful<RMAX>((const float *)p.G, p.S, p.g, p.draws[i], qf, lane, frac);
                t = leaf_scan<RMAX, T>(p.U, R, p.g, c, frac, lane_query<RMAX, T>(xT, R, lane), lane, empty);
            }
        }
        if (lane == 0) p.samples[i] = (uint64_t)t;
#pragma unroll
        for (int q = 0; q < XPL; ++q) {
            int col = lane + 32 * q;
            if (col < R) p.h[i * R + col] *= p.U[t * R + col];
        }
        __syncwarp();
    }
}

__global__ void philox_fill_dev_kernel(double *out, int64_t n, uint64_t seed, const uint64_t *ctr_dev) {
    const uint64_t ctr = *ctr_dev;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = philox_uniform(seed, ctr + (uint64_t)i);
}

__global__ void counter_add_kernel(uint64_t *ctr_dev, uint64_t inc) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *ctr_dev += inc;
}

__global__ void philox_fill_kernel(double *out, int64_t n, uint64_t seed, uint64_t ctr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = philox_uniform(seed, ctr + (uint64_t)i);
}

template <int RMAX, typename T, bool DIAG = false>
static size_t desc_smem() {
    return (NodeShape<RMAX, T>::SMAX * sizeof(uint16_t) + 15) / 16 * 16 +
           (size_t)Blk<RMAX, T>::WARPS * WarpSlot<RMAX, T, DIAG>::bytes;
}

// The fast FP32 DIAG32 draw kernels use registers only (no dynamic shared
// memory) and their own block shape; the fix-up kernels run the generic path.
template <int RMAX, typename T, bool DIAG>
struct FastD32 {
    static constexpr bool value = DIAG && sizeof(T) == 4;
};

template <bool S32, int NC, bool SW>
static int launch_d32(const DrawParams &p, cudaStream_t st) {
    using Sh = D32Shape<NC, SW>;
    constexpr int W = Sh::WARPS;
    const int arc = ensure_smem((const void *)krp_draw_d32_kernel<S32, NC, SW>, Sh::SMEM, "krp_draw_d32_kernel");
    if (arc) return arc;
    int64_t blocks = (p.J + (int64_t)W * NC - 1) / ((int64_t)W * NC);
    blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)num_sms() * 64));
    krp_draw_d32_kernel<S32, NC, SW><<<(unsigned)blocks, W * 32, Sh::SMEM, st>>>(p);
    return FTL_OK;
}

template <int RMAX, typename T, bool S32, bool DIAG>
static int launch_draw(const DrawParams &p, cudaStream_t st) {
    const int warps = Blk<RMAX, T>::WARPS;
    size_t smem = desc_smem<RMAX, T, DIAG>();
    if constexpr (FastD32<RMAX, T, DIAG>::value) {
        int lrc;
        switch (tuned_variant(FTL_TUNE_DRAW, p.R, FTL_PREC_FP32)) {
            case 0: lrc = launch_d32<S32, 1, false>(p, st); break;
            case 1: lrc = launch_d32<S32, 2, false>(p, st); break;
            case 3: lrc = launch_d32<S32, 3, true>(p, st); break;
            case 4: lrc = launch_d32<S32, 4, true>(p, st); break;
            case 5: lrc = launch_d32<S32, 6, true>(p, st); break;
            default: lrc = launch_d32<S32, 3, false>(p, st); break;
        }
        if (lrc) return lrc;
    } else {
        const int arc = ensure_smem((const void *)krp_draw_kernel<RMAX, T, S32, DIAG>, smem, "krp_draw_kernel");
        if (arc) return arc;
        int64_t blocks = (p.J + warps - 1) / warps;
        blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)num_sms() * 64));
        krp_draw_kernel<RMAX, T, S32, DIAG><<<(unsigned)blocks, warps * 32, smem, st>>>(p);
    }
    int rc = check_launch("krp_draw_kernel");
    if (rc || sizeof(T) == 8) return rc;
    {
        const int arc = ensure_smem((const void *)krp_fixup_kernel<RMAX, S32, DIAG>, smem, "krp_fixup_kernel");
        if (arc) return arc;
    }
    int64_t fblocks = (p.J + 32 * warps - 1) / (32 * warps);
    fblocks = std::max<int64_t>(1, std::min<int64_t>(fblocks, (int64_t)num_sms() * 8));
    krp_fixup_kernel<RMAX, S32, DIAG><<<(unsigned)fblocks, warps * 32, smem, st>>>(p);
    return check_launch("krp_fixup_kernel");
}

template <int RMAX, typename T, bool S32, bool DIAG>
static int launch_multi(const MultiDrawParams &mp, cudaStream_t st) {
    const int warps = Blk<RMAX, T>::WARPS;
    size_t smem = desc_smem<RMAX, T, DIAG>();
    const int64_t total = mp.cum[mp.n];
    {
        constexpr bool fast = FastD32<RMAX, T, DIAG>::value;
        const int dwarps = Blk<RMAX, T, DIAG>::WARPS;
        const size_t dsmem = fast ? 0 : smem;
        const int arc =
            ensure_smem((const void *)krp_draw_multi_kernel<RMAX, T, S32, DIAG>, dsmem, "krp_draw_multi_kernel");
        if (arc) return arc;
        int64_t blocks = (total + dwarps - 1) / dwarps;
        blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)num_sms() * 64));
        krp_draw_multi_kernel<RMAX, T, S32, DIAG><<<(unsigned)blocks, dwarps * 32, dsmem, st>>>(mp);
    }
    int rc = check_launch("krp_draw_multi_kernel");
    if (rc || sizeof(T) == 8) return rc;
    {
        const int arc = ensure_smem((const void *)krp_fixup_multi_kernel<RMAX, S32, DIAG>, smem, "krp_fixup_multi_kernel");
        if (arc) return arc;
    }
    int64_t fblocks = (total + 32 * warps - 1) / (32 * warps);
    fblocks = std::max<int64_t>(1, std::min<int64_t>(fblocks, (int64_t)num_sms() * 8));
    krp_fixup_multi_kernel<RMAX, S32, DIAG><<<(unsigned)fblocks, warps * 32, smem, st>>>(mp);
    return check_launch("krp_fixup_multi_kernel");
}

template <int RMAX, typename T, bool DIAG>
static int launch_tree_sample(const TreeSampleParams &p, cudaStream_t st) {
    const int warps = Blk<RMAX, T>::WARPS;
    size_t smem = desc_smem<RMAX, T, DIAG>();
    {
        const int arc = ensure_smem((const void *)tree_sample_kernel<RMAX, T, DIAG>, smem, "tree_sample_kernel");
        if (arc) return arc;
    }
    int64_t blocks = (p.J + warps - 1) / warps;
    blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)num_sms() * 64));
    tree_sample_kernel<RMAX, T, DIAG><<<(unsigned)blocks, warps * 32, smem, st>>>(p);
    return check_launch("tree_sample_kernel");
}

// FP32 draws read the leaf blocks from the FP32 factor copies when every
// sampled mode has one (the values are the same FP32 roundings the scan
// would make of the FP64 rows, so the results are identical).
static bool shadows_ready(const DrawParams &p) {
    for (int k = 0; k < p.N; ++k)
        if ((uint32_t)k != p.j && p.U32[k] == nullptr) return false;
    return true;
}

template <typename T>
static int dispatch_draw(const DrawParams &p, cudaStream_t st) {
    if constexpr (sizeof(T) == 4) {
        const bool diag = node_layout(p.R, sizeof(T)) == FTL_LAYOUT_DIAG32;
        if (shadows_ready(p)) {
            if (diag) return launch_draw<32, T, true, true>(p, st);
            if (p.R <= 32) return launch_draw<32, T, true, false>(p, st);
            if (p.R <= 64) return launch_draw<64, T, true, false>(p, st);
            return launch_draw<128, T, true, false>(p, st);
        }
        if (diag) return launch_draw<32, T, false, true>(p, st);
    }
    if (p.R <= 32) return launch_draw<32, T, false, false>(p, st);
    if (p.R <= 64) return launch_draw<64, T, false, false>(p, st);
    return launch_draw<128, T, false, false>(p, st);
}

// The register/shared-memory shapes are chosen by max(R, F): a lane handles
// RMAX/32 vector entries and RMAX/32 rows of a leaf block.
template <typename T>
static int dispatch_tree_sample(const TreeSampleParams &p, cudaStream_t st) {
    const int64_t RF = std::max<int64_t>(p.R, p.g.F);
    if constexpr (sizeof(T) == 4)
        if (node_layout(p.R, sizeof(T)) == FTL_LAYOUT_DIAG32 && RF <= 32) return launch_tree_sample<32, T, true>(p, st);
    if (RF <= 32) return launch_tree_sample<32, T, false>(p, st);
    if (RF <= 64) return launch_tree_sample<64, T, false>(p, st);
    return launch_tree_sample<128, T, false>(p, st);
}

static int validate_plan(const ftl_krp_plan *plan) {
    FTL_CHECK_ARG(plan != nullptr, "krp: plan is NULL");
    FTL_CHECK_ARG(plan->N >= 1 && plan->N <= FTL_MAX_MODES, "krp: N=%d outside [1, %d]", plan->N,
                  FTL_MAX_MODES);
    FTL_CHECK_ARG(plan->R >= 1 && plan->R <= FTL_MAX_RANK, "krp: R=%d outside [1, %d]", plan->R,
                  FTL_MAX_RANK);
    FTL_CHECK_ARG(plan->J >= 1, "krp: J=%lld must be positive", (long long)plan->J);
    FTL_CHECK_ARG(plan->prec == FTL_PREC_FP64 || plan->prec == FTL_PREC_FP32, "krp: bad precision %d",
                  plan->prec);
    FTL_CHECK_ARG(plan->eig_G && plan->M && plan->lambda && plan->pinv32, "krp: null workspace pointer");
    FTL_CHECK_ARG(aligned16(plan->eig_G) && aligned16(plan->M) && aligned16(plan->pinv32),
                  "krp: eig_G, M and pinv32 must be 16-byte aligned");
    for (int k = 0; k < plan->N; ++k) {
        FTL_CHECK_ARG(plan->dims[k] >= 1, "krp: dims[%d]=%lld must be positive", k, (long long)plan->dims[k]);
        FTL_CHECK_ARG(plan->U[k] && plan->gram_G[k], "krp: null factor or tree pointer for mode %d", k);
        FTL_CHECK_ARG(aligned16(plan->gram_G[k]), "krp: tree of mode %d must be 16-byte aligned", k);
    }
    return FTL_OK;
}

static uint32_t normalise_j(const ftl_krp_plan *plan, uint32_t j) {
    return j < (uint32_t)plan->N ? j : (uint32_t)plan->N + 1;
}

}  // namespace ftl

using namespace ftl;

extern "C" int ftl_krp_plan_sizes(int N, int R, int prec, size_t *eig_bytes, size_t *M_bytes,
                                  size_t *lambda_bytes, size_t *pinv32_bytes) {
    FTL_CHECK_ARG(N >= 1 && N <= FTL_MAX_MODES && R >= 1 && R <= FTL_MAX_RANK,
                  "ftl_krp_plan_sizes: bad N=%d R=%d", N, R);
    FTL_CHECK_ARG(valid_prec(prec), "ftl_krp_plan_sizes: bad precision");
    const int esize = prec_bytes(prec);
    if (eig_bytes) *eig_bytes = (size_t)N * (2 * R - 1) * node_stride(R, esize) * esize;
    if (M_bytes) *M_bytes = (cm_pinv64_offset(N, R) + node_stride(R, 8)) * sizeof(double);
    if (lambda_bytes) *lambda_bytes = (size_t)(N + 1) * R * sizeof(double);
    if (pinv32_bytes) *pinv32_bytes = (size_t)node_stride(R, 4) * sizeof(float);
    return FTL_OK;
}

extern "C" int ftl_krp_compute_m(const ftl_krp_plan *plan, uint32_t j, void *stream) {
    int rc = validate_plan(plan);
    if (rc) return rc;
    uint32_t jn = normalise_j(plan, j);
    int included = 0;
    for (int k = 0; k < plan->N; ++k) included += ((uint32_t)k != jn);
    FTL_CHECK_ARG(included >= 1, "krp: no mode left to sample (N=%d, j=%u)", plan->N, j);
    return computem_launch(plan, jn, (cudaStream_t)stream);
}

static void fill_draw_params(DrawParams &p, const ftl_krp_plan *plan, uint32_t j, uint64_t *samples, double *h,
                             double *weights, const double *draws, uint64_t seed, uint64_t ctr);

extern "C" int ftl_krp_sample(const ftl_krp_plan *plan, uint32_t j, uint64_t *samples, double *h,
                              double *weights, const double *draws, uint64_t seed, uint64_t ctr,
                              void *stream) {
    int rc = validate_plan(plan);
    if (rc) return rc;
    FTL_CHECK_ARG(samples != nullptr, "ftl_krp_sample: samples is NULL");
    DrawParams p;
    fill_draw_params(p, plan, j, samples, h, weights, draws, seed, ctr);
    cudaStream_t st = (cudaStream_t)stream;
    if (plan->prec == FTL_PREC_FP64) return dispatch_draw<double>(p, st);
    return dispatch_draw<float>(p, st);
}

static void fill_draw_params(DrawParams &p, const ftl_krp_plan *plan, uint32_t j, uint64_t *samples, double *h,
                             double *weights, const double *draws, uint64_t seed, uint64_t ctr) {
    p.N = plan->N;
    p.R = plan->R;
    p.P = packed_size(plan->R);
    p.S = node_stride(plan->R, plan->prec == FTL_PREC_FP64 ? 8 : 4);
    p.j = normalise_j(plan, j);
    p.J = plan->J;
    for (int k = 0; k < FTL_MAX_MODES; ++k) {
        if (k < plan->N) {
            Geom g = make_geom(plan->dims[k], std::min<int64_t>(plan->R, plan->dims[k]));
            p.gram[k] = to_dgeom(g);
            p.U[k] = plan->U[k];
            p.U32[k] = plan->prec == FTL_PREC_FP32 ? plan->U32[k] : nullptr;
            p.gram_G[k] = plan->gram_G[k];
            p.offset[k] = ((uint32_t)(k + 1) == p.j) ? k + 2 : k + 1;
        } else {
            p.U[k] = nullptr;
            p.U32[k] = nullptr;
            p.gram_G[k] = nullptr;
            p.offset[k] = 0;
        }
    }
    p.eig = to_dgeom(make_geom(plan->R, 1));
    p.eig_G = plan->eig_G;
    p.M = plan->M;
    p.pinv32 = plan->pinv32;
    p.samples = samples;
    p.h = h;
    p.weights = weights;
    p.draws = draws;
    p.seed = seed;
    p.ctr = ctr;
}

static int sample_packed(const ftl_krp_plan *const *plans, int n, const uint32_t *js, uint64_t *const *samples,
                         double *const *h, double *const *weights, const double *const *draws, const uint64_t *seeds,
                         const uint64_t *ctrs, const uint32_t *const *cancel, uint64_t budget_ns,
                         ftl_pack_status *status, void *stream);

extern "C" int ftl_krp_sample_packed(const ftl_krp_plan *const *plans, int n, const uint32_t *js,
                                     uint64_t *const *samples, double *const *h, double *const *weights,
                                     const double *const *draws, const uint64_t *seeds, const uint64_t *ctrs,
                                     void *stream) {
    return sample_packed(plans, n, js, samples, h, weights, draws, seeds, ctrs, nullptr, 0, nullptr, stream);
}

extern "C" int ftl_krp_sample_packed_ctl(const ftl_krp_plan *const *plans, int n, const uint32_t *js,
                                         uint64_t *const *samples, double *const *h, double *const *weights,
                                         const double *const *draws, const uint64_t *seeds, const uint64_t *ctrs,
                                         const uint32_t *const *cancel, uint64_t budget_ns, ftl_pack_status *status,
                                         void *stream) {
    FTL_CHECK_ARG(status != nullptr, "ftl_krp_sample_packed_ctl: status is NULL");
    FTL_CHECK_ARG(((uintptr_t)status & 7u) == 0, "ftl_krp_sample_packed_ctl: status must be 8-byte aligned");
    return sample_packed(plans, n, js, samples, h, weights, draws, seeds, ctrs, cancel, budget_ns, status, stream);
}

static int sample_packed(const ftl_krp_plan *const *plans, int n, const uint32_t *js, uint64_t *const *samples,
                         double *const *h, double *const *weights, const double *const *draws, const uint64_t *seeds,
                         const uint64_t *ctrs, const uint32_t *const *cancel, uint64_t budget_ns,
                         ftl_pack_status *status, void *stream) {
    FTL_CHECK_ARG(plans && js && samples && h && weights && seeds && ctrs, "ftl_krp_sample_packed: null array");
    FTL_CHECK_ARG(n >= 1 && n <= FTL_MAX_PACK, "ftl_krp_sample_packed: n=%d outside [1, %d]", n, FTL_MAX_PACK);
    MultiDrawParams mp;
    mp.n = n;
    mp.ctl = status;
    mp.budget_ns = budget_ns;
    for (int i = 0; i < FTL_MAX_PACK; ++i) mp.cancel[i] = (cancel && i < n) ? cancel[i] : nullptr;
    if (status) {
        cudaError_t err = cudaMemsetAsync(status, 0, sizeof(ftl_pack_status), (cudaStream_t)stream);
        if (err != cudaSuccess)
            return fail(FTL_E_CUDA, "ftl_krp_sample_packed_ctl: clearing the status: %s", cudaGetErrorString(err));
    }
    mp.cum[0] = 0;
    for (int i = 0; i < n; ++i) {
        int rc = validate_plan(plans[i]);
        if (rc) return rc;
        FTL_CHECK_ARG(plans[i]->R == plans[0]->R && plans[i]->prec == plans[0]->prec,
                      "ftl_krp_sample_packed: request %d has R=%d prec=%d, request 0 R=%d prec=%d", i,
                      plans[i]->R, plans[i]->prec, plans[0]->R, plans[0]->prec);
        FTL_CHECK_ARG(samples[i] != nullptr, "ftl_krp_sample_packed: samples[%d] is NULL", i);
        fill_draw_params(mp.req[i], plans[i], js[i], samples[i], h[i], weights[i], draws ? draws[i] : nullptr,
                         seeds[i], ctrs[i]);
        mp.cum[i + 1] = mp.cum[i] + plans[i]->J;
    }
    for (int i = n; i < FTL_MAX_PACK; ++i) mp.cum[i + 1] = mp.cum[n];
    cudaStream_t st = (cudaStream_t)stream;
    const int R = plans[0]->R;
    if (plans[0]->prec == FTL_PREC_FP64) {
        if (R <= 32) return launch_multi<32, double, false, false>(mp, st);
        if (R <= 64) return launch_multi<64, double, false, false>(mp, st);
        return launch_multi<128, double, false, false>(mp, st);
    }
    bool s32 = true;
    for (int i = 0; i < n; ++i) s32 = s32 && shadows_ready(mp.req[i]);
    const bool diag = node_layout(R, 4) == FTL_LAYOUT_DIAG32;
    if (s32) {
        if (diag) return launch_multi<32, float, true, true>(mp, st);
        if (R <= 32) return launch_multi<32, float, true, false>(mp, st);
        if (R <= 64) return launch_multi<64, float, true, false>(mp, st);
        return launch_multi<128, float, true, false>(mp, st);
    }
    if (diag) return launch_multi<32, float, false, true>(mp, st);
    if (R <= 32) return launch_multi<32, float, false, false>(mp, st);
    if (R <= 64) return launch_multi<64, float, false, false>(mp, st);
    return launch_multi<128, float, false, false>(mp, st);
}

extern "C" int ftl_krp_draw(const ftl_krp_plan *plan, uint32_t j, uint64_t *samples, double *h,
                            double *weights, const double *draws, uint64_t seed, uint64_t ctr,
                            void *stream) {
    int rc = ftl_krp_compute_m(plan, j, stream);
    if (rc) return rc;
    return ftl_krp_sample(plan, j, samples, h, weights, draws, seed, ctr, stream);
}

extern "C" int ftl_tree_sample(const void *G, int prec, const double *U, int64_t n, int R, int64_t F,
                               double *h, const double *scaled_h, uint64_t *samples,
                               const double *draws, int64_t J, void *stream) {
    FTL_CHECK_ARG(G && U && h && scaled_h && samples && draws, "ftl_tree_sample: null pointer");
    FTL_CHECK_ARG(aligned16(G), "ftl_tree_sample: the tree must be 16-byte aligned");
    FTL_CHECK_ARG(n >= 1 && R >= 1 && R <= FTL_MAX_RANK && F >= 1 && F <= FTL_MAX_RANK && J >= 0,
                  "ftl_tree_sample: bad shape n=%lld R=%d F=%lld J=%lld (need R, F in [1, %d])",
                  (long long)n, R, (long long)F, (long long)J, FTL_MAX_RANK);
    if (J == 0) return FTL_OK;
    TreeSampleParams p;
    p.G = G;
    p.U = U;
    p.R = R;
    p.P = packed_size(R);
    FTL_CHECK_ARG(valid_prec(prec), "ftl_tree_sample: bad precision %d", prec);
    prec = storage_prec(prec);
    p.S = node_stride(R, prec_bytes(prec));
    p.g = to_dgeom(make_geom(n, F));
    p.h = h;
    p.scaled_h = scaled_h;
    p.samples = samples;
    p.draws = draws;
    p.J = J;
    cudaStream_t st = (cudaStream_t)stream;
    if (prec == FTL_PREC_FP64) return dispatch_tree_sample<double>(p, st);
    if (prec == FTL_PREC_FP32) return dispatch_tree_sample<float>(p, st);
    return fail(FTL_E_ARG, "ftl_tree_sample: bad precision %d", prec);
}

extern "C" int ftl_philox_uniforms(double *out, int64_t n, uint64_t seed, uint64_t ctr, void *stream) {
    FTL_CHECK_ARG(out != nullptr && n >= 0, "ftl_philox_uniforms: bad arguments");
    if (n == 0) return FTL_OK;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 16);
    philox_fill_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(out, n, seed, ctr);
    return check_launch("philox_fill_kernel");
}

extern "C" int ftl_philox_uniforms_dev(double *out, int64_t n, uint64_t seed, uint64_t *ctr_dev, void *stream) {
    FTL_CHECK_ARG(out != nullptr && ctr_dev != nullptr && n >= 0, "ftl_philox_uniforms_dev: bad arguments");
    if (n == 0) return FTL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 16);
    philox_fill_dev_kernel<<<blocks, 256, 0, st>>>(out, n, seed, ctr_dev);
    counter_add_kernel<<<1, 32, 0, st>>>(ctr_dev, (uint64_t)n);
    return check_launch("philox_fill_dev_kernel");
}

namespace ftl {
__global__ void shadow_kernel(const double *__restrict__ U, int64_t n, float *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)U[i];
}
}  // namespace ftl

extern "C" int ftl_factor_shadow(const double *U, int64_t count, float *out, void *stream) {
    FTL_CHECK_ARG(U && out && count >= 0, "ftl_factor_shadow: bad arguments");
    if (count == 0) return FTL_OK;
    int blocks = (int)std::min<int64_t>((count + 255) / 256, (int64_t)num_sms() * 16);
    shadow_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(U, count, out);
    return check_launch("shadow_kernel");
}
