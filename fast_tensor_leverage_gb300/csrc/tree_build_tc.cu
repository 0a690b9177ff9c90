// Leaf Grams of a partition tree on the tensor cores (tcgen05), for factors
// of R <= 32 columns with leaves of F <= R rows.
//
// PartitionTree::build_tree (cpp_ext/partition_tree.hpp:120-170) forms
// G_leaf = U_blk^T U_blk for every leaf block (dsyrk) and sums children up
// the tree.  Here the leaf level runs as a persistent kernel, one CTA of 16
// warps per SM (the conversion is bound by instruction latency):
//
//   * TMA brings tiles of four consecutive leaf blocks (4F rows x R FP64
//     values, contiguous in U) into a four-stage shared-memory ring
//     (cp.async.bulk.tensor over a 2-D tensor map of U when R is even, the
//     untiled cp.async.bulk otherwise), completion tracked by mbarriers.
//   * Warps w, w+4, w+8, w+12 convert leaf w of the tile (8 of its 32 rows
//     each): lane c takes column c, rounds the
//     FP64 values to FP32 with integer operations (no FP64 instruction), and
//     writes them as the K-major operand X^T (M = 128 rows: 32 columns of
//     each of the four leaves; K = 32: the leaf's rows, zero padded) in the
//     128-byte-swizzled canonical layout; the FP32 copy of U for the descent's
//     leaf scans is written to global memory on the way.
//   * One thread issues tcgen05.mma with M = N = 128: D = X^T X in TMEM, whose
//     four 32 x 32 diagonal blocks are the four leaf Grams (the off-diagonal
//     blocks are wasted work: the leaf level is bound by HBM traffic, not by
//     the tensor pipe).  3xTF32: the FP32 inputs split as hi + lo (hi = the
//     FP32 value truncated to TF32), D = hi hi + hi lo + lo hi; BF16: inputs
//     rounded to BF16, one product.  Accumulation in FP32.
//   * Warp w then reads its diagonal block from TMEM (tcgen05.ld, its own lane
//     quarter) and writes the leaf node in the tree's FP32 layout.
//   Two accumulators and two operand buffers let the MMA of tile i run while
//   tile i+1 is converted and tile i-1 is written back.
//
// Every mbarrier wait is bounded by a clock budget: when it runs out the
// kernel sets a device status bit (ftl_device_status), stops, waits (again
// bounded) for its own copies and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "ftl_common.cuh"

namespace ftl {

__device__ unsigned int g_device_status;  // bit 0: a bounded wait of the tensor-core build ran out

namespace tc {

constexpr int kThreads = 512;
constexpr int kStages = 4;
constexpr int kStageBytes = 128 * 32 * 8;   // 4 leaves x 32 rows x 32 FP64 columns
constexpr int kOpBytes = 128 * 128;         // 128 operand rows x 128 bytes
constexpr int kTmemCols = 256;              // two 128 x 128 FP32 accumulators
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz

// shared memory map (offsets from a 1024-byte aligned base)
constexpr int kOffStage = 0;
constexpr int kOffOp = kOffStage + kStages * kStageBytes;  // [buffer][hi, lo]
constexpr int kOffBar = kOffOp + 4 * kOpBytes;             // full[kStages], mma[2]
constexpr int kOffMisc = kOffBar + 64 * 8;                 // tmem base, abort flag
constexpr int kOffXpose = kOffMisc + 64;                   // 4 warps x 32 x 33 floats
constexpr int kSmemBytes = kOffXpose + 4 * 32 * 33 * 4 + 1024;  // + alignment slack

struct Params {
    const double *U;
    int64_t n;
    int R, F;
    int64_t leaf_count, ntiles;
    DGeom g;
    float *G;      // tree nodes (FP32)
    int S;         // node stride
    int layout;    // FTL_LAYOUT_*
    float *U32;    // FP32 copy of U, or null
    int use_tmap;  // 2-D tensor-map copies (R even) or untiled bulk copies
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Wait for phase `parity` of `bar` to complete, at most kWaitCycles; false
// (and the CTA's abort flag and the device status set) when it runs out or
// another thread of the CTA has already given up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    const long long t0 = clock64();
    while (!mbar_test(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > kWaitCycles) {
            atomicOr(&g_device_status, 1u);
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), start address >> 4 in bits 0-13,
// descriptor version 1 (bits 46-47), swizzle mode 2 = 128B (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(const void *p) {
    const uint64_t addr = (uint64_t)(smem_u32(p) & 0x3FFFF) >> 4;
    const uint64_t lbo = 1;              // unused by swizzled K-major layouts
    const uint64_t sbo = 1024 >> 4;
    return addr | (lbo << 16) | (sbo << 32) | (1ull << 46) | (2ull << 61);
}

// Instruction descriptor: D FP32 (bits 4-5 = 1), A and B formats (bits 7-9,
// 10-12), both K-major, N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t idesc(uint32_t ab_format, int M, int N) {
    return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}
constexpr uint32_t kIdescTF32 = idesc(2, 128, 128);  // kind::tf32, TF32 inputs
constexpr uint32_t kIdescBF16 = idesc(1, 128, 128);  // kind::f16, BF16 inputs

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint32_t f2bf_rn(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u + 0x7fffu + ((u >> 16) & 1u)) >> 16;
}

// Byte offset of 16-byte chunk `chunk` of operand row m (128-byte swizzle).
__device__ __forceinline__ int op_off(int m, int chunk) {
    return (m >> 3) * 1024 + (m & 7) * 128 + ((chunk ^ (m & 7)) << 4);
}

// MODE 0: 3xTF32; MODE 1: BF16.
template <int MODE>
__global__ void __launch_bounds__(kThreads, 1) leaf_gram_tc_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                  Params p) {
    extern __shared__ unsigned char smem_dyn[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_dyn + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + kOffBar);
    uint64_t *mmad = full + kStages;
    uint32_t *tmem_slot = (uint32_t *)(smem + kOffMisc);
    volatile int *abort_flag = (volatile int *)(smem + kOffMisc + 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int R = p.R, F = p.F;

    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(full + s, 1);
        mbar_init(mmad, 1);
        mbar_init(mmad + 1, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const int64_t ntl = p.ntiles > blockIdx.x ? (p.ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    const int tile_rows = 4 * F;

    // bytes the untiled copy of local tile i brings (a multiple of 16; the
    // tail of the last tile past it is read from global memory)
    auto bulk_bytes = [&](int64_t i) -> uint32_t {
        const int64_t row0 = (blockIdx.x + i * (int64_t)gridDim.x) * tile_rows;
        const int64_t rows = min((int64_t)tile_rows, p.n - row0);
        return (uint32_t)((rows * R * 8) & ~(int64_t)15);
    };
    auto issue_load = [&](int64_t i) {
        const int s = (int)(i % kStages);
        const int64_t row0 = (blockIdx.x + i * (int64_t)gridDim.x) * tile_rows;
        void *dst = smem + kOffStage + s * kStageBytes;
        if (p.use_tmap) {
            mbar_expect_tx(full + s, (uint32_t)(tile_rows * R * 8));
            tma_load_2d(dst, &tmap, 0, (int)row0, full + s);
        } else {
            const uint32_t bytes = bulk_bytes(i);
            if (bytes) {
                mbar_expect_tx(full + s, bytes);
                bulk_load(dst, p.U + row0 * R, bytes, full + s);
            } else {
                mbar_arrive(full + s);
            }
        }
    };

    if (tid == 0)
        for (int64_t i = 0; i < min((int64_t)(kStages), (int64_t)(ntl)); ++i) issue_load(i);

    // Epilogue of local tile i: warp w < 4 writes leaf w's node from
    // accumulator i % 2 (warp w reads TMEM lanes 32w..32w+31).  The TMEM load
    // is warp-collective: a warp whose wait failed in any lane skips it as a
    // whole.
    auto epilogue = [&](int64_t i) -> bool {
        if (warp >= 4) return true;
        const int b = (int)(i & 1);
        const bool waited = mbar_wait(mmad + b, (uint32_t)((i >> 1) & 1), abort_flag);
        if (!__all_sync(0xffffffffu, waited)) return false;
        tc_fence_after();
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(b * 128 + 32 * warp), v);
        tc_fence_before();
        const int64_t leaf = (blockIdx.x + i * (int64_t)gridDim.x) * 4 + warp;  // warp < 4
        if (leaf < p.leaf_count) {
            float *xp = (float *)(smem + kOffXpose) + warp * 32 * 33;
#pragma unroll
            for (int j = 0; j < 32; ++j) xp[lane * 33 + j] = v[j];
            __syncwarp();
            float *node = p.G + leaf_node(p.g, leaf) * (int64_t)p.S;
            if (p.layout == FTL_LAYOUT_DIAG32) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float4 o;
                    o.x = xp[lane * 33 + ((lane + 4 * q + 0) & 31)];
                    o.y = xp[lane * 33 + ((lane + 4 * q + 1) & 31)];
                    o.z = xp[lane * 33 + ((lane + 4 * q + 2) & 31)];
                    o.w = xp[lane * 33 + ((lane + 4 * q + 3) & 31)];
                    reinterpret_cast<float4 *>(node)[32 * q + lane] = o;
                }
                node[512 + lane] = xp[lane * 33 + ((lane + 16) & 31)];
            } else {
                // packed upper triangle, one row per lane, then the padding
                if (lane < R) {
                    float *row = node + packed_row_offset(lane, R);
                    for (int bb = lane; bb < R; ++bb) row[bb - lane] = xp[lane * 33 + bb];
                }
                for (int e = packed_size(R) + lane; e < p.S; e += 32) node[e] = 0.0f;
            }
            __syncwarp();
        }
        return true;
    };

    // Every exit decision is taken at a block-wide barrier (__syncthreads_or),
    // so all threads leave the loop together.
    bool ok = true, epi_ok = true;
    int64_t issued_mma = 0;                              // MMA batches committed
    int64_t issued_loads = min((int64_t)(kStages), (int64_t)(ntl));   // tile loads issued (thread 0)
    for (int64_t i = 0; i < ntl; ++i) {
        const int s = (int)(i % kStages);
        const int b = (int)(i & 1);
        // operand buffer b was last read by the MMA of tile i - 2: every warp
        // waits for it (the epilogue warps already have) before overwriting it
        bool waited = i < 2 || mbar_wait(mmad + b, (uint32_t)(((i - 2) >> 1) & 1), abort_flag);
        waited = waited && mbar_wait(full + s, (uint32_t)((i / kStages) & 1), abort_flag);
        // convert: warp w = leaf w % 4 of the tile, rows 8 (w / 4) .. +7, lane = column
        if (waited) {
            const int lw = warp & 3, kg = warp >> 2;
            const int64_t tile = blockIdx.x + i * (int64_t)gridDim.x;
            const int64_t row0 = tile * tile_rows;
            const int64_t leaf = tile * 4 + lw;
            const int rows_leaf = leaf < p.leaf_count ? (int)min((int64_t)F, p.n - leaf * F) : 0;
            const double *st = (const double *)(smem + kOffStage + s * kStageBytes);
            const uint32_t copied = p.use_tmap ? 0xffffffffu : bulk_bytes(i);
            const int c = lane;
            const int m = 32 * lw + c;
            unsigned char *op_hi = smem + kOffOp + (b * 2 + 0) * kOpBytes;
            unsigned char *op_lo = smem + kOffOp + (b * 2 + 1) * kOpBytes;
            // full 32 x 32 leaf copied by the tensor map (the common case):
            // no per-value bounds, copy or fallback checks
            const bool full = p.use_tmap && R == 32 && F == 32 && rows_leaf == 32;
            const double *srow = st + (lw * 32) * 32 + c;
            float *u32 = (full && p.U32) ? p.U32 + row0 * 32 + (lw * 32) * 32 + c : nullptr;
#pragma unroll
            for (int q = 2 * kg; q < 2 * kg + 2; ++q) {
                float v[4];
                if (full) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        v[j] = d2f_rn(srow[(4 * q + j) * 32]);
                        if (u32) u32[(4 * q + j) * 32] = v[j];
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int k = 4 * q + j;
                        double x = 0.0;
                        if (c < R && k < rows_leaf) {
                            const int e = (lw * F + k) * R + c;  // element of the staged tile
                            x = ((uint32_t)e * 8u + 8u <= copied) ? st[e] : p.U[row0 * R + e];
                        }
                        v[j] = d2f_rn(x);
                        if (p.U32 && c < R && k < rows_leaf) p.U32[row0 * R + (lw * F + k) * R + c] = v[j];
                    }
                }
                if (MODE == 0) {
                    float4 h, l;
                    h.x = __uint_as_float(__float_as_uint(v[0]) & 0xffffe000u);
                    h.y = __uint_as_float(__float_as_uint(v[1]) & 0xffffe000u);
                    h.z = __uint_as_float(__float_as_uint(v[2]) & 0xffffe000u);
                    h.w = __uint_as_float(__float_as_uint(v[3]) & 0xffffe000u);
                    l.x = v[0] - h.x;
                    l.y = v[1] - h.y;
                    l.z = v[2] - h.z;
                    l.w = v[3] - h.w;
                    *reinterpret_cast<float4 *>(op_hi + op_off(m, q)) = h;
                    *reinterpret_cast<float4 *>(op_lo + op_off(m, q)) = l;
                } else {
                    // 8 BF16 values per 16-byte chunk: rows 4q..4q+3 fill half of chunk q/2
                    const uint32_t w0 = f2bf_rn(v[0]) | (f2bf_rn(v[1]) << 16);
                    const uint32_t w1 = f2bf_rn(v[2]) | (f2bf_rn(v[3]) << 16);
                    *reinterpret_cast<uint2 *>(op_hi + op_off(m, q >> 1) + (q & 1) * 8) = make_uint2(w0, w1);
                }
            }
        }
        fence_proxy_async();
        tc_fence_before();
        if (__syncthreads_or(!waited || !epi_ok || *abort_flag)) {
            ok = false;
            break;
        }
        if (tid == 0) {
            if (i + kStages < ntl) {
                issue_load(i + kStages);
                issued_loads = i + kStages + 1;
            }
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(b * 128);
            const uint64_t a_hi = sw128_desc(smem + kOffOp + (b * 2 + 0) * kOpBytes);
            if (MODE == 0) {
                const uint64_t a_lo = sw128_desc(smem + kOffOp + (b * 2 + 1) * kOpBytes);
#pragma unroll
                for (int ks = 0; ks < 4; ++ks) {  // K = 32 in steps of 8 (32 bytes)
                    const uint64_t adv = (uint64_t)(2 * ks);
                    mma_tf32(d, a_hi + adv, a_lo + adv, kIdescTF32, ks > 0);
                    mma_tf32(d, a_lo + adv, a_hi + adv, kIdescTF32, 1);
                    mma_tf32(d, a_hi + adv, a_hi + adv, kIdescTF32, 1);
                }
            } else {
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {  // K = 32 in steps of 16 (32 bytes)
                    const uint64_t adv = (uint64_t)(2 * ks);
                    mma_f16(d, a_hi + adv, a_hi + adv, kIdescBF16, ks > 0);
                }
            }
            mma_commit(mmad + b);
        }
        issued_mma = i + 1;
        if (i >= 1) epi_ok = epilogue(i - 1);
    }
    if (ok && ntl > 0) epi_ok = epilogue(ntl - 1);
    ok = !__syncthreads_or(!ok || !epi_ok);

    if (!ok) {
        // stop: let this CTA's own copies and MMAs in flight finish (bounded)
        // before the shared memory and TMEM are released
        if (tid == 0) {
            const long long t0 = clock64();
            for (int64_t i = issued_mma; i < issued_loads; ++i) {  // loads issued, not consumed
                const int s = (int)(i % kStages);
                while (!mbar_test(full + s, (uint32_t)((i / kStages) & 1)) && clock64() - t0 < kWaitCycles) {
                }
            }
            for (int64_t i = max((int64_t)(0), (int64_t)(issued_mma - 2)); i < issued_mma; ++i)
                while (!mbar_test(mmad + (i & 1), (uint32_t)((i >> 1) & 1)) && clock64() - t0 < kWaitCycles) {
                }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

}  // namespace tc

// Leaf level of an FP32 tree on the tensor cores: mode 0 = 3xTF32, 1 = BF16.
// U32 (n x R FP32, may be null) receives the FP32 copy of U.  Requires
// R <= 32 and F <= R (one leaf block fits a 32-row K extent).
int tc_leaf_grams(const double *U, int64_t n, int R, int64_t F, int mode, float *G, float *U32, cudaStream_t st) {
    using namespace tc;
    if (R > 32 || F > R || F < 1)
        return fail(FTL_E_UNSUPPORTED, "tensor-core leaf build: needs F <= R <= 32 (R=%d F=%lld)", R, (long long)F);
    if (((uintptr_t)U & 15u) != 0) return fail(FTL_E_ARG, "tensor-core leaf build: U must be 16-byte aligned");
    if (n >= ((int64_t)1 << 31))
        return fail(FTL_E_UNSUPPORTED, "tensor-core leaf build: n=%lld rows exceed the 32-bit copy coordinates",
                    (long long)n);
    Geom geom = make_geom(n, F);
    Params p;
    p.U = U;
    p.n = n;
    p.R = R;
    p.F = (int)F;
    p.leaf_count = geom.leaf_count;
    p.ntiles = (geom.leaf_count + 3) / 4;
    p.g = to_dgeom(geom);
    p.G = G;
    p.S = node_stride(R, 4);
    p.layout = node_layout(R, 4);
    p.U32 = U32;
    p.use_tmap = (R % 2) == 0;
    alignas(64) CUtensorMap map;
    memset(&map, 0, sizeof(map));
    if (p.use_tmap) {
        PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
        if (!enc) return fail(FTL_E_CUDA, "tensor-core leaf build: cuTensorMapEncodeTiled is not available");
        cuuint64_t gdim[2] = {(cuuint64_t)R, (cuuint64_t)n};
        cuuint64_t gstride[1] = {(cuuint64_t)R * 8};
        cuuint32_t box[2] = {(cuuint32_t)R, (cuuint32_t)(4 * F)};
        cuuint32_t estride[2] = {1, 1};
        CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void *)U, gdim, gstride, box, estride,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(FTL_E_CUDA, "tensor-core leaf build: tensor map encoding failed (%d)", (int)r);
    }
    const void *fn = mode == 0 ? (const void *)leaf_gram_tc_kernel<0> : (const void *)leaf_gram_tc_kernel<1>;
    int rc = ensure_smem(fn, kSmemBytes, "leaf_gram_tc_kernel");
    if (rc) return rc;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(p.ntiles, num_sms()));
    if (mode == 0)
        leaf_gram_tc_kernel<0><<<grid, kThreads, kSmemBytes, st>>>(map, p);
    else
        leaf_gram_tc_kernel<1><<<grid, kThreads, kSmemBytes, st>>>(map, p);
    return check_launch("leaf_gram_tc_kernel");
}

}  // namespace ftl

extern "C" int ftl_device_status(uint32_t *status_out) {
    FTL_CHECK_ARG(status_out != nullptr, "ftl_device_status: status_out is NULL");
    unsigned int v = 0;
    cudaError_t err = cudaMemcpyFromSymbol(&v, ftl::g_device_status, sizeof(v));
    if (err != cudaSuccess) return ftl::fail(FTL_E_CUDA, "ftl_device_status: %s", cudaGetErrorString(err));
    const unsigned int zero = 0;
    err = cudaMemcpyToSymbol(ftl::g_device_status, &zero, sizeof(zero));
    if (err != cudaSuccess) return ftl::fail(FTL_E_CUDA, "ftl_device_status: %s", cudaGetErrorString(err));
    *status_out = v;
    return FTL_OK;
}
