// Weighted Gram G = Y^T Y, Y = diag(s) F, of an FP32 factor on the tcgen05
// tensor cores (the A and B Grams of the bistochastic EVD).
//
// Precision: 3xTF32 with the weights on one side, G = (diag(s^2) F)^T F.
// The tensor core reads an FP32 operand as tf32 by dropping its low 13
// mantissa bits, so an element v is used as hi = trunc_tf32(v) when passed
// as it is, and lo = v - hi is exact in FP32 (its own read drops at most
// 2^-21 |v|).  The a operand is y = s_i^2 F[i][a] (hi: y itself, lo: y -
// trunc(y), both in Tensor Memory); the b operand is the raw F tile (hi: the
// TMA tile as loaded, lo: F - trunc(F) in the b-lo tile).  A 128 x 128 output
// tile accumulates hi_a lo_b^T + lo_a hi_b^T + hi_a hi_b^T in FP32 in Tensor
// Memory; the dropped parts (lo_a lo_b, the truncation of the lo reads) are
// below 2^-20 of each product and shrink its magnitude by about 5e-7 on
// average.  The tensor-core accumulator rounds each update with a one-sided
// bias, so the FP32 partial is kept short: every 2048 rows it is added into
// an FP64 tile in global memory and the long sum over N rows is FP64 (the
// Gram accumulators of the reference are FP64, ks_kevd.cu:1152-1158).  The
// relative error of a Gram entry is about 4e-5 (1024-row partials halve it
// and cost 14 % more time at N = 2M, k = 2000); eigenvalues are then refined
// in FP64 by Rayleigh-Ritz (kevd_evd.cu).
//
// CTA roles (448 threads):
//   warps 0-3   epilogue: TMEM -> registers -> FP64 tile (warp q owns TMEM
//               lanes 32q..32q+31 = tile rows)
//   warps 4-7   a converters: thread m owns row m of the a tile (factor column
//               a0+m, 32 rows of F): row weights and the hi/lo split, written
//               to the stage's Tensor Memory a-slot (tcgen05.st, hi and lo
//               columns)
//   warp 8      TMA producer
//   warp 9      TMEM allocation and the single MMA-issuing thread (A from
//               Tensor Memory, B from shared memory)
//   warps 10-13 b converters: row m of the b tile, its lo part into the b-lo
//               tile (the raw tile is the hi operand)
// The conversion and the MMA issue are the per-stage critical paths: two
// groups of four converter warps (one per SM sub-partition each), and the
// MMA thread issues a stage's 12 MMAs back to back from precomputed
// descriptors (measured on GB300: a kind::tf32 MMA of 128 x 128 x 8 takes 64
// cycles when issued back to back, 128 x 64 x 8 takes 48, and each dependent
// instruction between two MMAs adds its latency).
// A 4-stage ring (shared-memory tiles and their Tensor Memory a-slots) and a
// double-buffered TMEM accumulator (2 x 128 columns) are handed over with
// mbarriers; every wait is bounded and sets an error flag on timeout.
// Keeping the a operand out of shared memory removes its split stores and the
// MMA's a-operand reads (about 80 KB of shared-memory traffic per stage).
#include "kevd_internal.cuh"
#include "kevd_tc.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

namespace kevd {

namespace {

constexpr int kTT = 128;               // output tile edge
constexpr int kTK = 32;                // rows of F per stage (MMA K per stage)
constexpr int kStages = 4;
constexpr int kPrefetch = 0;          // stages of F prefetched into L2 ahead of the ring (0: off;
                                      // at N = 2M, k = 2000 a 6-stage prefetch cost 1.8x: it
                                      // broke the L2 sharing of panels between CTAs)
constexpr int kFlushStages = 64;       // 2048 rows per FP32 TMEM partial
constexpr int kOpBytes = kTT * kTK * 4;     // one operand tile, 16 KB
constexpr int kStageBytes = 3 * kOpBytes;   // a (raw), b hi, b lo
constexpr int kEpiWarps = 4;        // warps 0-3
constexpr int kCvtWarp0 = 4;        // warps 4-7: a operand -> Tensor Memory
constexpr int kProdWarp = 8;
constexpr int kMmaWarp = 9;
constexpr int kCvtBWarp0 = 10;      // warps 10-13: b operand, in shared memory
constexpr int kCvtWarps = 8;        // arrivals per stage on the "converted" barrier
constexpr int kThreads = 14 * 32;
constexpr uint32_t kTmemCols = 512;       // accumulators [0,256), a-operand slots [256,512)
constexpr uint32_t kTmemA = 256;
constexpr uint32_t kTmemASlot = 64;       // hi columns [0,32), lo [32,64)
static_assert(kTmemA + kStages * kTmemASlot <= kTmemCols, "Tensor Memory holds 512 columns");
constexpr uint64_t kTimeoutNs = 4000000000ull;

struct Barriers {
    alignas(16) float w2[kStages][32];   // squared row weights of each stage (bulk copy with the tiles)
    uint64_t tma[kStages];
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t accf[2];
    uint64_t acce[2];
    uint64_t done;
    uint32_t tmem_base;
};

constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + sizeof(Barriers) + 1024;
static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");

__device__ __forceinline__ void tile_of(int64_t t, int64_t& ta, int64_t& tb) {
    int64_t i = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    ta = i;
    tb = t - i * (i + 1) / 2;
}

// Per stage (32 rows of F = 32 columns of FT):
//   [a 16 KB][b 16 KB][b lo 16 KB]
// The TMA writes the raw FT boxes (128 factor columns x 32 rows, K-major,
// SWIZZLE_128B) into the a and b tiles.  With y = s_i^2 F[i][c], the a
// converters write y and y - trunc(y) into the stage's Tensor Memory a-slot;
// the b converters write F - trunc(F) of the b tile into the b-lo tile and
// leave the b tile as it is (on a diagonal tile b = a: the a converters also
// write the b-lo tile).  Element (m, k) of a tile sits at sw128_off(m, k), so a
// 16-byte chunk holds 4 consecutive rows k of one column m.
constexpr int kStageAlloc = kStageBytes;   // a multiple of 1024: every stage stays 1024-aligned

// Row m of a K-major SW128 tile: its 8 16-byte chunks (K = 4c .. 4c+3).
__device__ __forceinline__ void load_row(const uint8_t* tile, int m, float (&x)[32]) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const float4 v = *reinterpret_cast<const float4*>(tile + tc::sw128_off((uint32_t)m, 4u * c));
        x[4 * c] = v.x;
        x[4 * c + 1] = v.y;
        x[4 * c + 2] = v.z;
        x[4 * c + 3] = v.w;
    }
}

__device__ __forceinline__ void store_row(uint8_t* tile, int m, const float (&x)[32]) {
#pragma unroll
    for (int c = 0; c < 8; ++c)
        *reinterpret_cast<float4*>(tile + tc::sw128_off((uint32_t)m, 4u * c)) =
            make_float4(x[4 * c], x[4 * c + 1], x[4 * c + 2], x[4 * c + 3]);
}

__global__ void __launch_bounds__(kThreads, 1)
gram_tc_kernel(const __grid_constant__ CUtensorMap tmF, const float* __restrict__ w2, int64_t N, int64_t k,
               int n_tiles, int64_t rows_per, double* __restrict__ partial, int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    Barriers* bar = reinterpret_cast<Barriers*>(base + (size_t)kStages * kStageAlloc);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int64_t tix = blockIdx.x % n_tiles;
    const int64_t split = blockIdx.x / n_tiles;
    int64_t ta, tb;
    tile_of(tix, ta, tb);
    const bool diag = (ta == tb);
    const int64_t a0 = ta * kTT, b0 = tb * kTT;
    const int64_t r0 = split * rows_per;
    const int64_t r1 = min(N, r0 + rows_per);
    const int64_t n_stages = (r1 > r0) ? (r1 - r0 + kTK - 1) / kTK : 0;
    const int64_t n_chunks = (n_stages + kFlushStages - 1) / kFlushStages;
    double* out = partial + (int64_t)blockIdx.x * kTT * kTT;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&bar->tma[s], 1);
            tc::mbar_init(&bar->full[s], kCvtWarps);
            tc::mbar_init(&bar->empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&bar->accf[b], 1);
            tc::mbar_init(&bar->acce[b], kEpiWarps * 32);
        }
        tc::mbar_init(&bar->done, 1);
        tc::mbar_fence_init();
    }
    if (warp == kMmaWarp) {
        tc::tmem_alloc(&bar->tmem_base, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tbase = bar->tmem_base;

    if (warp == kProdWarp) {
        // ---------------- TMA producer
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)(diag ? kOpBytes : 2 * kOpBytes);
            for (int64_t s = 0; s < n_stages; ++s) {
                const int slot = (int)(s % kStages);
                const uint32_t use = (uint32_t)(s / kStages);
                if (!tc::mbar_wait(&bar->empty[slot], (use & 1u) ^ 1u, kTimeoutNs)) {
                    atomicExch(err, 1);
                    break;
                }
                uint8_t* st = base + (size_t)slot * kStageAlloc;
                const int x = (int)(r0 + s * kTK);
                if (kPrefetch > 0 && s + kPrefetch < n_stages) {
                    const int xp = (int)(r0 + (s + kPrefetch) * kTK);
                    tc::tma_prefetch_2d(&tmF, xp, (int)a0);
                    if (!diag) tc::tma_prefetch_2d(&tmF, xp, (int)b0);
                }
                tc::mbar_arrive_expect_tx(&bar->tma[slot], bytes + kTK * 4);
                tc::bulk_load(bar->w2[slot], w2 + x, kTK * 4, &bar->tma[slot]);
                tc::tma_load_2d(st, &tmF, x, (int)a0, &bar->tma[slot]);
                if (!diag) tc::tma_load_2d(st + kOpBytes, &tmF, x, (int)b0, &bar->tma[slot]);
            }
        }
        __syncwarp();
    } else if ((warp >= kCvtWarp0 && warp < kCvtWarp0 + 4) || warp >= kCvtBWarp0) {
        // ---------------- converters: thread m owns row m of the a tile (warps
        // 4-7, to Tensor Memory) or of the b tile (warps 10-13, lo part only)
        const bool grp_a = warp < kProdWarp;
        const int m = 32 * (warp & 3) + lane;
        const uint32_t tlane = tbase + ((uint32_t)(32 * (warp & 3)) << 16);   // this warp's TMEM lanes
        for (int64_t s = 0; s < n_stages; ++s) {
            const int slot = (int)(s % kStages);
            const uint32_t use = (uint32_t)(s / kStages);
            float x[32], l[32];
            if (!tc::mbar_wait(&bar->tma[slot], use & 1u, kTimeoutNs)) {
                atomicExch(err, 5);
                break;
            }
            uint8_t* st = base + (size_t)slot * kStageAlloc;
            if (grp_a) {
                // a operand -> Tensor Memory: y = s^2 x as the hi operand (the
                // tensor core reads its top 19 bits) and y - trunc(y) as lo; on a
                // diagonal tile the raw a tile is also b, whose lo part goes to
                // the b-lo tile
                const uint32_t ta = tlane + kTmemA + (uint32_t)slot * kTmemASlot;
                load_row(st, m, x);
                float y[32];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const float4 wv = reinterpret_cast<const float4*>(bar->w2[slot])[c];
                    y[4 * c + 0] = x[4 * c + 0] * wv.x;
                    y[4 * c + 1] = x[4 * c + 1] * wv.y;
                    y[4 * c + 2] = x[4 * c + 2] * wv.z;
                    y[4 * c + 3] = x[4 * c + 3] * wv.w;
                }
#pragma unroll
                for (int u = 0; u < 32; ++u) l[u] = y[u] - tc::tf32_trunc(y[u]);
                tc::tmem_st32(ta, y);
                tc::tmem_st32(ta + 32, l);
                if (diag) {
#pragma unroll
                    for (int u = 0; u < 32; ++u) l[u] = x[u] - tc::tf32_trunc(x[u]);
                    store_row(st + 2 * kOpBytes, m, l);
                }
                tc::tmem_wait_st();
                tc::tc_fence_before();
            } else if (!diag) {
                load_row(st + kOpBytes, m, x);
#pragma unroll
                for (int u = 0; u < 32; ++u) l[u] = x[u] - tc::tf32_trunc(x[u]);
                store_row(st + 2 * kOpBytes, m, l);
            }
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&bar->full[slot]);
        }
    } else if (warp == kMmaWarp) {
        // ---------------- MMA issuer.  The tensor core takes an MMA only when
        // the previous one is nearly done, so every address of a stage is in a
        // register before its 12 MMAs are issued back to back.
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_tf32(kTT, kTT);
            // low descriptor words of each slot's b-hi (raw b, or raw a on a
            // diagonal tile) and b-lo tiles; the high word is a constant
            uint32_t bh0[kStages], bl0[kStages];
#pragma unroll
            for (int sl = 0; sl < kStages; ++sl) {
                uint8_t* stg = base + (size_t)sl * kStageAlloc;
                bh0[sl] = tc::desc_lo_sw128(tc::smem_u32(diag ? stg : stg + kOpBytes));
                bl0[sl] = tc::desc_lo_sw128(tc::smem_u32(stg + 2 * kOpBytes));
            }
            bool ok = true;
            for (int64_t c = 0; c < n_chunks && ok; ++c) {
                const int tb_ = (int)(c & 1);
                const uint32_t tuse = (uint32_t)(c >> 1);
                if (!tc::mbar_wait(&bar->acce[tb_], (tuse & 1u) ^ 1u, kTimeoutNs)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t d = tbase + (uint32_t)(tb_ * kTT);
                const int64_t s0 = c * kFlushStages;   // a multiple of kStages: slot = s - s0 (mod kStages)
                const int64_t s1 = min(n_stages, s0 + kFlushStages);
                for (int64_t sb = s0; sb < s1 && ok; sb += kStages) {
                    const uint32_t use = (uint32_t)(sb / kStages);
#pragma unroll
                    for (int sl = 0; sl < kStages; ++sl) {
                        if (sb + sl >= s1) break;
                        if (!tc::mbar_wait(&bar->full[sl], use & 1u, kTimeoutNs)) {
                            ok = false;
                            break;
                        }
                        tc::tc_fence_after();
                        const uint32_t ahi = tbase + kTmemA + (uint32_t)sl * kTmemASlot, alo = ahi + 32;
                        uint64_t dbh[kTK / 8], dbl[kTK / 8];
#pragma unroll
                        for (int j = 0; j < kTK / 8; ++j) {   // +32 bytes of K per MMA: +2 in the address field
                            dbh[j] = tc::desc_sw128_from_lo(bh0[sl] + 2u * j);
                            dbl[j] = tc::desc_sw128_from_lo(bl0[sl] + 2u * j);
                            tc::reg_pin(dbh[j]);
                            tc::reg_pin(dbl[j]);
                        }
                        const uint32_t acc0 = (sb + sl > s0) ? 1u : 0u;
#pragma unroll
                        for (int j = 0; j < kTK / 8; ++j) {
                            tc::mma_tf32_tmem_a(d, ahi + 8 * j, dbl[j], idesc, j > 0 ? 1u : acc0);
                            tc::mma_tf32_tmem_a(d, alo + 8 * j, dbh[j], idesc, 1u);
                            tc::mma_tf32_tmem_a(d, ahi + 8 * j, dbh[j], idesc, 1u);
                        }
                        tc::mma_commit(&bar->empty[sl]);
                    }
                }
                if (ok) tc::mma_commit(&bar->accf[tb_]);
            }
            if (!ok) atomicExch(err, 2);
            // retire every issued MMA before the TMEM is released
            tc::mma_commit(&bar->done);
            if (!tc::mbar_wait(&bar->done, 0u, kTimeoutNs)) atomicExch(err, 3);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: warp q owns tile rows 32q..32q+31; the FP64
        // tile is stored column-major ([n][m]) so a warp's accesses coalesce
        const int m = warp * 32 + lane;
        double* orow = out + m;
        for (int n = 0; n < kTT; ++n) orow[n * kTT] = 0.0;
        for (int64_t c = 0; c < n_chunks; ++c) {
            const int tb_ = (int)(c & 1);
            const uint32_t use = (uint32_t)(c >> 1);
            if (!tc::mbar_wait(&bar->accf[tb_], use & 1u, kTimeoutNs)) {
                atomicExch(err, 4);
                break;
            }
            tc::tc_fence_after();
#pragma unroll 1
            for (int cb = 0; cb < kTT / 32; ++cb) {
                float v[32];
                tc::tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(tb_ * kTT + 32 * cb), v);
                tc::tmem_wait_ld();
#pragma unroll
                for (int n = 0; n < 32; ++n) tc::red_add(orow + (32 * cb + n) * kTT, (double)v[n]);
            }
            tc::tc_fence_before();
            tc::mbar_arrive(&bar->acce[tb_]);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == kMmaWarp) tc::tmem_dealloc(tbase, kTmemCols);
}

// ---------------------------------------------------------------------------
// Two weighted Grams of the same factor in one pass: G_A = F^T diag(sA)^2 F and
// G_B = F^T diag(sB)^2 F (the A and B Grams of the bistochastic EVD share F and
// differ only in the row weights).  Every F tile is loaded and its b side
// converted once for both: the stage's a tile is scaled twice into Tensor
// Memory (hi/lo of sA^2 F and of sB^2 F), the raw b tile and its lo part serve
// both, and 24 MMAs per stage accumulate the two output tiles.  Same precision
// scheme and FP64 flush as gram_tc_kernel.
//
// Tensor Memory: accumulators A [0,128) and B [128,256) (single-buffered: at a
// flush the MMA waits until the epilogue has read the accumulator it is about
// to overwrite); two a-slots of 128 columns at [256,512) (hi A, lo A, hi B, lo
// B, 32 each), handed back by the MMA through tfree barriers.
namespace dual {

constexpr int kTSlots = 2;
constexpr uint32_t kTSlotCols = 128;

struct Barriers {
    alignas(16) float w2[kStages][2][32];   // squared row weights of each stage, A then B
    uint64_t tma[kStages];
    uint64_t full[kStages];
    uint64_t empty[kStages];
    uint64_t tfree[kTSlots];
    uint64_t accf;
    uint64_t acce[2];
    uint64_t done;
    uint32_t tmem_base;
};

constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + sizeof(Barriers) + 1024;
static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");
static_assert(2 * kTT + kTSlots * kTSlotCols <= kTmemCols, "Tensor Memory holds 512 columns");
static_assert(kFlushStages % kStages == 0 && kStages % kTSlots == 0, "slot indices are compile-time per stage");

}  // namespace dual

__global__ void __launch_bounds__(kThreads, 1)
gram2_tc_kernel(const __grid_constant__ CUtensorMap tmF, const float* __restrict__ w2a, const float* __restrict__ w2b,
                int64_t N, int64_t k, int n_tiles, int64_t rows_per, double* __restrict__ partial,
                float* __restrict__ scratch, int n_scratch, int* __restrict__ err) {
    using dual::kTSlots;
    using dual::kTSlotCols;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    dual::Barriers* bar = reinterpret_cast<dual::Barriers*>(base + (size_t)kStages * kStageAlloc);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int64_t tix = blockIdx.x % n_tiles;
    const int64_t split = blockIdx.x / n_tiles;
    int64_t ta, tb;
    tile_of(tix, ta, tb);
    const bool diag = (ta == tb);
    const int64_t a0 = ta * kTT, b0 = tb * kTT;
    const int64_t r0 = split * rows_per;
    const int64_t r1 = min(N, r0 + rows_per);
    const int64_t n_stages = (r1 > r0) ? (r1 - r0 + kTK - 1) / kTK : 0;
    const int64_t n_chunks = (n_stages + kFlushStages - 1) / kFlushStages;
    double* out = partial + (int64_t)blockIdx.x * 2 * kTT * kTT;   // [G][n][m]
    // FP32 staging of the two accumulators at a flush, one per SM (one CTA per
    // SM: shared memory and Tensor Memory both admit only one)
    uint32_t smid, nsmid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
    if (nsmid > (uint32_t)n_scratch) {
        if (threadIdx.x == 0) atomicExch(err, 7);
        return;
    }
    float* scr = scratch + (size_t)smid * 2 * kTT * kTT;   // [G][n][m]

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&bar->tma[s], 1);
            tc::mbar_init(&bar->full[s], kCvtWarps);
            tc::mbar_init(&bar->empty[s], 1);
        }
        for (int t = 0; t < kTSlots; ++t) tc::mbar_init(&bar->tfree[t], 1);
        tc::mbar_init(&bar->accf, 1);
        tc::mbar_init(&bar->acce[0], kEpiWarps * 32);
        tc::mbar_init(&bar->acce[1], kEpiWarps * 32);
        tc::mbar_init(&bar->done, 1);
        tc::mbar_fence_init();
    }
    if (warp == kMmaWarp) {
        tc::tmem_alloc(&bar->tmem_base, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tbase = bar->tmem_base;

    if (warp == kProdWarp) {
        // ---------------- TMA producer: raw a and b tiles and both weight rows
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)(diag ? kOpBytes : 2 * kOpBytes) + 2 * kTK * 4;
            for (int64_t s = 0; s < n_stages; ++s) {
                const int slot = (int)(s % kStages);
                const uint32_t use = (uint32_t)(s / kStages);
                if (!tc::mbar_wait(&bar->empty[slot], (use & 1u) ^ 1u, kTimeoutNs)) {
                    atomicExch(err, 1);
                    break;
                }
                uint8_t* st = base + (size_t)slot * kStageAlloc;
                const int x = (int)(r0 + s * kTK);
                tc::mbar_arrive_expect_tx(&bar->tma[slot], bytes);
                tc::bulk_load(bar->w2[slot][0], w2a + x, kTK * 4, &bar->tma[slot]);
                tc::bulk_load(bar->w2[slot][1], w2b + x, kTK * 4, &bar->tma[slot]);
                tc::tma_load_2d(st, &tmF, x, (int)a0, &bar->tma[slot]);
                if (!diag) tc::tma_load_2d(st + kOpBytes, &tmF, x, (int)b0, &bar->tma[slot]);
            }
        }
        __syncwarp();
    } else if ((warp >= kCvtWarp0 && warp < kCvtWarp0 + 4) || warp >= kCvtBWarp0) {
        // ---------------- converters (a: both scaled copies into the stage's
        // Tensor Memory a-slot; b: lo part into the b-lo tile)
        const bool grp_a = warp < kProdWarp;
        const int m = 32 * (warp & 3) + lane;
        const uint32_t tlane = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
        for (int64_t s = 0; s < n_stages; ++s) {
            const int slot = (int)(s % kStages);
            const uint32_t use = (uint32_t)(s / kStages);
            float x[32], l[32];
            if (!tc::mbar_wait(&bar->tma[slot], use & 1u, kTimeoutNs)) {
                atomicExch(err, 5);
                break;
            }
            uint8_t* st = base + (size_t)slot * kStageAlloc;
            if (grp_a) {
                const int ts = (int)(s % kTSlots);
                const uint32_t tuse = (uint32_t)(s / kTSlots);
                load_row(st, m, x);
                if (!tc::mbar_wait(&bar->tfree[ts], (tuse & 1u) ^ 1u, kTimeoutNs)) {
                    atomicExch(err, 6);
                    break;
                }
                tc::tc_fence_after();
                const uint32_t ta_ = tlane + kTmemA + (uint32_t)ts * kTSlotCols;
#pragma unroll
                for (int gsel = 0; gsel < 2; ++gsel) {
                    float y[32];
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const float4 wv = reinterpret_cast<const float4*>(bar->w2[slot][gsel])[c];
                        y[4 * c + 0] = x[4 * c + 0] * wv.x;
                        y[4 * c + 1] = x[4 * c + 1] * wv.y;
                        y[4 * c + 2] = x[4 * c + 2] * wv.z;
                        y[4 * c + 3] = x[4 * c + 3] * wv.w;
                    }
#pragma unroll
                    for (int u = 0; u < 32; ++u) l[u] = y[u] - tc::tf32_trunc(y[u]);
                    tc::tmem_st32(ta_ + 64u * gsel, y);
                    tc::tmem_st32(ta_ + 64u * gsel + 32u, l);
                }
                if (diag) {
#pragma unroll
                    for (int u = 0; u < 32; ++u) l[u] = x[u] - tc::tf32_trunc(x[u]);
                    store_row(st + 2 * kOpBytes, m, l);
                }
                tc::tmem_wait_st();
                tc::tc_fence_before();
            } else if (!diag) {
                load_row(st + kOpBytes, m, x);
#pragma unroll
                for (int u = 0; u < 32; ++u) l[u] = x[u] - tc::tf32_trunc(x[u]);
                store_row(st + 2 * kOpBytes, m, l);
            }
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&bar->full[slot]);
        }
    } else if (warp == kMmaWarp) {
        // ---------------- MMA issuer: per stage 12 MMAs into accumulator A,
        // then 12 into B, from descriptors held in registers
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_tf32(kTT, kTT);
            uint32_t bh0[kStages], bl0[kStages];
#pragma unroll
            for (int sl = 0; sl < kStages; ++sl) {
                uint8_t* stg = base + (size_t)sl * kStageAlloc;
                bh0[sl] = tc::desc_lo_sw128(tc::smem_u32(diag ? stg : stg + kOpBytes));
                bl0[sl] = tc::desc_lo_sw128(tc::smem_u32(stg + 2 * kOpBytes));
            }
            bool ok = true;
            for (int64_t c = 0; c < n_chunks && ok; ++c) {
                const int64_t s0 = c * kFlushStages;
                const int64_t s1 = min(n_stages, s0 + kFlushStages);
                for (int64_t sb = s0; sb < s1 && ok; sb += kStages) {
                    const uint32_t use = (uint32_t)(sb / kStages);
#pragma unroll
                    for (int sl = 0; sl < kStages; ++sl) {
                        if (sb + sl >= s1) break;
                        const int ts = sl % kTSlots;   // sb is a multiple of kStages, hence of kTSlots
                        uint64_t dbh[kTK / 8], dbl[kTK / 8];
#pragma unroll
                        for (int j = 0; j < kTK / 8; ++j) {   // +32 bytes of K per MMA: +2 in the address field
                            dbh[j] = tc::desc_sw128_from_lo(bh0[sl] + 2u * j);
                            dbl[j] = tc::desc_sw128_from_lo(bl0[sl] + 2u * j);
                            tc::reg_pin(dbh[j]);
                            tc::reg_pin(dbl[j]);
                        }
                        if (!tc::mbar_wait(&bar->full[sl], use & 1u, kTimeoutNs)) {
                            ok = false;
                            break;
                        }
                        tc::tc_fence_after();
                        const bool first = (sb + sl == s0);
#pragma unroll
                        for (int gsel = 0; gsel < 2; ++gsel) {
                            if (first && c > 0) {
                                // the epilogue has read this accumulator's previous chunk
                                if (!tc::mbar_wait(&bar->acce[gsel], (uint32_t)((c - 1) & 1), kTimeoutNs)) {
                                    ok = false;
                                    break;
                                }
                                tc::tc_fence_after();
                            }
                            const uint32_t d = tbase + (uint32_t)(gsel * kTT);
                            const uint32_t ahi = tbase + kTmemA + (uint32_t)ts * kTSlotCols + 64u * gsel;
                            const uint32_t alo = ahi + 32u;
                            const uint32_t acc0 = first ? 0u : 1u;
#pragma unroll
                            for (int j = 0; j < kTK / 8; ++j) {
                                tc::mma_tf32_tmem_a(d, ahi + 8 * j, dbl[j], idesc, j > 0 ? 1u : acc0);
                                tc::mma_tf32_tmem_a(d, alo + 8 * j, dbh[j], idesc, 1u);
                                tc::mma_tf32_tmem_a(d, ahi + 8 * j, dbh[j], idesc, 1u);
                            }
                        }
                        if (!ok) break;
                        tc::mma_commit(&bar->empty[sl]);
                        tc::mma_commit(&bar->tfree[ts]);
                    }
                }
                if (ok) tc::mma_commit(&bar->accf);
            }
            if (!ok) atomicExch(err, 2);
            // retire every issued MMA before the TMEM is released
            tc::mma_commit(&bar->done);
            if (!tc::mbar_wait(&bar->done, 0u, kTimeoutNs)) atomicExch(err, 3);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: warp q owns tile rows 32q..32q+31 of both
        // accumulators; FP64 tiles column-major ([n][m]), A then B
        const int m = warp * 32 + lane;
        for (int n = 0; n < kTT; ++n) {
            out[n * kTT + m] = 0.0;
            out[kTT * kTT + n * kTT + m] = 0.0;
        }
        bool ok = true;
        for (int64_t c = 0; c < n_chunks && ok; ++c) {
            if (!tc::mbar_wait(&bar->accf, (uint32_t)(c & 1), kTimeoutNs)) {
                atomicExch(err, 4);
                ok = false;
                break;
            }
            tc::tc_fence_after();
            // 1. both FP32 accumulators -> this SM's scratch (plain stores, no
            //    waiting on memory), each handed back to the MMA as soon as it
            //    is read
#pragma unroll 1
            for (int gsel = 0; gsel < 2; ++gsel) {
                const uint32_t tacc = tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(gsel * kTT);
                float* srow = scr + (size_t)gsel * kTT * kTT + m;
#pragma unroll 1
                for (int cb = 0; cb < kTT / 32; ++cb) {
                    float v[32];
                    tc::tmem_ld32(tacc + 32u * cb, v);
                    tc::tmem_wait_ld();
                    if (cb == kTT / 32 - 1) {
                        tc::tc_fence_before();
                        tc::mbar_arrive(&bar->acce[gsel]);
                    }
#pragma unroll
                    for (int n = 0; n < 32; ++n) srow[(32 * cb + n) * kTT] = v[n];
                }
            }
            // 2. fold into the FP64 tiles while the MMA runs the next chunk (the
            //    thread reads back only what it wrote)
#pragma unroll 1
            for (int e0 = 0; e0 < 2 * kTT; e0 += 16) {
                double o[16];
                float v[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    o[u] = out[(size_t)(e0 + u) * kTT + m];
                    v[u] = scr[(size_t)(e0 + u) * kTT + m];
                }
#pragma unroll
                for (int u = 0; u < 16; ++u) out[(size_t)(e0 + u) * kTT + m] = o[u] + (double)v[u];
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == kMmaWarp) tc::tmem_dealloc(tbase, kTmemCols);
}

// w2[i] = s_i^2 rounded to FP32 for i < N, zero up to len (the last stage of
// the last row split may run past N).
__global__ void gram_w2_kernel(const double* __restrict__ s, const double* __restrict__ s2, int64_t N, int64_t len,
                               float* __restrict__ w2, float* __restrict__ w22) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
        w2[i] = (i < N) ? (float)(s[i] * s[i]) : 0.f;
        if (s2) w22[i] = (i < N) ? (float)(s2[i] * s2[i]) : 0.f;
    }
}

// Sum the row-split partial tiles and write the full symmetric k x k matrix
// (column-major).
// Partial tile of (split p, tile t, Gram g) at ((p * n_tiles + t) * nG + g) * kTT^2.
__global__ void gram_tc_reduce_kernel(const double* __restrict__ partial, int n_tiles, int n_split, int nG, int g,
                                      int64_t k, double* __restrict__ G) {
    const int64_t t = blockIdx.x;
    int64_t ta, tb;
    tile_of(t, ta, tb);
    for (int e = threadIdx.x; e < kTT * kTT; e += blockDim.x) {
        const int ib = e / kTT, ia = e - ib * kTT;   // partial tiles are [n][m]
        const int64_t ga = ta * kTT + ia, gb = tb * kTT + ib;
        if (ga >= k || gb >= k) continue;
        // the weights sit on the a side only, so a diagonal tile is not exactly
        // symmetric: its lower triangle (ga >= gb) is mirrored
        if (ta == tb && ia < ib) continue;
        double s = 0.0;
        for (int p = 0; p < n_split; ++p) s += partial[(((int64_t)p * n_tiles + t) * nG + g) * kTT * kTT + e];
        G[gb * k + ga] = s;
        G[ga * k + gb] = s;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    // resolved once per process (thread-safe static initialisation)
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    return fn;
}

// FT[c * ldT + i] = F[i * ldF + c]: 64 x 64 tiles through shared memory, read
// and written in 16-byte pieces where a piece lies inside the matrix and its
// row stride allows (F rows: ldF % 4 == 0; FT rows: ldT % 4 == 0 always), else
// element by element.
__global__ void __launch_bounds__(256) transpose_kernel(const float* __restrict__ F, int64_t ldF, int64_t N,
                                                        int64_t k, float* __restrict__ FT, int64_t ldT) {
    __shared__ float t[64][65];
    const int64_t n_ti = (N + 63) / 64, n_tc = (k + 63) / 64;
    const bool vec_in = (ldF % 4) == 0 && ((uintptr_t)F % 16) == 0;
    const bool vec_out = (ldT % 4) == 0 && ((uintptr_t)FT % 16) == 0;
    const int tid = threadIdx.x;
    for (int64_t tile = blockIdx.x; tile < n_ti * n_tc; tile += gridDim.x) {
        const int64_t i0 = (tile % n_ti) * 64, c0 = (tile / n_ti) * 64;
        __syncthreads();
        for (int e = tid; e < 64 * 16; e += 256) {
            const int r = e >> 4, c4 = (e & 15) * 4;   // row r, columns c4..c4+3 of the tile
            const int64_t i = i0 + r, c = c0 + c4;
            if (i < N && vec_in && c + 3 < k) {
                const float4 v = *reinterpret_cast<const float4*>(F + i * ldF + c);
                t[r][c4] = v.x; t[r][c4 + 1] = v.y; t[r][c4 + 2] = v.z; t[r][c4 + 3] = v.w;
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) t[r][c4 + u] = (i < N && c + u < k) ? F[i * ldF + c + u] : 0.f;
            }
        }
        __syncthreads();
        for (int e = tid; e < 64 * 16; e += 256) {
            const int cc = e >> 4, r4 = (e & 15) * 4;   // FT row c0 + cc, rows i0 + r4..+3
            const int64_t c = c0 + cc, i = i0 + r4;
            if (c >= k) continue;
            if (vec_out && i + 3 < ldT) {
                *reinterpret_cast<float4*>(FT + c * ldT + i) =
                    make_float4(t[r4][cc], t[r4 + 1][cc], t[r4 + 2][cc], t[r4 + 3][cc]);
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (i + u < ldT) FT[c * ldT + i + u] = t[r4 + u][cc];
            }
        }
    }
}

}  // namespace

// Column-major copy FT (k x ldT, ldT = N rounded up to 4) of a row-major FP32 factor.
int run_transpose_f32(kevd_ctx* ctx, const float* F, int64_t ldF, int64_t N, int64_t k, float* FT, int64_t ldT,
                      cudaStream_t st) {
    ProfScope ps(ctx, "ev_transpose", st);
    const int64_t tiles = ((N + 63) / 64) * ((k + 63) / 64);
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 8);
    transpose_kernel<<<grid, 256, 0, st>>>(F, ldF, N, k, FT, ldT);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

// Shared host path of the one- and two-Gram kernels (s2 == nullptr: one).
static int gram_tc_impl(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const double* s,
                        const double* s2, double* G, double* G2, cudaStream_t st) {
    const int nG = s2 ? 2 : 1;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return set_error(ctx, KEVD_ERR_CUDA, "gram_tc: cuTensorMapEncodeTiled unavailable");
    if ((ldT % 4) != 0 || ((uintptr_t)FT % 16) != 0)
        return set_error(ctx, KEVD_ERR_ARG, "gram_tc: FT must be 16-byte aligned with ldT %% 4 == 0");
    CUtensorMap tmF;
    {
        const cuuint64_t gdim[2] = {(cuuint64_t)N, (cuuint64_t)k};
        const cuuint64_t gstride[1] = {(cuuint64_t)ldT * 4};
        const cuuint32_t box[2] = {(cuuint32_t)kTK, (cuuint32_t)kTT};
        const cuuint32_t estr[2] = {1, 1};
        CUresult cr = enc(&tmF, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)FT, gdim, gstride, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (cr != CUDA_SUCCESS) return set_error(ctx, KEVD_ERR_CUDA, "gram_tc: tensor map (F) failed (%d)", (int)cr);
    }
    const int nt = ceil_div(k, kTT);
    const int n_tiles = nt * (nt + 1) / 2;
    // Row chunks: CTA (tile, chunk) has blockIdx = chunk * n_tiles + tile, so the
    // hardware issues CTAs chunk by chunk and the CTAs that share a column panel
    // stream the same rows at about the same time (the chunk's rows, about
    // 64k x k x 4 bytes, stay in L2 while its tiles run).  At least 8 waves of
    // CTAs keep the tail short.
    int64_t n_split64 = std::max<int64_t>((N + 65535) / 65536, ((int64_t)ctx->num_sms * 8 + n_tiles - 1) / n_tiles);
    n_split64 = std::min<int64_t>(n_split64, std::max<int64_t>(1, N / 1024));
    const int n_split = (int)std::max<int64_t>(1, n_split64);
    const int64_t rows_per = ((N + n_split - 1) / n_split + kTK - 1) / kTK * kTK;
    int rc = KEVD_OK;
    double* partial = arena_get<double>(ctx, "tc.gpart", (size_t)n_split * n_tiles * nG * kTT * kTT, &rc);
    int* err = arena_get<int>(ctx, "tc.err", 1, &rc);
    // squared weights, one 128-byte bulk copy per stage (row offsets are
    // multiples of 32, so every copy is 128-byte aligned)
    const int64_t w2_len = (N + kTK - 1) / kTK * kTK + kTK;
    float* w2 = arena_get<float>(ctx, "tc.w2", (size_t)w2_len, &rc);
    float* w22 = s2 ? arena_get<float>(ctx, "tc.w2b", (size_t)w2_len, &rc) : nullptr;
    if (rc != KEVD_OK) return set_error(ctx, rc, "gram_tc: out of device memory");
    KEVD_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(int), st));
    gram_w2_kernel<<<(int)std::min<int64_t>((w2_len + 255) / 256, (int64_t)ctx->num_sms * 8), 256, 0, st>>>(
        s, s2, N, w2_len, w2, w22);
    KEVD_LAUNCH(ctx);
    if (nG == 1) {
        KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&gram_tc_kernel), (int)kSmemBytes));
        ProfScope ps(ctx, "gram_tc", st);
        gram_tc_kernel<<<n_tiles * n_split, kThreads, kSmemBytes, st>>>(tmF, w2, N, k, n_tiles, rows_per, partial,
                                                                       err);
        KEVD_LAUNCH(ctx);
    } else {
        KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&gram2_tc_kernel), (int)dual::kSmemBytes));
        ProfScope ps(ctx, "gram_tc", st);
        // FP32 flush staging indexed by SM id (ids below %nsmid; the kernel
        // checks the bound and reports code 7 if it is exceeded)
        const int n_scratch = std::max(256, 2 * ctx->num_sms);
        float* scratch = arena_get<float>(ctx, "tc.gscr", (size_t)n_scratch * 2 * kTT * kTT, &rc);
        if (rc != KEVD_OK) return set_error(ctx, rc, "gram_tc: out of device memory");
        gram2_tc_kernel<<<n_tiles * n_split, kThreads, dual::kSmemBytes, st>>>(tmF, w2, w22, N, k, n_tiles,
                                                                              rows_per, partial, scratch,
                                                                              n_scratch, err);
        KEVD_LAUNCH(ctx);
    }
    for (int g = 0; g < nG; ++g) {
        gram_tc_reduce_kernel<<<n_tiles, 256, 0, st>>>(partial, n_tiles, n_split, nG, g, k, g ? G2 : G);
        KEVD_LAUNCH(ctx);
    }
    int herr = 0;
    KEVD_CUDA(ctx, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    KEVD_CUDA(ctx, cudaStreamSynchronize(st));
    if (herr != 0) return set_error(ctx, KEVD_ERR_TIMEOUT, "gram_tc: pipeline wait timed out (code %d)", herr);
    return KEVD_OK;
}

// G (k x k, column-major, full) = F^T diag(s)^2 F from the column-major FP32
// factor FT (k x ldT).  s: device, N doubles.
int run_gram_tc(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const double* s, double* G,
                cudaStream_t st) {
    return gram_tc_impl(ctx, FT, ldT, N, k, s, nullptr, G, nullptr, st);
}

// G = F^T diag(s)^2 F and G2 = F^T diag(s2)^2 F in one pass over F.
int run_gram2_tc(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const double* s,
                 const double* s2, double* G, double* G2, cudaStream_t st) {
    return gram_tc_impl(ctx, FT, ldT, N, k, s, s2, G, G2, st);
}

}  // namespace kevd
