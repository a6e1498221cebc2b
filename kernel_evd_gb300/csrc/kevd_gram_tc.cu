// Weighted Grams G = Y^T Y, Y = diag(s) F, of an FP32 factor on the tcgen05
// tensor cores (the A and B Grams of the bistochastic EVD, ks_kevd.cu:1152-1158,
// and the single weighted Gram of the API).
//
// Precision, with the weights on one side, G = (diag(s^2) F)^T F:
//   f16 split (when every Gram's s^2 spans at most 2^16): every factor column
//   is scaled by its own power of two into the f16 range (b side: F(:, c)
//   2^eb_c with 2^eb_c max|F(:, c)| <= 2^14; a side: s^2 F(:, c) 2^ea_c with
//   2^ea_c max(s^2) max|F(:, c)| <= 2^14), so late columns, orders of
//   magnitude smaller than the first ones, stay clear of the f16 subnormal
//   range; hi = rn_f16(v), lo = rn_f16(v - hi) carry 22 significant bits, the
//   precision of a two-term tf32 split, at twice the kind::tf32 rate and half
//   the operand bytes.  The scales 2^(ea_a + eb_b) of entry (a, b) are removed
//   exactly when the row-split partials are summed.
//   tf32 split (any weights: the bistochastic weights of a nearly diagonal
//   kernel span 1e17, beyond any f16 scale): v as the tensor core reads it
//   (hi, its 13 low mantissa bits dropped) and lo = v - trunc_tf32(v), exact in
//   FP32.
// A 128 x 128 output tile accumulates per 32-row stage the cross terms
// hi_a lo_b^T and lo_a hi_b^T and hi_a hi_b^T in FP32 in Tensor Memory; the
// dropped lo_a lo_b is below 2^-20 of each product.  The tensor-core
// accumulator rounds each update with a one-sided bias, so the FP32 partial is
// kept short: every 1920 rows it is added into an FP64 tile in global memory
// and the long sum over N rows is FP64 (the Gram accumulators of the reference
// are FP64).  Eigenvalues are then refined in FP64 by Rayleigh-Ritz
// (kevd_evd.cu).
//
// CTA roles (448 threads):
//   warps 0-3   epilogue: TMEM -> registers -> FP64 tile (warp q owns TMEM
//               lanes 32q..32q+31 = tile rows)
//   warps 4-7   a converters: thread m owns row m of the a tile (factor column
//               a0+m, 32 rows of F): row weights and the hi/lo split, written
//               to the stage's Tensor Memory a-slot (tcgen05.st, packed pairs)
//   warp 8      TMA producer
//   warp 9      TMEM allocation and the single MMA-issuing thread (A from
//               Tensor Memory, B from shared memory)
//   warps 10-13 b converters: row m of the b tile split into the f16 b-hi and
//               b-lo tiles (SWIZZLE_64B), or its tf32 lo part into an FP32
//               b-lo tile (the raw tile is then b-hi); on a diagonal tile
//               (b = a) the a converters write them
// A ring of 6 (f16) or 4 (tf32) stages of shared-memory tiles, 4 (f16) or 2
// (tf32) Tensor Memory a-slots and one TMEM accumulator per Gram are handed
// over with mbarriers; every wait is bounded and sets an error flag on timeout.
#include "kevd_internal.cuh"
#include "kevd_tc.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>

namespace kevd {

namespace {

constexpr int kTT = 128;               // output tile edge
constexpr int kTK = 32;                // rows of F per stage (MMA K per stage)
constexpr int kMaxStages = 6;
constexpr int kFlushStages = 60;       // 1920 rows per FP32 TMEM partial (a multiple of both ring depths)
constexpr int kOpBytes = kTT * kTK * 4;     // one raw FP32 operand tile, 16 KB
constexpr int kHalfBytes = kTT * kTK * 2;   // one f16 operand tile, 8 KB
constexpr int kOffB = kOpBytes;             // the b region of a stage
// Stage layout (every stage 1024-aligned for the TMA's SWIZZLE_128B boxes):
//   f16:  [a raw 16 KB][b raw 16 KB, split in place]: rows 8i..8i+7 of the raw
//         b tile occupy bytes [1024 i, 1024 i + 1024) of the b region, and the
//         b converters replace them by the SW64 atoms of the same rows, b-hi at
//         1024 i, b-lo at 1024 i + 512 (each warp's 32 rows stay inside its own
//         4 KB, so a warp-level sync orders the reads before the writes);
//         6 stages
//   tf32: [a raw 16 KB][b raw 16 KB = b-hi][b-lo FP32 16 KB]; 4 stages
template <bool F16> struct Layout {
    static constexpr int stages = F16 ? 6 : 4;
    static constexpr int stage_bytes = F16 ? 2 * kOpBytes : 3 * kOpBytes;
    static constexpr int off_blo32 = 2 * kOpBytes;   // tf32 b-lo tile
    static_assert(stage_bytes % 1024 == 0 && stages <= kMaxStages && kFlushStages % stages == 0, "ring shape");
};
constexpr int kEpiWarps = 4;        // warps 0-3
constexpr int kCvtWarp0 = 4;        // warps 4-7: a operand -> Tensor Memory
constexpr int kProdWarp = 8;
constexpr int kMmaWarp = 9;
constexpr int kCvtBWarp0 = 10;      // warps 10-13: b operand, in shared memory
constexpr int kCvtWarps = 8;        // arrivals per stage on the "converted" barrier
constexpr int kThreads = 14 * 32;
constexpr uint32_t kTmemCols = 512;       // accumulators [0, 256), a-slots [256, 512)
constexpr uint32_t kTmemA = 256;
// a-slots: f16 split, one per ring stage, per Gram 16 columns of packed hi
// pairs and 16 of lo; tf32 split, one per two stages, per Gram 32 hi and 32 lo
template <bool F16> struct Slots {
    static constexpr int n = F16 ? 4 : 2;
    static constexpr uint32_t cols = F16 ? 64 : 128;
    static constexpr uint32_t gram_cols = F16 ? 32 : 64;   // one Gram's hi + lo
    static constexpr uint32_t lo_off = F16 ? 16 : 32;
    static_assert(kTmemA + n * cols <= kTmemCols, "Tensor Memory holds 512 columns");

};
// Weight ranges (max s^2 / min s^2) above this take the tf32 split: the f16
// split keeps a factor column's values within 2^-28 .. 2^14 of its own scale at
// full precision, and the row weights multiply into that range.
constexpr float kF16WeightRange = 65536.f;
constexpr uint64_t kTimeoutNs = 4000000000ull;

struct Barriers {
    alignas(16) float w2[kMaxStages][2][32];   // squared row weights of each stage, A then B
    uint64_t tma[kMaxStages];
    uint64_t full[kMaxStages];
    uint64_t empty[kMaxStages];
    uint64_t tfree[4];
    uint64_t accf;
    uint64_t acce[2];
    uint64_t done;
    uint32_t tmem_base;
};

template <bool F16>
constexpr size_t smem_bytes() {
    return (size_t)Layout<F16>::stages * Layout<F16>::stage_bytes + sizeof(Barriers) + 1024;
}
static_assert(smem_bytes<true>() <= 227 * 1024 && smem_bytes<false>() <= 227 * 1024, "shared memory per CTA");

// Power-of-two scale exponents of one Gram call (device, per factor column c):
// eb[c] for the b side, ea[g][c] for the a side of Gram g.
struct GramExp {
    const int* eb;
    const int* ea0;
    const int* ea1;
};

__device__ __forceinline__ void tile_of(int64_t t, int64_t& ta, int64_t& tb) {
    int64_t i = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    ta = i;
    tb = t - i * (i + 1) / 2;
}

// Row m of a K-major SW128 tile of FP32: its 8 16-byte chunks (K = 4c .. 4c+3).
// The TMA writes the raw FT boxes (128 factor columns x 32 rows) this way, so
// a 16-byte chunk holds 4 consecutive rows k of one column m.
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

// Row m of the interleaved b-hi / b-lo atoms of a b region (f16 layout) from
// the 32 raw values of b row m.
__device__ __forceinline__ void store_b_split(uint8_t* breg, int m, const float (&x)[32], float bscale) {
    uint32_t h[16], l[16];
#pragma unroll
    for (int p = 0; p < 16; ++p) tc::split_f16x2(x[2 * p] * bscale, x[2 * p + 1] * bscale, h[p], l[p]);
    // sw64_off16 places row m at (m >> 3) * 512 + ...; the atoms here are 1024 apart
    const uint32_t atom = (uint32_t)(m >> 3) * 1024u;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const uint32_t off = atom + (tc::sw64_off16((uint32_t)(m & 7), 8u * c));
        *reinterpret_cast<uint4*>(breg + off) = make_uint4(h[4 * c], h[4 * c + 1], h[4 * c + 2], h[4 * c + 3]);
        *reinterpret_cast<uint4*>(breg + off + 512) = make_uint4(l[4 * c], l[4 * c + 1], l[4 * c + 2], l[4 * c + 3]);
    }
}

// NG weighted Grams of the same factor in one pass: G_g = F^T diag(s_g)^2 F.
// Every F tile is loaded and its b side split once for all of them: the
// stage's a tile is weighted NG times into Tensor Memory and each Gram's
// output tile accumulates the stage's products.
//   F16 (weights within kF16WeightRange): two-term f16 split of per-column
//     scaled values, 6 kind::f16 MMAs (K = 16) per stage and Gram; b-hi and
//     b-lo f16 tiles (SWIZZLE_64B) in shared memory.
//   tf32 (any weights): the tensor core reads an FP32 operand as tf32 by
//     dropping its 13 low mantissa bits, so an element v enters as hi = v as it
//     is and lo = v - trunc_tf32(v) (exact in FP32); 12 kind::tf32 MMAs (K = 8)
//     per stage and Gram; the raw b tile is b-hi, b-lo an FP32 tile.
template <int NG, bool F16>
__global__ void __launch_bounds__(kThreads, 1)
gram_tc_kernel(const __grid_constant__ CUtensorMap tmF, const float* __restrict__ w2a, const float* __restrict__ w2b,
               GramExp ex, int64_t N, int64_t k, int n_tiles, int64_t rows_per,
               double* __restrict__ partial, float* __restrict__ scratch, int n_scratch, int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    using LY = Layout<F16>;
    constexpr int kStages = LY::stages;
    constexpr int kStageBytes = LY::stage_bytes;
    Barriers* bar = reinterpret_cast<Barriers*>(base + (size_t)kStages * kStageBytes);
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
    double* out = partial + (int64_t)blockIdx.x * NG * kTT * kTT;   // [G][n][m]
    // FP32 staging of the accumulators at a flush, one per SM (one CTA per
    // SM: shared memory and Tensor Memory both admit only one)
    uint32_t smid, nsmid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
    if (nsmid > (uint32_t)n_scratch) {
        if (threadIdx.x == 0) atomicExch(err, 7);
        return;
    }
    float* scr = scratch + (size_t)smid * NG * kTT * kTT;   // [G][n][m]

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&bar->tma[s], 1);
            tc::mbar_init(&bar->full[s], kCvtWarps);
            tc::mbar_init(&bar->empty[s], 1);
        }
        for (int t = 0; t < Slots<F16>::n; ++t) tc::mbar_init(&bar->tfree[t], 1);
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
        // ---------------- TMA producer: raw a and b tiles and the weight rows
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)(diag ? kOpBytes : 2 * kOpBytes) + NG * kTK * 4;
            for (int64_t s = 0; s < n_stages; ++s) {
                const int slot = (int)(s % kStages);
                const uint32_t use = (uint32_t)(s / kStages);
                if (!tc::mbar_wait(&bar->empty[slot], (use & 1u) ^ 1u, kTimeoutNs)) {
                    atomicExch(err, 1);
                    break;
                }
                uint8_t* st = base + (size_t)slot * kStageBytes;
                const int x = (int)(r0 + s * kTK);
                tc::mbar_arrive_expect_tx(&bar->tma[slot], bytes);
                tc::bulk_load(bar->w2[slot][0], w2a + x, kTK * 4, &bar->tma[slot]);
                if (NG == 2) tc::bulk_load(bar->w2[slot][1], w2b + x, kTK * 4, &bar->tma[slot]);
                tc::tma_load_2d(st, &tmF, x, (int)a0, &bar->tma[slot]);
                if (!diag) tc::tma_load_2d(st + kOffB, &tmF, x, (int)b0, &bar->tma[slot]);
            }
        }
        __syncwarp();
    } else if ((warp >= kCvtWarp0 && warp < kCvtWarp0 + 4) || warp >= kCvtBWarp0) {
        // ---------------- converters (a: the weighted copies into the stage's
        // Tensor Memory a-slot; b: the split into the b-hi and b-lo tiles)
        const bool grp_a = warp < kProdWarp;
        const int m = 32 * (warp & 3) + lane;
        const uint32_t tlane = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
        // this thread's column scales (a converters: column a0 + m, which is
        // also the b column of a diagonal tile; b converters: column b0 + m)
        const int64_t cm = (grp_a ? a0 : b0) + m;
        const bool cin = cm < k;
        const float bscale = (F16 && cin) ? ldexpf(1.f, ex.eb[cm]) : 1.f;
        const float as0 = (F16 && grp_a && cin) ? ldexpf(1.f, ex.ea0[cm]) : 1.f;
        const float as1 = (F16 && grp_a && cin && NG == 2) ? ldexpf(1.f, ex.ea1[cm]) : 1.f;
        using SL = Slots<F16>;
        for (int64_t s = 0; s < n_stages; ++s) {
            const int slot = (int)(s % kStages);
            const uint32_t use = (uint32_t)(s / kStages);
            float x[32];
            if (!tc::mbar_wait(&bar->tma[slot], use & 1u, kTimeoutNs)) {
                atomicExch(err, 5);
                break;
            }
            uint8_t* st = base + (size_t)slot * kStageBytes;
            if (grp_a) {
                const int ts = (int)(s % SL::n);
                const uint32_t tuse = (uint32_t)(s / SL::n);
                load_row(st, m, x);
                if (!tc::mbar_wait(&bar->tfree[ts], (tuse & 1u) ^ 1u, kTimeoutNs)) {
                    atomicExch(err, 6);
                    break;
                }
                tc::tc_fence_after();
                const uint32_t ta_ = tlane + kTmemA + (uint32_t)ts * SL::cols;
#pragma unroll
                for (int gsel = 0; gsel < NG; ++gsel) {
                    if constexpr (F16) {
                        // y = (s^2 F) 2^ea: the power of two scales the rounded
                        // product exactly.  Words 0..15: hi pairs (rows 2p,
                        // 2p+1), words 16..31: lo pairs
                        const float as = gsel ? as1 : as0;
                        uint32_t w[32];
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            const float4 wv = reinterpret_cast<const float4*>(bar->w2[slot][gsel])[c];
                            tc::split_f16x2((x[4 * c + 0] * wv.x) * as, (x[4 * c + 1] * wv.y) * as, w[2 * c],
                                            w[16 + 2 * c]);
                            tc::split_f16x2((x[4 * c + 2] * wv.z) * as, (x[4 * c + 3] * wv.w) * as, w[2 * c + 1],
                                            w[17 + 2 * c]);
                        }
                        tc::tmem_st32u(ta_ + SL::gram_cols * gsel, w);
                    } else {
                        float y[32], l[32];
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
                        tc::tmem_st32(ta_ + SL::gram_cols * gsel, y);
                        tc::tmem_st32(ta_ + SL::gram_cols * gsel + 32u, l);
                    }
                }
                if (diag) {
                    if constexpr (F16) {
                        store_b_split(st + kOffB, m, x, bscale);
                    } else {
                        float l[32];
#pragma unroll
                        for (int u = 0; u < 32; ++u) l[u] = x[u] - tc::tf32_trunc(x[u]);
                        store_row(st + LY::off_blo32, m, l);
                    }
                }
                tc::tmem_wait_st();
                tc::tc_fence_before();
            } else if (!diag) {
                load_row(st + kOffB, m, x);
                if constexpr (F16) {
                    __syncwarp();   // the warp's raw rows are read before its atoms are rewritten
                    store_b_split(st + kOffB, m, x, bscale);
                } else {
                    float l[32];
#pragma unroll
                    for (int u = 0; u < 32; ++u) l[u] = x[u] - tc::tf32_trunc(x[u]);
                    store_row(st + LY::off_blo32, m, l);
                }
            }
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&bar->full[slot]);
        }
    } else if (warp == kMmaWarp) {
        // ---------------- MMA issuer: per stage 6 (f16) or 12 (tf32) MMAs into
        // each accumulator from descriptors held in registers
        if (lane == 0) {
            using SL = Slots<F16>;
            constexpr uint32_t idesc = F16 ? tc::idesc_f16(kTT, kTT) : tc::idesc_tf32(kTT, kTT);
            constexpr int kSteps = F16 ? kTK / 16 : kTK / 8;   // 32 bytes of K per MMA either way
            bool ok = true;
            for (int64_t c = 0; c < n_chunks && ok; ++c) {
                const int64_t s0 = c * kFlushStages;
                const int64_t s1 = min(n_stages, s0 + kFlushStages);
                for (int64_t sb = s0; sb < s1 && ok; sb += kStages) {
                    const uint32_t use = (uint32_t)(sb / kStages);
#pragma unroll
                    for (int sl = 0; sl < kStages; ++sl) {
                        if (sb + sl >= s1) break;
                        const int ts = (int)((sb + sl) % SL::n);
                        uint64_t dbh[kSteps], dbl[kSteps];
                        uint8_t* stg = base + (size_t)sl * kStageBytes;
#pragma unroll
                        for (int j = 0; j < kSteps; ++j) {   // +32 bytes of K per MMA
                            if constexpr (F16) {
                                // interleaved atoms: b-hi at +0, b-lo at +512, 1024 apart
                                const uint32_t bh = tc::smem_u32(stg + kOffB);
                                dbh[j] = tc::desc_sw64_sbo1024(bh + 32u * j);
                                dbl[j] = tc::desc_sw64_sbo1024(bh + 512u + 32u * j);
                            } else {
                                // b-hi: the raw b tile (the raw a tile on a diagonal
                                // tile); b-lo: the FP32 tile
                                const uint32_t bh = tc::desc_lo_sw128(tc::smem_u32(diag ? stg : stg + kOffB));
                                const uint32_t bl = tc::desc_lo_sw128(tc::smem_u32(stg + LY::off_blo32));
                                dbh[j] = tc::desc_sw128_from_lo(bh + 2u * j);
                                dbl[j] = tc::desc_sw128_from_lo(bl + 2u * j);
                            }
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
                        for (int gsel = 0; gsel < NG; ++gsel) {
                            if (first && c > 0) {
                                // the epilogue has read this accumulator's previous chunk
                                if (!tc::mbar_wait(&bar->acce[gsel], (uint32_t)((c - 1) & 1), kTimeoutNs)) {
                                    ok = false;
                                    break;
                                }
                                tc::tc_fence_after();
                            }
                            const uint32_t d = tbase + (uint32_t)(gsel * kTT);
                            const uint32_t ahi = tbase + kTmemA + (uint32_t)ts * SL::cols + SL::gram_cols * gsel;
                            const uint32_t alo = ahi + SL::lo_off;
                            const uint32_t acc0 = first ? 0u : 1u;
                            if constexpr (F16) {
#pragma unroll
                                for (int j = 0; j < kSteps; ++j) {
                                    tc::mma_f16_tmem_a(d, ahi + 8u * j, dbl[j], idesc, j > 0 ? 1u : acc0);
                                    tc::mma_f16_tmem_a(d, alo + 8u * j, dbh[j], idesc, 1u);
                                }
#pragma unroll
                                for (int j = 0; j < kSteps; ++j)
                                    tc::mma_f16_tmem_a(d, ahi + 8u * j, dbh[j], idesc, 1u);
                            } else {
#pragma unroll
                                for (int j = 0; j < kSteps; ++j) {
                                    tc::mma_tf32_tmem_a(d, ahi + 8u * j, dbl[j], idesc, j > 0 ? 1u : acc0);
                                    tc::mma_tf32_tmem_a(d, alo + 8u * j, dbh[j], idesc, 1u);
                                    tc::mma_tf32_tmem_a(d, ahi + 8u * j, dbh[j], idesc, 1u);
                                }
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
        // ---------------- epilogue: warp q owns tile rows 32q..32q+31 of the
        // accumulators; FP64 tiles column-major ([n][m]), Gram after Gram
        const int m = warp * 32 + lane;
        for (int n = 0; n < NG * kTT; ++n) out[n * kTT + m] = 0.0;
        bool ok = true;
        for (int64_t c = 0; c < n_chunks && ok; ++c) {
            if (!tc::mbar_wait(&bar->accf, (uint32_t)(c & 1), kTimeoutNs)) {
                atomicExch(err, 4);
                ok = false;
                break;
            }
            tc::tc_fence_after();
            // 1. the FP32 accumulators -> this SM's scratch (plain stores, no
            //    waiting on memory), each handed back to the MMA as soon as it
            //    is read
#pragma unroll 1
            for (int gsel = 0; gsel < NG; ++gsel) {
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
            for (int e0 = 0; e0 < NG * kTT; e0 += 16) {
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

// max and min of s_i^2 over i < N of each weight vector: mx[g] (atomicMax,
// starts at 0) and mx[2 + g] (atomicMin, starts at all ones), float bits of
// non-negative values, so unsigned order is float order.
__global__ void gram_wmax_kernel(const double* __restrict__ s, const double* __restrict__ s2, int64_t N,
                                 unsigned* __restrict__ mx) {
    float m0 = 0.f, m1 = 0.f, n0 = INFINITY, n1 = INFINITY;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const float a = (float)(s[i] * s[i]);
        m0 = fmaxf(m0, a);
        n0 = fminf(n0, a);
        if (s2) {
            const float b = (float)(s2[i] * s2[i]);
            m1 = fmaxf(m1, b);
            n1 = fminf(n1, b);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
        m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
        n0 = fminf(n0, __shfl_xor_sync(0xffffffffu, n0, o));
        n1 = fminf(n1, __shfl_xor_sync(0xffffffffu, n1, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(mx, __float_as_uint(m0));
        atomicMin(mx + 2, __float_as_uint(n0));
        if (s2) {
            atomicMax(mx + 1, __float_as_uint(m1));
            atomicMin(mx + 3, __float_as_uint(n1));
        }
    }
}

// e with 2^e v <= 2^14 < 2^(e+1) v for v > 0 (v = 0 or not finite: 0).
__device__ __forceinline__ int f16_range_exp(double v) {
    if (!(v > 0.0) || !isfinite(v)) return 0;
    int e;
    frexp(v, &e);   // v = f 2^e, 0.5 <= f < 1
    return 14 - e;
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

// Per-column scale exponents from max |F(:, c)| (colmax, float bits) and
// max s^2 of each Gram (wmax, float bits).
__global__ void gram_exp_kernel(const unsigned* __restrict__ colmax, const unsigned* __restrict__ wmax, int nG,
                                int64_t k, int* __restrict__ eb, int* __restrict__ ea0, int* __restrict__ ea1) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    const double cm = (double)__uint_as_float(colmax[c]);
    eb[c] = f16_range_exp(cm);
    ea0[c] = f16_range_exp(cm * (double)__uint_as_float(wmax[0]));
    if (nG == 2) ea1[c] = f16_range_exp(cm * (double)__uint_as_float(wmax[1]));
}

// Sum the row-split partial tiles, remove the scale, and write the full
// symmetric k x k matrix (column-major).
// Partial tile of (split p, tile t, Gram g) at ((p * n_tiles + t) * nG + g) * kTT^2.
__global__ void gram_tc_reduce_kernel(const double* __restrict__ partial, int n_tiles, int n_split, int nG, int g,
                                      int64_t k, const int* __restrict__ ea, const int* __restrict__ eb,
                                      double* __restrict__ G) {
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
        s = ldexp(s, -(ea[ga] + eb[gb]));   // the a side scales column ga, the b side column gb
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
// element by element.  Also max |F(:, c)| of every column into colmax[c]
// (bits of a non-negative float, so unsigned order is float order; colmax
// starts at 0): thread tid writes rows 4 (tid & 15) .. +3 of tile columns
// (tid >> 4) + 16 j, the same columns in every tile, so it keeps their maxima
// while its tiles stay in one column panel and flushes them (16-lane
// reduction, one atomic per column) when the panel changes.
__device__ __forceinline__ void flush_colmax(float (&mx)[4], int64_t c0, int64_t k, int tid,
                                             unsigned* __restrict__ colmax) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float m = mx[j];
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        const int64_t c = c0 + (tid >> 4) + 16 * j;
        if ((tid & 15) == 0 && c < k) atomicMax(colmax + c, __float_as_uint(m));
        mx[j] = 0.f;
    }
}

__global__ void __launch_bounds__(256) transpose_kernel(const float* __restrict__ F, int64_t ldF, int64_t N,
                                                        int64_t k, float* __restrict__ FT, int64_t ldT,
                                                        unsigned* __restrict__ colmax) {
    __shared__ float t[64][65];
    float mx[4] = {0.f, 0.f, 0.f, 0.f};
    int64_t cur_c0 = -1;
    const int64_t n_ti = (N + 63) / 64, n_tc = (k + 63) / 64;
    const bool vec_in = (ldF % 4) == 0 && ((uintptr_t)F % 16) == 0;
    const bool vec_out = (ldT % 4) == 0 && ((uintptr_t)FT % 16) == 0;
    const int tid = threadIdx.x;
    for (int64_t tile = blockIdx.x; tile < n_ti * n_tc; tile += gridDim.x) {
        const int64_t i0 = (tile % n_ti) * 64, c0 = (tile / n_ti) * 64;
        if (c0 != cur_c0) {   // uniform over the CTA
            if (cur_c0 >= 0) flush_colmax(mx, cur_c0, k, tid, colmax);
            cur_c0 = c0;
        }
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
            mx[e >> 8] = fmaxf(mx[e >> 8], fmaxf(fmaxf(fabsf(t[r4][cc]), fabsf(t[r4 + 1][cc])),
                                                 fmaxf(fabsf(t[r4 + 2][cc]), fabsf(t[r4 + 3][cc]))));
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
    if (cur_c0 >= 0) flush_colmax(mx, cur_c0, k, tid, colmax);
}
}  // namespace

// Column-major copy FT (k x ldT, ldT = N rounded up to 4) of a row-major FP32
// factor, and max |F(:, c)| into colmax[c] (k float bits; the call resets them).
int run_transpose_f32(kevd_ctx* ctx, const float* F, int64_t ldF, int64_t N, int64_t k, float* FT, int64_t ldT,
                      unsigned* colmax, cudaStream_t st) {
    ProfScope ps(ctx, "ev_transpose", st);
    KEVD_CUDA(ctx, cudaMemsetAsync(colmax, 0, (size_t)k * sizeof(unsigned), st));
    const int64_t tiles = ((N + 63) / 64) * ((k + 63) / 64);
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 8);
    transpose_kernel<<<grid, 256, 0, st>>>(F, ldF, N, k, FT, ldT, colmax);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

// Shared host path of the one- and two-Gram kernels (s2 == nullptr: one).
static int gram_tc_impl(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const unsigned* colmax,
                        const double* s, const double* s2, double* G, double* G2, cudaStream_t st) {
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
    unsigned* wmax = arena_get<unsigned>(ctx, "tc.wmax", 4, &rc);   // max, max, min, min
    int* exps = arena_get<int>(ctx, "tc.exps", (size_t)3 * k, &rc);   // eb, ea0, ea1
    // squared weights, one 128-byte bulk copy per stage (row offsets are
    // multiples of 32, so every copy is 128-byte aligned)
    const int64_t w2_len = (N + kTK - 1) / kTK * kTK + kTK;
    float* w2 = arena_get<float>(ctx, "tc.w2", (size_t)w2_len, &rc);
    float* w22 = s2 ? arena_get<float>(ctx, "tc.w2b", (size_t)w2_len, &rc) : nullptr;
    // FP32 flush staging indexed by SM id (ids below %nsmid; the kernel checks
    // the bound and reports code 7 if it is exceeded)
    const int n_scratch = std::max(256, 2 * ctx->num_sms);
    float* scratch = arena_get<float>(ctx, "tc.gscr", (size_t)n_scratch * nG * kTT * kTT, &rc);
    if (rc != KEVD_OK) return set_error(ctx, rc, "gram_tc: out of device memory");
    KEVD_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(int), st));
    KEVD_CUDA(ctx, cudaMemsetAsync(wmax, 0, 2 * sizeof(unsigned), st));
    KEVD_CUDA(ctx, cudaMemsetAsync(wmax + 2, 0xFF, 2 * sizeof(unsigned), st));
    const int wgrid = (int)std::min<int64_t>((w2_len + 255) / 256, (int64_t)ctx->num_sms * 8);
    gram_wmax_kernel<<<wgrid, 256, 0, st>>>(s, s2, N, wmax);
    KEVD_LAUNCH(ctx);
    gram_w2_kernel<<<wgrid, 256, 0, st>>>(s, s2, N, w2_len, w2, w22);
    KEVD_LAUNCH(ctx);
    // the split: f16 when every Gram's weights span at most kF16WeightRange
    // (the host reads the four extremes), else tf32
    unsigned hw[4];
    KEVD_CUDA(ctx, cudaMemcpyAsync(hw, wmax, sizeof(hw), cudaMemcpyDeviceToHost, st));
    KEVD_CUDA(ctx, cudaStreamSynchronize(st));
    bool f16 = true;
    for (int g = 0; g < nG; ++g) {
        float mx, mn;
        std::memcpy(&mx, &hw[g], sizeof(float));
        std::memcpy(&mn, &hw[2 + g], sizeof(float));
        f16 = f16 && mn > 0.f && std::isfinite(mx) && mx <= kF16WeightRange * mn;
    }
    const GramExp ex{exps, exps + k, exps + 2 * k};
    if (f16) {
        gram_exp_kernel<<<ceil_div(k, 256), 256, 0, st>>>(colmax, wmax, nG, k, exps, exps + k, exps + 2 * k);
        KEVD_LAUNCH(ctx);
    } else {
        KEVD_CUDA(ctx, cudaMemsetAsync(exps, 0, (size_t)3 * k * sizeof(int), st));
    }
    {
        ProfScope ps(ctx, f16 ? "gram_tc" : "gram_tc_tf32", st);
        const int grid = n_tiles * n_split;
        auto launch = [&](auto kern) -> int {
            const size_t smem = f16 ? smem_bytes<true>() : smem_bytes<false>();
            KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(kern), (int)smem));
            kern<<<grid, kThreads, smem, st>>>(tmF, w2, nG == 2 ? w22 : w2, ex, N, k, n_tiles, rows_per,
                                                      partial, scratch, n_scratch, err);
            KEVD_LAUNCH(ctx);
            return KEVD_OK;
        };
        if (nG == 1) {
            KEVD_TRY(f16 ? launch(&gram_tc_kernel<1, true>) : launch(&gram_tc_kernel<1, false>));
        } else {
            KEVD_TRY(f16 ? launch(&gram_tc_kernel<2, true>) : launch(&gram_tc_kernel<2, false>));
        }
    }
    for (int g = 0; g < nG; ++g) {
        gram_tc_reduce_kernel<<<n_tiles, 256, 0, st>>>(partial, n_tiles, n_split, nG, g, k, g ? ex.ea1 : ex.ea0,
                                                        ex.eb, g ? G2 : G);
        KEVD_LAUNCH(ctx);
    }
    int herr = 0;
    KEVD_CUDA(ctx, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    KEVD_CUDA(ctx, cudaStreamSynchronize(st));
    if (herr != 0) return set_error(ctx, KEVD_ERR_TIMEOUT, "gram_tc: pipeline wait timed out (code %d)", herr);
    return KEVD_OK;
}

// G (k x k, column-major, full) = F^T diag(s)^2 F from the column-major FP32
// factor FT (k x ldT) and its column maxima (colmax, device float bits, as
// written by run_transpose_f32).  s: device, N doubles.
int run_gram_tc(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const unsigned* colmax,
                const double* s, double* G, cudaStream_t st) {
    return gram_tc_impl(ctx, FT, ldT, N, k, colmax, s, nullptr, G, nullptr, st);
}

// G = F^T diag(s)^2 F and G2 = F^T diag(s2)^2 F in one pass over F.
int run_gram2_tc(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const unsigned* colmax,
                 const double* s, const double* s2, double* G, double* G2, cudaStream_t st) {
    return gram_tc_impl(ctx, FT, ldT, N, k, colmax, s, s2, G, G2, st);
}

}  // namespace kevd
