// Residual update of one block-RPCholesky round for an FP32 factor, on the
// tcgen05 tensor cores (the row-block loop of ks_arpclm.cu:933-995 with the
// factor stored):
//
//   for every 128-row block R:
//     P = F(R, 0:r) F(S_i, 0:r)^T                    tcgen05, two-term f16 split
//     T = K(R, S_i) - P      (K(:, S_i) by update_kcols_kernel, FP32 direct distances)
//     G = T L_i^{-T};  F(R, r:r+nacc) = G
//     d(R) <- max(d(R) - rowsq(G), 0)  (FP64);  block sum of d for the sampler
//
// Precision.  F elements are scaled by 2^14 and split in two f16 parts,
// hi = rn_f16(a), lo = rn_f16(a - hi): 22 significant bits, the precision of
// a two-term tf32 split, at twice the kind::tf32 rate and half its operand
// bytes (|F| <= 1 keeps every scaled value inside the f16 range).  Each
// 32-column stage accumulates, into a fresh TMEM partial, hi_a hi_b in one
// 64-column accumulator and the cross terms hi_a lo_b + lo_a hi_b (2^-11
// smaller) in a second; the epilogue sums the partials in FP32 registers with
// round-to-nearest, so the tensor core's one-sided accumulator rounding never
// builds up over r, and removes the 2^28 scale exactly.  That bias is
// systematic, so it does not average out in the eigenvalues: top-32 error
// against FP64 on the same pivots at N = 2M, k = 2000 over five seeds, max
// (median): cross terms in the hi_a hi_b accumulator 1.13e-8 (9.7e-9), in one
// accumulator per 128-row block 1.09e-8 (1.0e-8), a fresh one per stage
// 9.2e-9 (8.4e-9).
//
// CTA (576 threads, persistent over row blocks):
//   warp 0     TMA producer: F(R, c:c+32) tiles (128 x 32 fp32, SWIZZLE_128B)
//              and the pre-split S_i tiles (bulk copy, f16 SWIZZLE_64B)
//   warp 1     TMEM allocation and the single MMA-issuing thread (A from
//              Tensor Memory, B from shared memory); a stage's 4 kind::f16
//              MMAs (K = 16) are issued back to back from descriptors
//              computed before its wait
//   warps 2,3,8,9 and 10-13  converters, two groups of four taking alternate
//              stages: thread m owns row m of the F tile (its TMEM lane
//              quarter is warp % 4), zeroes columns >= r and writes the packed
//              hi and lo pairs into the stage's Tensor Memory a-slot
//              (tcgen05.st)
//   warps 4-7  epilogue (TMEM lane quarter = warp % 4 = tile rows): sums the
//              partials of a row block and leaves T = K - P in the K tile
//   warps 14-17 tail: G = T L_i^{-T}, the d update, the F write and the block
//              sum of d for one row block while the other roles run ahead on
//              the next ones; also the TMA loads of the K(R, S_i) tiles (a
//              second producer lane in warp 0 would share that warp's issue
//              slots with the F-ring producer's waits)
// Ring of 6 stages (shared-memory tiles + Tensor Memory a-slots of 32 columns)
// and 2 TMEM partial buffers of 128 columns, handed over with mbarriers; every
// wait is bounded (error flag on timeout).  The F tile never goes back to
// shared memory split, so per stage the shared-memory traffic is the TMA
// writes (16 KB of F, 8 KB of S_i), one read of F by the converters and the
// MMA's B reads.
#include "kevd_internal.cuh"
#include "kevd_tc.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

namespace kevd {

namespace {

constexpr int kRows = 128;          // rows per block (MMA M)
constexpr int kCols = 64;           // accepted columns per round (MMA N), nacc <= 64
constexpr int kKs = 32;             // F columns per stage
// Pipeline shape (tuning parameters; Tensor Memory holds kBufs partial buffers
// of 128 columns and kStages a-slots of 32 columns)
#ifndef KEVD_UPD_STAGES
#define KEVD_UPD_STAGES 6
#endif
#ifndef KEVD_UPD_BUFS
#define KEVD_UPD_BUFS 2
#endif
constexpr int kStages = KEVD_UPD_STAGES;
constexpr int kPrefetch = 8;        // F tiles prefetched into L2 ahead of the ring
constexpr int kBufs = KEVD_UPD_BUFS;              // TMEM partial buffers (one per stage in flight)
// A partial buffer holds two 64-column FP32 accumulators side by side:
// [0, 64) hi_a hi_b, [64, 128) the cross terms hi_a lo_b + lo_a hi_b (one
// N = 128 MMA of hi_a against the b-hi and b-lo tiles, which lie back to back
// in shared memory as one 128-row operand, and one N = 64 MMA of lo_a hi_b)
constexpr int kPartCols = 2 * kCols;
static_assert((kBufs & (kBufs - 1)) == 0, "partial-buffer count is a power of two");
constexpr uint32_t kASlotCols = 32;               // a-slot: 16 columns of packed hi pairs, then 16 of lo
constexpr uint32_t kTmemA = kBufs * kPartCols;    // a-slots after the partials
static_assert(kTmemA + kStages * kASlotCols <= 512, "Tensor Memory holds 512 columns");
constexpr uint32_t kTmemCols = 512;       // allocated and freed as one block
constexpr int kAOp = kRows * kKs * 4;     // raw F tile, 16 KB
constexpr int kBTile = kCols * kKs * 2;   // one f16 operand tile of the S_i rows (64 rows x 64 B), 4 KB
constexpr int kStageBytes = kAOp + 2 * kBTile;   // raw F tile, b_hi, b_lo
static_assert(kStageBytes % 1024 == 0, "stage tiles keep the 1024-byte alignment of SWIZZLE_128B");
// The split works on F 2^14 (every |F(i, a)| <= 1 for a unit-diagonal kernel,
// so the scaled values stay far below the f16 maximum, 65504, and above its
// normal range down to |F| = 2^-28); each product carries 2^28, removed
// exactly in the epilogue.
constexpr float kSplitScale = 16384.f;
constexpr float kSplitUnscale = 1.0f / (16384.f * 16384.f);
constexpr int kThreads = 576;
constexpr uint64_t kTimeoutNs = 4000000000ull;
constexpr int kMaxD = kMaxFeatures;
constexpr int kFeatChunk = 64;      // features staged at a time by update_kcols_kernel
constexpr int kGPitch = kCols + 1;  // row pitch of the new-column staging buffer (conflict-free by row and column)

struct Bars {
    uint64_t tma_full[kStages];
    uint64_t cvt_full[kStages];
    uint64_t empty[kStages];
    uint64_t accf[kBufs];
    uint64_t acce[kBufs];
    uint64_t kfull;     // K(R, S_i) tile landed
    uint64_t tready;    // epilogue left T = K - P in the K tile
    uint64_t done;
    uint32_t tmem_base;
};

// converter warps: group 0 = {2, 3, 8, 9} takes the even stages, group 1 =
// {10, 11, 12, 13} the odd ones; warp % 4 is the TMEM lane quarter it writes
__device__ __forceinline__ bool is_cvt_warp(int w) { return w == 2 || w == 3 || (w >= 8 && w <= 13); }
__device__ __forceinline__ int cvt_group(int w) { return w >= 10 ? 1 : 0; }

struct RoundView {   // must match the RoundState layout of kevd_rpchol.cu
    int64_t rank;
    int64_t r_old;
    int32_t nacc;
    int32_t done;
    int32_t rounds;
    int32_t pad;
    double total;
};

// Update pass g of a round that accepted more than kCols columns: columns
// r_old + kCols g .. against the factor's first r_old + kCols g columns (the
// same split as the SIMT update in kevd_rpchol.cu).  False when the pass has
// no column.
__device__ __forceinline__ bool pass_view(const RoundView* st, int group, int64_t& r, int& nacc) {
    if (st->done) return false;
    r = st->r_old + (int64_t)kCols * group;
    nacc = min(kCols, st->nacc - kCols * group);
    return nacc > 0;
}

// K(R, S_i) for row block rb: two 128 x 32 SWIZZLE_128B boxes into the K tile
__device__ __forceinline__ void load_ktile(const CUtensorMap* tmk, uint8_t* ktile, uint64_t* kfull, int64_t rb) {
    tc::mbar_arrive_expect_tx(kfull, 2 * kAOp);
    tc::tma_load_2d(ktile, tmk, 0, (int)(rb * kRows), kfull);
    tc::tma_load_2d(ktile + kAOp, tmk, 32, (int)(rb * kRows), kfull);
}

__global__ void __launch_bounds__(kThreads, 1)
update_tc_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap tmk,
                 float* __restrict__ F, int64_t ldF, int64_t N, const float* __restrict__ minv_f, int b,
                 const uint8_t* __restrict__ bprep, const RoundView* st, double* __restrict__ dvec,
                 double* __restrict__ dblk, int* __restrict__ err, int group) {
    int64_t r;
    int nacc;
    if (!pass_view(st, group, r, nacc)) return;
    const int n_st = (int)((r + kKs - 1) / kKs);
    const int64_t nblk = (N + kRows - 1) / kRows;

    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // K(R, S_i) tile: two 128 x 32 SWIZZLE_128B halves (TMA), then G in place
    uint8_t* ktile = base + (size_t)kStages * kStageBytes;
    float* mv = reinterpret_cast<float*>(ktile + 2 * kAOp);                      // kCols x kCols
    float* gbuf = mv + kCols * kCols;                                            // kRows x kGPitch: new columns
    Bars* bar = reinterpret_cast<Bars*>(gbuf + kRows * kGPitch);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // L_i^{-1} (FP32) for the epilogue, transposed: mv[q][a] = L_i^{-1}[a][q]
    // (zero above the diagonal and beyond nacc)
    for (int e = threadIdx.x; e < kCols * kCols; e += kThreads) {
        const int q = e / kCols, a = e - q * kCols;
        mv[e] = (a < nacc && q <= a) ? minv_f[a * b + q] : 0.f;
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&bar->tma_full[s], 1);
            tc::mbar_init(&bar->cvt_full[s], 4);
            tc::mbar_init(&bar->empty[s], 1);
        }
        for (int t = 0; t < kBufs; ++t) {
            tc::mbar_init(&bar->accf[t], 1);
            tc::mbar_init(&bar->acce[t], 128);
        }

        tc::mbar_init(&bar->kfull, 1);
        tc::mbar_init(&bar->tready, 128);
        tc::mbar_init(&bar->done, 1);
        tc::mbar_fence_init();
    }
    if (warp == 1) {
        tc::tmem_alloc(&bar->tmem_base, kTmemCols);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tbase = bar->tmem_base;

    if (warp == 0) {
        // ---------------- TMA producer
        if (lane == 0) {
            int64_t g = 0;
            bool ok = true;
            for (int64_t rb = blockIdx.x; rb < nblk && ok; rb += gridDim.x) {
                for (int s = 0; s < n_st; ++s, ++g) {
                    const int slot = (int)(g % kStages);
                    const uint32_t use = (uint32_t)(g / kStages);
                    if (!tc::mbar_wait(&bar->empty[slot], (use & 1u) ^ 1u, kTimeoutNs)) {
                        ok = false;
                        break;
                    }
                    uint8_t* stg = base + (size_t)slot * kStageBytes;
                    {   // L2 prefetch kPrefetch stages ahead (possibly in the next row block)
                        const int sp = s + kPrefetch;
                        const int64_t rbp = rb + (int64_t)(sp / n_st) * gridDim.x;
                        if (rbp < nblk) tc::tma_prefetch_2d(&tmap, (sp % n_st) * kKs, (int)(rbp * kRows));
                    }
                    tc::mbar_arrive_expect_tx(&bar->tma_full[slot], kAOp + 2 * kBTile);
                    tc::tma_load_2d(stg, &tmap, s * kKs, (int)(rb * kRows), &bar->tma_full[slot]);
                    tc::bulk_load(stg + kAOp, bprep + (size_t)s * 2 * kBTile, 2 * kBTile, &bar->tma_full[slot]);
                }
            }
            if (!ok) atomicExch(err, 11);
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------- MMA issuer.  The stages of this CTA run as one flat
        // sequence g = 0, 1, ... (row block after row block) taken kStages at a
        // time, so the ring slot of each stage, and with it every operand
        // descriptor, is a compile-time index into registers filled once.
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_f16(kRows, kCols);
            constexpr uint32_t idesc2 = tc::idesc_f16(kRows, kPartCols);
            constexpr int kSteps = kKs / 16;   // K = 16 per kind::f16 MMA
            uint64_t dbh[kStages][kSteps];   // b-hi and b-lo tiles as one 128-row operand
#pragma unroll
            for (int sl = 0; sl < kStages; ++sl)
#pragma unroll
                for (int j = 0; j < kSteps; ++j) {   // +32 bytes of K per MMA
                    const uint32_t bh = tc::smem_u32(base + (size_t)sl * kStageBytes + kAOp) + 32u * j;
                    dbh[sl][j] = tc::desc_sw64(bh);
                    tc::reg_pin(dbh[sl][j]);
                }
            const int64_t my_blocks = (nblk - blockIdx.x + gridDim.x - 1) / gridDim.x;
            const int64_t total = my_blocks * n_st;
            // per-stage bookkeeping in 32-bit counters (the issuing thread runs
            // it between two MMA bursts, so every dependent instruction counts)
            uint32_t s = 0;            // stage within the current row block
            uint32_t pg = 0;           // partial buffers used so far
            const uint32_t last_s = (uint32_t)n_st - 1u;
            bool ok = true;
            for (int64_t g0 = 0; g0 < total && ok; g0 += kStages) {
                const uint32_t use = (uint32_t)(g0 / kStages);
#pragma unroll
                for (int sl = 0; sl < kStages; ++sl) {
                    if (g0 + sl >= total) break;
                    // both sums into a fresh partial buffer every stage
                    const uint32_t tb = pg & (uint32_t)(kBufs - 1);
                    const uint32_t tpar = ((pg / (uint32_t)kBufs) & 1u) ^ 1u;
                    const uint32_t ahi = tbase + kTmemA + (uint32_t)sl * kASlotCols, alo = ahi + 16u;
                    const uint32_t dt = tbase + tb * (uint32_t)kPartCols;
                    if (!tc::mbar_wait(&bar->acce[tb], tpar, kTimeoutNs) ||
                        !tc::mbar_wait(&bar->cvt_full[sl], use & 1u, kTimeoutNs)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
#pragma unroll
                    for (int j = 0; j < kSteps; ++j) {
                        // [hi_a hi_b | hi_a lo_b] (N = 128), then lo_a hi_b into the second half
                        tc::mma_f16_tmem_a(dt, ahi + 8u * j, dbh[sl][j], idesc2, j > 0 ? 1u : 0u);
                        tc::mma_f16_tmem_a(dt + (uint32_t)kCols, alo + 8u * j, dbh[sl][j], idesc, 1u);
                    }
                    tc::mma_commit(&bar->empty[sl]);
                    tc::mma_commit(&bar->accf[tb]);
                    ++pg;
                    s = (s == last_s) ? 0u : s + 1u;
                }
            }
            if (!ok) atomicExch(err, 12);
            tc::mma_commit(&bar->done);
            if (!tc::mbar_wait(&bar->done, 0u, kTimeoutNs)) atomicExch(err, 13);
        }
        __syncwarp();
    } else if (is_cvt_warp(warp)) {
        // ---------------- converters: thread m owns row m of the F tile
        const int m = 32 * (warp & 3) + lane;
        const uint32_t tlane = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
        const int grp = cvt_group(warp);
        int64_t g = 0;
        for (int64_t rb = blockIdx.x; rb < nblk; rb += gridDim.x) {
            bool ok = true;
            for (int s = 0; s < n_st; ++s, ++g) {
                if ((int)(g & 1) != grp) continue;
                const int slot = (int)(g % kStages);
                const uint32_t use = (uint32_t)(g / kStages);
                if (!tc::mbar_wait(&bar->tma_full[slot], use & 1u, kTimeoutNs)) {
                    atomicExch(err, 14);
                    ok = false;
                    break;
                }
                const uint8_t* stg = base + (size_t)slot * kStageBytes;
                const int64_t cbase = (int64_t)s * kKs;
                float x[32];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const float4 a =
                        *reinterpret_cast<const float4*>(stg + tc::sw128_off((uint32_t)m, (uint32_t)(4 * c)));
                    x[4 * c + 0] = a.x;
                    x[4 * c + 1] = a.y;
                    x[4 * c + 2] = a.z;
                    x[4 * c + 3] = a.w;
                }
                if (cbase + kKs > r) {   // the last stage of a row block: columns >= r are zero
#pragma unroll
                    for (int u = 0; u < 32; ++u)
                        if (cbase + u >= r) x[u] = 0.f;
                }
                // words 0..15: hi pairs (K = 2p, 2p+1), words 16..31: lo pairs
                uint32_t w[32];
#pragma unroll
                for (int p2 = 0; p2 < 16; ++p2)
                    tc::split_f16x2(x[2 * p2] * kSplitScale, x[2 * p2 + 1] * kSplitScale, w[p2], w[16 + p2]);
                tc::tmem_st32u(tlane + kTmemA + (uint32_t)slot * kASlotCols, w);
                tc::tmem_wait_st();
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&bar->cvt_full[slot]);
            }
            if (!ok) break;
        }
    } else if (warp < 8) {
        // ---------------- epilogue: warps 4..7, TMEM lane quarter q = warp - 4.
        // Sums each row block's partials as they land and leaves T = K - P in
        // the K tile (this thread's row, in place) for the tail warps.  After a
        // timed-out wait the warp stops waiting but keeps walking the row
        // blocks and arriving, so no other role waits for it in vain.
        const int q = warp - 4;
        const int rloc = 32 * q + lane;
        const int n_part = n_st;   // one partial per stage
        int64_t g = 0;
        int64_t kit = 0;
        bool ok = true;
        for (int64_t rb = blockIdx.x; rb < nblk; rb += gridDim.x) {
            float acc[kCols];
#pragma unroll
            for (int j = 0; j < kCols; ++j) acc[j] = 0.f;
            for (int s = 0; s < n_part; ++s, ++g) {
                if (!ok) continue;
                const int tb = (int)(g % kBufs);
                const uint32_t use = (uint32_t)(g / kBufs);
                if (!tc::mbar_wait(&bar->accf[tb], use & 1u, kTimeoutNs)) {
                    atomicExch(err, 15);
                    ok = false;
                    continue;
                }
                tc::tc_fence_after();
                float v[16];
                const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)(tb * kPartCols);
                // 16 columns at a time (register budget of 576 threads): the
                // hi_a hi_b sums, then the cross-term sums of the same columns
#pragma unroll
                for (int h = 0; h < kPartCols / 16; ++h) {
                    tc::tmem_ld16(ta + (uint32_t)(16 * h), v);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < 16; ++j) acc[16 * (h & 3) + j] += v[j];
                }
                tc::tc_fence_before();
                tc::mbar_arrive(&bar->acce[tb]);
            }
            if (ok && !tc::mbar_wait(&bar->kfull, (uint32_t)(kit & 1), kTimeoutNs)) {
                atomicExch(err, 17);
                ok = false;
            }
            if (ok) {
                // T = K(i, S_i) - P over the K tile's row (K(:, S_i) by
                // update_kcols_kernel, TMA tile in smem); P = acc 2^-28 exactly
#pragma unroll
                for (int c4 = 0; c4 < kCols / 4; ++c4) {
                    float4* kp = reinterpret_cast<float4*>(
                        ktile + (c4 >> 3) * kAOp + tc::sw128_off((uint32_t)rloc, (uint32_t)(4 * (c4 & 7))));
                    float4 kv = *kp;
                    kv.x = fmaf(-acc[4 * c4 + 0], kSplitUnscale, kv.x);
                    kv.y = fmaf(-acc[4 * c4 + 1], kSplitUnscale, kv.y);
                    kv.z = fmaf(-acc[4 * c4 + 2], kSplitUnscale, kv.z);
                    kv.w = fmaf(-acc[4 * c4 + 3], kSplitUnscale, kv.w);
                    *kp = kv;
                }
                // the tile is written by TMA again once the tail warps release it
                tc::fence_async_smem();
            }
            tc::mbar_arrive(&bar->tready);
            ++kit;
        }
    } else {
        // ---------------- tail: warps 14..17, row 32q + lane of each row block.
        // G = T L_i^{-T}, the d update, the F write and the block sum of d,
        // overlapped with the MMA and the epilogue working on the next row
        // blocks.  The tail also loads the K tiles (single-buffered): the next
        // row block's tile is issued as soon as the four warps hold their T
        // rows in registers.
        const int q = warp - 14;
        const int rloc = 32 * q + lane;
        int64_t it = 0;
        bool ok = true;
        __shared__ double wsum[2][4];
        if (rloc == 0) load_ktile(&tmk, ktile, &bar->kfull, blockIdx.x);
        for (int64_t rb = blockIdx.x; rb < nblk; rb += gridDim.x) {
            const int64_t row0 = rb * kRows;
            const int64_t i = row0 + rloc;
            const double d_old = (i < N) ? dvec[i] : 0.0;
            if (ok && !tc::mbar_wait(&bar->tready, (uint32_t)(it & 1), kTimeoutNs)) {
                atomicExch(err, 18);
                ok = false;
            }
            const bool live = ok && i < N;
            // T row -> this thread's staging row (pitch kGPitch: the 32 rows of
            // a warp fall in distinct banks for every column)
            float* grow = gbuf + rloc * kGPitch;
            if (live) {
#pragma unroll
                for (int c4 = 0; c4 < kCols / 4; ++c4) {
                    const float4 tv = *reinterpret_cast<const float4*>(
                        ktile + (c4 >> 3) * kAOp + tc::sw128_off((uint32_t)rloc, (uint32_t)(4 * (c4 & 7))));
                    grow[4 * c4 + 0] = tv.x;
                    grow[4 * c4 + 1] = tv.y;
                    grow[4 * c4 + 2] = tv.z;
                    grow[4 * c4 + 3] = tv.w;
                }
            }
            // every tail thread has copied its T row: the next K tile may land
            // (the epilogue's writes of T were fenced for the async proxy
            // before tready; these reads are ordered before the TMA by the
            // barrier)
            asm volatile("bar.sync 2, 128;" ::: "memory");
            if (rloc == 0 && rb + gridDim.x < nblk) {
                tc::fence_async_smem();
                load_ktile(&tmk, ktile, &bar->kfull, rb + gridDim.x);
            }
            double nd = d_old;
            if (live) {
                // G = T L_i^{-T} in place in the staging row, blocks of eight
                // outputs from the last to the first: block a0 reads T[0 ..
                // a0+7] and overwrites T[a0 .. a0+7], which no earlier block
                // needs.  Eight independent FMA chains per block, each G[a]
                // summing e = 0..a in increasing order (the zero terms above
                // the diagonal leave it unchanged); runtime loops keep the code
                // small (fully unrolled, the 2,080 FMAs of a row took 11k cycles
                // per row block against 2k of FP32 pipe time).
                const int nb = (nacc + 7) >> 3;
                float sq = 0.f;
                for (int blk = nb - 1; blk >= 0; --blk) {
                    const int a0 = 8 * blk;
                    float g8[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) g8[u] = 0.f;
                    const float* mcol = mv + a0;
#pragma unroll 4
                    for (int e = 0; e < a0 + 8; ++e) {
                        const float te = grow[e];
                        const float4 m0 = *reinterpret_cast<const float4*>(mcol + e * kCols);
                        const float4 m1 = *reinterpret_cast<const float4*>(mcol + e * kCols + 4);
                        g8[0] = fmaf(te, m0.x, g8[0]);
                        g8[1] = fmaf(te, m0.y, g8[1]);
                        g8[2] = fmaf(te, m0.z, g8[2]);
                        g8[3] = fmaf(te, m0.w, g8[3]);
                        g8[4] = fmaf(te, m1.x, g8[4]);
                        g8[5] = fmaf(te, m1.y, g8[5]);
                        g8[6] = fmaf(te, m1.z, g8[6]);
                        g8[7] = fmaf(te, m1.w, g8[7]);
                    }
                    float sb = 0.f;
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        grow[a0 + u] = g8[u];
                        if (a0 + u < nacc) sb = fmaf(g8[u], g8[u], sb);
                    }
                    sq += sb;
                }
                nd = fmax(d_old - (double)sq, 0.0);
                dvec[i] = nd;
            }
            __syncwarp();   // this warp's 32 rows of G staged
            // coalesced store of the new columns: warp q writes its own rows
            // 32q .. 32q+31, so no other warp has to be waited for
            if (ok) {
                // lane owns columns lane and lane + 32; eight rows per batch so
                // the shared loads of a batch are in flight together
                const int nr = (int)min((int64_t)32, N - row0 - 32 * q);
                float* fbase = F + (row0 + 32 * q) * ldF + r;
                const bool c1 = lane < nacc, c2 = lane + 32 < nacc;
#pragma unroll 8
                for (int rr = 0; rr < 32; ++rr) {
                    if (rr < nr) {
                        const float* grow = gbuf + (32 * q + rr) * kGPitch;
                        const float v1 = grow[lane], v2 = grow[lane + 32];
                        if (c1) fbase[(int64_t)rr * ldF + lane] = v1;
                        if (c2) fbase[(int64_t)rr * ldF + lane + 32] = v2;
                    }
                }
            }
            __syncwarp();
            ++it;
            // block sum of the new d over the 128 tail threads
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) nd += __shfl_xor_sync(0xffffffffu, nd, o);
            double* ws = wsum[it & 1];   // alternate buffers: one barrier per row block
            if (lane == 0) ws[q] = nd;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (rloc == 0) dblk[rb] = (ws[0] + ws[1]) + (ws[2] + ws[3]);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (warp == 1) tc::tmem_dealloc(tbase, kTmemCols);
}

// K(:, S_i) for the round, FP32 from direct differences: Kc[i][c], 64 columns
// per row (zero beyond nacc); the scale enters as an FP32 pair (kexp_scaled).
// CTA = 128 rows x 64 pivots; thread (ty, tx) of 16 x 16 computes rows
// ty + 16a (a < 8) and columns tx + 16c (c < 4).  Features are staged 64 at
// a time with a row pitch of 68 floats, so a thread reads four features of a
// row in one 16-byte shared load (8 + 4 loads per four features for 256 FP32
// operations) and the pivot loads of a quarter warp fall in distinct banks;
// each squared distance still sums its features in increasing order (the
// zero padding of a ragged last chunk adds exact zeros).
constexpr int kKcPitch = kFeatChunk + 4;

__global__ void __launch_bounds__(256)
update_kcols_kernel(const float* __restrict__ X, int64_t N, int d, ScalePair scale, const int64_t* __restrict__ sacc,
                    const RoundView* st, float* __restrict__ Kc, int group) {
    int64_t r_unused;
    int nacc;
    if (!pass_view(st, group, r_unused, nacc)) return;
    sacc += (int64_t)kCols * group;
    extern __shared__ __align__(16) float ksm[];
    float* xr = ksm;                      // 128 x kKcPitch
    float* xq = ksm + kRows * kKcPitch;   // 64 x kKcPitch
    const int64_t row0 = (int64_t)blockIdx.x * kRows;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const bool vec = (d & 3) == 0 && ((uintptr_t)X & 15) == 0;   // rows start on 16-byte boundaries
    float acc[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][c] = 0.f;
    for (int c0 = 0; c0 < d; c0 += kFeatChunk) {
        const int w = min(kFeatChunk, d - c0);
        const int w4 = (w + 3) & ~3;
        __syncthreads();
        if (vec) {
            const int nq = w4 >> 2;
            for (int e = threadIdx.x; e < (kRows + kCols) * nq; e += 256) {
                const int rr = e / nq, k4 = (e - rr * nq) << 2;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (rr < kRows) {
                    const int64_t i = row0 + rr;
                    if (i < N) v = __ldg(reinterpret_cast<const float4*>(X + i * d + c0 + k4));
                    *reinterpret_cast<float4*>(xr + rr * kKcPitch + k4) = v;
                } else {
                    const int q = rr - kRows;
                    if (q < nacc) v = __ldg(reinterpret_cast<const float4*>(X + sacc[q] * d + c0 + k4));
                    *reinterpret_cast<float4*>(xq + q * kKcPitch + k4) = v;
                }
            }
        } else {
            for (int e = threadIdx.x; e < (kRows + kCols) * w4; e += 256) {
                const int rr = e / w4, kk = e - rr * w4;
                if (rr < kRows) {
                    const int64_t i = row0 + rr;
                    xr[rr * kKcPitch + kk] = (i < N && kk < w) ? X[i * d + c0 + kk] : 0.f;
                } else {
                    const int q = rr - kRows;
                    xq[q * kKcPitch + kk] = (q < nacc && kk < w) ? X[sacc[q] * d + c0 + kk] : 0.f;
                }
            }
        }
        __syncthreads();
        for (int kk = 0; kk < w4; kk += 4) {
            float4 vr[8], vq[4];
#pragma unroll
            for (int a = 0; a < 8; ++a) vr[a] = *reinterpret_cast<const float4*>(xr + (ty + 16 * a) * kKcPitch + kk);
#pragma unroll
            for (int c = 0; c < 4; ++c) vq[c] = *reinterpret_cast<const float4*>(xq + (tx + 16 * c) * kKcPitch + kk);
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float t = vr[a].x - vq[c].x;
                    acc[a][c] = fmaf(t, t, acc[a][c]);
                    t = vr[a].y - vq[c].y;
                    acc[a][c] = fmaf(t, t, acc[a][c]);
                    t = vr[a].z - vq[c].z;
                    acc[a][c] = fmaf(t, t, acc[a][c]);
                    t = vr[a].w - vq[c].w;
                    acc[a][c] = fmaf(t, t, acc[a][c]);
                }
        }
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        const int64_t i = row0 + ty + 16 * a;
        if (i >= N) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int col = tx + 16 * c;
            Kc[i * kCols + col] = (col < nacc) ? kexp_scaled(acc[a][c], scale) : 0.f;
        }
    }
}

// Split the accepted rows F(S_i, 0:r) into pre-swizzled hi / lo tiles:
// stage s -> [hi: 64 rows x 32 cols][lo], K-major SW128 (rows >= nacc and
// columns >= r are zero).
__global__ void update_prep_kernel(const float* __restrict__ F, int64_t ldF, const int64_t* __restrict__ sacc,
                                   const RoundView* st, int n_stages_max, uint8_t* __restrict__ bprep, int group) {
    int64_t r;
    int nacc;
    if (!pass_view(st, group, r, nacc)) return;
    sacc += (int64_t)kCols * group;
    const int n_st = (int)((r + kKs - 1) / kKs);
    const int64_t total = (int64_t)n_st * kCols * kKs;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(e / (kCols * kKs));
        const int rem = (int)(e - (int64_t)s * kCols * kKs);
        const int qrow = rem / kKs, kk = rem - qrow * kKs;
        const int64_t c = (int64_t)s * kKs + kk;
        const float v = (qrow < nacc && c < r) ? F[sacc[qrow] * ldF + c] : 0.f;
        uint32_t h, l;   // the converters' split of the same value (low halves)
        tc::split_f16x2(v * kSplitScale, 0.f, h, l);
        uint8_t* t = bprep + (size_t)s * 2 * kBTile;
        const uint32_t off = tc::sw64_off16((uint32_t)qrow, (uint32_t)kk);
        *reinterpret_cast<uint16_t*>(t + off) = (uint16_t)(h & 0xFFFFu);
        *reinterpret_cast<uint16_t*>(t + kBTile + off) = (uint16_t)(l & 0xFFFFu);
    }
    (void)n_stages_max;
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
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

}  // namespace

constexpr size_t kUpdSmem =
    (size_t)kStages * kStageBytes + 2 * kAOp + kCols * kCols * 4 + kRows * kGPitch * 4 + sizeof(Bars) + 1024;
static_assert(kUpdSmem <= 227 * 1024, "shared memory per CTA");
static_assert(kUpdSmem <= 227 * 1024, "shared memory per CTA");

// Whether the tensor-core update can run for this factor layout.
bool update_tc_supported(const float* F, int64_t ldF, int d) {
    return get_encode() != nullptr && (ldF % 4) == 0 && ((uintptr_t)F % 16) == 0 && d <= kMaxD &&
           ldF * 4 < (1ll << 40);
}

// Enqueue one round's residual update (reads nacc / r_old from the device
// round state).  k_max bounds the number of stages of the pre-split buffer.
int launch_update_tc(kevd_ctx* ctx, float* F, int64_t ldF, int64_t N, int64_t k_max, const float* X, int d,
                     double scale, const int64_t* sacc, const float* minv_f, int b, const void* round_state,
                     double* dvec, double* dblk, int* err, cudaStream_t s) {
    static thread_local const void* last_F = nullptr;
    static thread_local int64_t last_ld = -1, last_N = -1;
    static thread_local CUtensorMap tmap;
    if (F != last_F || ldF != last_ld || N != last_N) {
        PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode();
        if (!enc) return set_error(ctx, KEVD_ERR_CUDA, "update_tc: cuTensorMapEncodeTiled unavailable");
        const cuuint64_t gdim[2] = {(cuuint64_t)ldF, (cuuint64_t)N};
        const cuuint64_t gstride[1] = {(cuuint64_t)ldF * 4};
        const cuuint32_t box[2] = {(cuuint32_t)kKs, (cuuint32_t)kRows};
        const cuuint32_t estr[2] = {1, 1};
        CUresult cr = enc(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)F, gdim, gstride, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (cr != CUDA_SUCCESS) return set_error(ctx, KEVD_ERR_CUDA, "update_tc: tensor map encode failed (%d)", (int)cr);
        last_F = F;
        last_ld = ldF;
        last_N = N;
    }
    const int n_stages_max = (int)((k_max + kKs - 1) / kKs);
    const int n_groups = (b + kCols - 1) / kCols;
    int rc = KEVD_OK;
    uint8_t* bprep = arena_get<uint8_t>(ctx, "utc.bprep", (size_t)std::max(1, n_stages_max) * 2 * kBTile, &rc);
    if (rc != KEVD_OK) return set_error(ctx, rc, "update_tc: out of device memory");
    const RoundView* rv = static_cast<const RoundView*>(round_state);
    // K(R, S_i): update_kcols_kernel writes an N x 64 buffer that the update
    // kernel loads by TMA, one 128-row tile per row block
    float* Kc = nullptr;
    static thread_local const void* last_K = nullptr;
    static thread_local int64_t last_KN = -1;
    static thread_local CUtensorMap tmk;
    {
        Kc = arena_get<float>(ctx, "utc.kc", (size_t)N * kCols, &rc);
        if (rc != KEVD_OK) return set_error(ctx, rc, "update_tc: out of device memory");
        if (Kc != last_K || N != last_KN) {
            const cuuint64_t gdim[2] = {(cuuint64_t)kCols, (cuuint64_t)N};
            const cuuint64_t gstride[1] = {(cuuint64_t)kCols * 4};
            const cuuint32_t box[2] = {32, (cuuint32_t)kRows};
            const cuuint32_t estr[2] = {1, 1};
            CUresult cr = get_encode()(&tmk, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)Kc, gdim, gstride, box, estr,
                                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (cr != CUDA_SUCCESS)
                return set_error(ctx, KEVD_ERR_CUDA, "update_tc: tensor map (K) encode failed (%d)", (int)cr);
            last_K = Kc;
            last_KN = N;
        }
    }
    const size_t ksm = (size_t)(kRows + kCols) * kKcPitch * sizeof(float);
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&update_kcols_kernel), (int)ksm));
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&update_tc_kernel), (int)kUpdSmem));
    const int64_t nblk = (N + kRows - 1) / kRows;
    const int grid = (int)std::min<int64_t>(nblk, ctx->num_sms);
    // one pass per 64 accepted columns (passes beyond the round's count return at once)
    for (int g = 0; g < n_groups; ++g) {
        const float* minv_g = minv_f + (size_t)kCols * g * b + (size_t)kCols * g;
        {
            ProfScope ps(ctx, "rp_update_kcols", s);
            update_kcols_kernel<<<(int)nblk, 256, ksm, s>>>(X, N, d, split_scale(scale), sacc, rv, Kc, g);
            KEVD_LAUNCH(ctx);
        }
        {
            ProfScope ps(ctx, "rp_update_prep", s);
            update_prep_kernel<<<std::max(1, std::min(n_stages_max * 8, ctx->num_sms * 4)), 256, 0, s>>>(
                F, ldF, sacc, rv, n_stages_max, bprep, g);
            KEVD_LAUNCH(ctx);
        }
        {
            ProfScope ps(ctx, "rp_update", s);
            update_tc_kernel<<<grid, kThreads, kUpdSmem, s>>>(tmap, tmk, F, ldF, N, minv_g, b, bprep, rv, dvec, dblk,
                                                              err, g);
            KEVD_LAUNCH(ctx);
        }
    }
    return KEVD_OK;
}

}  // namespace kevd
