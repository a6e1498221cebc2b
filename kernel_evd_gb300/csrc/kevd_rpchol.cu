// Stage 2: block randomly pivoted Cholesky with a stored factor.
//
// Semantics follow ks_arpclm.cu's round (propose, residual block, accept /
// reject + factor, residual-diagonal update, trace error), with the factor F
// kept in HBM instead of regenerating K(R, S) every round:
//
//   round:  sample   b proposals ~ d                    (1 CTA)
//           hgram    F(S',:) F(S',:)^T split over column chunks, and K(S',S')
//           factor   H = K(S',S') - F F^T, accept/reject, Cholesky, L_i^{-1}
//           update   G = (K(R,S_i) - F(R,:) F(S_i,:)^T) L_i^{-T} for every row
//                    block R; F(R, r:r+nacc) = G; d(R) -= rowsq(G), clamped;
//                    per-block sums of d for the next sampler
//
// All round state stays on the device: kernels read the rank and accepted
// count from a RoundState, and after the stop condition every kernel returns
// immediately, so the host enqueues rounds without a per-round sync (the
// reference synchronises and copies nacc to the host every round,
// ks_arpclm.cu:877-886).
//
// T = double is the plain FP64 form; T = float the mixed form (F, the F F^T
// products and G in FP32; H, its Cholesky and inverse, the residual diagonal
// and all sums in FP64).
#include "kevd_internal.cuh"
#include "kevd_rng.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace kevd {

bool update_tc_supported(const float* F, int64_t ldF, int d);
int launch_update_tc(kevd_ctx* ctx, float* F, int64_t ldF, int64_t N, int64_t k_max, const float* X, int d,
                     double scale, const int64_t* sacc, const float* minv_f, int b, const void* round_state,
                     double* dvec, double* dblk, int* err, cudaStream_t s);

constexpr int kRowBlock = 128;   // rows per update CTA (= rows per d partial sum)
constexpr int kMaxBlock = 512;   // proposals per round (the reference's default BLK, ks_arpclm.cu:38)
constexpr int kGroup = 64;       // accepted columns per update pass: a round with more runs several passes
constexpr int kSmallBlock = 64;  // rounds up to this size factor their block in shared memory
constexpr int kFactorThreads = 256;   // rp_factor_kernel: 16 x 16 threads over the trailing update
constexpr int kBigFactorThreads = 1024;   // rp_factor_big_kernel: 32 x 32 threads
static_assert(kFactorThreads == 256 && kSmallBlock * kSmallBlock % kFactorThreads == 0, "factor thread layout");
constexpr int kColChunk = 32;    // F columns per hgram CTA
constexpr int kFeat = 64;        // features staged at a time by the SIMT update
constexpr int kSampleThreads = 1024;

// Acceptance floor of the mixed form, relative to K(S',S')_ii (= 1 for the
// Gaussian kernel).  In the mixed form H = K(S',S') - F(S',:) F(S',:)^T is
// formed from the FP32 factor, whose rounding leaves noise of a few 1e-7 in
// H_ii; a proposal whose H_ii is at that level would be accepted on noise and
// give a column of noise / sqrt(noise).  The mixed form therefore rejects
// H_ii <= 16 u32 K_ii (u32 = 2^-24, about 9.5e-7) and stops once the trace
// error, the mean residual diagonal, has fallen below the same level.  The
// FP64 form keeps the reference's tolerance alone (ks_arpclm.cu:329-331).
constexpr double kMixedFloor = 16.0 / 16777216.0;

struct RoundState {
    int64_t rank;    // columns of F written
    int64_t r_old;   // rank before this round's update
    int32_t nacc;    // accepted this round
    int32_t done;    // set once the factorisation has stopped
    int32_t rounds;  // rounds executed
    int32_t pad;
    double total;    // sum of d after the last update
};

// Host side of a capture-safe factorisation: no host read inside the round
// loop (all max_rounds rounds are enqueued; the kernels return at once after
// the stop), results copied to these pinned buffers at the end.
struct RpcholDeferred {
    RoundState* state_h;
    int* tcerr_h;
    int64_t* piv_h;
};

// Kernel values of a fixed pseudo-random sample of kDensityPairs pairs (i, j),
// i != j, counted when K(i, j) >= 2^-24.  A factorisation whose kernel is
// nearly diagonal (fewer than half the sampled values reach 2^-24) keeps the
// FP32 SIMT residual update: the tensor-core update splits F into f16 parts
// scaled to |F| <= 1, which hold F's tiny entries only to about 2^-39
// absolutely, and the bistochastic weights 1/dtil^2 of such kernels amplify
// exactly those rows (top-16 eigenvalue errors of 1e-6 .. 1e-5 against FP64
// on the same pivots, against at most 7e-7 with the SIMT update).
constexpr int kDensityPairs = 4096;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {   // splitmix64 finaliser
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) kernel_density_kernel(const float* __restrict__ X, int64_t N, int d,
                                                              double scale, int* __restrict__ count) {
    int c = 0;
    for (int t = threadIdx.x; t < kDensityPairs; t += blockDim.x) {
        const int64_t i = (int64_t)(mix64(2 * (uint64_t)t + 1) % (uint64_t)N);
        int64_t j = (int64_t)(mix64(2 * (uint64_t)t + 2) % (uint64_t)N);
        if (j == i) j = (i + 1) % N;
        float d2 = 0.f;
        for (int f = 0; f < d; ++f) {
            const float u = X[i * d + f] - X[j * d + f];
            d2 = fmaf(u, u, d2);
        }
        c += (exp(-scale * (double)d2) >= 5.9604644775390625e-8) ? 1 : 0;   // 2^-24
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(count, c);
}

// Whether the kernel is nearly diagonal (see kernel_density_kernel); one
// small launch and a 4-byte copy.  Must not run inside a stream capture.
static int kernel_nearly_diagonal(kevd_ctx* ctx, const float* X, int64_t N, int d, double scale, cudaStream_t s,
                                  bool* out) {
    *out = false;
    if (N < 2) return KEVD_OK;
    int st = KEVD_OK;
    int* cnt = arena_get<int>(ctx, "rp.density", 1, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "rpchol: out of device memory");
    KEVD_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int), s));
    kernel_density_kernel<<<1, 256, 0, s>>>(X, N, d, scale, cnt);
    KEVD_LAUNCH(ctx);
    int* h = static_cast<int*>(ctx->pinned);
    KEVD_CUDA(ctx, cudaMemcpyAsync(h, cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    *out = 2 * *h < kDensityPairs;
    return KEVD_OK;
}

__global__ void rp_init_kernel(double* __restrict__ d, double* __restrict__ dblk, int64_t N,
                               int64_t nblk, RoundState* st) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x)
        d[i] = 1.0;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblk;
         b += (int64_t)gridDim.x * blockDim.x)
        dblk[b] = (double)min((int64_t)kRowBlock, N - b * kRowBlock);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->rank = 0;
        st->r_old = 0;
        st->nacc = 0;
        st->done = 0;
        st->rounds = 0;
        st->total = (double)N;
    }
}

// ---- sampler ---------------------------------------------------------------
// Inverse-CDF proposals (ks_arpclm.cu:197-224): pivot = smallest i with
// cumsum(d)[i] >= u * sum(d), else N - 1.  The prefix is hierarchical: a scan
// over per-thread chunks of the block sums, a sequential walk over the chunk,
// then a warp scan inside the 128-row block.  Also records the trace error of
// the previous round and decides the stop.
__global__ void __launch_bounds__(kSampleThreads)
rp_sample_kernel(const double* __restrict__ d, const double* __restrict__ dblk, int64_t N,
                 int64_t nblk, int round, int b, uint64_t seed,
                 const double* __restrict__ uniforms, int64_t* __restrict__ props,
                 RoundState* st, int64_t k_max, int max_rounds, double err_target,
                 double err_floor, double* __restrict__ err) {
    __shared__ double incl[kSampleThreads];
    __shared__ int s_stop;
    if (st->done) return;
    const int tid = threadIdx.x;
    const int64_t chunk = (nblk + kSampleThreads - 1) / kSampleThreads;
    const int64_t c0 = min(nblk, (int64_t)tid * chunk), c1 = min(nblk, c0 + chunk);
    double s = 0.0;
    for (int64_t q = c0; q < c1; ++q) s += dblk[q];
    incl[tid] = s;
    __syncthreads();
    for (int off = 1; off < kSampleThreads; off <<= 1) {
        const double v = (tid >= off) ? incl[tid - off] : 0.0;
        __syncthreads();
        incl[tid] += v;
        __syncthreads();
    }
    const double total = incl[kSampleThreads - 1];
    if (tid == 0) {
        const double e = total / (double)N;
        if (round > 0) err[round - 1] = e;
        st->total = total;
        const bool stop = (round >= max_rounds) || (st->rank >= k_max) ||
                          (err_target > 0.0 && round > 0 && e <= err_target) ||
                          (err_floor > 0.0 && round > 0 && e <= err_floor);
        if (stop) {
            st->done = 1;
            st->rounds = round;
        }
        s_stop = stop;
    }
    __syncthreads();
    if (s_stop) return;
    const int lane = tid & 31, warp = tid >> 5;
    for (int t = warp; t < b; t += kSampleThreads / 32) {
        const double u = uniforms ? uniforms[((int64_t)round * 2) * b + t]
                                  : philox_uniform(seed, (uint32_t)round, 0u, (uint32_t)t);
        const double target = u * total;
        int64_t pick = N - 1;
        if (target <= total) {
            // smallest chunk owner c with incl[c] >= target
            int lo = 0, hi = kSampleThreads - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (incl[mid] >= target) hi = mid; else lo = mid + 1;
            }
            double base = (lo > 0) ? incl[lo - 1] : 0.0;
            const int64_t q0 = min(nblk, (int64_t)lo * chunk), q1 = min(nblk, q0 + chunk);
            int64_t blk = q1 - 1;
            for (int64_t q = q0; q < q1; ++q) {
                const double nb = base + dblk[q];
                if (nb >= target) { blk = q; break; }
                base = nb;
            }
            if (blk >= q0) {
                // within block: lane l holds rows 4l..4l+3
                const int64_t r0 = blk * kRowBlock;
                double v[4], ls = 0.0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int64_t row = r0 + 4 * lane + j;
                    v[j] = (row < N) ? d[row] : 0.0;
                    ls += v[j];
                }
                double pre = ls;  // inclusive warp scan of lane sums
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const double y = __shfl_up_sync(0xffffffffu, pre, o);
                    if (lane >= o) pre += y;
                }
                double cum = base + pre - ls;
                int hit = -1;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    cum += v[j];
                    if (hit < 0 && cum >= target && v[j] > 0.0) hit = j;
                }
                const unsigned m = __ballot_sync(0xffffffffu, hit >= 0);
                if (m) {
                    const int src = __ffs(m) - 1;
                    const int hj = __shfl_sync(0xffffffffu, hit, src);
                    pick = r0 + 4 * src + hj;
                } else {
                    // rounding left the target past this block's recomputed
                    // sum: take its last row with d > 0
                    const unsigned mz = __ballot_sync(0xffffffffu, ls > 0.0);
                    if (mz) {
                        const int src = 31 - __clz(mz);
                        int jj = 3;
                        double vv[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) vv[j] = __shfl_sync(0xffffffffu, v[j], src);
                        while (jj > 0 && !(vv[jj] > 0.0)) --jj;
                        pick = r0 + 4 * src + jj;
                    }
                }
            }
        }
        if (lane == 0) props[t] = min(pick, N - 1);
    }
}

// ---- proposal block: F(S',c-chunk) F(S',c-chunk)^T and K(S',S') -----------
constexpr int kHgramStageRows = 128;
template <typename T>
static size_t hgram_smem(int b) {
    const size_t f = (size_t)b * (kColChunk + 1) * sizeof(T);
    const size_t x = b <= kHgramStageRows ? (size_t)b * 129 * sizeof(float) : 0;
    return std::max(f, x);
}
template <typename T>
__global__ void __launch_bounds__(256)
rp_hgram_kernel(const T* __restrict__ F, int64_t ldF, const float* __restrict__ X, int d,
                double scale, const int64_t* __restrict__ props, int b, int n_split,
                const RoundState* st, double* __restrict__ hpart, double* __restrict__ kss) {
    if (st->done) return;
    // one buffer, used either for an F column chunk or for the X rows of S'
    extern __shared__ __align__(16) unsigned char raw[];
    T* fs = reinterpret_cast<T*>(raw);
    float* xs = reinterpret_cast<float*>(raw);
    const int tid = threadIdx.x;
    if ((int)blockIdx.x < n_split) {
        const int64_t r = st->rank;
        const int64_t c0 = (int64_t)blockIdx.x * kColChunk;
        if (c0 >= r) return;
        const int nc = (int)min((int64_t)kColChunk, r - c0);
        for (int e = tid; e < b * kColChunk; e += 256) {
            const int p = e / kColChunk, c = e - p * kColChunk;
            fs[p * (kColChunk + 1) + c] = (c < nc) ? F[props[p] * ldF + c0 + c] : (T)0;
        }
        __syncthreads();
        for (int e = tid; e < b * b; e += 256) {
            const int p = e / b, q = e - p * b;
            T acc = 0;
#pragma unroll 8
            for (int c = 0; c < kColChunk; ++c)
                acc += fs[p * (kColChunk + 1) + c] * fs[q * (kColChunk + 1) + c];
            hpart[((int64_t)blockIdx.x * b + p) * b + q] = (double)acc;
        }
    } else {
        // K(S', S') in FP64, rows split over the remaining CTAs
        const int nk = gridDim.x - n_split;
        const int part = blockIdx.x - n_split;
        // rows of S' staged in shared memory up to 128 features and 128
        // proposals, read from global memory (L2-resident, b rows) beyond;
        // same summation order
        const bool staged = d <= 128 && b <= kHgramStageRows;
        if (staged)
            for (int e = tid; e < b * d; e += 256) {
                const int p = e / d, k = e - p * d;
                xs[p * 129 + k] = X[props[p] * d + k];
            }
        __syncthreads();
        for (int e = tid; e < b * b; e += 256) {
            const int p = e / b, q = e - p * b;
            if (p % nk != part) continue;
            double acc = 0.0;
            if (staged) {
                for (int k = 0; k < d; ++k) {
                    const double t = (double)xs[p * 129 + k] - (double)xs[q * 129 + k];
                    acc += t * t;
                }
            } else {
                const float* xp = X + props[p] * d;
                const float* xq = X + props[q] * d;
                for (int k = 0; k < d; ++k) {
                    const double t = (double)__ldg(xp + k) - (double)__ldg(xq + k);
                    acc += t * t;
                }
            }
            kss[p * b + q] = exp(-scale * acc);
        }
    }
}

// ---- accept / reject, Cholesky, inverse of the compacted factor ------------
// ks_arpclm.cu:305-408.  H lives in shared memory; accepted columns are
// overwritten in place by the Cholesky column (only accepted columns are
// read back).  Minv (b x b, row-major [a][e], zeros above the diagonal).
__global__ void __launch_bounds__(256)
rp_factor_kernel(const double* __restrict__ kss, const double* __restrict__ hpart, int b,
                 int round, uint64_t seed, const double* __restrict__ uniforms, double tol,
                 double floor_rel, int64_t k_max, const int64_t* __restrict__ props, RoundState* st,
                 double* __restrict__ minv, float* __restrict__ minv_f,
                 int64_t* __restrict__ sacc, int64_t* __restrict__ piv,
                 int32_t* __restrict__ hm) {
    if (st->done) return;
    extern __shared__ double H[];         // b x b, the b x b inverse being formed, the compacted factor
    double* MS = H + b * b;
    double* LC = MS + b * b;
    __shared__ double H0[kSmallBlock];
    __shared__ double us[kSmallBlock];    // the round's acceptance uniforms
    __shared__ double kfl[kSmallBlock];   // acceptance floor per proposal (0 in the FP64 form)
    __shared__ int accpos[kSmallBlock];
    const int tid = threadIdx.x;
    const int64_t r = st->rank;
    const int nz = (int)((r + kColChunk - 1) / kColChunk);
    {
        // 256 threads x 16 elements (b <= 64): the 16 chains of a thread advance
        // together over the column chunks, so 16 loads are in flight per step;
        // each element still subtracts its chunks in increasing order
        constexpr int kPer = kSmallBlock * kSmallBlock / 256;
        double v[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int e = tid + 256 * j;
            v[j] = (e < b * b) ? kss[e] : 0.0;
        }
        for (int z = 0; z < nz; ++z) {
            const double* hz = hpart + (int64_t)z * b * b;
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const int e = tid + 256 * j;
                if (e < b * b) v[j] -= hz[e];
            }
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const int e = tid + 256 * j;
            if (e < b * b) H[e] = v[j];
        }
    }
    __syncthreads();
    for (int p = tid; p < b; p += blockDim.x) {
        H0[p] = H[p * b + p];
        kfl[p] = floor_rel * kss[p * b + p];
        us[p] = uniforms ? uniforms[((int64_t)round * 2 + 1) * b + p] : philox_uniform(seed, (uint32_t)round, 1u, (uint32_t)p);
    }
    const int64_t cap = k_max - r;
    // Every thread takes the same decisions (H_ii is final once the previous
    // accepted step's trailing update has passed its barrier), so a rejected
    // proposal costs no barrier and an accepted one a single barrier.  The
    // trailing update forms the scaled column l_j = H_ji f in registers, the
    // same product that is stored into column i after the barrier (the next
    // steps never touch column i, so that write overlaps them).
    int m = 0;
    __syncthreads();
    for (int i = 0; i < b; ++i) {
        const double hii = H[i * b + i];
        const bool acc = (m < cap) && (H0[i] * us[i] < hii) && (hii > tol) && (hii > kfl[i]);
        if (!acc) continue;
        if (tid == 0) accpos[m] = i;
        ++m;
        const double f = 1.0 / sqrt(hii);
        // trailing update of the lower triangle, 16 x 16 threads over (jj, kk)
        for (int jj = i + 1 + (tid >> 4); jj < b; jj += 16) {
            const double lj = H[jj * b + i] * f;
            for (int kk = i + 1 + (tid & 15); kk <= jj; kk += 16) {
                const double lk = H[kk * b + i] * f;
                H[jj * b + kk] -= lj * lk;
            }
        }
        __syncthreads();
        for (int j = i + tid; j < b; j += blockDim.x) H[j * b + i] *= f;
    }
    __syncthreads();   // the last scaled column is written
    const int nacc = m;
    // forward substitution, one column per thread, in shared memory (the
    // sequential dot products read what the same thread wrote a step earlier)
    // on the compacted factor LC (no index indirection inside the chains)
    for (int e = tid; e < b * b; e += blockDim.x) {
        MS[e] = 0.0;
        const int a = e / b, c = e - a * b;
        LC[e] = (a < nacc && c < nacc) ? H[accpos[a] * b + accpos[c]] : 0.0;
    }
    __syncthreads();
    if (tid < nacc) {
        const int t = tid;
        MS[t * b + t] = 1.0 / LC[t * b + t];
        for (int a = t + 1; a < nacc; ++a) {
            const double* la = LC + a * b;
            double s = 0.0;
            for (int e = t; e < a; ++e) s += la[e] * MS[e * b + t];
            MS[a * b + t] = -s / la[a];
        }
    }
    __syncthreads();
    for (int e = tid; e < b * b; e += blockDim.x) {
        minv[e] = MS[e];
        minv_f[e] = (float)MS[e];
    }
    if (tid < nacc) {
        const int64_t sp = props[accpos[tid]];
        sacc[tid] = sp;
        piv[r + tid] = sp;
    }
    if (tid == 0) {
        st->r_old = r;
        st->nacc = nacc;
        st->rank = r + nacc;
        hm[round] = nacc;
    }
}

// Accept / reject, Cholesky and inverse for 64 < b <= kMaxBlock: the steps and
// the per-element operation order of rp_factor_kernel, with H, the compacted
// factor LC and the inverse MS in a global workspace (b^2 doubles each,
// L2-resident) instead of shared memory, and 32 x 32 threads over the
// trailing update.  __syncthreads orders the CTA's global accesses as it does
// its shared ones.
__global__ void __launch_bounds__(kBigFactorThreads)
rp_factor_big_kernel(const double* __restrict__ kss, const double* __restrict__ hpart, int b,
                     int round, uint64_t seed, const double* __restrict__ uniforms, double tol,
                     double floor_rel, int64_t k_max, const int64_t* __restrict__ props, RoundState* st,
                     double* __restrict__ minv, float* __restrict__ minv_f,
                     int64_t* __restrict__ sacc, int64_t* __restrict__ piv,
                     int32_t* __restrict__ hm, double* H, double* MS, double* LC) {
    if (st->done) return;
    __shared__ double H0[kMaxBlock];
    __shared__ double us[kMaxBlock];
    __shared__ double kfl[kMaxBlock];
    __shared__ int accpos[kMaxBlock];
    __shared__ int s_dec, s_m;
    const int tid = threadIdx.x;
    const int nt = blockDim.x;
    const int64_t r = st->rank;
    const int nz = (int)((r + kColChunk - 1) / kColChunk);
    for (int e = tid; e < b * b; e += nt) {
        double v = kss[e];
        for (int z = 0; z < nz; ++z) v -= hpart[(int64_t)z * b * b + e];
        H[e] = v;
    }
    __syncthreads();
    for (int p = tid; p < b; p += nt) {
        H0[p] = H[p * b + p];
        kfl[p] = floor_rel * kss[p * b + p];
        us[p] = uniforms ? uniforms[((int64_t)round * 2 + 1) * b + p] : philox_uniform(seed, (uint32_t)round, 1u, (uint32_t)p);
    }
    if (tid == 0) s_m = 0;
    __syncthreads();
    const int64_t cap = k_max - r;
    for (int i = 0; i < b; ++i) {
        __syncthreads();
        if (tid == 0) {
            const double u = us[i];
            const double hii = H[i * b + i];
            const int acc = (s_m < cap) && (H0[i] * u < hii) && (hii > tol) && (hii > kfl[i]);
            s_dec = acc;
            if (acc) accpos[s_m++] = i;
        }
        __syncthreads();
        if (s_dec) {
            const double f = 1.0 / sqrt(H[i * b + i]);
            __syncthreads();
            for (int j = i + tid; j < b; j += nt) H[j * b + i] *= f;
            __syncthreads();
            for (int jj = i + 1 + (tid >> 5); jj < b; jj += 32)
                for (int kk = i + 1 + (tid & 31); kk <= jj; kk += 32) H[jj * b + kk] -= H[jj * b + i] * H[kk * b + i];
            __syncthreads();
        }
    }
    const int nacc = s_m;
    for (int e = tid; e < b * b; e += nt) {
        MS[e] = 0.0;
        const int a = e / b, c = e - a * b;
        LC[e] = (a < nacc && c < nacc) ? H[accpos[a] * b + accpos[c]] : 0.0;
    }
    __syncthreads();
    if (tid < nacc) {
        const int t = tid;
        MS[t * b + t] = 1.0 / LC[t * b + t];
        for (int a = t + 1; a < nacc; ++a) {
            const double* la = LC + a * b;
            double sum = 0.0;
            for (int e = t; e < a; ++e) sum += la[e] * MS[e * b + t];
            MS[a * b + t] = -sum / la[a];
        }
    }
    __syncthreads();
    for (int e = tid; e < b * b; e += nt) {
        minv[e] = MS[e];
        minv_f[e] = (float)MS[e];
    }
    if (tid < nacc) {
        const int64_t sp = props[accpos[tid]];
        sacc[tid] = sp;
        piv[r + tid] = sp;
    }
    if (tid == 0) {
        st->r_old = r;
        st->nacc = nacc;
        st->rank = r + nacc;
        hm[round] = nacc;
    }
}

// ---- residual update over all row blocks -----------------------------------
// CTA = 128 rows x up to 64 accepted columns; thread (ty, tx) of 16 x 16 owns
// rows ty + 16i (i < 8) and columns tx + 16j (j < 4).
//
// A round that accepts more than 64 columns is updated in passes of 64
// (group g = columns r + 64g ...).  With L_i = [[L00, 0], [L10, L11]] the new
// columns satisfy G0 = T0 L00^{-T} and G1 = (T1 - G0 L10^T) L11^{-T}; pass g
// therefore runs the one-group update against the factor's first r + 64g
// columns (which include the previous passes' output, whose rows at S_g are
// L10) with the pivots of group g and the diagonal block g of L_i^{-1}.
__device__ __forceinline__ bool group_view(int64_t r_old, int nacc_all, int group, int64_t& r, int& nacc) {
    r = r_old + (int64_t)kGroup * group;
    nacc = min(kGroup, nacc_all - kGroup * group);
    return nacc > 0;
}
template <typename T>
struct UpdSmem {
    static constexpr int KC = 32;
};

template <typename T>
__global__ void __launch_bounds__(256)
rp_update_kernel(T* __restrict__ F, int64_t ldF, const float* __restrict__ X, int64_t N, int d,
                 double scale, const int64_t* __restrict__ sacc, const double* __restrict__ minv,
                 const float* __restrict__ minv_f, int b, const RoundState* st,
                 double* __restrict__ dvec, double* __restrict__ dblk, int group) {
    if (st->done) return;
    int64_t r;
    int nacc;
    if (!group_view(st->r_old, st->nacc, group, r, nacc)) return;
    {   // this pass's pivots and diagonal block of L_i^{-1} (leading dimension b)
        const int64_t o = (int64_t)kGroup * group;
        sacc += o;
        minv += o * b + o;
        minv_f += o * b + o;
    }
    constexpr int KC = UpdSmem<T>::KC;
    extern __shared__ __align__(16) unsigned char smraw[];
    // region 1 (phase A: X rows, kFeat features at a time; phase B: F tiles),
    // then Tm, then Minv
    constexpr int dp = kFeat + 1;
    const size_t reg1_a = (size_t)(kRowBlock + kGroup) * dp * sizeof(float);
    const size_t reg1_b = (size_t)(kRowBlock + kGroup) * (KC + 1) * sizeof(T);
    const size_t reg1 = (reg1_a > reg1_b ? reg1_a : reg1_b + 0);
    float* xr = reinterpret_cast<float*>(smraw);
    float* xs = xr + kRowBlock * dp;
    T* At = reinterpret_cast<T*>(smraw);
    T* Bt = At + kRowBlock * (KC + 1);
    T* Tm = reinterpret_cast<T*>(smraw + ((reg1 + 15) / 16) * 16);   // 128 x (64+1)
    T* Mv = Tm + kRowBlock * (kGroup + 1);                         // 64 x (64+1)
    __shared__ double rowsq_s[kRowBlock];

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t row0 = (int64_t)blockIdx.x * kRowBlock;
    const int nrows = (int)min((int64_t)kRowBlock, N - row0);

    // phase A: K(R, S_i) into Tm
    for (int e = tid; e < nacc * nacc; e += 256) {
        const int a = e / nacc, q = e - a * nacc;
        Mv[a * (kGroup + 1) + q] = sizeof(T) == 8 ? (T)minv[a * b + q] : (T)minv_f[a * b + q];
    }
    {
        T acc[8][4];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0;
        for (int c0 = 0; c0 < d; c0 += kFeat) {
            const int w = min(kFeat, d - c0);
            __syncthreads();
            for (int e = tid; e < kRowBlock * w; e += 256) {
                const int rr = e / w, k = e - rr * w;
                xr[rr * dp + k] = (rr < nrows) ? X[(row0 + rr) * d + c0 + k] : 0.f;
            }
            for (int e = tid; e < nacc * w; e += 256) {
                const int q = e / w, k = e - q * w;
                xs[q * dp + k] = X[sacc[q] * d + c0 + k];
            }
            __syncthreads();
            for (int k = 0; k < w; ++k) {
                T vr[8], vs[4];
#pragma unroll
                for (int i = 0; i < 8; ++i) vr[i] = (T)xr[(ty + 16 * i) * dp + k];
#pragma unroll
                for (int j = 0; j < 4; ++j) vs[j] = (T)xs[min(tx + 16 * j, kGroup - 1) * dp + k];
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const T t = vr[i] - vs[j];
                        acc[i][j] += t * t;
                    }
            }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = tx + 16 * j;
                T kv = 0;
                if (c < nacc) {
                    if (sizeof(T) == 8) kv = (T)exp(-scale * (double)acc[i][j]);
                    else kv = (T)kexp_scaled((float)acc[i][j], split_scale(scale));
                }
                Tm[(ty + 16 * i) * (kGroup + 1) + c] = kv;
            }
    }
    __syncthreads();

    // phase B: acc = F(R, 0:r) F(S_i, 0:r)^T
    T acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0;
    for (int64_t c0 = 0; c0 < r; c0 += KC) {
        const int nc = (int)min((int64_t)KC, r - c0);
        for (int e = tid; e < kRowBlock * KC; e += 256) {
            const int rr = e / KC, c = e - rr * KC;
            At[rr * (KC + 1) + c] = (rr < nrows && c < nc) ? F[(row0 + rr) * ldF + c0 + c] : (T)0;
        }
        for (int e = tid; e < kGroup * KC; e += 256) {
            const int q = e / KC, c = e - q * KC;
            Bt[q * (KC + 1) + c] = (q < nacc && c < nc) ? F[sacc[q] * ldF + c0 + c] : (T)0;
        }
        __syncthreads();
#pragma unroll 4
        for (int c = 0; c < KC; ++c) {
            T va[8], vb[4];
#pragma unroll
            for (int i = 0; i < 8; ++i) va[i] = At[(ty + 16 * i) * (KC + 1) + c];
#pragma unroll
            for (int j = 0; j < 4; ++j) vb[j] = Bt[(tx + 16 * j) * (KC + 1) + c];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] += va[i] * vb[j];
        }
        __syncthreads();
    }
    // phase C: Tm -= acc (own entries)
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) Tm[(ty + 16 * i) * (kGroup + 1) + tx + 16 * j] -= acc[i][j];
    __syncthreads();
    // phase D: G = Tm Minv^T
    T g[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) g[i][j] = 0;
    for (int e = 0; e < nacc; ++e) {
        T vt[8], vm[4];
#pragma unroll
        for (int i = 0; i < 8; ++i) vt[i] = Tm[(ty + 16 * i) * (kGroup + 1) + e];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int a = tx + 16 * j;
            vm[j] = (a < nacc) ? Mv[a * (kGroup + 1) + e] : (T)0;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) g[i][j] += vt[i] * vm[j];
    }
    // phase E: store the new columns, update d, block sum
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int rr = ty + 16 * i;
        double sq = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int a = tx + 16 * j;
            if (a < nacc && rr < nrows) {
                F[(row0 + rr) * ldF + r + a] = g[i][j];
                sq += (double)g[i][j] * (double)g[i][j];
            }
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
        if (tx == 0) rowsq_s[rr] = sq;
    }
    __syncthreads();
    double nd = 0.0;
    if (tid < kRowBlock && tid < nrows) {
        const int64_t gi = row0 + tid;
        nd = fmax(dvec[gi] - rowsq_s[tid], 0.0);
        dvec[gi] = nd;
    }
    // block sum of the new d over the first 128 threads (4 warps)
    __shared__ double wsum[8];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nd += __shfl_xor_sync(0xffffffffu, nd, o);
    if ((tid & 31) == 0) wsum[tid >> 5] = nd;
    __syncthreads();
    if (tid == 0) dblk[blockIdx.x] = ((wsum[0] + wsum[1]) + (wsum[2] + wsum[3]));
}

template <typename T>
static size_t update_smem(int d) {
    (void)d;
    const int dp = kFeat + 1;
    const size_t reg1_a = (size_t)(kRowBlock + kGroup) * dp * sizeof(float);
    const size_t reg1_b = (size_t)(kRowBlock + kGroup) * (UpdSmem<T>::KC + 1) * sizeof(T);
    const size_t reg1 = ((std::max(reg1_a, reg1_b) + 15) / 16) * 16;
    return reg1 + (size_t)kRowBlock * (kGroup + 1) * sizeof(T) +
           (size_t)kGroup * (kGroup + 1) * sizeof(T);
}

template <typename T>
static int rpchol_impl(kevd_ctx* ctx, const float* X, int64_t N, int d, double scale,
                       const kevd_rpchol_params* p, T* F, int64_t ldF, int64_t* piv_h,
                       double* err_h, int32_t* hm_h, kevd_rpchol_result* res, cudaStream_t s,
                       RpcholDeferred* defer = nullptr, bool tc_allowed = true) {
    const int b = p->block;
    const double floor_rel = sizeof(T) == 4 ? kMixedFloor : 0.0;
    const int64_t nblk = (N + kRowBlock - 1) / kRowBlock;
    const int n_split = (int)((p->k_max + kColChunk - 1) / kColChunk);
    const int n_kss = 32;   // CTAs sharing the FP64 K(S', S') block (one element per thread, same order)
    int st = KEVD_OK;
    double* dvec = arena_get<double>(ctx, "rp.d", N, &st);
    double* dblk = arena_get<double>(ctx, "rp.dblk", nblk, &st);
    RoundState* rs = arena_get<RoundState>(ctx, "rp.state", 1, &st);
    int64_t* props = arena_get<int64_t>(ctx, "rp.props", kMaxBlock, &st);
    int64_t* sacc = arena_get<int64_t>(ctx, "rp.sacc", kMaxBlock, &st);
    int64_t* piv = arena_get<int64_t>(ctx, "rp.piv", p->k_max, &st);
    double* hpart = arena_get<double>(ctx, "rp.hpart", (size_t)std::max(n_split, 1) * b * b, &st);
    double* kss = arena_get<double>(ctx, "rp.kss", (size_t)b * b, &st);
    double* minv = arena_get<double>(ctx, "rp.minv", (size_t)b * b, &st);
    float* minv_f = arena_get<float>(ctx, "rp.minvf", (size_t)b * b, &st);
    double* err = arena_get<double>(ctx, "rp.err", p->max_rounds, &st);
    int32_t* hm = arena_get<int32_t>(ctx, "rp.hm", p->max_rounds, &st);
    double* unif = nullptr;
    if (p->uniforms) unif = arena_get<double>(ctx, "rp.unif", (size_t)p->max_rounds * 2 * b, &st);
    if (st != KEVD_OK) return st;
    if (unif)
        KEVD_CUDA(ctx, cudaMemcpyAsync(unif, p->uniforms, (size_t)p->max_rounds * 2 * b * sizeof(double),
                                       cudaMemcpyHostToDevice, s));
    KEVD_CUDA(ctx, cudaMemsetAsync(err, 0, p->max_rounds * sizeof(double), s));
    KEVD_CUDA(ctx, cudaMemsetAsync(hm, 0, p->max_rounds * sizeof(int32_t), s));
    rp_init_kernel<<<ctx->num_sms * 4, 256, 0, s>>>(dvec, dblk, N, nblk, rs);
    KEVD_LAUNCH(ctx);

    const bool big = b > kSmallBlock;
    const size_t fsm = big ? 0 : (size_t)3 * b * b * sizeof(double);
    double* hbig = nullptr;   // H, the compacted factor and the inverse of a large block
    if (big) {
        hbig = arena_get<double>(ctx, "rp.hbig", (size_t)3 * b * b, &st);
        if (st != KEVD_OK) return st;
    } else {
        KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&rp_factor_kernel), (int)std::max(fsm, (size_t)1024)));
    }
    const size_t hsm = hgram_smem<T>(b);
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&rp_hgram_kernel<T>), (int)hsm));
    const int n_groups = (b + kGroup - 1) / kGroup;
    const size_t usm = update_smem<T>(d);
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&rp_update_kernel<T>), (int)usm));
    int* done_h = static_cast<int*>(ctx->pinned);
    // FP32 factors take the tensor-core residual update when the layout allows
    // TMA and the kernel is not nearly diagonal (kernel_density_kernel)
    const bool use_tc =
        sizeof(T) == 4 && tc_allowed && update_tc_supported(reinterpret_cast<const float*>(F), ldF, d);
    int* tc_err = arena_get<int>(ctx, "rp.tcerr", 1, &st);
    if (st != KEVD_OK) return st;
    KEVD_CUDA(ctx, cudaMemsetAsync(tc_err, 0, sizeof(int), s));
    int round = 0;
    for (; round < p->max_rounds; ++round) {
        {
            ProfScope ps(ctx, "rp_sample", s);
            rp_sample_kernel<<<1, kSampleThreads, 0, s>>>(dvec, dblk, N, nblk, round, b, p->seed,
                                                          unif, props, rs, p->k_max, p->max_rounds,
                                                          p->err_target, floor_rel, err);
            KEVD_LAUNCH(ctx);
        }
        {
            ProfScope ps(ctx, "rp_hgram", s);
            rp_hgram_kernel<T><<<n_split + n_kss, 256, hsm, s>>>(F, ldF, X, d, scale, props, b,
                                                               n_split, rs, hpart, kss);
            KEVD_LAUNCH(ctx);
        }
        {
            ProfScope ps(ctx, "rp_factor", s);
            if (big)
                rp_factor_big_kernel<<<1, kBigFactorThreads, 0, s>>>(kss, hpart, b, round, p->seed, unif, p->tol,
                                                                      floor_rel, p->k_max, props, rs, minv, minv_f,
                                                                      sacc, piv, hm, hbig, hbig + (size_t)b * b,
                                                                      hbig + (size_t)2 * b * b);
            else
                rp_factor_kernel<<<1, kFactorThreads, fsm, s>>>(kss, hpart, b, round, p->seed, unif, p->tol,
                                                                floor_rel, p->k_max, props, rs, minv, minv_f, sacc,
                                                                piv, hm);
            KEVD_LAUNCH(ctx);
        }
        if (use_tc) {
            KEVD_TRY(launch_update_tc(ctx, reinterpret_cast<float*>(F), ldF, N, p->k_max, X, d, scale, sacc,
                                      minv_f, b, rs, dvec, dblk, tc_err, s));
        } else {
            ProfScope ps(ctx, "rp_update", s);
            for (int g = 0; g < n_groups; ++g) {
                rp_update_kernel<T><<<(int)nblk, 256, usm, s>>>(F, ldF, X, N, d, scale, sacc, minv,
                                                               minv_f, b, rs, dvec, dblk, g);
                KEVD_LAUNCH(ctx);
            }
        }
        if (!defer && (round & 3) == 3) {
            KEVD_CUDA(ctx, cudaMemcpyAsync(done_h, &rs->done, sizeof(int), cudaMemcpyDeviceToHost, s));
            KEVD_CUDA(ctx, cudaStreamSynchronize(s));
            if (*done_h) break;
        }
    }
    // closing sampler call: records the last round's error and the stop
    rp_sample_kernel<<<1, kSampleThreads, 0, s>>>(dvec, dblk, N, nblk, std::min(round, p->max_rounds),
                                                  0, p->seed, unif, props, rs, p->k_max,
                                                  std::min(round, p->max_rounds), p->err_target, floor_rel, err);
    KEVD_LAUNCH(ctx);
    if (defer) {
        // capture-safe: results go to pinned host memory, read after the stream completes
        KEVD_CUDA(ctx, cudaMemcpyAsync(defer->state_h, rs, sizeof(RoundState), cudaMemcpyDeviceToHost, s));
        KEVD_CUDA(ctx, cudaMemcpyAsync(defer->tcerr_h, tc_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        KEVD_CUDA(ctx, cudaMemcpyAsync(defer->piv_h, piv, p->k_max * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        return KEVD_OK;
    }
    RoundState hs;
    int herr = 0;
    KEVD_CUDA(ctx, cudaMemcpyAsync(&hs, rs, sizeof(RoundState), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(&herr, tc_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    if (herr != 0)
        return set_error(ctx, KEVD_ERR_TIMEOUT, "rpchol: tensor-core update pipeline timed out (code %d)", herr);
    if (hs.rank > 0 && piv_h)
        KEVD_CUDA(ctx, cudaMemcpy(piv_h, piv, hs.rank * sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (err_h) KEVD_CUDA(ctx, cudaMemcpy(err_h, err, hs.rounds * sizeof(double), cudaMemcpyDeviceToHost));
    if (hm_h) KEVD_CUDA(ctx, cudaMemcpy(hm_h, hm, hs.rounds * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (res) {
        res->rank = hs.rank;
        res->rounds = hs.rounds;
        res->trace_error = hs.total / (double)N;
    }
    return KEVD_OK;
}

int run_rpchol(kevd_ctx* ctx, const float* X, int64_t N, int d, double scale,
               const kevd_rpchol_params* p, void* F, int64_t ldF, int64_t* piv, double* err,
               int32_t* accepted, kevd_rpchol_result* res, cudaStream_t s) {
    if (!X || !p || !F || N < 1 || d < 1 || d > kMaxFeatures)
        return set_error(ctx, KEVD_ERR_ARG, "rpchol: need X, F, N >= 1 and 1 <= d <= %d", kMaxFeatures);
    if (p->block < 1 || p->block > kMaxBlock)
        return set_error(ctx, KEVD_ERR_ARG, "rpchol: block must be in [1, %d]", kMaxBlock);
    if (p->k_max < 1 || ldF < p->k_max || p->max_rounds < 1)
        return set_error(ctx, KEVD_ERR_ARG, "rpchol: need k_max >= 1, ldF >= k_max, max_rounds >= 1");
    if (p->precision == KEVD_FP64)
        return rpchol_impl<double>(ctx, X, N, d, scale, p, (double*)F, ldF, piv, err, accepted, res, s);
    if (p->precision == KEVD_MIXED) {
        bool diag = false;
        if (update_tc_supported((const float*)F, ldF, d)) KEVD_TRY(kernel_nearly_diagonal(ctx, X, N, d, scale, s, &diag));
        return rpchol_impl<float>(ctx, X, N, d, scale, p, (float*)F, ldF, piv, err, accepted, res, s, nullptr, !diag);
    }
    return set_error(ctx, KEVD_ERR_ARG, "rpchol: unknown precision %d", p->precision);
}

// Many factorisations at once.  Each job gets its own workspace context and
// stream; with use_graph the whole set of round loops is captured as parallel
// branches of one CUDA graph (fork from the caller's stream, join back) and
// launched once, so the GPU overlaps the jobs' small launches without a host
// thread per job.  Without use_graph the same work is issued directly on the
// per-job streams.
int run_rpchol_batched(kevd_ctx* ctx, kevd_rpchol_job* jobs, int n_jobs, int use_graph, cudaStream_t s) {
    if (!jobs || n_jobs < 1 || n_jobs > 1024) return set_error(ctx, KEVD_ERR_ARG, "rpchol_batched: 1..1024 jobs");
    for (int q = 0; q < n_jobs; ++q) {
        const kevd_rpchol_job& j = jobs[q];
        if (!j.X || !j.F || !j.piv || j.N < 1 || j.d < 1 || j.d > kMaxFeatures || j.block < 1 || j.block > kMaxBlock ||
            j.k_max < 1 || j.ldF < j.k_max || j.max_rounds < 1 || !(j.scale > 0.0))
            return set_error(ctx, KEVD_ERR_ARG, "rpchol_batched: bad job %d", q);
    }
    struct Slot {
        kevd_ctx* c = nullptr;
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        RoundState* state_h = nullptr;
        int* tcerr_h = nullptr;
        int64_t* piv_h = nullptr;
    };
    std::vector<Slot> sl(n_jobs);
    int rc = KEVD_OK;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (fork) cudaEventDestroy(fork);
        for (auto& x : sl) {
            if (x.ev) cudaEventDestroy(x.ev);
            if (x.st) cudaStreamDestroy(x.st);
            if (x.state_h) cudaFreeHost(x.state_h);
            if (x.tcerr_h) cudaFreeHost(x.tcerr_h);
            if (x.piv_h) cudaFreeHost(x.piv_h);
            if (x.c) {
                x.c->arena.release();
                delete x.c;
            }
        }
    };
    for (int q = 0; q < n_jobs && rc == KEVD_OK; ++q) {
        Slot& x = sl[q];
        x.c = new kevd_ctx();
        x.c->device = ctx->device;
        x.c->num_sms = ctx->num_sms;
        if (cudaStreamCreateWithFlags(&x.st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&x.ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaMallocHost(&x.state_h, sizeof(RoundState)) != cudaSuccess ||
            cudaMallocHost(&x.tcerr_h, sizeof(int)) != cudaSuccess ||
            cudaMallocHost(&x.piv_h, jobs[q].k_max * sizeof(int64_t)) != cudaSuccess)
            rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: stream / pinned buffer setup failed");
    }
    if (rc == KEVD_OK && cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess)
        rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: event setup failed");
    // the residual-update form of every job, decided before any capture
    std::vector<char> tc_ok(n_jobs, 1);
    for (int q = 0; q < n_jobs && rc == KEVD_OK; ++q) {
        const kevd_rpchol_job& j = jobs[q];
        bool diag = false;
        if (update_tc_supported((const float*)j.F, j.ldF, j.d)) rc = kernel_nearly_diagonal(ctx, j.X, j.N, j.d, j.scale, s, &diag);
        tc_ok[q] = diag ? 0 : 1;
    }
    // the capture runs on a stream of its own (the caller's stream may be the
    // legacy default stream, which cannot be captured); it is ordered after the
    // caller's work and the graph is launched on the caller's stream
    cudaStream_t cs = nullptr;
    if (rc == KEVD_OK && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
        rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: capture stream setup failed");
    auto enqueue_all = [&](int rounds_override, cudaStream_t root) -> int {
        if (cudaEventRecord(fork, root) != cudaSuccess) return set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: fork");
        for (int q = 0; q < n_jobs; ++q) {
            const kevd_rpchol_job& j = jobs[q];
            Slot& x = sl[q];
            if (cudaStreamWaitEvent(x.st, fork, 0) != cudaSuccess)
                return set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: fork wait");
            kevd_rpchol_params p;
            std::memset(&p, 0, sizeof(p));
            p.k_max = j.k_max;
            p.block = j.block;
            p.max_rounds = rounds_override > 0 ? rounds_override : j.max_rounds;
            p.tol = 1e-10;
            p.seed = j.seed;
            p.precision = KEVD_MIXED;
            RpcholDeferred df{x.state_h, x.tcerr_h, x.piv_h};
            const int r = rpchol_impl<float>(x.c, j.X, j.N, j.d, j.scale, &p, (float*)j.F, j.ldF, nullptr, nullptr,
                                             nullptr, nullptr, x.st, &df, tc_ok[q] != 0);
            ctx->launches += x.c->launches;
            x.c->launches = 0;
            if (r != KEVD_OK) return set_error(ctx, r, "rpchol_batched: job %d: %s", q, x.c->last_error.c_str());
            if (cudaEventRecord(x.ev, x.st) != cudaSuccess || cudaStreamWaitEvent(root, x.ev, 0) != cudaSuccess)
                return set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: join");
        }
        return KEVD_OK;
    };
    if (rc == KEVD_OK) {
        if (use_graph) {
            // one uncaptured round per job allocates every workspace buffer (their
            // sizes do not depend on the round count), so nothing is allocated
            // inside the capture; the captured run starts again from rp_init
            rc = enqueue_all(1, s);
            if (rc == KEVD_OK && cudaStreamSynchronize(s) != cudaSuccess)
                rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: workspace pass failed");
            if (rc == KEVD_OK) {
                if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
                    rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: begin capture");
                } else {
                    rc = enqueue_all(0, cs);
                    const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
                    if (rc == KEVD_OK && ce != cudaSuccess)
                        rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: end capture: %s", cudaGetErrorString(ce));
                }
            }
            if (rc == KEVD_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
                rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: graph instantiate");
            if (rc == KEVD_OK && cudaGraphLaunch(exec, s) != cudaSuccess)
                rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: graph launch");
        } else {
            rc = enqueue_all(0, s);
        }
    }
    if (rc == KEVD_OK && cudaStreamSynchronize(s) != cudaSuccess)
        rc = set_error(ctx, KEVD_ERR_CUDA, "rpchol_batched: %s", cudaGetErrorString(cudaGetLastError()));
    if (rc == KEVD_OK) {
        for (int q = 0; q < n_jobs; ++q) {
            const Slot& x = sl[q];
            kevd_rpchol_job& j = jobs[q];
            if (*x.tcerr_h != 0 && rc == KEVD_OK)
                rc = set_error(ctx, KEVD_ERR_TIMEOUT, "rpchol_batched: job %d tensor-core pipeline timed out", q);
            j.result.rank = x.state_h->rank;
            j.result.rounds = x.state_h->rounds;
            j.result.trace_error = x.state_h->total / (double)j.N;
            std::memcpy(j.piv, x.piv_h, (size_t)x.state_h->rank * sizeof(int64_t));
        }
    }
    cleanup();
    if (cs) cudaStreamDestroy(cs);
    return rc;
}

// Gather rows idx of F (first ncols columns) into a column-major FP64 n x ncols
// matrix (ld n): used for L = F(S, :).
template <typename T>
__global__ void gather_rows_kernel(const T* __restrict__ F, int64_t ldF,
                                   const int64_t* __restrict__ idx, int64_t n, int64_t ncols,
                                   double* __restrict__ out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * ncols;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e / n, q = e - c * n;
        out[e] = (double)F[idx[q] * ldF + c];
    }
}

int run_gather_rows(kevd_ctx* ctx, const void* F, int precision, int64_t ldF, const int64_t* idx,
                    int64_t n, int64_t ncols, double* out, cudaStream_t s) {
    const int grid = (int)std::min<int64_t>((n * ncols + 255) / 256, (int64_t)ctx->num_sms * 16);
    if (grid < 1) return KEVD_OK;
    if (precision == KEVD_FP64)
        gather_rows_kernel<double><<<grid, 256, 0, s>>>((const double*)F, ldF, idx, n, ncols, out);
    else
        gather_rows_kernel<float><<<grid, 256, 0, s>>>((const float*)F, ldF, idx, n, ncols, out);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

}  // namespace kevd
