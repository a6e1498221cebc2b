// Stage 1: fused bandwidth-calibration pair sums and the pair-distance median.
//
// The reference writes every strict-lower-triangle distance to HBM
// (dmat_comp, ks_bandwidth.cu:181-232) and re-reads the whole buffer once per
// bandwidth (kernelsum_comp x 36, :276-325, :566-572).  Here each 128 x 128
// pair tile is evaluated once into registers and every scale of the sweep is
// accumulated from those registers in the same pass: no distance buffer, one
// read of X (L2-resident), and the work is bound by the exp2 (MUFU) rate.
//
// Tiles cover the lower triangle ti >= tj of the 128-row tile grid; pairs with
// i <= l, or outside [0, N), are masked to D = +inf (exp2(-inf) = 0).  Each
// CTA is persistent over a static stride of tiles and keeps one FP64
// accumulator per scale; warp partials are FP32 (<= 2048 terms of <= 1).  The
// per-CTA FP64 partials go to a scratch array and a second kernel reduces them
// in a fixed order, so the result is deterministic.
#include "kevd_internal.cuh"
#include "kevd_pairtile.cuh"

#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

namespace kevd {

constexpr int kCalTile = 128;
constexpr int kCalMaxScales = 256;
constexpr int kCalMaxD = 1024;
constexpr int kFC = 64;            // feature chunk staged in shared memory
constexpr int kFP = kFC + 1;       // its row pitch (bank-conflict padding)

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Tile index t of the lower-triangular tile grid -> (ti, tj), ti >= tj.
__device__ __forceinline__ void tri_tile(int64_t t, int64_t& ti, int64_t& tj) {
    int64_t i = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > t) --i;
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    ti = i;
    tj = t - i * (i + 1) / 2;
}

// Loads features [c0, c0 + w) of rows [r0, r0+128) of X into a [128][kFP]
// shared tile (zeros past N).
__device__ __forceinline__ void load_chunk(const float* __restrict__ X, int64_t N, int d, int64_t r0, int c0,
                                           int w, float* dst) {
    for (int e = threadIdx.x; e < kCalTile * w; e += blockDim.x) {
        const int rr = e / w, kk = e - rr * w;
        const int64_t r = r0 + rr;
        dst[rr * kFP + kk] = (r < N) ? X[r * d + c0 + kk] : 0.f;
    }
}

__global__ void __launch_bounds__(256, 2)
calibrate_tiles_kernel(const float* __restrict__ X, int64_t N, int d,
                       const float* __restrict__ c2, int n_scales, int64_t n_tiles,
                       double* __restrict__ partial) {
    extern __shared__ __align__(16) float sm[];
    float* xi = sm;
    float* xj = sm + kPtTile * kPtPitch;
    float* cs = xj + kPtTile * kPtPitch;                 // n_scales
    float* red = cs + kCalMaxScales;                     // 8 warps x n_scales
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = threadIdx.x; j < n_scales; j += blockDim.x) cs[j] = c2[j];
    double acc = 0.0;  // thread j < n_scales owns scale j
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        int64_t ti, tj;
        tri_tile(t, ti, tj);
        float D[8][8];
        pt_dist(X, N, d, ti * kCalTile, tj * kCalTile, xi, xj, ty, tx, D);
        const int64_t gi0 = ti * kCalTile + ty, gj0 = tj * kCalTile + tx;
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const int64_t gi = gi0 + 16 * a, gj = gj0 + 16 * b;
                if (!(gi < N && gi > gj)) D[a][b] = __int_as_float(0x7f800000);  // +inf
            }
        for (int j = 0; j < n_scales; ++j) {
            const float c = -cs[j];
            float s = 0.f;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) s += ex2_approx(D[a][b] * c);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) red[warp * kCalMaxScales + j] = s;
        }
        __syncthreads();
        if (threadIdx.x < n_scales) {
            double w = 0.0;
#pragma unroll
            for (int q = 0; q < 8; ++q) w += (double)red[q * kCalMaxScales + threadIdx.x];
            acc += w;
        }
    }
    if (threadIdx.x < n_scales) partial[(int64_t)blockIdx.x * n_scales + threadIdx.x] = acc;
}

__global__ void reduce_partials_kernel(const double* __restrict__ partial, int n_parts,
                                       int n_scales, double* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_scales) return;
    double s = 0.0;
    for (int p = 0; p < n_parts; ++p) s += partial[(int64_t)p * n_scales + j];
    out[j] = s;
}

// Plain FP64 form of the same pass (FP64 direct distances, FP64 exp): the
// precision reference of the fused FP32 / exp2 kernel above.  Same tiles and
// masking; 64 FP64 distances per thread, so one CTA per SM.
__global__ void __launch_bounds__(256, 1)
calibrate_tiles_fp64_kernel(const float* __restrict__ X, int64_t N, int d, const double* __restrict__ sc,
                            int n_scales, int64_t n_tiles, double* __restrict__ partial) {
    extern __shared__ float sm[];
    float* xi = sm;
    float* xj = sm + kCalTile * kFP;
    double* cs = reinterpret_cast<double*>(xj + kCalTile * kFP + 2);   // 8-byte aligned (2 x 128 x kFP floats is even)
    double* red = cs + kCalMaxScales;                                   // 8 warps x n_scales
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = threadIdx.x; j < n_scales; j += blockDim.x) cs[j] = sc[j];
    double acc = 0.0;
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        int64_t ti, tj;
        tri_tile(t, ti, tj);
        double D[8][8];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < 8; ++b) D[a][b] = 0.0;
        for (int c0 = 0; c0 < d; c0 += kFC) {
            const int w = min(kFC, d - c0);
            __syncthreads();
            load_chunk(X, N, d, ti * kCalTile, c0, w, xi);
            load_chunk(X, N, d, tj * kCalTile, c0, w, xj);
            __syncthreads();
            for (int k = 0; k < w; ++k) {
                double vi[8], vj[8];
#pragma unroll
                for (int a = 0; a < 8; ++a) vi[a] = (double)xi[(ty + 16 * a) * kFP + k];
#pragma unroll
                for (int b = 0; b < 8; ++b) vj[b] = (double)xj[(tx + 16 * b) * kFP + k];
#pragma unroll
                for (int a = 0; a < 8; ++a)
#pragma unroll
                    for (int b = 0; b < 8; ++b) {
                        const double u = vi[a] - vj[b];
                        D[a][b] = fma(u, u, D[a][b]);
                    }
            }
        }
        const int64_t gi0 = ti * kCalTile + ty, gj0 = tj * kCalTile + tx;
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const int64_t gi = gi0 + 16 * a, gj = gj0 + 16 * b;
                if (!(gi < N && gi > gj)) D[a][b] = __longlong_as_double(0x7ff0000000000000ll);  // +inf
            }
        for (int j = 0; j < n_scales; ++j) {
            const double c = -cs[j];
            double s = 0.0;
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) s += exp(D[a][b] * c);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) red[warp * kCalMaxScales + j] = s;
        }
        __syncthreads();
        if (threadIdx.x < n_scales) {
            double w = 0.0;
#pragma unroll
            for (int q = 0; q < 8; ++q) w += red[q * kCalMaxScales + threadIdx.x];
            acc += w;
        }
    }
    if (threadIdx.x < n_scales) partial[(int64_t)blockIdx.x * n_scales + threadIdx.x] = acc;
}

static size_t calib_smem_fp64(int d) {
    (void)d;
    return 2 * kCalTile * (size_t)kFP * sizeof(float) + 16 + 9 * kCalMaxScales * sizeof(double);
}

int run_calibrate_fp64(kevd_ctx* ctx, const float* X, int64_t N, int d, const double* scales, int n_scales,
                       double* sums, cudaStream_t s) {
    if (!X || !scales || !sums || N < 1 || d < 1 || d > kCalMaxD || n_scales < 1 || n_scales > kCalMaxScales)
        return set_error(ctx, KEVD_ERR_ARG, "calibrate_fp64: need N >= 1, 1 <= d <= %d, 1 <= n_scales <= %d",
                         kCalMaxD, kCalMaxScales);
    for (int j = 0; j < n_scales; ++j)
        if (!(scales[j] > 0.0)) return set_error(ctx, KEVD_ERR_ARG, "calibrate_fp64: scales must be positive");
    const int64_t nt = (N + kCalTile - 1) / kCalTile;
    const int64_t n_tiles = nt * (nt + 1) / 2;
    const int grid = (int)std::min<int64_t>(n_tiles, (int64_t)ctx->num_sms);
    int st = KEVD_OK;
    double* sc = arena_get<double>(ctx, "cal64.sc", kCalMaxScales, &st);
    double* partial = arena_get<double>(ctx, "cal64.partial", (size_t)grid * n_scales, &st);
    double* out = arena_get<double>(ctx, "cal64.out", kCalMaxScales, &st);
    if (st != KEVD_OK) return st;
    KEVD_CUDA(ctx, cudaMemcpyAsync(sc, scales, n_scales * sizeof(double), cudaMemcpyHostToDevice, s));
    const size_t smem = calib_smem_fp64(d);
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&calibrate_tiles_fp64_kernel), (int)smem));
    {
        ProfScope ps(ctx, "calibrate_tiles_fp64", s);
        calibrate_tiles_fp64_kernel<<<grid, 256, smem, s>>>(X, N, d, sc, n_scales, n_tiles, partial);
        KEVD_LAUNCH(ctx);
    }
    reduce_partials_kernel<<<1, kCalMaxScales, 0, s>>>(partial, grid, n_scales, out);
    KEVD_LAUNCH(ctx);
    KEVD_CUDA(ctx, cudaMemcpyAsync(sums, out, n_scales * sizeof(double), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    return KEVD_OK;
}

static size_t calib_smem(int d) {
    (void)d;
    return (2 * kPtTile * (size_t)kPtPitch + kCalMaxScales + 8 * kCalMaxScales) * sizeof(float);
}

int run_calibrate(kevd_ctx* ctx, const float* X, int64_t N, int d, const double* scales,
                  int n_scales, double* sums, cudaStream_t s) {
    if (!X || !scales || !sums || N < 1 || d < 1 || d > kCalMaxD || n_scales < 1 ||
        n_scales > kCalMaxScales)
        return set_error(ctx, KEVD_ERR_ARG,
                         "calibrate: need N >= 1, 1 <= d <= %d, 1 <= n_scales <= %d", kCalMaxD,
                         kCalMaxScales);
    const int64_t nt = (N + kCalTile - 1) / kCalTile;
    const int64_t n_tiles = nt * (nt + 1) / 2;
    const int grid = (int)std::min<int64_t>(n_tiles, (int64_t)ctx->num_sms * 2);
    int st = KEVD_OK;
    float* c2 = arena_get<float>(ctx, "cal.c2", kCalMaxScales, &st);
    double* partial = arena_get<double>(ctx, "cal.partial", (size_t)grid * n_scales, &st);
    double* out = arena_get<double>(ctx, "cal.out", kCalMaxScales, &st);
    if (st != KEVD_OK) return st;
    std::vector<float> hc(n_scales);
    for (int j = 0; j < n_scales; ++j) {
        if (!(scales[j] > 0.0))
            return set_error(ctx, KEVD_ERR_ARG, "calibrate: scales must be positive");
        hc[j] = (float)(scales[j] * 1.4426950408889634);  // exp(-x s) = exp2(-x s log2 e)
    }
    KEVD_CUDA(ctx, cudaMemcpyAsync(c2, hc.data(), n_scales * sizeof(float),
                                   cudaMemcpyHostToDevice, s));
    const size_t smem = calib_smem(d);
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&calibrate_tiles_kernel), (int)smem));
    {
        ProfScope ps(ctx, "calibrate_tiles", s);
        calibrate_tiles_kernel<<<grid, 256, smem, s>>>(X, N, d, c2, n_scales, n_tiles, partial);
        KEVD_LAUNCH(ctx);
    }
    reduce_partials_kernel<<<1, kCalMaxScales, 0, s>>>(partial, grid, n_scales, out);
    KEVD_LAUNCH(ctx);
    KEVD_CUDA(ctx, cudaMemcpyAsync(sums, out, n_scales * sizeof(double), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    return KEVD_OK;
}

// ---- calibration without allocation -------------------------------------
// Some callers cannot allocate device memory: processes whose device memory is
// fully reserved by a pool they do not own (another framework's caching
// allocator, a host application that hands the plugin a fixed budget), and
// services that forbid allocation once they have started.  For them the
// pair-sum sweep has a variant whose scratch (per-CTA FP64 partials, the
// device copy of the scales and the reduced sums) lives in fixed file-scope
// device arrays instead of workspace buffers.  Limits: at most kNaMaxScales
// scales per call and a grid of at most kNaGrid CTAs (about 160 KB held by
// every GPU that loads the library, until the process exits).  Each call
// overwrites every entry it reads, so no entry has to start at zero; calls
// share the arrays, so calls that overlap on the GPU (different streams, or
// several host threads) race.
constexpr int kNaMaxScales = 64;
constexpr int kNaGrid = 304;
static __device__ __align__(256) double g_na_partial[kNaGrid * kNaMaxScales];
static __device__ __align__(256) float g_na_scales[kNaMaxScales];
static __device__ __align__(256) double g_na_sums[kNaMaxScales];

struct NoAllocScratch {
    double* partial = nullptr;
    float* scales = nullptr;
    double* sums = nullptr;
};

// The current CUDA context, through the driver entry point (no link against
// the driver library): the module holding the arrays is loaded once per
// context, so their device addresses are only valid in the context that
// resolved them.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
static CtxGetCurrentFn ctx_get_current() {
    static const CtxGetCurrentFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<CtxGetCurrentFn>(p);
        return (CtxGetCurrentFn) nullptr;
    }();
    return fn;
}

// Device addresses of the arrays, resolved with cudaGetSymbolAddress once per
// device and context, with that device current (a host-side use of the
// symbols is a host stand-in, not a device address).  A caller that switches
// to another context on the same device (cuCtxCreate) gets them resolved
// again for that context.
static int noalloc_scratch(NoAllocScratch* out) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static CUcontext owner[kMaxDevices] = {};
    static NoAllocScratch table[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return KEVD_ERR_CUDA;
    CUcontext cur = nullptr;
    const CtxGetCurrentFn get = ctx_get_current();
    if (get && get(&cur) != CUDA_SUCCESS) cur = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (owner[dev] == nullptr || owner[dev] != cur) {
        NoAllocScratch t;
        if (cudaGetSymbolAddress((void**)&t.partial, g_na_partial) != cudaSuccess ||
            cudaGetSymbolAddress((void**)&t.scales, g_na_scales) != cudaSuccess ||
            cudaGetSymbolAddress((void**)&t.sums, g_na_sums) != cudaSuccess)
            return KEVD_ERR_CUDA;
        // the first symbol access made the context current if none was
        if (get && cur == nullptr && get(&cur) != CUDA_SUCCESS) cur = nullptr;
        table[dev] = t;
        owner[dev] = cur;
    }
    *out = table[dev];
    return KEVD_OK;
}

int run_calibrate_noalloc(const float* X, int64_t N, int d, const double* scales, int n_scales, double* sums,
                          cudaStream_t s) {
    if (!X || !scales || !sums || N < 1 || d < 1 || d > kCalMaxD || n_scales < 1 || n_scales > kNaMaxScales)
        return KEVD_ERR_ARG;
    for (int j = 0; j < n_scales; ++j)
        if (!(scales[j] > 0.0)) return KEVD_ERR_ARG;
    // An error left pending by earlier work on this thread would make this
    // call's launch check ambiguous: report it and leave it in place.
    if (cudaPeekAtLastError() != cudaSuccess) return KEVD_ERR_CUDA;
    NoAllocScratch sc;
    if (noalloc_scratch(&sc) != KEVD_OK) {
        cudaGetLastError();   // this call's own failure
        return KEVD_ERR_CUDA;
    }
    float hc[kNaMaxScales];
    for (int j = 0; j < n_scales; ++j) hc[j] = (float)(scales[j] * 1.4426950408889634);
    const int64_t nt = (N + kCalTile - 1) / kCalTile;
    const int64_t n_tiles = nt * (nt + 1) / 2;
    const int grid = (int)std::min<int64_t>(n_tiles, kNaGrid);
    const size_t smem = calib_smem(d);
    // hc lives on this stack frame: the copy is complete (pageable source) or
    // staged before cudaMemcpyAsync returns, and the stream is synchronised
    // below before the frame goes away
    if (cudaMemcpyAsync(sc.scales, hc, n_scales * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        raise_smem_limit(reinterpret_cast<const void*>(&calibrate_tiles_kernel), (int)smem) !=
            cudaSuccess) {
        cudaGetLastError();
        return KEVD_ERR_CUDA;
    }
    calibrate_tiles_kernel<<<grid, 256, smem, s>>>(X, N, d, sc.scales, n_scales, n_tiles, sc.partial);
    reduce_partials_kernel<<<1, kCalMaxScales, 0, s>>>(sc.partial, grid, n_scales, sc.sums);
    if (cudaPeekAtLastError() != cudaSuccess ||
        cudaMemcpyAsync(sums, sc.sums, n_scales * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();   // nothing was pending on entry: the error is this call's
        return KEVD_ERR_CUDA;
    }
    return KEVD_OK;
}

// ---- pair-distance median by radix selection over FP32 bit patterns -------
//
// Non-negative floats order like their uint32 bit patterns.  Three passes
// histogram bits [31:20], [19:8], [7:0] of the distances whose higher bits
// match the prefix found so far; the host walks each histogram to the bin
// holding the wanted rank.  Distances are recomputed in every pass (cheap
// next to the 4096-bin shared-memory histogram).

constexpr int kHistBins = 4096;

__device__ __forceinline__ void hist_add(unsigned* h, float D, int shift, unsigned mask,
                                         unsigned prefix, int hi_shift) {
    const unsigned u = __float_as_uint(D);
    const bool match = (hi_shift >= 32) ? true : ((u >> hi_shift) == prefix);
    if (match) atomicAdd(&h[(u >> shift) & mask], 1u);
}

__global__ void __launch_bounds__(256, 2)
median_tiles_kernel(const float* __restrict__ X, int64_t N, int d, int64_t n_tiles, int shift,
                    unsigned mask, unsigned prefix, int hi_shift, unsigned* __restrict__ hist) {
    extern __shared__ __align__(16) float sm[];
    float* xi = sm;
    float* xj = sm + kPtTile * kPtPitch;
    unsigned* h = reinterpret_cast<unsigned*>(xj + kPtTile * kPtPitch);
    for (int e = threadIdx.x; e < kHistBins; e += blockDim.x) h[e] = 0u;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        int64_t ti, tj;
        tri_tile(t, ti, tj);
        float D[8][8];
        pt_dist(X, N, d, ti * kCalTile, tj * kCalTile, xi, xj, ty, tx, D);
        const int64_t gi0 = ti * kCalTile + ty, gj0 = tj * kCalTile + tx;
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const int64_t gi = gi0 + 16 * a, gj = gj0 + 16 * b;
                if (gi < N && gi > gj) hist_add(h, D[a][b], shift, mask, prefix, hi_shift);
            }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kHistBins; e += blockDim.x)
        if (h[e]) atomicAdd(&hist[e], h[e]);
}

__global__ void median_pairs_kernel(const float* __restrict__ X, int d,
                                    const int64_t* __restrict__ pi, const int64_t* __restrict__ pl,
                                    int64_t n_pairs, int shift, unsigned mask, unsigned prefix,
                                    int hi_shift, unsigned* __restrict__ hist) {
    __shared__ unsigned h[kHistBins];
    for (int e = threadIdx.x; e < kHistBins; e += blockDim.x) h[e] = 0u;
    __syncthreads();
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_pairs;
         p += (int64_t)gridDim.x * blockDim.x) {
        const float* a = X + pi[p] * d;
        const float* b = X + pl[p] * d;
        float D = 0.f;
        for (int k = 0; k < d; ++k) {
            const float t = a[k] - b[k];
            D = fmaf(t, t, D);
        }
        hist_add(h, D, shift, mask, prefix, hi_shift);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kHistBins; e += blockDim.x)
        if (h[e]) atomicAdd(&hist[e], h[e]);
}

int run_pair_median(kevd_ctx* ctx, const float* X, int64_t N, int d, const int64_t* pi,
                    const int64_t* pl, int64_t n_pairs, double* median, cudaStream_t s) {
    if (!X || !median || N < 2 || d < 1 || d > kCalMaxD || n_pairs < 0 ||
        (n_pairs > 0 && (!pi || !pl)))
        return set_error(ctx, KEVD_ERR_ARG, "pair_median: bad arguments");
    const bool exact = (n_pairs == 0);
    const int64_t nt = (N + kCalTile - 1) / kCalTile;
    const int64_t n_tiles = nt * (nt + 1) / 2;
    const uint64_t total = exact ? (uint64_t)N * (uint64_t)(N - 1) / 2 : (uint64_t)n_pairs;
    uint64_t rank = (total - 1) / 2;  // lower median
    int st = KEVD_OK;
    unsigned* hist = arena_get<unsigned>(ctx, "med.hist", kHistBins, &st);
    if (st != KEVD_OK) return st;
    const size_t smem = 2 * kPtTile * (size_t)kPtPitch * sizeof(float) + kHistBins * sizeof(unsigned);
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&median_tiles_kernel), (int)smem));
    const int shifts[3] = {20, 8, 0};
    const unsigned masks[3] = {0xfffu, 0xfffu, 0xffu};
    unsigned prefix = 0;
    int hi_shift = 32;
    std::vector<unsigned> hh(kHistBins);
    for (int pass = 0; pass < 3; ++pass) {
        KEVD_CUDA(ctx, cudaMemsetAsync(hist, 0, kHistBins * sizeof(unsigned), s));
        if (exact) {
            const int grid = (int)std::min<int64_t>(n_tiles, (int64_t)ctx->num_sms * 2);
            median_tiles_kernel<<<grid, 256, smem, s>>>(X, N, d, n_tiles, shifts[pass],
                                                        masks[pass], prefix, hi_shift, hist);
        } else {
            const int grid = (int)std::min<int64_t>((n_pairs + 255) / 256, (int64_t)ctx->num_sms * 4);
            median_pairs_kernel<<<grid, 256, 0, s>>>(X, d, pi, pl, n_pairs, shifts[pass],
                                                     masks[pass], prefix, hi_shift, hist);
        }
        KEVD_LAUNCH(ctx);
        KEVD_CUDA(ctx, cudaMemcpyAsync(hh.data(), hist, kHistBins * sizeof(unsigned),
                                       cudaMemcpyDeviceToHost, s));
        KEVD_CUDA(ctx, cudaStreamSynchronize(s));
        uint64_t cum = 0;
        int bin = -1;
        for (int b = 0; b <= (int)masks[pass]; ++b) {
            if (cum + hh[b] > rank) {
                bin = b;
                break;
            }
            cum += hh[b];
        }
        if (bin < 0) return set_error(ctx, KEVD_ERR_CUDA, "pair_median: histogram lost counts");
        rank -= cum;
        prefix = (hi_shift >= 32 ? 0u : (prefix << (hi_shift - shifts[pass]))) | (unsigned)bin;
        hi_shift = shifts[pass];
    }
    float m;
    unsigned bits = prefix;
    std::memcpy(&m, &bits, sizeof(float));
    *median = (double)m;
    return KEVD_OK;
}

}  // namespace kevd
