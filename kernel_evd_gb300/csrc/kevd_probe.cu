// Issue-rate probes for the roofline denominators that no library call
// measures: the MUFU ex2 rate (the bound of the calibration pair sums), the
// FP32 FMA rate (the SIMT distance loops) and the FP64 FMA rate (the plain FP64
// form).  Each probe runs independent dependency chains, eight per thread,
// 2048 threads per SM, long enough (tens of milliseconds) for CUDA events to
// time it; the result is operations per second at whatever clock the GPU runs.
// A fourth probe measures packed FP32 FMAs (fma.rn.f32x2, counted as two).
#include "kevd_internal.cuh"

namespace kevd {

namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeCtasPerSm = 8;
constexpr int kChains = 8;
constexpr int kUnroll = 16;

__global__ void __launch_bounds__(kProbeThreads)
probe_ex2_kernel(float* __restrict__ out, int iters) {
    float x[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) x[j] = 0.25f + 1e-6f * (float)(threadIdx.x * kChains + j);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int j = 0; j < kChains; ++j) {
                // x <- 2^-x keeps x in [0.5, 1); the negation is an operand modifier
                float y;
                asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-x[j]));
                x[j] = y;
            }
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < kChains; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
__global__ void __launch_bounds__(kProbeThreads)
probe_fma_kernel(T* __restrict__ out, int iters, T a, T b) {
    T x[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) x[j] = (T)1 + (T)1e-6 * (T)(threadIdx.x * kChains + j);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int j = 0; j < kChains; ++j) x[j] = fma(x[j], a, b);   // converges to b / (1 - a)
    }
    T s = 0;
#pragma unroll
    for (int j = 0; j < kChains; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Packed FP32 pairs (fma.rn.f32x2): two FMAs per instruction.
__global__ void __launch_bounds__(kProbeThreads)
probe_fma2_kernel(float* __restrict__ out, int iters, float a, float b) {
    uint64_t x[kChains];
    const uint64_t av = ((uint64_t)__float_as_uint(a) << 32) | __float_as_uint(a);
    const uint64_t bv = ((uint64_t)__float_as_uint(b) << 32) | __float_as_uint(b);
#pragma unroll
    for (int j = 0; j < kChains; ++j) {
        const float v = 1.f + 1e-6f * (float)(threadIdx.x * kChains + j);
        x[j] = ((uint64_t)__float_as_uint(v) << 32) | __float_as_uint(v + 0.5f);
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int j = 0; j < kChains; ++j) asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[j]) : "l"(av), "l"(bv));
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < kChains; ++j) s += __uint_as_float((uint32_t)x[j]) + __uint_as_float((uint32_t)(x[j] >> 32));
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

int run_peak_rate(kevd_ctx* ctx, int kind, double* rate, double* ms_out, cudaStream_t s) {
    if (!rate || kind < 0 || kind > 3)
        return set_error(ctx, KEVD_ERR_ARG, "peak_rate: kind 0 (ex2), 1 (fp32 fma), 2 (fp64 fma), 3 (packed fp32 fma)");
    const int grid = ctx->num_sms * kProbeCtasPerSm;
    int st = KEVD_OK;
    double* out = arena_get<double>(ctx, "probe.out", (size_t)grid * kProbeThreads, &st);
    if (st != KEVD_OK) return st;
    // iterations per launch: a few tens of milliseconds at nominal rates
    const int iters = kind == 0 ? 4096 : kind == 1 ? 16384 : kind == 2 ? 512 : 16384;
    cudaEvent_t a = nullptr, b = nullptr;
    KEVD_CUDA(ctx, cudaEventCreate(&a));
    KEVD_CUDA(ctx, cudaEventCreate(&b));
    auto launch = [&]() -> int {
        if (kind == 0)
            probe_ex2_kernel<<<grid, kProbeThreads, 0, s>>>(reinterpret_cast<float*>(out), iters);
        else if (kind == 1)
            probe_fma_kernel<float><<<grid, kProbeThreads, 0, s>>>(reinterpret_cast<float*>(out), iters, 0.999f, 1e-3f);
        else if (kind == 2)
            probe_fma_kernel<double><<<grid, kProbeThreads, 0, s>>>(out, iters, 0.999, 1e-3);
        else
            probe_fma2_kernel<<<grid, kProbeThreads, 0, s>>>(reinterpret_cast<float*>(out), iters, 0.999f, 1e-3f);
        KEVD_LAUNCH(ctx);
        return KEVD_OK;
    };
    int rc = launch();   // warm-up (clocks ramp, module load)
    float best = 0.f;
    for (int rep = 0; rep < 3 && rc == KEVD_OK; ++rep) {
        cudaEventRecord(a, s);
        rc = launch();
        cudaEventRecord(b, s);
        if (rc == KEVD_OK && cudaEventSynchronize(b) == cudaSuccess) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (best == 0.f || ms < best) best = ms;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc != KEVD_OK) return rc;
    if (!(best > 0.f)) return set_error(ctx, KEVD_ERR_CUDA, "peak_rate: timing failed");
    const double ops = (double)grid * kProbeThreads * kChains * kUnroll * (double)iters * (kind == 3 ? 2.0 : 1.0);
    *rate = ops / (best * 1e-3);
    if (ms_out) *ms_out = best;
    return KEVD_OK;
}

}  // namespace kevd
