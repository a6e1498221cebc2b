// The extern "C" boundary (include/kevd.h): argument checks, context and
// workspace management, and the host orchestration that is not a kernel.
#include "kevd_internal.cuh"

#include <map>
#include <mutex>

#include <algorithm>
#include <cmath>
#include <iterator>
#include <cstdarg>
#include <cstring>
#include <vector>

namespace kevd {

int set_error(kevd_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return code;
}

void* Arena::get(const std::string& name, size_t bytes, int* status) {
    if (*status != KEVD_OK) return nullptr;
    Buf& b = bufs_[name];
    if (bytes == 0) bytes = 1;
    if (b.n >= bytes) return b.p;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    // round up to 2 MiB to limit regrowth
    const size_t want = (bytes + (2u << 20) - 1) & ~(size_t)((2u << 20) - 1);
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        *status = KEVD_ERR_NOMEM;
        return nullptr;
    }
    b.n = want;
    return b.p;
}

cudaError_t raise_smem_limit(const void* func, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> limit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = limit[{dev, func}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

void Arena::release() {
    for (auto& kv : bufs_)
        if (kv.second.p) cudaFree(kv.second.p);
    bufs_.clear();
}

// Nystrom model: landmark rows, Z' = L^{-T} Z and p1' = L^{-T} c1 packed as
// the r x (k_out + 1) column-major matrix [Z' | p1'].
struct Model {
    int64_t r = 0;
    int d = 0;
    int k_out = 0;
    double scale = 0.0;
    float* xs = nullptr;   // r x d
    double* zp = nullptr;  // r x (k_out + 1), column-major
};

}  // namespace kevd

struct kevd_model {
    kevd::Model m;
};

using namespace kevd;

#define KEVD_CHECK_CTX(ctx) \
    if (!(ctx)) return KEVD_ERR_ARG

static void resolve_profile(kevd_ctx* ctx) {
    for (auto& r : ctx->pending) {
        float ms = 0.f;
        cudaEventSynchronize(r.b);
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            auto& acc = ctx->prof_acc[r.name];
            acc.first += ms;
            acc.second += 1;
        } else {
            cudaGetLastError();
        }
        ctx->pool.push_back(r.a);
        ctx->pool.push_back(r.b);
    }
    ctx->pending.clear();
}


extern "C" {

int kevd_abi_version(void) { return 1; }

const char* kevd_status_name(int status) {
    switch (status) {
        case KEVD_OK: return "KEVD_OK";
        case KEVD_ERR_ARG: return "KEVD_ERR_ARG";
        case KEVD_ERR_CUDA: return "KEVD_ERR_CUDA";
        case KEVD_ERR_NONPOS_DTIL: return "KEVD_ERR_NONPOS_DTIL";
        case KEVD_ERR_POTRF: return "KEVD_ERR_POTRF";
        case KEVD_ERR_NONPOS_QTIL: return "KEVD_ERR_NONPOS_QTIL";
        case KEVD_ERR_SYEVD: return "KEVD_ERR_SYEVD";
        case KEVD_ERR_NOMEM: return "KEVD_ERR_NOMEM";
        case KEVD_ERR_TIMEOUT: return "KEVD_ERR_TIMEOUT";
        default: return "KEVD_ERR_UNKNOWN";
    }
}

int kevd_ctx_create(int device, kevd_ctx** out) {
    if (!out) return KEVD_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return KEVD_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return KEVD_ERR_CUDA;
    kevd_ctx* ctx = new kevd_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cublasCreate(&ctx->blas) != CUBLAS_STATUS_SUCCESS ||
        cusolverDnCreate(&ctx->solver) != CUSOLVER_STATUS_SUCCESS ||
        cudaMallocHost(&ctx->pinned, 4096) != cudaSuccess) {
        kevd_ctx_destroy(ctx);
        return KEVD_ERR_CUDA;
    }
    ctx->pinned_bytes = 4096;
    *out = ctx;
    return KEVD_OK;
}

void kevd_ctx_destroy(kevd_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    resolve_profile(ctx);
    for (cudaEvent_t e : ctx->pool) cudaEventDestroy(e);
    ctx->arena.release();
    if (ctx->blas) cublasDestroy(ctx->blas);
    if (ctx->solver) cusolverDnDestroy(ctx->solver);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    delete ctx;
}

const char* kevd_last_error(const kevd_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int kevd_profile_enable(kevd_ctx* ctx, int on) {
    KEVD_CHECK_CTX(ctx);
    resolve_profile(ctx);
    ctx->prof_acc.clear();
    ctx->prof = on != 0;
    return KEVD_OK;
}

int kevd_profile_read(kevd_ctx* ctx, int idx, char* name, int name_len, double* total_ms,
                      int64_t* count) {
    KEVD_CHECK_CTX(ctx);
    resolve_profile(ctx);
    if (idx < 0 || idx >= (int)ctx->prof_acc.size()) return KEVD_ERR_ARG;
    auto it = ctx->prof_acc.begin();
    std::advance(it, idx);
    if (name && name_len > 0) {
        std::strncpy(name, it->first.c_str(), name_len - 1);
        name[name_len - 1] = 0;
    }
    if (total_ms) *total_ms = it->second.first;
    if (count) *count = it->second.second;
    return KEVD_OK;
}

int64_t kevd_launch_count(const kevd_ctx* ctx) { return ctx ? ctx->launches : 0; }

int kevd_peak_rate(kevd_ctx* ctx, int32_t kind, double* ops_per_s, double* ms, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_peak_rate(ctx, kind, ops_per_s, ms, as_stream(stream));
}

int kevd_hankel_rows(kevd_ctx* ctx, const float* u, int64_t Ndata, int64_t M, int64_t Nq, float* X,
                     void* stream) {
    KEVD_CHECK_CTX(ctx);
    return launch_hankel_rows(ctx, u, Ndata, M, Nq, X, as_stream(stream));
}

int kevd_kernel_block(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, double scale,
                      const int64_t* rows, int64_t row0, int64_t nrows, const int64_t* cols,
                      int64_t ncols, int32_t precision, void* out, int64_t ld, void* stream) {
    KEVD_CHECK_CTX(ctx);
    if (!cols) return set_error(ctx, KEVD_ERR_ARG, "kernel_block: cols is required");
    if (precision != KEVD_FP64 && precision != KEVD_MIXED)
        return set_error(ctx, KEVD_ERR_ARG, "kernel_block: unknown precision");
    return launch_kernel_block(ctx, X, N, d, scale, rows, row0, nrows, cols, ncols, precision, out,
                               ld, as_stream(stream));
}

int kevd_calibrate(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, const double* scales,
                   int32_t n_scales, double* sums, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_calibrate(ctx, X, N, d, scales, n_scales, sums, as_stream(stream));
}

int kevd_calibrate_batched(kevd_ctx* ctx, const kevd_calib_job* jobs, int32_t n_jobs, int32_t tiles_per_item,
                           void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_calibrate_batched(ctx, jobs, n_jobs, tiles_per_item, as_stream(stream));
}

int kevd_calibrate_fp64(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, const double* scales,
                        int32_t n_scales, double* sums, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_calibrate_fp64(ctx, X, N, d, scales, n_scales, sums, as_stream(stream));
}

int kevd_calibrate_noalloc(const float* X, int64_t N, int32_t d, const double* scales, int32_t n_scales,
                           double* sums, void* stream) {
    return run_calibrate_noalloc(X, N, d, scales, n_scales, sums, as_stream(stream));
}

int kevd_calibrate_select(const double* bw, const double* sums, int32_t n, int64_t NM,
                          double* logS, double* slope, int32_t* idmax, double* eopt,
                          double* mdim) {
    if (!bw || !sums || n < 3 || NM < 1 || !logS || !slope || !idmax || !eopt || !mdim)
        return KEVD_ERR_ARG;
    for (int i = 0; i < n; ++i) logS[i] = std::log(2.0 * sums[i] / (double)NM + 1.0);
    for (int i = 1; i < n - 1; ++i)
        slope[i - 1] = (logS[i + 1] - logS[i - 1]) / (std::log(bw[i + 1]) - std::log(bw[i - 1]));
    int im = 0;
    for (int i = 1; i < n - 2; ++i)
        if (slope[i] > slope[im]) im = i;
    *idmax = im;
    *eopt = bw[im + 1];
    *mdim = 2.0 * slope[im];
    return KEVD_OK;
}

int kevd_pair_median(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, const int64_t* pi,
                     const int64_t* pl, int64_t n_pairs, double* median, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_pair_median(ctx, X, N, d, pi, pl, n_pairs, median, as_stream(stream));
}

int kevd_rpchol(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, double scale,
                const kevd_rpchol_params* params, void* F, int64_t ldF, int64_t* piv, double* err,
                int32_t* accepted, kevd_rpchol_result* result, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_rpchol(ctx, X, N, d, scale, params, F, ldF, piv, err, accepted, result,
                      as_stream(stream));
}

int kevd_rpchol_batched(kevd_ctx* ctx, kevd_rpchol_job* jobs, int32_t n_jobs, int32_t use_graph, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_rpchol_batched(ctx, jobs, n_jobs, use_graph, as_stream(stream));
}

int kevd_linv_from_factor(kevd_ctx* ctx, const void* F, int32_t precision, int64_t ldF,
                          const int64_t* piv, int64_t r, double* Linv, void* stream) {
    KEVD_CHECK_CTX(ctx);
    if (!F || !piv || !Linv || r < 1 || ldF < r || (precision != KEVD_FP64 && precision != KEVD_MIXED))
        return set_error(ctx, KEVD_ERR_ARG, "linv_from_factor: bad arguments");
    cudaStream_t s = as_stream(stream);
    int st = KEVD_OK;
    int64_t* idx = arena_get<int64_t>(ctx, "li.idx", r, &st);
    double* L = arena_get<double>(ctx, "li.L", (size_t)r * r, &st);
    double* I = arena_get<double>(ctx, "li.I", (size_t)r * r, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "linv_from_factor: out of device memory");
    KEVD_CUDA(ctx, cudaMemcpyAsync(idx, piv, r * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    KEVD_TRY(run_gather_rows(ctx, F, precision, ldF, idx, r, r, L, s));
    std::vector<double> eye((size_t)r * r, 0.0);
    for (int64_t i = 0; i < r; ++i) eye[(size_t)i * r + i] = 1.0;
    KEVD_CUDA(ctx, cudaMemcpyAsync(I, eye.data(), eye.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    KEVD_BLAS(ctx, cublasSetStream(ctx->blas, s));
    const double one = 1.0;
    KEVD_BLAS(ctx, cublasDtrsm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                               CUBLAS_DIAG_NON_UNIT, (int)r, (int)r, &one, L, (int)r, I, (int)r));
    KEVD_CUDA(ctx, cudaMemcpyAsync(Linv, I, (size_t)r * r * sizeof(double), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    for (int64_t c = 0; c < r; ++c)
        for (int64_t q = 0; q < c; ++q) Linv[(size_t)c * r + q] = 0.0;  // strict upper
    return KEVD_OK;
}

int kevd_bistochastic_evd(kevd_ctx* ctx, const void* F, int32_t precision, int64_t N, int64_t k,
                          int64_t ldF, int32_t k_out, double* lam, float* U, kevd_evd_info* info,
                          kevd_evd_dump* dump, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_bistochastic_evd(ctx, F, precision, N, k, ldF, k_out, lam, U, info, dump,
                                as_stream(stream));
}

int kevd_weighted_gram(kevd_ctx* ctx, const void* F, int32_t precision, int64_t N, int64_t k, int64_t ldF,
                       const double* s, double* G, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_weighted_gram(ctx, F, precision, N, k, ldF, s, G, as_stream(stream));
}

int kevd_ks_generate(kevd_ctx* ctx, int32_t n_traj, int32_t M, int32_t precision, const double* coef,
                     const double* g, const double* vhat0, int64_t n_warm, const int64_t* n_snap, float* const* out,
                     void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_ks_generate(ctx, n_traj, M, precision, coef, g, vhat0, n_warm, n_snap, out, as_stream(stream));
}

int kevd_weighted_gram2(kevd_ctx* ctx, const void* F, int32_t precision, int64_t N, int64_t k, int64_t ldF,
                        const double* s, const double* s2, double* G, double* G2, void* stream) {
    KEVD_CHECK_CTX(ctx);
    return run_weighted_gram2(ctx, F, precision, N, k, ldF, s, s2, G, G2, as_stream(stream));
}

__global__ void cast_d2f_kernel(const double* __restrict__ a, int64_t rows, int64_t cols,
                                int64_t lda, float* __restrict__ b, int64_t ldb) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / cols, c = e - i * cols;
        b[i * ldb + c] = (float)a[i * lda + c];
    }
}

int kevd_factor_from_linv(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, double scale,
                          const int64_t* piv, int64_t r, const double* Linv, int32_t precision,
                          void* F, int64_t ldF, void* stream) {
    KEVD_CHECK_CTX(ctx);
    if (!X || !piv || !Linv || !F || N < 1 || r < 1 || ldF < r ||
        (precision != KEVD_FP64 && precision != KEVD_MIXED))
        return set_error(ctx, KEVD_ERR_ARG, "factor_from_linv: bad arguments");
    cudaStream_t s = as_stream(stream);
    // panels of rows sized to ~256 MiB of FP64
    int64_t rows = std::max<int64_t>(1, (256ll << 20) / (r * 8));
    rows = std::min(rows, N);
    int st = KEVD_OK;
    int64_t* idx = arena_get<int64_t>(ctx, "fl.idx", r, &st);
    double* Li = arena_get<double>(ctx, "fl.Linv", (size_t)r * r, &st);
    double* Kp = arena_get<double>(ctx, "fl.K", (size_t)rows * r, &st);
    double* Fp = precision == KEVD_MIXED ? arena_get<double>(ctx, "fl.F", (size_t)rows * r, &st) : nullptr;
    if (st != KEVD_OK) return set_error(ctx, st, "factor_from_linv: out of device memory");
    KEVD_CUDA(ctx, cudaMemcpyAsync(idx, piv, r * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(Li, Linv, (size_t)r * r * sizeof(double), cudaMemcpyHostToDevice, s));
    KEVD_BLAS(ctx, cublasSetStream(ctx->blas, s));
    const double one = 1.0;
    for (int64_t r0 = 0; r0 < N; r0 += rows) {
        const int64_t nr = std::min(rows, N - r0);
        KEVD_TRY(launch_kernel_block(ctx, X, N, d, scale, nullptr, r0, nr, idx, r, KEVD_FP64, Kp, r, s));
        // (F panel)^T = Linv * (K panel)^T  in column-major terms; Linv is lower
        // triangular (its upper part is never read), half the FP64 work of a GEMM
        double* dst = precision == KEVD_FP64 ? (double*)F + r0 * ldF : Fp;
        const int64_t ldd = precision == KEVD_FP64 ? ldF : r;
        KEVD_BLAS(ctx, cublasDtrmm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                                   CUBLAS_DIAG_NON_UNIT, (int)r, (int)nr, &one, Li, (int)r, Kp, (int)r, dst,
                                   (int)ldd));
        if (precision == KEVD_MIXED) {
            const int grid = (int)std::min<int64_t>((nr * r + 255) / 256, (int64_t)ctx->num_sms * 16);
            cast_d2f_kernel<<<grid, 256, 0, s>>>(Fp, nr, r, r, (float*)F + r0 * ldF, ldF);
            KEVD_LAUNCH(ctx);
        }
    }
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    return KEVD_OK;
}

int kevd_factor_from_pivots(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, double scale,
                            const int64_t* piv, int64_t r, int32_t precision, void* F, int64_t ldF,
                            void* stream) {
    KEVD_CHECK_CTX(ctx);
    if (!X || !piv || !F || N < 1 || r < 1 || r > N || ldF < r ||
        (precision != KEVD_FP64 && precision != KEVD_MIXED))
        return set_error(ctx, KEVD_ERR_ARG, "factor_from_pivots: bad arguments");
    cudaStream_t s = as_stream(stream);
    int64_t rows = std::max<int64_t>(1, (256ll << 20) / (r * 8));
    rows = std::min(rows, N);
    int st = KEVD_OK;
    int64_t* idx = arena_get<int64_t>(ctx, "fp.idx", r, &st);
    double* L = arena_get<double>(ctx, "fp.L", (size_t)r * r, &st);
    double* Kp = arena_get<double>(ctx, "fp.K", (size_t)rows * r, &st);
    int* info = arena_get<int>(ctx, "fp.info", 1, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "factor_from_pivots: out of device memory");
    KEVD_CUDA(ctx, cudaMemcpyAsync(idx, piv, r * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    // L L^T = K(S, S): row-major K(S,S) is its own column-major transpose (symmetric)
    KEVD_TRY(launch_kernel_block(ctx, X, N, d, scale, idx, 0, r, idx, r, KEVD_FP64, L, r, s));
    KEVD_SOLVER(ctx, cusolverDnSetStream(ctx->solver, s));
    KEVD_BLAS(ctx, cublasSetStream(ctx->blas, s));
    int lwork = 0;
    KEVD_SOLVER(ctx, cusolverDnDpotrf_bufferSize(ctx->solver, CUBLAS_FILL_MODE_LOWER, (int)r, L, (int)r, &lwork));
    double* work = arena_get<double>(ctx, "fp.work", (size_t)lwork + 1, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "factor_from_pivots: out of device memory");
    KEVD_SOLVER(ctx, cusolverDnDpotrf(ctx->solver, CUBLAS_FILL_MODE_LOWER, (int)r, L, (int)r, work, lwork, info));
    int hinfo = 0;
    KEVD_CUDA(ctx, cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    if (hinfo != 0) return set_error(ctx, KEVD_ERR_POTRF, "factor_from_pivots: K(S,S) not positive definite (%d)", hinfo);
    const double one = 1.0;
    for (int64_t r0 = 0; r0 < N; r0 += rows) {
        const int64_t nr = std::min(rows, N - r0);
        KEVD_TRY(launch_kernel_block(ctx, X, N, d, scale, nullptr, r0, nr, idx, r, KEVD_FP64, Kp, r, s));
        // (F panel)^T solves L Y = K(R,S)^T (column-major r x nr)
        KEVD_BLAS(ctx, cublasDtrsm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                                   CUBLAS_DIAG_NON_UNIT, (int)r, (int)nr, &one, L, (int)r, Kp, (int)r));
        if (precision == KEVD_FP64) {
            KEVD_CUDA(ctx, cudaMemcpy2DAsync((double*)F + r0 * ldF, ldF * sizeof(double), Kp, r * sizeof(double),
                                             r * sizeof(double), nr, cudaMemcpyDeviceToDevice, s));
        } else {
            const int grid = (int)std::min<int64_t>((nr * r + 255) / 256, (int64_t)ctx->num_sms * 16);
            cast_d2f_kernel<<<grid, 256, 0, s>>>(Kp, nr, r, r, (float*)F + r0 * ldF, ldF);
            KEVD_LAUNCH(ctx);
        }
    }
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    return KEVD_OK;
}

__global__ void landmark_gather_kernel(const float* __restrict__ X, const int64_t* __restrict__ idx, int64_t r, int d,
                                       float* __restrict__ xs) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < r * d; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = e / d;
        xs[e] = X[idx[q] * d + (e - q * d)];
    }
}

int kevd_nystrom_prepare(kevd_ctx* ctx, const float* X, int64_t N, int32_t d, double scale,
                         const void* F, int32_t precision, int64_t ldF, const int64_t* piv,
                         int64_t r, int32_t k_out, kevd_model** model, void* stream) {
    KEVD_CHECK_CTX(ctx);
    if (!X || !F || !piv || !model || r < 1 || k_out < 1 || k_out > 64 || k_out > r)
        return set_error(ctx, KEVD_ERR_ARG, "nystrom_prepare: bad arguments");
    cudaStream_t s = as_stream(stream);
    std::vector<double> c1(r), Z((size_t)r * k_out), lam(r);
    kevd_evd_dump dump;
    std::memset(&dump, 0, sizeof(dump));
    dump.c1 = c1.data();
    dump.Z = Z.data();
    int st = KEVD_OK;
    float* U = arena_get<float>(ctx, "ny.U", (size_t)N * k_out, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "nystrom_prepare: out of device memory");
    KEVD_TRY(run_bistochastic_evd(ctx, F, precision, N, r, ldF, k_out, lam.data(), U, nullptr, &dump, s));
    // L = F(S, :) on the device; [Z' | p1'] = L^{-T} [Z | c1]
    int64_t* idx = arena_get<int64_t>(ctx, "ny.idx", r, &st);
    double* L = arena_get<double>(ctx, "ny.L", (size_t)r * r, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "nystrom_prepare: out of device memory");
    kevd_model* m = new kevd_model();
    m->m.r = r;
    m->m.d = d;
    m->m.k_out = k_out;
    m->m.scale = scale;
    if (cudaMalloc(&m->m.xs, (size_t)r * d * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->m.zp, (size_t)r * (k_out + 1) * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        kevd_model_destroy(m);
        return set_error(ctx, KEVD_ERR_NOMEM, "nystrom_prepare: out of device memory");
    }
    std::vector<double> zp((size_t)r * (k_out + 1));
    std::memcpy(zp.data(), Z.data(), Z.size() * sizeof(double));
    std::memcpy(zp.data() + (size_t)r * k_out, c1.data(), r * sizeof(double));
    int rc = KEVD_OK;
    do {
        if (cudaMemcpyAsync(idx, piv, r * sizeof(int64_t), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(m->m.zp, zp.data(), zp.size() * sizeof(double), cudaMemcpyHostToDevice, s) !=
                cudaSuccess) {
            rc = set_error(ctx, KEVD_ERR_CUDA, "nystrom_prepare: copy failed");
            break;
        }
        rc = run_gather_rows(ctx, F, precision, ldF, idx, r, r, L, s);
        if (rc != KEVD_OK) break;
        const double one = 1.0;
        if (cublasSetStream(ctx->blas, s) != CUBLAS_STATUS_SUCCESS ||
            cublasDtrsm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                        CUBLAS_DIAG_NON_UNIT, (int)r, k_out + 1, &one, L, (int)r, m->m.zp,
                        (int)r) != CUBLAS_STATUS_SUCCESS) {
            rc = set_error(ctx, KEVD_ERR_CUDA, "nystrom_prepare: trsm failed");
            break;
        }
        // landmark rows X[piv]
        landmark_gather_kernel<<<(unsigned)std::min<int64_t>((r * d + 255) / 256, (int64_t)ctx->num_sms * 8), 256, 0,
                                 s>>>(X, idx, r, d, m->m.xs);
        ++ctx->launches;
        if (cudaGetLastError() != cudaSuccess) {
            rc = set_error(ctx, KEVD_ERR_CUDA, "nystrom_prepare: landmark gather failed");
            break;
        }
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = set_error(ctx, KEVD_ERR_CUDA, "nystrom_prepare: sync");
    } while (0);
    if (rc != KEVD_OK) {
        kevd_model_destroy(m);
        return rc;
    }
    *model = m;
    return KEVD_OK;
}

// Fused out-of-sample evaluation.  One CTA serves 32 query rows: for each
// chunk of 32 landmarks it forms K(y, s_j) from FP32 direct differences summed
// over the feature index in increasing order and an FP32 exp (relative error
// about 1e-7 in K, far below the FP32 output's), and accumulates
// P[row][c] = sum_j K(y, s_j) [Z'|p1'][j][c] in FP64 with j ascending in one
// register per output: [Z'|p1'] = L^{-T}[Z|c1] has large entries of both
// signs, so the sum stays FP64.  No thread ever combines two query rows, so a
// row's result is bit-identical whatever batch it is evaluated in and wherever
// it sits in the batch.
constexpr int kNyRows = 32;
constexpr int kNyLm = 32;
constexpr int kNyMaxOut = 9;   // ceil(32 * 65 / 256) outputs per thread
constexpr int kNyFeat = 128;   // features staged at a time

__global__ void __launch_bounds__(256) nystrom_eval_kernel(const float* __restrict__ Y, int64_t n,
                                                           const float* __restrict__ xs, const double* __restrict__ zp,
                                                           int64_t r, int d, int k_out, double scale,
                                                           float* __restrict__ Uy) {
    extern __shared__ __align__(16) unsigned char ny_smem[];
    constexpr int dp = kNyFeat + 1;
    const int kc = k_out + 1;
    double* kv = reinterpret_cast<double*>(ny_smem);     // 32 x 33
    double* zc = kv + kNyRows * (kNyLm + 1);             // 32 landmarks x kc
    float* ys = reinterpret_cast<float*>(zc + kNyLm * kc);  // 32 x dp (one feature chunk)
    float* xc = ys + kNyRows * dp;                       // 32 x dp
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const ScalePair fscale = split_scale(scale);
    const int64_t row0 = (int64_t)blockIdx.x * kNyRows;
    // with one feature chunk the query rows are staged once for all landmarks
    const bool one_chunk = d <= kNyFeat;
    if (one_chunk)
        for (int e = threadIdx.x; e < kNyRows * d; e += 256) {
            const int rr = e / d, kk = e - rr * d;
            ys[rr * dp + kk] = (row0 + rr < n) ? Y[(row0 + rr) * d + kk] : 0.f;
        }
    double acc[kNyMaxOut];
#pragma unroll
    for (int q = 0; q < kNyMaxOut; ++q) acc[q] = 0.0;
    const int n_out = kNyRows * kc;
    for (int64_t j0 = 0; j0 < r; j0 += kNyLm) {
        __syncthreads();
        for (int e = threadIdx.x; e < kNyLm * kc; e += 256) {
            const int jj = e / kc, c = e - jj * kc;
            zc[jj * kc + c] = (j0 + jj < r) ? zp[(int64_t)c * r + j0 + jj] : 0.0;
        }
        // K(row ty + 8i, landmark tx): features kNyFeat at a time, in increasing order
        float dist[4] = {0.f, 0.f, 0.f, 0.f};
        for (int f0 = 0; f0 < d; f0 += kNyFeat) {
            const int w = min(kNyFeat, d - f0);
            __syncthreads();
            if (!one_chunk)
                for (int e = threadIdx.x; e < kNyRows * w; e += 256) {
                    const int rr = e / w, kk = e - rr * w;
                    ys[rr * dp + kk] = (row0 + rr < n) ? Y[(row0 + rr) * d + f0 + kk] : 0.f;
                }
            for (int e = threadIdx.x; e < kNyLm * w; e += 256) {
                const int jj = e / w, kk = e - jj * w;
                xc[jj * dp + kk] = (j0 + jj < r) ? xs[(j0 + jj) * d + f0 + kk] : 0.f;
            }
            __syncthreads();
            for (int kk = 0; kk < w; ++kk) {
                const float c = xc[tx * dp + kk];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float t = ys[(ty + 8 * i) * dp + kk] - c;
                    dist[i] = fmaf(t, t, dist[i]);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
            kv[(ty + 8 * i) * (kNyLm + 1) + tx] = (j0 + tx < r) ? (double)kexp_scaled(dist[i], fscale) : 0.0;
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kNyMaxOut; ++q) {
            const int o = threadIdx.x + 256 * q;
            if (o < n_out) {
                const int rr = o / kc, c = o - rr * kc;
                double a = acc[q];
#pragma unroll 8
                for (int jj = 0; jj < kNyLm; ++jj) a += kv[rr * (kNyLm + 1) + jj] * zc[jj * kc + c];
                acc[q] = a;
            }
        }
    }
    __syncthreads();
    double* P = kv;   // reuse: 32 x kc doubles fit in kv + zc
#pragma unroll
    for (int q = 0; q < kNyMaxOut; ++q) {
        const int o = threadIdx.x + 256 * q;
        if (o < n_out) P[o] = acc[q];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kNyRows * k_out; e += 256) {
        const int rr = e / k_out, c = e - rr * k_out;
        if (row0 + rr < n) Uy[(row0 + rr) * k_out + c] = (float)(P[rr * kc + c] / P[rr * kc + k_out]);
    }
}

static size_t nystrom_smem(int d, int k_out) {
    (void)d;
    return (size_t)kNyRows * (kNyLm + 1) * 8 + (size_t)kNyLm * (k_out + 1) * 8 + 2 * (size_t)kNyRows * (kNyFeat + 1) * 4;
}

int kevd_nystrom_eval(kevd_ctx* ctx, const kevd_model* model, const float* Y, int64_t n, float* Uy,
                      void* stream) {
    KEVD_CHECK_CTX(ctx);
    if (!model || !Y || !Uy || n < 0) return set_error(ctx, KEVD_ERR_ARG, "nystrom_eval: bad arguments");
    if (n == 0) return KEVD_OK;
    const Model& m = model->m;
    const int64_t n_blocks = (n + kNyRows - 1) / kNyRows;
    const size_t smem = nystrom_smem(m.d, m.k_out);
    if (smem > 227 * 1024 || n_blocks > (int64_t)INT32_MAX)
        return set_error(ctx, KEVD_ERR_ARG, "nystrom_eval: unsupported size (d=%d, n=%lld)", m.d, (long long)n);
    cudaStream_t s = as_stream(stream);
    if (smem > 48 * 1024)
        KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&nystrom_eval_kernel), (int)smem));
    nystrom_eval_kernel<<<(unsigned)n_blocks, 256, smem, s>>>(Y, n, m.xs, m.zp, m.r, m.d, m.k_out,
                                                                         m.scale, Uy);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

void kevd_model_destroy(kevd_model* model) {
    if (!model) return;
    if (model->m.xs) cudaFree(model->m.xs);
    if (model->m.zp) cudaFree(model->m.zp);
    delete model;
}

}  // extern "C"
