// Internal declarations shared by the kevd CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/kevd.h"

namespace kevd {

// Largest sample dimension d (features per state) the kernels accept; rows
// are staged in shared memory a fixed-width chunk of features at a time.
constexpr int kMaxFeatures = 1024;

constexpr int kNumSMs = 152;

// Status with a message stored in the context.
struct Error {
    int code;
    std::string msg;
};

// One named, growable device buffer per purpose.  Buffers are reused across
// calls and only grow; they are released with the context.
class Arena {
  public:
    ~Arena() { release(); }
    void* get(const std::string& name, size_t bytes, int* status);
    void release();
    size_t total() const {
        size_t t = 0;
        for (const auto& kv : bufs_) t += kv.second.n;
        return t;
    }

  private:
    struct Buf {
        void* p = nullptr;
        size_t n = 0;
    };
    std::map<std::string, Buf> bufs_;
};

}  // namespace kevd

struct kevd_ctx {
    int device = 0;
    int num_sms = kevd::kNumSMs;
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
    kevd::Arena arena;
    void* pinned = nullptr;  // small pinned host staging area
    size_t pinned_bytes = 0;
    std::string last_error;
    // profiling: CUDA events recorded on the launching stream around each
    // kernel (only while enabled) and a count of this library's launches
    bool prof = false;
    int64_t launches = 0;
    struct Rec {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    std::map<std::string, std::pair<double, int64_t>> prof_acc;
};

namespace kevd {

int set_error(kevd_ctx* ctx, int code, const char* fmt, ...);

#define KEVD_CUDA(ctx, call)                                                          \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return ::kevd::set_error((ctx), KEVD_ERR_CUDA, "%s:%d %s: %s", __FILE__,  \
                                     __LINE__, #call, cudaGetErrorString(e_));        \
    } while (0)

#define KEVD_LAUNCH(ctx)                                                              \
    do {                                                                              \
        ++(ctx)->launches;                                                            \
        cudaError_t e_ = cudaGetLastError();                                          \
        if (e_ != cudaSuccess)                                                        \
            return ::kevd::set_error((ctx), KEVD_ERR_CUDA, "%s:%d launch: %s",        \
                                     __FILE__, __LINE__, cudaGetErrorString(e_));     \
    } while (0)

#define KEVD_BLAS(ctx, call)                                                          \
    do {                                                                              \
        cublasStatus_t s_ = (call);                                                   \
        if (s_ != CUBLAS_STATUS_SUCCESS)                                              \
            return ::kevd::set_error((ctx), KEVD_ERR_CUDA, "%s:%d %s: cublas status %d", \
                                     __FILE__, __LINE__, #call, (int)s_);             \
    } while (0)

#define KEVD_SOLVER(ctx, call)                                                        \
    do {                                                                              \
        cusolverStatus_t s_ = (call);                                                 \
        if (s_ != CUSOLVER_STATUS_SUCCESS)                                            \
            return ::kevd::set_error((ctx), KEVD_ERR_CUDA, "%s:%d %s: cusolver status %d", \
                                     __FILE__, __LINE__, #call, (int)s_);             \
    } while (0)

#define KEVD_TRY(expr)                 \
    do {                               \
        int st_ = (expr);              \
        if (st_ != KEVD_OK) return st_; \
    } while (0)

// Times the kernels launched on stream s during its lifetime under name, and
// marks the same span as an NVTX range (for ncu --nvtx filters; a no-op when
// no tool is attached).
class ProfScope {
  public:
    ProfScope(kevd_ctx* ctx, const char* name, cudaStream_t s) : ctx_(ctx), name_(name), s_(s) {
        nvtxRangePushA(name);
        if (ctx_->prof) {
            a_ = take();
            if (a_) cudaEventRecord(a_, s_);
        }
    }
    ~ProfScope() {
        nvtxRangePop();
        if (!a_) return;
        cudaEvent_t b = take();
        if (!b) return;
        cudaEventRecord(b, s_);
        ctx_->pending.push_back({name_, a_, b});
    }

  private:
    cudaEvent_t take() {
        if (!ctx_->pool.empty()) {
            cudaEvent_t e = ctx_->pool.back();
            ctx_->pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return e;
    }
    kevd_ctx* ctx_;
    const char* name_;
    cudaStream_t s_;
    cudaEvent_t a_ = nullptr;
};

template <typename T>
T* arena_get(kevd_ctx* ctx, const char* name, size_t count, int* st) {
    return static_cast<T*>(ctx->arena.get(name, count * sizeof(T), st));
}

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// The kernel scale 1/(Nq eps) of an FP32 kernel evaluation as an FP32 pair
// hi + lo (hi = fl32(s)).  Rounding s to FP32 alone moves eps by up to 6e-8
// relative for every entry of K alike, which shifts the spectrum
// systematically; the pair keeps s to about 2^-48.
struct ScalePair {
    float hi, lo;
};
__host__ __device__ inline ScalePair split_scale(double s) {
    const float hi = (float)s;
    return {hi, (float)(s - (double)hi)};
}

// exp(-s x) in FP32 for a squared distance x >= 0 and s = hi + lo: with
// a = fl(hi x), the product's rounding error (exact, by fma) and lo x form
// a_lo, and e^{-(a + a_lo)} = e^{-a} (1 - a_lo) to first order (|a_lo| is
// below 2^-22 a, so the dropped term a_lo^2/2 is below 2^-44 a^2 of the
// value).  The entry then carries only the rounding of x and of expf.
__device__ __forceinline__ float kexp_scaled(float x, ScalePair s) {
    const float a = __fmul_rn(s.hi, x);
    const float a_lo = fmaf(s.lo, x, fmaf(s.hi, x, -a));
    const float e = expf(-a);
    return fmaf(-e, a_lo, e);
}

// ---- stage entry points implemented in the .cu files (C++ linkage) --------
int launch_hankel_rows(kevd_ctx* ctx, const float* u, int64_t Ndata, int64_t M, int64_t Nq,
                       float* X, cudaStream_t s);
int launch_kernel_block(kevd_ctx* ctx, const float* X, int64_t N, int d, double scale,
                        const int64_t* rows, int64_t row0, int64_t nrows, const int64_t* cols,
                        int64_t ncols, int precision, void* out, int64_t ld, cudaStream_t s,
                        const float* Xc = nullptr);
// Raise (never lower) a kernel's dynamic shared-memory limit.  The attribute
// belongs to the kernel, not to the calling thread: a call sized for a small
// problem must not cut the limit that another thread's larger launch of the
// same kernel relies on.
cudaError_t raise_smem_limit(const void* func, size_t bytes);

int run_rpchol_batched(kevd_ctx* ctx, kevd_rpchol_job* jobs, int n_jobs, int use_graph, cudaStream_t s);
int run_calibrate_batched(kevd_ctx* ctx, const kevd_calib_job* jobs, int n_jobs, int tiles_per_item,
                          cudaStream_t s);
int run_calibrate_fp64(kevd_ctx* ctx, const float* X, int64_t N, int d, const double* scales, int n_scales,
                       double* sums, cudaStream_t s);
int run_calibrate(kevd_ctx* ctx, const float* X, int64_t N, int d, const double* scales,
                  int n_scales, double* sums, cudaStream_t s);
int run_calibrate_noalloc(const float* X, int64_t N, int d, const double* scales, int n_scales, double* sums,
                          cudaStream_t s);
int run_pair_median(kevd_ctx* ctx, const float* X, int64_t N, int d, const int64_t* pi,
                    const int64_t* pl, int64_t n_pairs, double* median, cudaStream_t s);
int run_rpchol(kevd_ctx* ctx, const float* X, int64_t N, int d, double scale,
               const kevd_rpchol_params* p, void* F, int64_t ldF, int64_t* piv, double* err,
               int32_t* accepted, kevd_rpchol_result* res, cudaStream_t s);
int run_bistochastic_evd(kevd_ctx* ctx, const void* F, int precision, int64_t N, int64_t k,
                         int64_t ldF, int k_out, double* lam, float* U, kevd_evd_info* info,
                         kevd_evd_dump* dump, cudaStream_t s);
int run_weighted_gram(kevd_ctx* ctx, const void* F, int precision, int64_t N, int64_t k, int64_t ldF,
                      const double* s_dev, double* G, cudaStream_t st);
int run_ks_generate(kevd_ctx* ctx, int32_t n_traj, int32_t M, int32_t precision, const double* coef,
                    const double* g, const double* vhat0, int64_t n_warm, const int64_t* n_snap,
                    float* const* out, cudaStream_t s);
int run_weighted_gram2(kevd_ctx* ctx, const void* F, int precision, int64_t N, int64_t k, int64_t ldF,
                       const double* s_dev, const double* s2_dev, double* G, double* G2, cudaStream_t st);
int run_peak_rate(kevd_ctx* ctx, int kind, double* rate, double* ms, cudaStream_t s);
int run_gather_rows(kevd_ctx* ctx, const void* F, int precision, int64_t ldF, const int64_t* idx,
                    int64_t n, int64_t ncols, double* out, cudaStream_t s);

}  // namespace kevd
