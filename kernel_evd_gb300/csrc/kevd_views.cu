// Sample views and generic kernel-block evaluation.
//
//  * hankel_rows: materialise the reference's delay-embedded samples as a
//    row-major matrix once, so every later kernel streams plain rows with
//    coalesced loads (ks_arpclm.cu:263-268 is the index map).
//  * kernel_block<T>: K(rows, cols) in T, from direct differences
//    (ks_arpclm.cu:242-280, ks_kevd.cu:302-340).  Both row and column samples
//    are staged through shared memory, one 32 x 32 tile per CTA.
#include "kevd_internal.cuh"

namespace kevd {

__global__ void hankel_rows_kernel(const float* __restrict__ u, int64_t Ndata, int64_t N,
                                   int64_t NM, int64_t Nq, float* __restrict__ X) {
    const int64_t total = NM * Nq;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx / Nq;
        const int64_t k = idx - i * Nq;
        X[idx] = u[(i / N) * Ndata + (i % N) + k];
    }
}

int launch_hankel_rows(kevd_ctx* ctx, const float* u, int64_t Ndata, int64_t M, int64_t Nq,
                       float* X, cudaStream_t s) {
    if (!u || !X || Ndata < 1 || M < 1 || Nq < 1 || Nq > Ndata)
        return set_error(ctx, KEVD_ERR_ARG, "hankel_rows: bad sizes Ndata=%lld M=%lld Nq=%lld",
                         (long long)Ndata, (long long)M, (long long)Nq);
    const int64_t N = Ndata - Nq + 1;
    const int64_t NM = N * M;
    int grid = (int)std::min<int64_t>((NM * Nq + 255) / 256, (int64_t)ctx->num_sms * 32);
    hankel_rows_kernel<<<grid, 256, 0, s>>>(u, Ndata, N, NM, Nq, X);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

constexpr int kBlkFeat = 128;   // features staged at a time

// One CTA computes a 32 x 32 tile; thread (tx, ty) computes rows ty + 8j.
template <typename T>
__global__ void __launch_bounds__(256) kernel_block_kernel(
    const float* __restrict__ Xr, const float* __restrict__ Xc, int d, double scale,
    const int64_t* __restrict__ rows, int64_t row0, int64_t nrows,
    const int64_t* __restrict__ cols, int64_t ncols, T* __restrict__ out, int64_t ld) {
    extern __shared__ float sm[];
    constexpr int dp = kBlkFeat + 1;
    float* xr = sm;             // 32 x dp
    float* xc = sm + 32 * dp;   // 32 x dp
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tx;
    const int64_t r_base = (int64_t)blockIdx.y * 32;
    const int64_t c_base = (int64_t)blockIdx.x * 32;
    T acc[4] = {0, 0, 0, 0};
    // features kBlkFeat at a time, summed in increasing order
    for (int c0 = 0; c0 < d; c0 += kBlkFeat) {
        const int w = min(kBlkFeat, d - c0);
        __syncthreads();
        for (int e = tid; e < 32 * w; e += 256) {
            const int rr = e / w, kk = e - rr * w;
            const int64_t r = r_base + rr;
            const int64_t c = c_base + rr;
            float vr = 0.f, vc = 0.f;
            if (r < nrows) vr = Xr[(rows ? rows[r] : row0 + r) * d + c0 + kk];
            if (c < ncols) vc = Xc[(cols ? cols[c] : c) * d + c0 + kk];
            xr[rr * dp + kk] = vr;
            xc[rr * dp + kk] = vc;
        }
        __syncthreads();
        for (int kk = 0; kk < w; ++kk) {
            const T c = (T)xc[tx * dp + kk];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T t = (T)xr[(ty + 8 * j) * dp + kk] - c;
                acc[j] += t * t;
            }
        }
    }
    const int64_t c = c_base + tx;
    if (c >= ncols) return;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int64_t r = r_base + ty + 8 * j;
        if (r < nrows) {
            if constexpr (sizeof(T) == 8)
                out[r * ld + c] = exp(-scale * (double)acc[j]);
            else
                out[r * ld + c] = kexp_scaled((float)acc[j], split_scale(scale));
        }
    }
}

int launch_kernel_block(kevd_ctx* ctx, const float* X, int64_t N, int d, double scale,
                        const int64_t* rows, int64_t row0, int64_t nrows, const int64_t* cols,
                        int64_t ncols, int precision, void* out, int64_t ld, cudaStream_t s,
                        const float* Xc) {
    if (!Xc) Xc = X;
    if (!X || !out || d < 1 || d > kMaxFeatures || nrows < 0 || ncols < 0 || ld < ncols)
        return set_error(ctx, KEVD_ERR_ARG, "kernel_block: bad arguments");
    if (!rows && (row0 < 0 || row0 + nrows > N))
        return set_error(ctx, KEVD_ERR_ARG, "kernel_block: row range outside [0, N)");
    if (nrows == 0 || ncols == 0) return KEVD_OK;
    dim3 grid(ceil_div(ncols, 32), ceil_div(nrows, 32));
    if (grid.y > 65535) return set_error(ctx, KEVD_ERR_ARG, "kernel_block: too many rows");
    size_t smem = 2 * 32 * (size_t)(kBlkFeat + 1) * sizeof(float);
    if (precision == KEVD_FP64) {
        if (smem > 48 * 1024)
            KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&kernel_block_kernel<double>), (int)smem));
        kernel_block_kernel<double><<<grid, dim3(32, 8), smem, s>>>(
            X, Xc, d, scale, rows, row0, nrows, cols, ncols, (double*)out, ld);
    } else {
        if (smem > 48 * 1024)
            KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&kernel_block_kernel<float>), (int)smem));
        kernel_block_kernel<float><<<grid, dim3(32, 8), smem, s>>>(
            X, Xc, d, scale, rows, row0, nrows, cols, ncols, (float*)out, ld);
    }
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

}  // namespace kevd
