// Stage 3: bistochastic normalisation + EVD of a stored factor F (N x k).
//
// Closed form of ks_kevd.cu (README_kevd.md:20-69) with Khat = F F^T:
//
//   c1   = F^T 1                 colsum pass
//   dtil = F c1                  rowdot pass (+ positivity check, abort code 2)
//   cq   = F^T dtil^{-1}         colsum pass
//   qtil = F cq                  rowdot pass (+ positivity check, abort code 4)
//   A    = F^T Dtil^{-2} F       weighted Gram
//   B    = F^T Qtil^{-1} F       weighted Gram
//   s    = DBL_EPSILON tr(A);  A + sI = L L^T (R = L^T)      (abort code 3)
//   W    = R B R^T; (lam, V) = syevd(W), ascending           (abort code 5)
//   Z    = R^{-1} V[:, k-k_out:];  U = Dtil^{-1} F Z (float, row-major)
//
// The streaming passes and Grams are this file's kernels; the k x k FP64
// factorisation, products and eigensolve use cuSOLVER / cuBLAS (the reference
// uses cuSOLVERMp / cuBLASMp for the same dense steps).  Cross-row sums are
// FP64; FP32 factors accumulate FP32 partials over 1024-row chunks that are
// then added in FP64.
#include "kevd_internal.cuh"
#include "kevd_tc.cuh"

#include <algorithm>
#include <cfloat>
#include <vector>

namespace kevd {

int run_gram_tc(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const unsigned* colmax,
                const double* s, double* G, cudaStream_t st);
int run_gram2_tc(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, const unsigned* colmax,
                 const double* s, const double* s2, double* G, double* G2, cudaStream_t st);
int run_transpose_f32(kevd_ctx* ctx, const float* F, int64_t ldF, int64_t N, int64_t k, float* FT, int64_t ldT,
                      unsigned* amax, cudaStream_t st);

// Column-major copy of an FP32 factor for the tensor-core Grams (K-major TMA
// tiles), and its column maxima (device float bits) for their f16 scaling.
static int transposed(kevd_ctx* ctx, const float* F, int64_t ldF, int64_t N, int64_t k, float** FT,
                      int64_t* ldT, unsigned** colmax, cudaStream_t s) {
    *ldT = (N + 3) / 4 * 4;
    int st = KEVD_OK;
    *FT = arena_get<float>(ctx, "ev.FT", (size_t)k * (size_t)(*ldT), &st);
    *colmax = arena_get<unsigned>(ctx, "ev.FTmax", (size_t)k, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "transpose: out of device memory");
    return run_transpose_f32(ctx, F, ldF, N, k, *FT, *ldT, *colmax, s);
}

// ---- column sums c = F^T w (w == nullptr: ones) ----------------------------
template <typename T>
__global__ void __launch_bounds__(256)
ev_colsum_kernel(const T* __restrict__ F, int64_t ldF, int64_t N, int64_t k,
                 const double* __restrict__ w, int64_t rows_per, double* __restrict__ partial) {
    const int64_t c = (int64_t)blockIdx.x * 256 + threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.y * rows_per;
    const int64_t r1 = min(N, r0 + rows_per);
    if (c >= k) return;
    double acc = 0.0;
    for (int64_t i = r0; i < r1; ++i) {
        const double f = (double)F[i * ldF + c];
        acc += w ? f * w[i] : f;
    }
    partial[(int64_t)blockIdx.y * k + c] = acc;
}

__global__ void ev_sum_partials_kernel(const double* __restrict__ partial, int n_parts, int64_t k,
                                       double* __restrict__ out) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    double s = 0.0;
    for (int p = 0; p < n_parts; ++p) s += partial[(int64_t)p * k + c];
    out[c] = s;
}

// ---- row dots y = F v, with y > 0 check and 1/y ----------------------------
template <typename T>
__global__ void __launch_bounds__(256)
ev_rowdot_kernel(const T* __restrict__ F, int64_t ldF, int64_t N, int64_t k,
                 const double* __restrict__ v, double* __restrict__ y, double* __restrict__ yinv,
                 int* __restrict__ bad) {
    extern __shared__ double vs[];
    for (int64_t c = threadIdx.x; c < k; c += blockDim.x) vs[c] = v[c];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < N; i += warps) {
        const T* row = F + i * ldF;
        double acc = 0.0;
        for (int64_t c = lane; c < k; c += 32) acc += (double)row[c] * vs[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            y[i] = acc;
            yinv[i] = 1.0 / acc;
            if (!(acc > 0.0)) atomicOr(bad, 1);
        }
    }
}

// ---- weighted Gram  G = sum_i w_i F_i^T F_i, lower 64 x 64 tiles -----------
// grid.x = lower tile index, grid.y = row split.  Thread (ty, tx) of 16 x 16
// owns rows ty + 16a and columns tx + 16b of the tile.
constexpr int kGT = 64;   // tile edge
constexpr int kGK = 32;   // rows per stage
constexpr int kGFlush = 1024;  // rows per FP32 partial (FP32 factors)

template <typename T>
__global__ void __launch_bounds__(256)
ev_gram_kernel(const T* __restrict__ F, int64_t ldF, int64_t N, int64_t k,
               const double* __restrict__ w, int64_t rows_per, double* __restrict__ partial) {
    __shared__ T As[kGK][kGT + 1];
    __shared__ T Bs[kGK][kGT + 1];
    // lower tile (ta >= tb) from the linear index
    const int64_t t = blockIdx.x;
    int64_t ta = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (ta * (ta + 1) / 2 > t) --ta;
    while ((ta + 1) * (ta + 2) / 2 <= t) ++ta;
    const int64_t tb = t - ta * (ta + 1) / 2;
    const int64_t a0 = ta * kGT, b0 = tb * kGT;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t r0 = (int64_t)blockIdx.y * rows_per;
    const int64_t r1 = min(N, r0 + rows_per);
    double acc64[4][4];
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) { acc64[i][j] = 0.0; acc[i][j] = 0; }
    int64_t since_flush = 0;
    for (int64_t i0 = r0; i0 < r1; i0 += kGK) {
        for (int e = threadIdx.x; e < kGK * kGT; e += 256) {
            const int rr = e / kGT, cc = e - rr * kGT;
            const int64_t i = i0 + rr;
            T fa = 0, fb = 0;
            if (i < r1) {
                const T wi = (T)w[i];
                if (a0 + cc < k) fa = F[i * ldF + a0 + cc] * wi;
                if (b0 + cc < k) fb = F[i * ldF + b0 + cc];
            }
            As[rr][cc] = fa;
            Bs[rr][cc] = fb;
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < kGK; ++rr) {
            T va[4], vb[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) va[a] = As[rr][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) vb[b] = Bs[rr][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += va[a] * vb[b];
        }
        __syncthreads();
        since_flush += kGK;
        if (sizeof(T) == 4 && since_flush >= kGFlush) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) { acc64[a][b] += (double)acc[a][b]; acc[a][b] = 0; }
            since_flush = 0;
        }
    }
    double* out = partial + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * kGT * kGT;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
            out[(ty + 16 * a) * kGT + tx + 16 * b] = acc64[a][b] + (double)acc[a][b];
}

// Sum the row-split partials of every lower tile into a full symmetric
// column-major k x k matrix.
__global__ void ev_gram_reduce_kernel(const double* __restrict__ partial, int n_tiles, int n_split,
                                      int64_t k, double* __restrict__ G) {
    const int64_t t = blockIdx.x;
    int64_t ta = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (ta * (ta + 1) / 2 > t) --ta;
    while ((ta + 1) * (ta + 2) / 2 <= t) ++ta;
    const int64_t tb = t - ta * (ta + 1) / 2;
    for (int e = threadIdx.x; e < kGT * kGT; e += blockDim.x) {
        const int ia = e / kGT, ib = e - ia * kGT;
        const int64_t ga = ta * kGT + ia, gb = tb * kGT + ib;
        if (ga >= k || gb >= k) continue;
        double s = 0.0;
        for (int p = 0; p < n_split; ++p) s += partial[((int64_t)p * n_tiles + t) * kGT * kGT + e];
        G[gb * k + ga] = s;   // (ga, gb)
        G[ga * k + gb] = s;   // (gb, ga)
    }
}

// ---- small helpers ---------------------------------------------------------
__global__ void ev_rsqrt_kernel(const double* __restrict__ q, double* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = 1.0 / sqrt(q[i]);
}

__global__ void ev_square_kernel(const double* __restrict__ x, double* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = x[i] * x[i];
}

__global__ void ev_trace_shift_kernel(double* __restrict__ A, int64_t k, double* __restrict__ out, double c) {
    // one CTA: out[0] = tr(A), out[1] = shift = c u tr(A); A += shift I
    __shared__ double red[1024];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < k; i += blockDim.x) s += A[i * k + i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double tr = red[0];
    const double sh = c * DBL_EPSILON * tr;
    for (int64_t i = threadIdx.x; i < k; i += blockDim.x) A[i * k + i] += sh;
    if (threadIdx.x == 0) {
        out[0] = tr;
        out[1] = sh;
    }
}

__global__ void ev_symmetrize_kernel(double* __restrict__ W, int64_t k) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < k * k;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e / k, r = e - c * k;
        if (r > c) {
            const double v = 0.5 * (W[c * k + r] + W[r * k + c]);
            W[c * k + r] = v;
            W[r * k + c] = v;
        }
    }
}

// ---- U = Dtil^{-1} F Z (row-major float, N x k_out) -------------------------
// CTA: 64 rows x 64 columns (column chunk blockIdx.y of k_out <= 256); Z
// chunks of 32 rows staged as T.
template <typename T>
__global__ void __launch_bounds__(256)
ev_u_kernel(const T* __restrict__ F, int64_t ldF, int64_t N, int64_t k, const double* __restrict__ Z,
            int k_out, const double* __restrict__ dinv, float* __restrict__ U) {
    __shared__ T Fs[64][33];
    __shared__ T Zs[32][65];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t row0 = (int64_t)blockIdx.x * 64;
    const int j0 = 64 * blockIdx.y;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0;
    for (int64_t c0 = 0; c0 < k; c0 += 32) {
        for (int e = threadIdx.x; e < 64 * 32; e += 256) {
            const int rr = e / 32, cc = e - rr * 32;
            const int64_t i = row0 + rr, c = c0 + cc;
            Fs[rr][cc] = (i < N && c < k) ? F[i * ldF + c] : (T)0;
        }
        for (int e = threadIdx.x; e < 32 * 64; e += 256) {
            const int cc = e / 64, j = e - cc * 64;
            const int64_t c = c0 + cc;
            Zs[cc][j] = (c < k && j0 + j < k_out) ? (T)Z[(int64_t)(j0 + j) * k + c] : (T)0;
        }
        __syncthreads();
#pragma unroll 8
        for (int cc = 0; cc < 32; ++cc) {
            T vf[4], vz[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) vf[a] = Fs[ty + 16 * a][cc];
#pragma unroll
            for (int b = 0; b < 4; ++b) vz[b] = Zs[cc][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += vf[a] * vz[b];
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int64_t i = row0 + ty + 16 * a;
        if (i >= N) continue;
        const double di = dinv[i];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int j = j0 + tx + 16 * b;
            if (j < k_out) U[i * k_out + j] = (float)((double)acc[a][b] * di);
        }
    }
}

// Compensated (Kahan) FP32 accumulation: the running sum is s - c.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// ---- streaming passes on the column-major FP32 factor FT (k x ldT) ------------
// Reads are coalesced along rows.  The bistochastic scaling vectors are FP64
// quantities: FP64 multipliers are carried as FP32 (hi, lo) pairs, each product
// x * hi keeps its exact rounding error (fma), and short sums are double-FP32
// pairs (two-sum), flushed into FP64.  The result is FP64-accurate (about
// 1e-14 relative) while the arithmetic stays on the FP32 pipe, so the passes
// remain HBM-bound.

// (s, c) += x exactly up to the rounding of c: s + c is the running sum.
__device__ __forceinline__ void df_add(float& s, float& c, float x) {
    const float t = s + x;
    const float z = t - s;
    c += (s - (t - z)) + (x - z);
    s = t;
}

// (s, c) += x * (wh + wl), with the product error of x * wh kept.
__device__ __forceinline__ void df_fma(float& s, float& c, float x, float wh, float wl) {
    const float p = __fmul_rn(x, wh);   // never contracted into the following add
    const float pe = fmaf(x, wh, -p);
    df_add(s, c, p);
    c = fmaf(x, wl, c + pe);
}

// Partial column sums c[j] = sum_i w_i FT[j][i] (w == nullptr: ones) over this
// CTA's row range.  CTA = 16 warps = 16 columns; the (hi, lo) weights of each
// 2048-row chunk are staged once in shared memory for all 16 columns; each lane
// sums 64 products as a double-FP32 pair, chunks are added in FP64.
__global__ void __launch_bounds__(512)
evt_colsum_kernel(const float* __restrict__ FT, int64_t ldT, int64_t N, int64_t k, const double* __restrict__ w,
                  int64_t rows_per, double* __restrict__ partial) {
    __shared__ float wsh[2048], wsl[2048];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t j = (int64_t)blockIdx.x * 16 + warp;
    const int64_t r0 = (int64_t)blockIdx.y * rows_per;
    const int64_t r1 = min(N, r0 + rows_per);
    double acc = 0.0;
    for (int64_t i0 = r0; i0 < r1; i0 += 2048) {
        const int n = (int)min((int64_t)2048, r1 - i0);
        __syncthreads();
        for (int t = threadIdx.x; t < n; t += 512) {
            const double x = w ? w[i0 + t] : 1.0;
            const float h = (float)x;
            wsh[t] = h;
            wsl[t] = (float)(x - (double)h);
        }
        __syncthreads();
        if (j < k) {
            const float* col = FT + j * ldT + i0;
            float ps = 0.f, pc = 0.f;
            for (int t = lane; t < n; t += 32) df_fma(ps, pc, col[t], wsh[t], wsl[t]);
            acc += (double)ps + (double)pc;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && j < k) partial[(int64_t)blockIdx.y * k + j] = acc;
}

// y_i = sum_j FT[j][i] v_j with v as an FP32 (hi, lo) pair; double-FP32 sums
// of 32 terms, FP64 across them; yinv = 1/y; bad |= (y <= 0).
__global__ void __launch_bounds__(256)
evt_rowdot_kernel(const float* __restrict__ FT, int64_t ldT, int64_t N, int64_t k, const double* __restrict__ v,
                  double* __restrict__ y, double* __restrict__ yinv, int* __restrict__ bad) {
    extern __shared__ float vhl[];   // 2k floats
    for (int64_t j = threadIdx.x; j < k; j += blockDim.x) {
        const float h = (float)v[j];
        vhl[2 * j] = h;
        vhl[2 * j + 1] = (float)(v[j] - (double)h);
    }
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    double acc = 0.0;
    for (int64_t j0 = 0; j0 < k; j0 += 32) {
        float ps = 0.f, pc = 0.f;
        const int64_t j1 = min(k, j0 + 32);
        int64_t j = j0;
        for (; j + 8 <= j1; j += 8) {   // eight loads in flight, then the compensated sums in order
            float f[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) f[u] = FT[(j + u) * ldT + i];
#pragma unroll
            for (int u = 0; u < 8; ++u) df_fma(ps, pc, f[u], vhl[2 * (j + u)], vhl[2 * (j + u) + 1]);
        }
        for (; j < j1; ++j) df_fma(ps, pc, FT[j * ldT + i], vhl[2 * j], vhl[2 * j + 1]);
        acc += (double)ps + (double)pc;
    }
    y[i] = acc;
    yinv[i] = 1.0 / acc;
    if (!(acc > 0.0)) atomicOr(bad, 1);
}

// U[i][:] = dinv_i * sum_j FT[j][i] Z[j][:]  (Z: k x m column-major FP64, m <= 32).
// CTA = 256 rows; thread t forms columns 16 h .. 16 h + 15 (h = t & 1) of rows
// p and p + 128 (p = t >> 1), so every broadcast load of a Z row feeds twice as
// many FMAs as with one full row per thread (there the shared-memory loads
// and the FMAs each filled their pipe) at the same 32 accumulators.
__global__ void __launch_bounds__(256)
evt_u_kernel(const float* __restrict__ FT, int64_t ldT, int64_t N, int64_t k, const double* __restrict__ Z, int m,
             const double* __restrict__ dinv, float* __restrict__ U, float* __restrict__ Y) {
    __shared__ __align__(16) float Zs[128][32];
    const int h = threadIdx.x & 1, p = threadIdx.x >> 1;
    const int64_t i0 = (int64_t)blockIdx.x * 256 + p, i1 = i0 + 128;
    const bool v0 = i0 < N, v1 = i1 < N;
    float acc0[16], acc1[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc0[q] = acc1[q] = 0.f;
    for (int64_t j0 = 0; j0 < k; j0 += 128) {
        __syncthreads();
        for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) {
            const int jj = e >> 5, q = e & 31;
            const int64_t j = j0 + jj;
            Zs[jj][q] = (j < k && q < m) ? (float)Z[(int64_t)q * k + j] : 0.f;
        }
        __syncthreads();
        if (v0) {
            const int jn = (int)min((int64_t)128, k - j0);
            // the F values of the next four columns are loaded before this
            // step's FMAs (columns past jn read as zero; Zs is zero there too)
            float g0[4], g1[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                g0[u] = (u < jn) ? FT[(j0 + u) * ldT + i0] : 0.f;
                g1[u] = (u < jn && v1) ? FT[(j0 + u) * ldT + i1] : 0.f;
            }
            for (int jj = 0; jj < jn; jj += 4) {
                float f0[4], f1[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    f0[u] = g0[u];
                    f1[u] = g1[u];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const bool in = jj + 4 + u < jn;
                    g0[u] = in ? FT[(j0 + jj + 4 + u) * ldT + i0] : 0.f;
                    g1[u] = (in && v1) ? FT[(j0 + jj + 4 + u) * ldT + i1] : 0.f;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4* zr = reinterpret_cast<const float4*>(Zs[jj + u] + 16 * h);
#pragma unroll
                    for (int q4 = 0; q4 < 4; ++q4) {
                        const float4 z = zr[q4];
                        acc0[4 * q4 + 0] = fmaf(f0[u], z.x, acc0[4 * q4 + 0]);
                        acc0[4 * q4 + 1] = fmaf(f0[u], z.y, acc0[4 * q4 + 1]);
                        acc0[4 * q4 + 2] = fmaf(f0[u], z.z, acc0[4 * q4 + 2]);
                        acc0[4 * q4 + 3] = fmaf(f0[u], z.w, acc0[4 * q4 + 3]);
                        acc1[4 * q4 + 0] = fmaf(f1[u], z.x, acc1[4 * q4 + 0]);
                        acc1[4 * q4 + 1] = fmaf(f1[u], z.y, acc1[4 * q4 + 1]);
                        acc1[4 * q4 + 2] = fmaf(f1[u], z.z, acc1[4 * q4 + 2]);
                        acc1[4 * q4 + 3] = fmaf(f1[u], z.w, acc1[4 * q4 + 3]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int64_t i = r ? i1 : i0;
        if (i >= N) continue;
        const double di = dinv[i];
#pragma unroll
        for (int qq = 0; qq < 16; ++qq) {
            const int q = 16 * h + qq;
            const float u = (float)((double)(r ? acc1[qq] : acc0[qq]) * di);
            if (q < m) U[i * m + q] = u;
            // Y = Dtil^{-1} U of the rounded U, 32 columns (zero beyond m), for the
            // Rayleigh-Ritz T1 pass
            if (Y) Y[i * 32 + q] = (q < m) ? (float)((double)u * di) : 0.f;
        }
    }
}

// Rayleigh-Ritz T1 partials: T1[j][q] = sum_i FT[j][i] Y[i][q] over this CTA's
// rows, Y = Dtil^{-1} U rounded to FP32 (N x 32, written by evt_u_kernel), for a
// block of 64 columns j.  128 threads, thread (jg, qg) owns columns 4 jg..4 jg+3
// and q = 4 qg..4 qg+3.  Tiles of 64 rows are staged with 16-byte cp.async into
// a double buffer (the next tile is in flight while this one is used): F as
// [column][row] with the 16-byte chunk index of a column XOR-ed with
// (column >> 1) & 7 (the four columns a warp reads at once land in four
// different bank groups), Y as [row][q].  FP32 products and 8-row FP32 partials
// (round to nearest: their errors are unbiased and average out in H); the
// partials are added with compensation over the CTA's row range.
constexpr int kT1Rows = 64;
constexpr size_t kT1Smem = 2 * (size_t)(64 * kT1Rows + kT1Rows * 32) * sizeof(float);
__global__ void __launch_bounds__(128)
evt_t1_kernel(const float* __restrict__ FT, int64_t ldT, int64_t N, int64_t k, const float* __restrict__ Y, int m,
              int64_t rows_per, double* __restrict__ partial) {
    extern __shared__ __align__(16) float t1sm[];
    const int tid = threadIdx.x;
    const int jg = tid >> 3, qg = tid & 7;
    const int64_t j0 = (int64_t)blockIdx.x * 64;
    const int64_t r0 = (int64_t)blockIdx.y * rows_per;
    const int64_t r1 = min(N, r0 + rows_per);
    const int64_t n_t = (r1 > r0) ? (r1 - r0 + kT1Rows - 1) / kT1Rows : 0;
    auto fbuf = [&](int b) { return t1sm + (size_t)b * (64 * kT1Rows + kT1Rows * 32); };
    auto stage = [&](int64_t t, int b) {
        float* Fs = fbuf(b);
        float* Ws = Fs + 64 * kT1Rows;
        const int64_t i0 = r0 + t * kT1Rows;
        for (int e = tid; e < 64 * 16 + kT1Rows * 8; e += 128) {
            if (e < 64 * 16) {
                const int jj = e >> 4, c = e & 15;   // column jj, rows 4c..4c+3
                const int64_t j = j0 + jj, i = i0 + 4 * c;
                const bool ok = (j < k) && (i < r1);
                const float* src = ok ? FT + j * ldT + i : FT;
                tc::cp_async16(Fs + jj * kT1Rows + 4 * (c ^ ((jj >> 1) & 7)), src, ok ? 16u : 0u);
            } else {
                const int e2 = e - 64 * 16;
                const int ii = e2 >> 3, c = e2 & 7;   // row ii, q 4c..4c+3
                const int64_t i = i0 + ii;
                const bool ok = i < r1;
                tc::cp_async16(Ws + ii * 32 + 4 * c, ok ? Y + i * 32 + 4 * c : Y, ok ? 16u : 0u);
            }
        }
    };
    float ks[4][4], kc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) ks[a][b] = kc[a][b] = 0.f;
    if (n_t > 0) stage(0, 0);
    tc::cp_async_commit();
    for (int64_t t = 0; t < n_t; ++t) {
        if (t + 1 < n_t) {
            stage(t + 1, (int)((t + 1) & 1));
            tc::cp_async_commit();
            tc::cp_async_wait<1>();
        } else {
            tc::cp_async_wait<0>();
        }
        __syncthreads();
        const float* Fs = fbuf((int)(t & 1));
        const float* Ws = Fs + 64 * kT1Rows;
#pragma unroll 1
        for (int i8 = 0; i8 < kT1Rows; i8 += 8) {
            float p[4][4];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) p[a][b] = 0.f;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int rc = (i8 >> 2) + h;   // 16-byte chunk of rows 4 rc..4 rc+3
                float fv[4][4], wv[4][4];
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const int jj = 4 * jg + a;
                    const float4 f = *reinterpret_cast<const float4*>(Fs + jj * kT1Rows + 4 * (rc ^ ((jj >> 1) & 7)));
                    fv[a][0] = f.x; fv[a][1] = f.y; fv[a][2] = f.z; fv[a][3] = f.w;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4 w = *reinterpret_cast<const float4*>(Ws + (4 * rc + u) * 32 + 4 * qg);
                    wv[u][0] = w.x; wv[u][1] = w.y; wv[u][2] = w.z; wv[u][3] = w.w;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) p[a][b] = fmaf(fv[a][u], wv[u][b], p[a][b]);
            }
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) kahan_add(ks[a][b], kc[a][b], p[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int64_t j = j0 + 4 * jg + a;
        if (j >= k) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int q = 4 * qg + b;
            if (q < m) partial[((int64_t)blockIdx.y * k + j) * m + q] = (double)ks[a][b] - (double)kc[a][b];
        }
    }
}

// Rayleigh-Ritz H and M partials over 64-row tiles: w_i = F_i (T1h + T1l)
// (T1 as an FP32 hi/lo pair, k x 32), H += (w/sqrt(q))(w/sqrt(q))^T, M += u u^T.
// 128 threads; for w thread (ig, qg) owns rows 4 ig..4 ig+3 and columns
// 4 qg..4 qg+3 (16-byte loads of F and of the T1 rows from shared memory, 8-term
// FP32 partials added with compensation); for H and M thread t owns entries
// t + 128 r of the 32 x 32 matrices, summed over the tile with compensation and
// across tiles in FP64.
constexpr int kHmRows = 64;
__global__ void __launch_bounds__(128)
evt_hm_kernel(const float* __restrict__ FT, int64_t ldT, int64_t N, int64_t k, const float* __restrict__ T1hl,
              int m, const float* __restrict__ U, const double* __restrict__ qinv, double* __restrict__ partial) {
    // double buffer of (F chunk [column j][row i], T1 hi/lo chunk), 16-byte
    // cp.async copies: the next (tile, column chunk) step is in flight while
    // this one is used
    __shared__ __align__(16) float Fsb[2][32][kHmRows];
    __shared__ __align__(16) float Tsb[2][2][32][32];
    __shared__ float Ws[kHmRows][33];
    const int tid = threadIdx.x;
    const int ig = tid >> 3, qg = tid & 7;
    double h64[8], m64[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) h64[r] = m64[r] = 0.0;
    const int64_t n_tiles = (N + kHmRows - 1) / kHmRows;
    const int nch = (int)((k + 31) / 32);
    auto stage = [&](int64_t t, int c, int b) {
        const int64_t i0 = t * kHmRows, j0 = (int64_t)c * 32;
        for (int e = tid; e < 32 * (kHmRows / 4) + 64 * 8; e += 128) {
            if (e < 32 * (kHmRows / 4)) {
                const int jj = e / (kHmRows / 4), rc = e % (kHmRows / 4);   // column jj, rows 4 rc..4 rc+3
                const int64_t j = j0 + jj, i = i0 + 4 * rc;
                const bool ok = (j < k) && (i < N);   // FT rows are padded to a multiple of 4 with zeros
                tc::cp_async16(&Fsb[b][jj][4 * rc], ok ? FT + j * ldT + i : FT, ok ? 16u : 0u);
            } else {
                const int e2 = e - 32 * (kHmRows / 4);
                const int r2 = e2 >> 3, c4 = e2 & 7;   // T1hl row 2 j + (hi, lo), q 4 c4..4 c4+3
                const int jj = r2 >> 1, hl = r2 & 1;
                const int64_t j = j0 + jj;
                const bool ok = j < k;
                tc::cp_async16(&Tsb[b][hl][jj][4 * c4], ok ? T1hl + (2 * j + hl) * 32 + 4 * c4 : T1hl, ok ? 16u : 0u);
            }
        }
    };
    int b = 0;
    if ((int64_t)blockIdx.x < n_tiles) stage(blockIdx.x, 0, 0);
    tc::cp_async_commit();
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const int64_t i0 = t * kHmRows;
        float ws[4][4], wc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int bb = 0; bb < 4; ++bb) ws[a][bb] = wc[a][bb] = 0.f;
        for (int c = 0; c < nch; ++c) {
            const int64_t nt = (c + 1 < nch) ? t : t + gridDim.x;
            const int nc = (c + 1 < nch) ? c + 1 : 0;
            if (nt < n_tiles) {
                stage(nt, nc, b ^ 1);
                tc::cp_async_commit();
                tc::cp_async_wait<1>();
            } else {
                tc::cp_async_wait<0>();
            }
            __syncthreads();
            float (*Fs)[kHmRows] = Fsb[b];
            float (*Ts)[32][32] = Tsb[b];
#pragma unroll 1
            for (int j8 = 0; j8 < 32; j8 += 8) {
                float p[4][4];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int bb = 0; bb < 4; ++bb) p[a][bb] = 0.f;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const float4 f = *reinterpret_cast<const float4*>(&Fs[j8 + u][4 * ig]);
                    const float4 th = *reinterpret_cast<const float4*>(&Ts[0][j8 + u][4 * qg]);
                    const float4 tl = *reinterpret_cast<const float4*>(&Ts[1][j8 + u][4 * qg]);
                    const float fv[4] = {f.x, f.y, f.z, f.w};
                    const float hv[4] = {th.x, th.y, th.z, th.w}, lv[4] = {tl.x, tl.y, tl.z, tl.w};
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int bb = 0; bb < 4; ++bb) p[a][bb] = fmaf(fv[a], hv[bb], fmaf(fv[a], lv[bb], p[a][bb]));
                }
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int bb = 0; bb < 4; ++bb) kahan_add(ws[a][bb], wc[a][bb], p[a][bb]);
            }
            __syncthreads();
            b ^= 1;
        }
        __syncthreads();
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int64_t i = i0 + 4 * ig + a;
            const float sq = (i < N) ? (float)sqrt(qinv[i]) : 0.f;
#pragma unroll
            for (int bb = 0; bb < 4; ++bb) {
                const int q = 4 * qg + bb;
                Ws[4 * ig + a][q] = (q < m) ? (ws[a][bb] - wc[a][bb]) * sq : 0.f;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int e = tid + 128 * r;
            const int ja = e >> 5, jb = e & 31;
            float hs = 0.f, hc = 0.f;
            for (int rr = 0; rr < kHmRows; ++rr) kahan_add(hs, hc, Ws[rr][ja] * Ws[rr][jb]);
            h64[r] += (double)hs - (double)hc;
        }
        __syncthreads();
        for (int e = tid; e < kHmRows * 32; e += 128) {
            const int rr = e >> 5, q = e & 31;
            const int64_t i = i0 + rr;
            Ws[rr][q] = (i < N && q < m) ? U[i * m + q] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const int e = tid + 128 * r;
            const int ja = e >> 5, jb = e & 31;
            float ms = 0.f, mc = 0.f;
            for (int rr = 0; rr < kHmRows; ++rr) kahan_add(ms, mc, Ws[rr][ja] * Ws[rr][jb]);
            m64[r] += (double)ms - (double)mc;
        }
    }
    double* out = partial + (int64_t)blockIdx.x * 2048;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        out[tid + 128 * r] = h64[r];
        out[1024 + tid + 128 * r] = m64[r];
    }
}

__global__ void evt_split_t1_kernel(const double* __restrict__ T1, int64_t k, int m, float* __restrict__ T1hl) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < k * 32;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e >> 5;
        const int q = (int)(e & 31);
        const double t = (q < m) ? T1[j * m + q] : 0.0;
        const float h = (float)t;
        T1hl[(2 * j) * 32 + q] = h;
        T1hl[(2 * j + 1) * 32 + q] = (float)(t - (double)h);
    }
}

// ---- Rayleigh-Ritz refinement of the leading eigenpairs (FP32 factor) -------
// With U = Dtil^{-1} F Z (N x m), U^T P U = T1^T B T1 where T1 = F^T Dtil^{-1} U
// (k x m) and B = F^T Qtil^{-1} F, so
//     H = U^T P U = sum_i w_i w_i^T / qtil_i,  w_i = F_i T1,
//     M = U^T U   = sum_i u_i u_i^T.
// Both are formed in streaming passes over F with FP32 products (round to
// nearest, unbiased) summed in FP64 across rows; the m x m pencil (H, M) gives
// Ritz values accurate to the square of the eigenvector error of the Gram path.

__global__ void rr_sum_kernel(const double* __restrict__ partial, int n_parts, int64_t len,
                              double* __restrict__ out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len;
         e += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int p = 0; p < n_parts; ++p) s += partial[(int64_t)p * len + e];
        out[e] = s;
    }
}

// U <- U C (N x m times m x m), C column-major.
__global__ void rr_rotate_kernel(float* __restrict__ U, int64_t N, int m, const double* __restrict__ C) {
    __shared__ double Cs[32 * 32];
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) Cs[e] = C[e];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        float u[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) u[j] = (j < m) ? U[i * m + j] : 0.f;
#pragma unroll 1
        for (int j = 0; j < m; ++j) {
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < 32; ++q)
                if (q < m) s = fmaf(u[q], (float)Cs[j * m + q], s);
            U[i * m + j] = s;
        }
    }
}

// On the column-major FP32 factor FT (k x ldT).
static int rayleigh_ritz(kevd_ctx* ctx, const float* FT, int64_t ldT, int64_t N, int64_t k, int m, float* U,
                         const float* Y, const double* qinv, double* lam_top, cudaStream_t s) {
    ProfScope ps(ctx, "ev_ritz", s);
    int st = KEVD_OK;
    const int ny = (int)std::min<int64_t>((N + 8191) / 8192, (int64_t)ctx->num_sms * 2);
    const int64_t rows_per = ((N + ny - 1) / ny + 63) / 64 * 64;
    double* tpart = arena_get<double>(ctx, "rr.tpart", (size_t)ny * k * m, &st);
    double* T1 = arena_get<double>(ctx, "rr.T1", (size_t)k * m, &st);
    float* T1hl = arena_get<float>(ctx, "rr.T1hl", (size_t)k * 64, &st);
    const int nhm = ctx->num_sms * 4;
    double* hmpart = arena_get<double>(ctx, "rr.hmpart", (size_t)nhm * 2048, &st);
    double* HM = arena_get<double>(ctx, "rr.HM", 2048, &st);
    double* w = arena_get<double>(ctx, "rr.w", 64, &st);
    int* info = arena_get<int>(ctx, "rr.info", 1, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "rayleigh_ritz: out of device memory");
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&evt_t1_kernel), kT1Smem));
    evt_t1_kernel<<<dim3(ceil_div(k, 64), ny), 128, kT1Smem, s>>>(FT, ldT, N, k, Y, m, rows_per, tpart);
    KEVD_LAUNCH(ctx);
    rr_sum_kernel<<<ceil_div(k * m, 256), 256, 0, s>>>(tpart, ny, k * m, T1);
    KEVD_LAUNCH(ctx);
    evt_split_t1_kernel<<<ceil_div(k * 32, 256), 256, 0, s>>>(T1, k, m, T1hl);
    KEVD_LAUNCH(ctx);
    evt_hm_kernel<<<nhm, 128, 0, s>>>(FT, ldT, N, k, T1hl, m, U, qinv, hmpart);
    KEVD_LAUNCH(ctx);
    rr_sum_kernel<<<8, 256, 0, s>>>(hmpart, nhm, 2048, HM);
    KEVD_LAUNCH(ctx);
    // H and M are stored 32 x 32 (row-major = column-major, symmetric); use the
    // leading m x m with leading dimension 32
    int lwork = 0;
    KEVD_SOLVER(ctx, cusolverDnDsygvd_bufferSize(ctx->solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                                 CUBLAS_FILL_MODE_LOWER, m, HM, 32, HM + 1024, 32, w, &lwork));
    double* work = arena_get<double>(ctx, "rr.work", (size_t)lwork + 1, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "rayleigh_ritz: out of device memory");
    KEVD_SOLVER(ctx, cusolverDnDsygvd(ctx->solver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                      CUBLAS_FILL_MODE_LOWER, m, HM, 32, HM + 1024, 32, w, work, lwork, info));
    // eigenvectors C (m x m, ld 32) -> compact ld m for the rotation
    double* C = arena_get<double>(ctx, "rr.C", (size_t)m * m, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "rayleigh_ritz: out of device memory");
    KEVD_CUDA(ctx, cudaMemcpy2DAsync(C, m * sizeof(double), HM, 32 * sizeof(double), m * sizeof(double), m,
                                     cudaMemcpyDeviceToDevice, s));
    rr_rotate_kernel<<<ctx->num_sms * 4, 128, 0, s>>>(U, N, m, C);
    KEVD_LAUNCH(ctx);
    int hinfo = 0;
    KEVD_CUDA(ctx, cudaMemcpyAsync(lam_top, w, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    if (hinfo != 0) return set_error(ctx, KEVD_ERR_SYEVD, "rayleigh_ritz: sygvd failed, info %d", hinfo);
    return KEVD_OK;
}

template <typename T>
static int colsum(kevd_ctx* ctx, const T* F, int64_t ldF, int64_t N, int64_t k, const double* w,
                  double* out, cudaStream_t s) {
    const int ny = (int)std::min<int64_t>((N + 1023) / 1024, (int64_t)ctx->num_sms * 4);
    const int64_t rows_per = (N + ny - 1) / ny;
    int st = KEVD_OK;
    double* partial = arena_get<double>(ctx, "ev.cpart", (size_t)ny * k, &st);
    if (st != KEVD_OK) return st;
    ProfScope ps(ctx, "ev_colsum", s);
    ev_colsum_kernel<T><<<dim3(ceil_div(k, 256), ny), 256, 0, s>>>(F, ldF, N, k, w, rows_per, partial);
    KEVD_LAUNCH(ctx);
    ev_sum_partials_kernel<<<ceil_div(k, 256), 256, 0, s>>>(partial, ny, k, out);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

template <typename T>
static int rowdot(kevd_ctx* ctx, const T* F, int64_t ldF, int64_t N, int64_t k, const double* v,
                  double* y, double* yinv, int* bad, cudaStream_t s) {
    const size_t smem = (size_t)k * sizeof(double);
    KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&ev_rowdot_kernel<T>), (int)smem));
    const int grid = (int)std::min<int64_t>((N + 7) / 8, (int64_t)ctx->num_sms * 8);
    ProfScope ps(ctx, "ev_rowdot", s);
    ev_rowdot_kernel<T><<<grid, 256, smem, s>>>(F, ldF, N, k, v, y, yinv, bad);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

template <typename T>
static int gram(kevd_ctx* ctx, const T* F, int64_t ldF, int64_t N, int64_t k, const double* w,
                double* G, cudaStream_t s) {
    const int nt = ceil_div(k, kGT);
    const int n_tiles = nt * (nt + 1) / 2;
    int n_split = (int)std::max<int64_t>(1, ((int64_t)ctx->num_sms * 8 + n_tiles - 1) / n_tiles);
    n_split = (int)std::min<int64_t>(n_split, std::max<int64_t>(1, N / 256));
    const int64_t rows_per = ((N + n_split - 1) / n_split + kGK - 1) / kGK * kGK;
    int st = KEVD_OK;
    double* partial = arena_get<double>(ctx, "ev.gpart", (size_t)n_split * n_tiles * kGT * kGT, &st);
    if (st != KEVD_OK) return st;
    {
        ProfScope ps(ctx, "ev_gram", s);
        ev_gram_kernel<T><<<dim3(n_tiles, n_split), 256, 0, s>>>(F, ldF, N, k, w, rows_per, partial);
        KEVD_LAUNCH(ctx);
    }
    ev_gram_reduce_kernel<<<n_tiles, 256, 0, s>>>(partial, n_tiles, n_split, k, G);
    KEVD_LAUNCH(ctx);
    return KEVD_OK;
}

static int d2h(kevd_ctx* ctx, double* host, const double* dev, size_t n, cudaStream_t s) {
    if (!host) return KEVD_OK;
    KEVD_CUDA(ctx, cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    return KEVD_OK;
}

// Element-wise copies between the FP64 and FP32 k x k workspaces (column-major).
__global__ void ev_d2f_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
__global__ void ev_f2d_kernel(const float* __restrict__ a, double* __restrict__ b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

// Leading eigenpairs of the FP64 matrix W (k x k) for an FP32 factor: an FP32
// divide-and-conquer eigensolve of W rounded to FP32 gives the whole spectrum
// (FP32-accurate) and the leading m-dimensional subspace; Rayleigh-Ritz on the
// FP64 W over that subspace (two Cholesky-QR passes, then H = V^T W V and an
// m x m FP64 eigensolve) gives the leading eigenpairs in FP64.  On return
// lam[0..k) holds the spectrum (ascending; the top m entries from the FP64
// Rayleigh-Ritz step) and V (k x m, column-major) the refined eigenvectors,
// ascending.  flag receives the solver info (non-zero: failure).
static int top_eigs_fp32_rr(kevd_ctx* ctx, const double* W, int64_t k, int m, double* lam, double* V, int* flag,
                            cudaStream_t s) {
    int st = KEVD_OK;
    float* Wf = arena_get<float>(ctx, "ev.Wf", (size_t)k * k, &st);
    float* lamf = arena_get<float>(ctx, "ev.lamf", k, &st);
    double* Y = arena_get<double>(ctx, "ev.rrY", (size_t)k * m, &st);
    double* H = arena_get<double>(ctx, "ev.rrH", (size_t)m * m, &st);
    double* mu = arena_get<double>(ctx, "ev.rrmu", m, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "bistochastic_evd: out of device memory");
    const int grid = ctx->num_sms * 4;
    ev_d2f_kernel<<<grid, 256, 0, s>>>(W, Wf, k * k);
    KEVD_LAUNCH(ctx);
    int lw = 0, lw2 = 0, lw3 = 0;
    KEVD_SOLVER(ctx, cusolverDnSsyevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                                 (int)k, Wf, (int)k, lamf, &lw));
    KEVD_SOLVER(ctx, cusolverDnDsyevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m,
                                                 H, m, mu, &lw2));
    KEVD_SOLVER(ctx, cusolverDnDpotrf_bufferSize(ctx->solver, CUBLAS_FILL_MODE_UPPER, m, H, m, &lw3));
    float* wf = arena_get<float>(ctx, "ev.swork", (size_t)lw + 1, &st);
    double* wd = arena_get<double>(ctx, "ev.rrwork", (size_t)std::max(lw2, lw3) + 1, &st);
    if (st != KEVD_OK) return set_error(ctx, st, "bistochastic_evd: out of device memory");
    {
        ProfScope p3(ctx, "dense_syevd", s);
        KEVD_SOLVER(ctx, cusolverDnSsyevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)k, Wf,
                                          (int)k, lamf, wf, lw, flag));
    }
    ProfScope pr(ctx, "dense_rr", s);
    ev_f2d_kernel<<<grid, 256, 0, s>>>(lamf, lam, k);
    KEVD_LAUNCH(ctx);
    ev_f2d_kernel<<<grid, 256, 0, s>>>(Wf + (k - m) * k, V, k * m);
    KEVD_LAUNCH(ctx);
    const double one = 1.0, zero = 0.0;
    // two Cholesky-QR passes: V <- V R^{-1}, R^T R = V^T V
    for (int pass = 0; pass < 2; ++pass) {
        KEVD_BLAS(ctx, cublasDsyrk(ctx->blas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, m, (int)k, &one, V, (int)k,
                                   &zero, H, m));
        KEVD_SOLVER(ctx, cusolverDnDpotrf(ctx->solver, CUBLAS_FILL_MODE_UPPER, m, H, m, wd, lw3, flag + 1));
        KEVD_BLAS(ctx, cublasDtrsm(ctx->blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N,
                                   CUBLAS_DIAG_NON_UNIT, (int)k, m, &one, H, m, V, (int)k));
    }
    // H = V^T W V, eigenpairs ascending; V <- V Q
    KEVD_BLAS(ctx, cublasDsymm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, (int)k, m, &one, W, (int)k, V,
                               (int)k, &zero, Y, (int)k));
    KEVD_BLAS(ctx, cublasDgemm(ctx->blas, CUBLAS_OP_T, CUBLAS_OP_N, m, m, (int)k, &one, V, (int)k, Y, (int)k, &zero,
                               H, m));
    KEVD_SOLVER(ctx, cusolverDnDsyevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, m, H, m, mu,
                                      wd, lw2, flag + 2));
    KEVD_BLAS(ctx, cublasDgemm(ctx->blas, CUBLAS_OP_N, CUBLAS_OP_N, (int)k, m, m, &one, V, (int)k, H, m, &zero, Y,
                               (int)k));
    KEVD_CUDA(ctx, cudaMemcpyAsync(V, Y, (size_t)k * m * sizeof(double), cudaMemcpyDeviceToDevice, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(lam + (k - m), mu, (size_t)m * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return KEVD_OK;
}

template <typename T>
static int evd_impl(kevd_ctx* ctx, const T* F, int64_t N, int64_t k, int64_t ldF, int k_out,
                    double* lam_h, float* U, kevd_evd_info* info, kevd_evd_dump* dump,
                    cudaStream_t s) {
    int st = KEVD_OK;
    double* c1 = arena_get<double>(ctx, "ev.c1", k, &st);
    double* cq = arena_get<double>(ctx, "ev.cq", k, &st);
    double* dtil = arena_get<double>(ctx, "ev.dtil", N, &st);
    double* dinv = arena_get<double>(ctx, "ev.dinv", N, &st);
    double* qtil = arena_get<double>(ctx, "ev.qtil", N, &st);
    double* qinv = arena_get<double>(ctx, "ev.qinv", N, &st);
    double* w2 = arena_get<double>(ctx, "ev.w2", N, &st);
    double* A = arena_get<double>(ctx, "ev.A", (size_t)k * k, &st);
    double* B = arena_get<double>(ctx, "ev.B", (size_t)k * k, &st);
    double* W = arena_get<double>(ctx, "ev.W", (size_t)k * k, &st);
    double* lam = arena_get<double>(ctx, "ev.lam", k, &st);
    double* Z = arena_get<double>(ctx, "ev.Z", (size_t)k * k_out, &st);
    double* trsh = arena_get<double>(ctx, "ev.trsh", 2, &st);
    int* flags = arena_get<int>(ctx, "ev.flags", 4, &st);
    if (st != KEVD_OK) return st;
    int* hflags = static_cast<int*>(ctx->pinned);
    KEVD_CUDA(ctx, cudaMemsetAsync(flags, 0, 4 * sizeof(int), s));

    // FP32 factors run every streaming pass on a column-major copy (coalesced
    // along rows, K-major tensor-core tiles for the Grams)
    float* FT = nullptr;
    int64_t ldT = 0;
    unsigned* colmax = nullptr;
    if (sizeof(T) == 4) {
        KEVD_TRY(transposed(ctx, (const float*)F, ldF, N, k, &FT, &ldT, &colmax, s));
        const size_t vsm = (size_t)2 * k * sizeof(float);
        KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&evt_rowdot_kernel), (int)std::max(vsm, (size_t)1024)));
        ProfScope ps(ctx, "ev_passes", s);
        const int ny = (int)std::min<int64_t>(16, std::max<int64_t>(1, N / 8192));
        const int64_t rows_per = (N + ny - 1) / ny;
        double* cpart = arena_get<double>(ctx, "ev.cpartT", (size_t)ny * k, &st);
        if (st != KEVD_OK) return set_error(ctx, st, "bistochastic_evd: out of device memory");
        const dim3 cgrid(ceil_div(k, 16), ny);
        evt_colsum_kernel<<<cgrid, 512, 0, s>>>(FT, ldT, N, k, nullptr, rows_per, cpart);
        KEVD_LAUNCH(ctx);
        ev_sum_partials_kernel<<<ceil_div(k, 256), 256, 0, s>>>(cpart, ny, k, c1);
        KEVD_LAUNCH(ctx);
        evt_rowdot_kernel<<<ceil_div(N, 256), 256, vsm, s>>>(FT, ldT, N, k, c1, dtil, dinv, flags + 0);
        KEVD_LAUNCH(ctx);
        evt_colsum_kernel<<<cgrid, 512, 0, s>>>(FT, ldT, N, k, dinv, rows_per, cpart);
        KEVD_LAUNCH(ctx);
        ev_sum_partials_kernel<<<ceil_div(k, 256), 256, 0, s>>>(cpart, ny, k, cq);
        KEVD_LAUNCH(ctx);
        evt_rowdot_kernel<<<ceil_div(N, 256), 256, vsm, s>>>(FT, ldT, N, k, cq, qtil, qinv, flags + 1);
        KEVD_LAUNCH(ctx);
    } else {
        // pass 1: c1 = F^T 1;  pass 2: dtil = F c1, cq = F^T dtil^{-1}
        KEVD_TRY(colsum<T>(ctx, F, ldF, N, k, nullptr, c1, s));
        KEVD_TRY(rowdot<T>(ctx, F, ldF, N, k, c1, dtil, dinv, flags + 0, s));
        KEVD_TRY(colsum<T>(ctx, F, ldF, N, k, dinv, cq, s));
        // pass 3: qtil = F cq
        KEVD_TRY(rowdot<T>(ctx, F, ldF, N, k, cq, qtil, qinv, flags + 1, s));
    }
    KEVD_CUDA(ctx, cudaMemcpyAsync(hflags, flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    if (hflags[0]) return set_error(ctx, KEVD_ERR_NONPOS_DTIL, "bistochastic_evd: nonpositive dtil");
    if (hflags[1]) return set_error(ctx, KEVD_ERR_NONPOS_QTIL, "bistochastic_evd: nonpositive qtil");

    // Grams: A = (Dtil^{-1} F)^T (Dtil^{-1} F), B = (Qtil^{-1/2} F)^T (Qtil^{-1/2} F)
    if (sizeof(T) == 4) {
        // FP32 factor: two-term f16 tcgen05 Grams with FP64 accumulation across row chunks
        ev_rsqrt_kernel<<<ctx->num_sms * 4, 256, 0, s>>>(qtil, w2, N);
        KEVD_LAUNCH(ctx);
        KEVD_TRY(run_gram2_tc(ctx, FT, ldT, N, k, colmax, dinv, w2, A, B, s));
    } else {
        ev_square_kernel<<<ctx->num_sms * 4, 256, 0, s>>>(dinv, w2, N);
        KEVD_LAUNCH(ctx);
        KEVD_TRY(gram<T>(ctx, F, ldF, N, k, w2, A, s));
        KEVD_TRY(gram<T>(ctx, F, ldF, N, k, qinv, B, s));
    }
    if (dump) {
        KEVD_TRY(d2h(ctx, dump->c1, c1, k, s));
        KEVD_TRY(d2h(ctx, dump->dtil, dtil, N, s));
        KEVD_TRY(d2h(ctx, dump->cq, cq, k, s));
        KEVD_TRY(d2h(ctx, dump->qtil, qtil, N, s));
        KEVD_TRY(d2h(ctx, dump->A, A, (size_t)k * k, s));
        KEVD_TRY(d2h(ctx, dump->B, B, (size_t)k * k, s));
    }

    // dense 1: shift, Cholesky A + sI = L L^T
    KEVD_SOLVER(ctx, cusolverDnSetStream(ctx->solver, s));
    KEVD_BLAS(ctx, cublasSetStream(ctx->blas, s));
    int lwork = 0, lwork2 = 0;
    KEVD_SOLVER(ctx, cusolverDnDpotrf_bufferSize(ctx->solver, CUBLAS_FILL_MODE_LOWER, (int)k, A,
                                                 (int)k, &lwork));
    KEVD_SOLVER(ctx, cusolverDnDsyevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR,
                                                 CUBLAS_FILL_MODE_LOWER, (int)k, W, (int)k, lam,
                                                 &lwork2));
    double* work = arena_get<double>(ctx, "ev.work", (size_t)std::max(lwork, lwork2) + 1, &st);
    if (st != KEVD_OK) return st;
    {
        // s = u tr(A) (ks_kevd.cu:1447-1499).  The tensor-core Grams of an FP32
        // factor carry about 1e-5 relative error, which can leave a numerically
        // rank-deficient A indefinite by more than u tr(A); there potrf is
        // retried from a saved A with the shift raised 1e3-fold per attempt (the
        // leading eigenpairs are refined against F in FP64 afterwards).  The FP64
        // factor keeps the single attempt.
        ProfScope p1(ctx, "dense_potrf", s);
        const int attempts = (sizeof(T) == 4) ? 4 : 1;
        if (attempts > 1)
            KEVD_CUDA(ctx, cudaMemcpyAsync(W, A, (size_t)k * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
        double c = 1.0;
        for (int a = 0; a < attempts; ++a, c *= 1e3) {
            if (a > 0) {
                KEVD_CUDA(ctx, cudaMemcpyAsync(A, W, (size_t)k * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
                KEVD_CUDA(ctx, cudaMemsetAsync(flags + 2, 0, sizeof(int), s));
            }
            ev_trace_shift_kernel<<<1, 1024, 0, s>>>(A, k, trsh, c);
            KEVD_LAUNCH(ctx);
            KEVD_SOLVER(ctx, cusolverDnDpotrf(ctx->solver, CUBLAS_FILL_MODE_LOWER, (int)k, A, (int)k, work,
                                              lwork, flags + 2));
            if (a + 1 < attempts) {
                KEVD_CUDA(ctx, cudaMemcpyAsync(hflags + 2, flags + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
                KEVD_CUDA(ctx, cudaStreamSynchronize(s));
                if (hflags[2] == 0) break;
            }
        }
    }
    // dense 2: W = L^T B L
    const double one = 1.0;
    if (sizeof(T) == 4) {
        // FP32 factor: W only has to deliver the leading subspace, which is
        // refined against F afterwards, and B carries the FP32-level error of
        // the tensor-core Gram, so W is formed in FP32 (two strmm) and widened back
        ProfScope p2(ctx, "dense_trmm", s);
        float* Lf = arena_get<float>(ctx, "ev.Lf", (size_t)k * k, &st);
        float* Bf = arena_get<float>(ctx, "ev.Bf", (size_t)k * k, &st);
        float* Wf = arena_get<float>(ctx, "ev.Wf32", (size_t)k * k, &st);
        if (st != KEVD_OK) return set_error(ctx, st, "bistochastic_evd: out of device memory");
        const int g = ctx->num_sms * 4;
        ev_d2f_kernel<<<g, 256, 0, s>>>(A, Lf, k * k);
        KEVD_LAUNCH(ctx);
        ev_d2f_kernel<<<g, 256, 0, s>>>(B, Bf, k * k);
        KEVD_LAUNCH(ctx);
        const float onef = 1.f;
        KEVD_BLAS(ctx, cublasStrmm(ctx->blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                                   CUBLAS_DIAG_NON_UNIT, (int)k, (int)k, &onef, Lf, (int)k, Bf, (int)k, Wf,
                                   (int)k));
        KEVD_BLAS(ctx, cublasStrmm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                                   CUBLAS_DIAG_NON_UNIT, (int)k, (int)k, &onef, Lf, (int)k, Wf, (int)k, Wf,
                                   (int)k));
        ev_f2d_kernel<<<g, 256, 0, s>>>(Wf, W, k * k);
        KEVD_LAUNCH(ctx);
    } else {
        ProfScope p2(ctx, "dense_trmm", s);
        KEVD_BLAS(ctx, cublasDtrmm(ctx->blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N,
                                   CUBLAS_DIAG_NON_UNIT, (int)k, (int)k, &one, A, (int)k, B, (int)k, W,
                                   (int)k));
        KEVD_BLAS(ctx, cublasDtrmm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                                   CUBLAS_DIAG_NON_UNIT, (int)k, (int)k, &one, A, (int)k, W, (int)k, W,
                                   (int)k));
    }
    ev_symmetrize_kernel<<<ctx->num_sms * 4, 256, 0, s>>>(W, k);
    KEVD_LAUNCH(ctx);
    if (dump) KEVD_TRY(d2h(ctx, dump->W, W, (size_t)k * k, s));
    if (sizeof(T) == 4) {
        // FP32 factor: FP32 eigensolve + FP64 Rayleigh-Ritz of the leading subspace
        const int m = (int)std::min<int64_t>(k, k_out + 16);
        double* V = arena_get<double>(ctx, "ev.rrV", (size_t)k * m, &st);
        int* rrflag = arena_get<int>(ctx, "ev.rrflag", 3, &st);
        if (st != KEVD_OK) return set_error(ctx, st, "bistochastic_evd: out of device memory");
        KEVD_CUDA(ctx, cudaMemsetAsync(rrflag, 0, 3 * sizeof(int), s));
        KEVD_TRY(top_eigs_fp32_rr(ctx, W, k, m, lam, V, rrflag, s));
        int hrr[3];
        KEVD_CUDA(ctx, cudaMemcpyAsync(hrr, rrflag, sizeof(hrr), cudaMemcpyDeviceToHost, s));
        KEVD_CUDA(ctx, cudaStreamSynchronize(s));
        if (hrr[0] != 0 || hrr[1] != 0 || hrr[2] != 0)
            return set_error(ctx, KEVD_ERR_SYEVD, "bistochastic_evd: eigensolve failed, info %d/%d/%d", hrr[0],
                             hrr[1], hrr[2]);
        // Z = L^{-T} V[:, m-k_out:]
        KEVD_CUDA(ctx, cudaMemcpyAsync(Z, V + (size_t)(m - k_out) * k, (size_t)k * k_out * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s));
    } else {
        {
            ProfScope p3(ctx, "dense_syevd", s);
            KEVD_SOLVER(ctx, cusolverDnDsyevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                              (int)k, W, (int)k, lam, work, lwork2, flags + 3));
        }
        // Z = L^{-T} V[:, k-k_out:]
        KEVD_CUDA(ctx, cudaMemcpyAsync(Z, W + (k - k_out) * k, (size_t)k * k_out * sizeof(double),
                                       cudaMemcpyDeviceToDevice, s));
    }
    KEVD_BLAS(ctx, cublasDtrsm(ctx->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T,
                               CUBLAS_DIAG_NON_UNIT, (int)k, k_out, &one, A, (int)k, Z, (int)k));
    // pass 4: U = Dtil^{-1} F Z
    float* Yrr = nullptr;   // Dtil^{-1} U for the Rayleigh-Ritz T1 pass (FP32 factor)
    float* Urr = nullptr;   // the leading columns the Rayleigh-Ritz refines (U itself for k_out <= 32)
    const int m_rr = (int)std::min<int64_t>(k_out, 32);
    {
        ProfScope ps(ctx, "ev_u", s);
        if (sizeof(T) == 4 && k_out <= 32) {
            Yrr = arena_get<float>(ctx, "ev.Yrr", (size_t)N * 32, &st);
            if (st != KEVD_OK) return set_error(ctx, st, "bistochastic_evd: out of device memory");
            evt_u_kernel<<<ceil_div(N, 256), 256, 0, s>>>(FT, ldT, N, k, Z, k_out, dinv, U, Yrr);
            Urr = U;
        } else {
            ev_u_kernel<T><<<dim3(ceil_div(N, 64), ceil_div(k_out, 64)), 256, 0, s>>>(F, ldF, N, k, Z, k_out, dinv, U);
            if (sizeof(T) == 4) {
                // FP32 factor with k_out > 32: the leading 32 columns once more, with
                // Y, for their refinement (Z's last 32 columns)
                KEVD_LAUNCH(ctx);
                Yrr = arena_get<float>(ctx, "ev.Yrr", (size_t)N * 32, &st);
                Urr = arena_get<float>(ctx, "ev.Urr", (size_t)N * 32, &st);
                if (st != KEVD_OK) return set_error(ctx, st, "bistochastic_evd: out of device memory");
                evt_u_kernel<<<ceil_div(N, 256), 256, 0, s>>>(FT, ldT, N, k, Z + (size_t)(k_out - 32) * k, 32, dinv,
                                                              Urr, Yrr);
            }
        }
        KEVD_LAUNCH(ctx);
    }
    if (dump) KEVD_TRY(d2h(ctx, dump->Z, Z, (size_t)k * k_out, s));
    double htr[2];
    KEVD_CUDA(ctx, cudaMemcpyAsync(htr, trsh, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(hflags, flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (lam_h) KEVD_CUDA(ctx, cudaMemcpyAsync(lam_h, lam, k * sizeof(double), cudaMemcpyDeviceToHost, s));
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    if (sizeof(T) == 4 && hflags[2] == 0 && hflags[3] == 0) {
        // FP32 factor: refine the leading min(k_out, 32) eigenpairs by Rayleigh-Ritz
        // in FP64; with k_out > 32 the refined columns replace U's last 32
        double top[32];
        KEVD_TRY(rayleigh_ritz(ctx, FT, ldT, N, k, m_rr, Urr, Yrr, qinv, top, s));
        if (Urr != U)
            KEVD_CUDA(ctx, cudaMemcpy2DAsync(U + (k_out - 32), (size_t)k_out * sizeof(float), Urr, 32 * sizeof(float),
                                             32 * sizeof(float), (size_t)N, cudaMemcpyDeviceToDevice, s));
        if (lam_h)
            for (int j = 0; j < m_rr; ++j) lam_h[k - m_rr + j] = top[j];
    }
    if (info) {
        info->trace_A = htr[0];
        info->shift = htr[1];
    }
    if (hflags[2] != 0)
        return set_error(ctx, KEVD_ERR_POTRF, "bistochastic_evd: potrf failed, info %d", hflags[2]);
    if (hflags[3] != 0)
        return set_error(ctx, KEVD_ERR_SYEVD, "bistochastic_evd: syevd failed, info %d", hflags[3]);
    return KEVD_OK;
}

int run_weighted_gram(kevd_ctx* ctx, const void* F, int precision, int64_t N, int64_t k, int64_t ldF,
                      const double* s_dev, double* G, cudaStream_t st) {
    if (!F || !s_dev || !G || N < 1 || k < 1 || ldF < k)
        return set_error(ctx, KEVD_ERR_ARG, "weighted_gram: bad arguments");
    if (precision == KEVD_MIXED) {
        float* FT = nullptr;
        int64_t ldT = 0;
        unsigned* colmax = nullptr;
        KEVD_TRY(transposed(ctx, (const float*)F, ldF, N, k, &FT, &ldT, &colmax, st));
        return run_gram_tc(ctx, FT, ldT, N, k, colmax, s_dev, G, st);
    }
    if (precision != KEVD_FP64) return set_error(ctx, KEVD_ERR_ARG, "weighted_gram: unknown precision");
    int rc = KEVD_OK;
    double* w2 = arena_get<double>(ctx, "wg.w2", N, &rc);
    if (rc != KEVD_OK) return set_error(ctx, rc, "weighted_gram: out of device memory");
    ev_square_kernel<<<ctx->num_sms * 4, 256, 0, st>>>(s_dev, w2, N);
    KEVD_LAUNCH(ctx);
    KEVD_TRY(gram<double>(ctx, (const double*)F, ldF, N, k, w2, G, st));
    KEVD_CUDA(ctx, cudaStreamSynchronize(st));
    return KEVD_OK;
}

int run_weighted_gram2(kevd_ctx* ctx, const void* F, int precision, int64_t N, int64_t k, int64_t ldF,
                       const double* s_dev, const double* s2_dev, double* G, double* G2, cudaStream_t st) {
    if (!F || !s_dev || !s2_dev || !G || !G2 || N < 1 || k < 1 || ldF < k)
        return set_error(ctx, KEVD_ERR_ARG, "weighted_gram2: bad arguments");
    if (precision == KEVD_MIXED) {
        float* FT = nullptr;
        int64_t ldT = 0;
        unsigned* colmax = nullptr;
        KEVD_TRY(transposed(ctx, (const float*)F, ldF, N, k, &FT, &ldT, &colmax, st));
        return run_gram2_tc(ctx, FT, ldT, N, k, colmax, s_dev, s2_dev, G, G2, st);
    }
    KEVD_TRY(run_weighted_gram(ctx, F, precision, N, k, ldF, s_dev, G, st));
    return run_weighted_gram(ctx, F, precision, N, k, ldF, s2_dev, G2, st);
}

int run_bistochastic_evd(kevd_ctx* ctx, const void* F, int precision, int64_t N, int64_t k,
                         int64_t ldF, int k_out, double* lam, float* U, kevd_evd_info* info,
                         kevd_evd_dump* dump, cudaStream_t s) {
    if (!F || !U || N < 1 || k < 1 || ldF < k || k_out < 1 || k_out > 256 || k_out > k || k > 8192)
        return set_error(ctx, KEVD_ERR_ARG,
                         "bistochastic_evd: need F, U, N >= 1, 1 <= k <= 8192, ldF >= k, "
                         "1 <= k_out <= min(k, 256)");
    if (precision == KEVD_FP64)
        return evd_impl<double>(ctx, (const double*)F, N, k, ldF, k_out, lam, U, info, dump, s);
    if (precision == KEVD_MIXED)
        return evd_impl<float>(ctx, (const float*)F, N, k, ldF, k_out, lam, U, info, dump, s);
    return set_error(ctx, KEVD_ERR_ARG, "bistochastic_evd: unknown precision %d", precision);
}

}  // namespace kevd
