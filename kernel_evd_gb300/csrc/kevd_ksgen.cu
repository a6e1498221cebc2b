// Kuramoto-Sivashinsky trajectories on the GPU: u_t = -u u_x - u_xx - u_xxxx
// (periodic), advanced in real-FFT coefficients by exponential time-differencing
// RK4 (Kassam & Trefethen 2005) with the quadratic term dealiased by the 3/2
// rule -- the scheme of the reference's data generator (ks_datagen.py:21-101)
// and of the host generator csrc/host/ksgen.c, in FP64.
//
// One warp per trajectory, four trajectories per CTA: each nonlinear evaluation
// is an inverse FFT onto Mext = 3M/2 points, a square and a forward FFT, done by
// a mixed-radix (2, 3) Stockham FFT in the warp's shared memory (butterflies
// spread over the 32 lanes, warp barriers between stages, no block-wide ones).  The phi-function coefficients E, E2, Q,
// f1, f2, f3 and the dealiased -1/2 d_x factor g are computed by the caller
// (contour integrals in FP64, as for the host generator).  Coefficient
// convention: NumPy's unnormalised rfft (u = irfft(uhat)).
//
// Precision: KEVD_FP64 steps in FP64 like the reference; on the GB300 an FP64
// warp instruction occupies the SM's FP64 pipe for many cycles and a step of
// M = 64 takes about 45 us, slower than the host generator for one trajectory.
// KEVD_MIXED steps in FP32 (FP64 coefficients rounded once), about 20x faster:
// the chaotic trajectory then leaves the FP64 one after a few Lyapunov times,
// while the sampled attractor is statistically the same.
#include "kevd_internal.cuh"

#include <cmath>
#include <vector>

namespace kevd {

namespace {

constexpr int kKsWarps = 4;                 // trajectories per CTA, one warp each
constexpr int kKsThreads = 32 * kKsWarps;
constexpr int kKsMaxM = 128;
constexpr int kKsMaxExt = 3 * kKsMaxM / 2;
constexpr int kKsMaxM2 = kKsMaxM / 2 + 1;

struct KsTraj {
    const double* coef;   // 6 x M2: E, E2, Q, f1, f2, f3
    const double* g;      // M2 complex (interleaved)
    const double* v0;     // M2 complex (interleaved)
    float* out;           // n_snap x M
    int64_t n_snap;
};

template <typename T> struct Cx;
template <> struct Cx<double> { using type = double2; };
template <> struct Cx<float> { using type = float2; };
template <typename T> using cx = typename Cx<T>::type;

template <typename T>
__device__ __forceinline__ cx<T> mk(T re, T im) {
    cx<T> r;
    r.x = re;
    r.y = im;
    return r;
}

template <typename T>
struct KsSmem {
    cx<T> buf[2][kKsMaxExt];
    cx<T> twe[kKsMaxExt];   // exp(+2 pi i t / Mext)
    cx<T> twm[kKsMaxM];     // exp(+2 pi i t / M)
    cx<T> v[kKsMaxM2], nv[kKsMaxM2], a[kKsMaxM2], na[kKsMaxM2];
    cx<T> b[kKsMaxM2], nb[kKsMaxM2], c[kKsMaxM2], nc[kKsMaxM2];
    cx<T> g[kKsMaxM2];
    T coef[6][kKsMaxM2];
};

template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> x, cx<T> y) {
    return mk<T>(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

// Stockham FFT of n = 2^p or 3 x 2^p points from x (radix 2 stages first, so Ns
// is a power of two at every stage), sign +1 (inverse, unscaled) or -1 (forward);
// tw[t] = exp(+2 pi i t / n).  One warp; returns the buffer holding the result
// (x or y) after a warp barrier.
template <typename T>
__device__ cx<T>* ks_fft(cx<T>* x, cx<T>* y, int n, const cx<T>* tw, int sign, int lane) {
    int lg = 0;   // log2 Ns
    int rem = n;
    while (rem > 1) {
        const int R = (rem % 2 == 0) ? 2 : 3;
        const int nr = n / R;
        const int Ns = 1 << lg;
        const int tstep = n / (Ns * R);
        for (int j = lane; j < nr; j += 32) {
            const int jm = j & (Ns - 1);
            cx<T> v0 = x[j], v1 = x[j + nr];
            cx<T> w1 = tw[jm * tstep];
            if (sign < 0) w1.y = -w1.y;
            v1 = cmul<T>(v1, w1);
            const int idx = ((j >> lg) << lg) * R + jm;
            if (R == 2) {
                y[idx] = mk<T>(v0.x + v1.x, v0.y + v1.y);
                y[idx + Ns] = mk<T>(v0.x - v1.x, v0.y - v1.y);
            } else {
                cx<T> v2 = x[j + 2 * nr];
                cx<T> w2 = tw[2 * jm * tstep];
                if (sign < 0) w2.y = -w2.y;
                v2 = cmul<T>(v2, w2);
                cx<T> c1 = tw[n / 3], c2 = tw[(2 * n) / 3];   // exp(+-2 pi i / 3), exp(+-4 pi i / 3)
                if (sign < 0) {
                    c1.y = -c1.y;
                    c2.y = -c2.y;
                }
                // V_q = v0 + v1 w^q + v2 w^(2q), w = exp(sign 2 pi i / 3)
                const cx<T> t1 = cmul<T>(v1, c1), t2 = cmul<T>(v2, c2);
                const cx<T> s1 = cmul<T>(v1, c2), s2 = cmul<T>(v2, c1);
                y[idx] = mk<T>(v0.x + v1.x + v2.x, v0.y + v1.y + v2.y);
                y[idx + Ns] = mk<T>(v0.x + t1.x + t2.x, v0.y + t1.y + t2.y);
                y[idx + 2 * Ns] = mk<T>(v0.x + s1.x + s2.x, v0.y + s1.y + s2.y);
            }
        }
        __syncwarp();
        cx<T>* t = x;
        x = y;
        y = t;
        ++lg;   // after a radix-3 stage (always the last) the loop ends
        rem /= R;
    }
    return x;
}

// Hermitian spectrum on n points from the m2 coefficients vh (as the host
// generator: the source's top coefficient is taken as real when it lands on this
// grid's Nyquist), then the inverse FFT; returns the buffer with n * u in .x.
template <typename T>
__device__ cx<T>* ks_irfft(KsSmem<T>& S, const cx<T>* vh, int m2, int n, const cx<T>* tw, int lane) {
    cx<T>* X = S.buf[0];
    for (int k = lane; k < n; k += 32) {
        cx<T> val = mk<T>(0, 0);
        if (k <= n / 2) {
            if (k < m2) val = vh[k];
            if ((n % 2) == 0 && k == n / 2 && m2 - 1 == n / 2) val.y = 0;
        } else {
            const int kk = n - k;
            if (kk >= 1 && kk < m2 && kk < (n + 1) / 2) val = mk<T>(vh[kk].x, -vh[kk].y);
        }
        X[k] = val;
    }
    __syncwarp();
    return ks_fft<T>(X, S.buf[1], n, tw, +1, lane);
}

// out = g * fft(irfft_Mext(vh)^2)[0:m2]
template <typename T>
__device__ void ks_nonlinear(KsSmem<T>& S, const cx<T>* vh, cx<T>* out, int m2, int ne, int lane) {
    cx<T>* U = ks_irfft<T>(S, vh, m2, ne, S.twe, lane);
    cx<T>* Y = (U == S.buf[0]) ? S.buf[1] : S.buf[0];
    for (int j = lane; j < ne; j += 32) {
        const T u = U[j].x / (T)ne;
        Y[j] = mk<T>(u * u, 0);
    }
    __syncwarp();
    cx<T>* F = ks_fft<T>(Y, U, ne, S.twe, -1, lane);
    for (int k = lane; k < m2; k += 32) out[k] = cmul<T>(S.g[k], F[k]);
    __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(kKsThreads) ks_etdrk4_kernel(const KsTraj* __restrict__ trajs, int n_traj, int M,
                                                               int64_t n_warm) {
    extern __shared__ __align__(16) unsigned char ks_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t_idx = blockIdx.x * kKsWarps + warp;
    if (t_idx >= n_traj) return;   // whole warps only: no block-wide barrier below
    KsSmem<T>& S = reinterpret_cast<KsSmem<T>*>(ks_raw)[warp];
    const KsTraj tj = trajs[t_idx];
    const int m2 = M / 2 + 1, ne = (3 * M) / 2;
    for (int t = lane; t < ne; t += 32) {
        double sv, cv;
        sincospi(2.0 * (double)t / (double)ne, &sv, &cv);
        S.twe[t] = mk<T>((T)cv, (T)sv);
    }
    for (int t = lane; t < M; t += 32) {
        double sv, cv;
        sincospi(2.0 * (double)t / (double)M, &sv, &cv);
        S.twm[t] = mk<T>((T)cv, (T)sv);
    }
    for (int k = lane; k < m2; k += 32) {
        S.v[k] = mk<T>((T)tj.v0[2 * k], (T)tj.v0[2 * k + 1]);
        S.g[k] = mk<T>((T)tj.g[2 * k], (T)tj.g[2 * k + 1]);
        for (int q = 0; q < 6; ++q) S.coef[q][k] = (T)tj.coef[q * m2 + k];
    }
    __syncwarp();
    const T *E = S.coef[0], *E2 = S.coef[1], *Q = S.coef[2], *f1 = S.coef[3], *f2 = S.coef[4], *f3 = S.coef[5];
    const int64_t total = n_warm + (tj.n_snap > 0 ? tj.n_snap - 1 : 0);
    int64_t saved = 0;
    for (int64_t n = 0; n <= total; ++n) {
        if (n >= n_warm && saved < tj.n_snap) {
            cx<T>* U = ks_irfft<T>(S, S.v, m2, M, S.twm, lane);
            for (int j = lane; j < M; j += 32) tj.out[saved * M + j] = (float)(U[j].x / (T)M);
            __syncwarp();
            ++saved;
        }
        if (n == total) break;
        ks_nonlinear<T>(S, S.v, S.nv, m2, ne, lane);
        for (int k = lane; k < m2; k += 32)
            S.a[k] = mk<T>(E2[k] * S.v[k].x + Q[k] * S.nv[k].x, E2[k] * S.v[k].y + Q[k] * S.nv[k].y);
        __syncwarp();
        ks_nonlinear<T>(S, S.a, S.na, m2, ne, lane);
        for (int k = lane; k < m2; k += 32)
            S.b[k] = mk<T>(E2[k] * S.v[k].x + Q[k] * S.na[k].x, E2[k] * S.v[k].y + Q[k] * S.na[k].y);
        __syncwarp();
        ks_nonlinear<T>(S, S.b, S.nb, m2, ne, lane);
        for (int k = lane; k < m2; k += 32)
            S.c[k] = mk<T>(E2[k] * S.a[k].x + Q[k] * ((T)2 * S.nb[k].x - S.nv[k].x),
                           E2[k] * S.a[k].y + Q[k] * ((T)2 * S.nb[k].y - S.nv[k].y));
        __syncwarp();
        ks_nonlinear<T>(S, S.c, S.nc, m2, ne, lane);
        for (int k = lane; k < m2; k += 32) {
            const cx<T> v = S.v[k], nv = S.nv[k], na = S.na[k], nb = S.nb[k], nc = S.nc[k];
            S.v[k] = mk<T>(E[k] * v.x + f1[k] * nv.x + f2[k] * (na.x + nb.x) + f3[k] * nc.x,
                           E[k] * v.y + f1[k] * nv.y + f2[k] * (na.y + nb.y) + f3[k] * nc.y);
        }
        __syncwarp();
    }
}

bool pow2(int n) { return n >= 4 && (n & (n - 1)) == 0; }

}  // namespace

int run_ks_generate(kevd_ctx* ctx, int32_t n_traj, int32_t M, int32_t precision, const double* coef,
                    const double* g, const double* vhat0, int64_t n_warm, const int64_t* n_snap,
                    float* const* out, cudaStream_t s) {
    if (precision != KEVD_FP64 && precision != KEVD_MIXED)
        return set_error(ctx, KEVD_ERR_ARG, "ks_generate: precision must be KEVD_FP64 or KEVD_MIXED (FP32 stepping)");
    if (n_traj < 1 || !coef || !g || !vhat0 || !n_snap || !out || n_warm < 0)
        return set_error(ctx, KEVD_ERR_ARG, "ks_generate: bad arguments");
    if (!pow2(M) || M > kKsMaxM)   // the FFTs run on M and 3M/2 = 3 x 2^p points
        return set_error(ctx, KEVD_ERR_ARG, "ks_generate: M must be a power of two in [4, %d]", kKsMaxM);
    const int m2 = M / 2 + 1;
    const size_t per = (size_t)(6 + 2 + 2) * m2;   // doubles per trajectory: coef, g, v0
    std::vector<double> h((size_t)n_traj * per);
    for (int t = 0; t < n_traj; ++t) {
        if (n_snap[t] < 0 || (n_snap[t] > 0 && !out[t]))
            return set_error(ctx, KEVD_ERR_ARG, "ks_generate: trajectory %d: bad output", t);
        double* d = h.data() + (size_t)t * per;
        for (int e = 0; e < 6 * m2; ++e) d[e] = coef[(size_t)t * 6 * m2 + e];
        for (int e = 0; e < 2 * m2; ++e) d[6 * m2 + e] = g[(size_t)t * 2 * m2 + e];
        for (int e = 0; e < 2 * m2; ++e) d[8 * m2 + e] = vhat0[(size_t)t * 2 * m2 + e];
    }
    int rc = KEVD_OK;
    double* dpar = arena_get<double>(ctx, "ks.par", h.size(), &rc);
    KsTraj* dtj = arena_get<KsTraj>(ctx, "ks.traj", (size_t)n_traj, &rc);
    if (rc != KEVD_OK) return set_error(ctx, rc, "ks_generate: out of device memory");
    std::vector<KsTraj> ht((size_t)n_traj);
    for (int t = 0; t < n_traj; ++t) {
        const double* d = dpar + (size_t)t * per;
        ht[t] = KsTraj{d, d + 6 * m2, d + 8 * m2, out[t], n_snap[t]};
    }
    KEVD_CUDA(ctx, cudaMemcpyAsync(dpar, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    KEVD_CUDA(ctx, cudaMemcpyAsync(dtj, ht.data(), ht.size() * sizeof(KsTraj), cudaMemcpyHostToDevice, s));
    {
        ProfScope ps(ctx, "ks_generate", s);
        const int grid = (n_traj + kKsWarps - 1) / kKsWarps;
        if (precision == KEVD_FP64) {
            const size_t sm = kKsWarps * sizeof(KsSmem<double>);
            KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&ks_etdrk4_kernel<double>), sm));
            ks_etdrk4_kernel<double><<<grid, kKsThreads, sm, s>>>(dtj, n_traj, M, n_warm);
        } else {
            const size_t sm = kKsWarps * sizeof(KsSmem<float>);
            KEVD_CUDA(ctx, raise_smem_limit(reinterpret_cast<const void*>(&ks_etdrk4_kernel<float>), sm));
            ks_etdrk4_kernel<float><<<grid, kKsThreads, sm, s>>>(dtj, n_traj, M, n_warm);
        }
        KEVD_LAUNCH(ctx);
    }
    // the host arrays are released on return: wait for the copies
    KEVD_CUDA(ctx, cudaStreamSynchronize(s));
    return KEVD_OK;
}

}  // namespace kevd
