/*
 * Kuramoto-Sivashinsky state generator for the synthetic workloads.
 *
 * Advances u_t = -u u_x - u_xx - u_xxxx (periodic) in real-FFT coefficients
 * with exponential time-differencing RK4 (Kassam & Trefethen 2005), the
 * quadratic term dealiased by the 3/2 rule -- the scheme of the reference's
 * ks_datagen.py:21-101.  The phi-function coefficients are computed by the
 * caller; this file does the time stepping with its own radix-2/3 FFT so a
 * trajectory of millions of states takes seconds instead of the minutes a
 * NumPy loop needs.
 *
 * Coefficient convention: NumPy's unnormalised rfft (u = irfft(uhat)).
 */
#include <math.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double re, im;
} cplx;

static cplx cmul(cplx a, cplx b) {
    cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}

/* Recursive decimation-in-time FFT (sign -1 forward, +1 inverse, unscaled)
 * over n = 2^a 3^b points read with stride s; tw[k] = exp(sign 2 pi i k / NT). */
static void fft_rec(const cplx* x, int n, int s, cplx* out, const cplx* tw, int NT) {
    if (n == 1) {
        out[0] = x[0];
        return;
    }
    if (n == 2) {
        out[0].re = x[0].re + x[s].re;
        out[0].im = x[0].im + x[s].im;
        out[1].re = x[0].re - x[s].re;
        out[1].im = x[0].im - x[s].im;
        return;
    }
    const int ts = NT / n;  /* twiddle stride of this level */
    if (n % 2 == 0) {
        const int h = n / 2;
        fft_rec(x, h, 2 * s, out, tw, NT);
        fft_rec(x + s, h, 2 * s, out + h, tw, NT);
        for (int k = 0; k < h; ++k) {
            const cplx e = out[k];
            const cplx o = cmul(tw[k * ts], out[k + h]);
            out[k].re = e.re + o.re;
            out[k].im = e.im + o.im;
            out[k + h].re = e.re - o.re;
            out[k + h].im = e.im - o.im;
        }
        return;
    }
    /* radix 3 */
    const int t = n / 3;
    fft_rec(x, t, 3 * s, out, tw, NT);
    fft_rec(x + s, t, 3 * s, out + t, tw, NT);
    fft_rec(x + 2 * s, t, 3 * s, out + 2 * t, tw, NT);
    cplx tmp[3];
    for (int k = 0; k < t; ++k) {
        const cplx y0 = out[k];
        const cplx y1 = cmul(tw[k * ts], out[k + t]);
        const cplx y2 = cmul(tw[2 * k * ts], out[k + 2 * t]);
        for (int m = 0; m < 3; ++m) {
            const cplx w1 = tw[m * (NT / 3)];
            const cplx w2 = tw[(2 * m % 3) * (NT / 3)];
            const cplx a = cmul(w1, y1), b = cmul(w2, y2);
            tmp[m].re = y0.re + a.re + b.re;
            tmp[m].im = y0.im + a.im + b.im;
        }
        out[k] = tmp[0];
        out[k + t] = tmp[1];
        out[k + 2 * t] = tmp[2];
    }
}

typedef struct {
    int M, M2, Mext;
    cplx *twf_ext, *twi_ext, *twi_M;
    cplx *buf, *buf2;
} Plan;

static void make_tw(cplx* tw, int n, double sign) {
    for (int k = 0; k < n; ++k) {
        const double a = sign * 2.0 * M_PI * (double)k / (double)n;
        tw[k].re = cos(a);
        tw[k].im = sin(a);
    }
}

/* irfft of M2 coefficients onto n points (n >= 2 (M2-1)), unnormalised inverse / n */
static void irfft_n(const Plan* p, const cplx* vhat, int n, const cplx* twi, double* u) {
    cplx* full = p->buf;
    memset(full, 0, sizeof(cplx) * n);
    const int nk = p->M2;
    for (int k = 0; k < nk && k <= n / 2; ++k) full[k] = vhat[k];
    /* Hermitian completion; the Nyquist coefficient of the source is used
     * as a real value only when it lands on this grid's Nyquist */
    for (int k = 1; k < nk && k < (n + 1) / 2; ++k) {
        full[n - k].re = vhat[k].re;
        full[n - k].im = -vhat[k].im;
    }
    if (n % 2 == 0 && nk - 1 == n / 2) full[n / 2].im = 0.0;
    fft_rec(full, n, 1, p->buf2, twi, n);
    for (int j = 0; j < n; ++j) u[j] = p->buf2[j].re / (double)n;
}

static void nonlinear(const Plan* p, const cplx* g, const cplx* vhat, cplx* out, double* up) {
    irfft_n(p, vhat, p->Mext, p->twi_ext, up);
    cplx* sq = p->buf;
    for (int j = 0; j < p->Mext; ++j) {
        sq[j].re = up[j] * up[j];
        sq[j].im = 0.0;
    }
    fft_rec(sq, p->Mext, 1, p->buf2, p->twf_ext, p->Mext);
    for (int k = 0; k < p->M2; ++k) out[k] = cmul(g[k], p->buf2[k]);
}

/* coef: 6 x M2 doubles (E, E2, Q, f1, f2, f3); g: M2 complex (interleaved);
 * vhat: M2 complex state, advanced in place.  Writes n_snap states, the first
 * after n_warm steps.  Returns 0 on success. */
int ks_run(int M, const double* coef, const double* g_il, double* vhat_il, int64_t n_warm,
           int64_t n_snap, float* out32, double* out64) {
    if (M < 4 || M % 2 != 0) return 1;
    Plan p;
    p.M = M;
    p.M2 = M / 2 + 1;
    p.Mext = (3 * M) / 2;
    const int n_big = p.Mext > M ? p.Mext : M;
    p.twf_ext = malloc(sizeof(cplx) * p.Mext);
    p.twi_ext = malloc(sizeof(cplx) * p.Mext);
    p.twi_M = malloc(sizeof(cplx) * M);
    p.buf = malloc(sizeof(cplx) * n_big);
    p.buf2 = malloc(sizeof(cplx) * n_big);
    double* up = malloc(sizeof(double) * n_big);
    cplx *v = malloc(sizeof(cplx) * p.M2), *g = malloc(sizeof(cplx) * p.M2);
    cplx *Nv = malloc(sizeof(cplx) * p.M2), *a = malloc(sizeof(cplx) * p.M2);
    cplx *Na = malloc(sizeof(cplx) * p.M2), *b = malloc(sizeof(cplx) * p.M2);
    cplx *Nb = malloc(sizeof(cplx) * p.M2), *c = malloc(sizeof(cplx) * p.M2);
    cplx* Nc = malloc(sizeof(cplx) * p.M2);
    if (!p.twf_ext || !p.twi_ext || !p.twi_M || !p.buf || !p.buf2 || !up || !v || !g || !Nv || !a ||
        !Na || !b || !Nb || !c || !Nc)
        return 2;
    make_tw(p.twf_ext, p.Mext, -1.0);
    make_tw(p.twi_ext, p.Mext, +1.0);
    make_tw(p.twi_M, M, +1.0);
    const int m2 = p.M2;
    const double *E = coef, *E2 = coef + m2, *Q = coef + 2 * m2, *f1 = coef + 3 * m2,
                 *f2 = coef + 4 * m2, *f3 = coef + 5 * m2;
    for (int k = 0; k < m2; ++k) {
        v[k].re = vhat_il[2 * k];
        v[k].im = vhat_il[2 * k + 1];
        g[k].re = g_il[2 * k];
        g[k].im = g_il[2 * k + 1];
    }
    const int64_t total = n_warm + (n_snap > 0 ? n_snap - 1 : 0);
    int64_t saved = 0;
    for (int64_t n = 0; n <= total; ++n) {
        if (n >= n_warm && saved < n_snap) {
            irfft_n(&p, v, M, p.twi_M, up);
            for (int j = 0; j < M; ++j) {
                if (out32) out32[saved * M + j] = (float)up[j];
                if (out64) out64[saved * M + j] = up[j];
            }
            ++saved;
        }
        if (n == total) break;
        nonlinear(&p, g, v, Nv, up);
        for (int k = 0; k < m2; ++k) {
            a[k].re = E2[k] * v[k].re + Q[k] * Nv[k].re;
            a[k].im = E2[k] * v[k].im + Q[k] * Nv[k].im;
        }
        nonlinear(&p, g, a, Na, up);
        for (int k = 0; k < m2; ++k) {
            b[k].re = E2[k] * v[k].re + Q[k] * Na[k].re;
            b[k].im = E2[k] * v[k].im + Q[k] * Na[k].im;
        }
        nonlinear(&p, g, b, Nb, up);
        for (int k = 0; k < m2; ++k) {
            c[k].re = E2[k] * a[k].re + Q[k] * (2.0 * Nb[k].re - Nv[k].re);
            c[k].im = E2[k] * a[k].im + Q[k] * (2.0 * Nb[k].im - Nv[k].im);
        }
        nonlinear(&p, g, c, Nc, up);
        for (int k = 0; k < m2; ++k) {
            v[k].re = E[k] * v[k].re + f1[k] * Nv[k].re + f2[k] * (Na[k].re + Nb[k].re) + f3[k] * Nc[k].re;
            v[k].im = E[k] * v[k].im + f1[k] * Nv[k].im + f2[k] * (Na[k].im + Nb[k].im) + f3[k] * Nc[k].im;
        }
    }
    for (int k = 0; k < m2; ++k) {
        vhat_il[2 * k] = v[k].re;
        vhat_il[2 * k + 1] = v[k].im;
    }
    free(p.twf_ext); free(p.twi_ext); free(p.twi_M); free(p.buf); free(p.buf2); free(up);
    free(v); free(g); free(Nv); free(a); free(Na); free(b); free(Nb); free(c); free(Nc);
    return 0;
}
