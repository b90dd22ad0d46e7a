/*
 * or_fft.c -- CPU discrete Fourier transform used by the oracle and by the
 * MEX stand-in that links the reference sources.  TEST INFRASTRUCTURE ONLY:
 * nothing in the shipped library calls this file.
 *
 * The reference k-space gateways hand the spread grids to MATLAB's fft2 and
 * ifft2 (PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:80-81,176-177,
 * PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:314-317,452-453).
 * MATLAB is a closed third-party dependency, so its published definition is
 * restated here:
 *
 *     fft :  X[k] = sum_j x[j] exp(-2*pi*i*j*k/n)
 *     ifft:  x[j] = (1/n) sum_k X[k] exp(+2*pi*i*j*k/n)
 *
 * fft2/ifft2 apply the 1-D transform along the columns (contiguous, length My)
 * and then along the rows (stride My) of a column-major My x Mx array.  The
 * complex data is held as separate real and imaginary arrays, the storage
 * MATLAB's mxGetPr/mxGetPi API exposes.
 *
 * Algorithm: recursive decimation-in-time mixed radix (Cooley & Tukey 1965)
 * for sizes whose prime factors are at most OR_FFT_MAXRADIX, and Bluestein's
 * chirp-z algorithm (Bluestein 1970) over a power-of-two length otherwise.
 * Twiddles are evaluated with reduced integer arguments so that the phase is
 * exact before the single sin/cos call.
 */
#include "or_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OR_FFT_MAXRADIX 13
#define OR_PI 3.14159265358979323846264338327950288

struct or_fft_plan {
    int n;
    int nfac;
    int fac[40];
    double* twr; /* exp(-2 pi i k / n), k = 0..n-1 */
    double* twi;
    /* Bluestein */
    int bluestein;
    int m;
    double* chr; /* chirp exp(-i pi k^2 / n), k = 0..n-1 */
    double* chi;
    double* bhr; /* FFT of the conjugate chirp, length m */
    double* bhi;
    struct or_fft_plan* sub; /* power-of-two plan of length m */
};

/* exp(-2 pi i num/den) with num reduced modulo den first. */
static void or_unit_root(long long num, long long den, double* c, double* s) {
    num %= den;
    if (num < 0) num += den;
    /* map to the nearest octant-friendly angle: use symmetric argument */
    double ang;
    if (2 * num <= den)
        ang = -2.0 * OR_PI * (double)num / (double)den;
    else
        ang = 2.0 * OR_PI * (double)(den - num) / (double)den;
    *c = cos(ang);
    *s = sin(ang);
}

static int or_factorize(int n, int* fac) {
    int nf = 0;
    /* radix 4 first for fewer passes, then the primes */
    while (n % 4 == 0) { fac[nf++] = 4; n /= 4; }
    for (int p = 2; p <= n && p <= OR_FFT_MAXRADIX; p++) {
        while (n % p == 0) { fac[nf++] = p; n /= p; }
    }
    if (n > 1) return -1; /* a prime factor larger than OR_FFT_MAXRADIX remains */
    return nf;
}

or_fft_plan* or_fft_plan_create(int n) {
    if (n <= 0) return NULL;
    or_fft_plan* p = (or_fft_plan*)calloc(1, sizeof(or_fft_plan));
    if (!p) return NULL;
    p->n = n;
    int nf = or_factorize(n, p->fac);
    if (nf >= 0) {
        p->nfac = nf;
        p->twr = (double*)malloc(sizeof(double) * (size_t)n);
        p->twi = (double*)malloc(sizeof(double) * (size_t)n);
        if (!p->twr || !p->twi) { or_fft_plan_destroy(p); return NULL; }
        for (int k = 0; k < n; k++) or_unit_root(k, n, &p->twr[k], &p->twi[k]);
        return p;
    }
    /* Bluestein over a power-of-two length m >= 2n-1 */
    p->bluestein = 1;
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    p->m = m;
    p->sub = or_fft_plan_create(m);
    p->chr = (double*)malloc(sizeof(double) * (size_t)n);
    p->chi = (double*)malloc(sizeof(double) * (size_t)n);
    p->bhr = (double*)calloc((size_t)m, sizeof(double));
    p->bhi = (double*)calloc((size_t)m, sizeof(double));
    if (!p->sub || !p->chr || !p->chi || !p->bhr || !p->bhi) { or_fft_plan_destroy(p); return NULL; }
    for (int k = 0; k < n; k++) {
        /* exp(-i pi k^2/n) = exp(-2 pi i (k^2 mod 2n) / (2n)) */
        long long k2 = ((long long)k * (long long)k) % (2LL * n);
        or_unit_root(k2, 2LL * n, &p->chr[k], &p->chi[k]);
    }
    /* b[k] = conj(chirp[k]) for k in (-n, n), wrapped into length m */
    p->bhr[0] = p->chr[0];
    p->bhi[0] = -p->chi[0];
    for (int k = 1; k < n; k++) {
        p->bhr[k] = p->chr[k];
        p->bhi[k] = -p->chi[k];
        p->bhr[m - k] = p->chr[k];
        p->bhi[m - k] = -p->chi[k];
    }
    or_fft_exec(p->sub, p->bhr, p->bhi, 1, 0);
    return p;
}

void or_fft_plan_destroy(or_fft_plan* p) {
    if (!p) return;
    free(p->twr);
    free(p->twi);
    free(p->chr);
    free(p->chi);
    free(p->bhr);
    free(p->bhi);
    if (p->sub) or_fft_plan_destroy(p->sub);
    free(p);
}

/*
 * Forward transform of length n read from (xr, xi) with stride `is`, written
 * contiguously to (yr, yi).  Twiddles come from the top-level table of length
 * N (tw stride = N/n).
 */
static void or_fft_rec(const or_fft_plan* P, int n, const int* fac, const double* xr, const double* xi,
                       long is, double* yr, double* yi, int twstride, double* scr, double* sci) {
    if (n == 1) {
        yr[0] = xr[0];
        yi[0] = xi[0];
        return;
    }
    int p = fac[0];
    int m = n / p;
    /* sub-transforms of the p decimated sequences */
    for (int q = 0; q < p; q++)
        or_fft_rec(P, m, fac + 1, xr + q * is, xi + q * is, is * p, yr + q * m, yi + q * m, twstride * p, scr, sci);
    /* butterflies: X[k + s m] = sum_q W_n^{q (k + s m)} Y_q[k] */
    const int N = P->n;
    double tr[OR_FFT_MAXRADIX], ti[OR_FFT_MAXRADIX];
    for (int k = 0; k < m; k++) {
        for (int q = 0; q < p; q++) {
            long tix = (long)q * k * twstride % N;
            double wr = P->twr[tix], wi = P->twi[tix];
            double ar = yr[q * m + k], ai = yi[q * m + k];
            tr[q] = ar * wr - ai * wi;
            ti[q] = ar * wi + ai * wr;
        }
        for (int s = 0; s < p; s++) {
            double sr = 0.0, si = 0.0;
            for (int q = 0; q < p; q++) {
                /* W_p^{q s} = W_N^{q s N/p} */
                long tix = ((long)q * s % p) * (N / p);
                double wr = P->twr[tix], wi = P->twi[tix];
                sr += tr[q] * wr - ti[q] * wi;
                si += tr[q] * wi + ti[q] * wr;
            }
            scr[s] = sr;
            sci[s] = si;
        }
        for (int s = 0; s < p; s++) {
            yr[k + s * m] = scr[s];
            yi[k + s * m] = sci[s];
        }
    }
}

static void or_fft_smooth(const or_fft_plan* P, double* re, double* im, int inverse) {
    int n = P->n;
    double* xr = (double*)malloc(sizeof(double) * (size_t)n * 2);
    double* xi = xr + n;
    double scr[OR_FFT_MAXRADIX], sci[OR_FFT_MAXRADIX];
    memcpy(xr, re, sizeof(double) * (size_t)n);
    if (inverse)
        for (int k = 0; k < n; k++) xi[k] = -im[k];
    else
        memcpy(xi, im, sizeof(double) * (size_t)n);
    or_fft_rec(P, n, P->fac, xr, xi, 1, re, im, 1, scr, sci);
    if (inverse)
        for (int k = 0; k < n; k++) im[k] = -im[k];
    free(xr);
}

static void or_fft_bluestein(const or_fft_plan* P, double* re, double* im, int inverse) {
    int n = P->n, m = P->m;
    double* ar = (double*)calloc((size_t)m * 2, sizeof(double));
    double* ai = ar + m;
    for (int k = 0; k < n; k++) {
        double xr = re[k], xi = inverse ? -im[k] : im[k];
        ar[k] = xr * P->chr[k] - xi * P->chi[k];
        ai[k] = xr * P->chi[k] + xi * P->chr[k];
    }
    or_fft_exec(P->sub, ar, ai, 1, 0);
    for (int k = 0; k < m; k++) {
        double xr = ar[k], xi = ai[k];
        ar[k] = xr * P->bhr[k] - xi * P->bhi[k];
        ai[k] = xr * P->bhi[k] + xi * P->bhr[k];
    }
    or_fft_exec(P->sub, ar, ai, 1, 1); /* unnormalised inverse */
    double inv_m = 1.0 / (double)m;
    for (int k = 0; k < n; k++) {
        double xr = ar[k] * inv_m, xi = ai[k] * inv_m;
        double yr = xr * P->chr[k] - xi * P->chi[k];
        double yi = xr * P->chi[k] + xi * P->chr[k];
        re[k] = yr;
        im[k] = inverse ? -yi : yi;
    }
    free(ar);
}

/* In-place 1-D transform of (re, im) with unit stride.  `inverse` selects
 * exp(+i...), `normalise` divides by n (MATLAB's ifft convention). */
void or_fft_exec(const or_fft_plan* P, double* re, double* im, int unit_stride_unused, int inverse) {
    (void)unit_stride_unused;
    if (P->bluestein)
        or_fft_bluestein(P, re, im, inverse);
    else
        or_fft_smooth(P, re, im, inverse);
}

/*
 * MATLAB fft2 / ifft2 on a column-major My x Mx complex array (separate
 * real/imaginary storage).  ifft2 includes the 1/(Mx*My) factor.
 */
int or_fft2(int My, int Mx, double* re, double* im, int inverse) {
    if (My <= 0 || Mx <= 0) return -1;
    or_fft_plan* py = or_fft_plan_create(My);
    or_fft_plan* px = or_fft_plan_create(Mx);
    if (!py || !px) { or_fft_plan_destroy(py); or_fft_plan_destroy(px); return -2; }
    /* columns: contiguous */
#pragma omp parallel for schedule(static)
    for (int x = 0; x < Mx; x++) or_fft_exec(py, re + (size_t)x * My, im + (size_t)x * My, 1, inverse);
    /* rows: gather stride My */
#pragma omp parallel
    {
        double* tr = (double*)malloc(sizeof(double) * (size_t)Mx * 2);
        double* ti = tr + Mx;
#pragma omp for schedule(static)
        for (int y = 0; y < My; y++) {
            for (int x = 0; x < Mx; x++) {
                tr[x] = re[(size_t)x * My + y];
                ti[x] = im[(size_t)x * My + y];
            }
            or_fft_exec(px, tr, ti, 1, inverse);
            for (int x = 0; x < Mx; x++) {
                re[(size_t)x * My + y] = tr[x];
                im[(size_t)x * My + y] = ti[x];
            }
        }
        free(tr);
    }
    if (inverse) {
        double s = 1.0 / ((double)Mx * (double)My);
        size_t n = (size_t)Mx * My;
#pragma omp parallel for schedule(static)
        for (long k = 0; k < (long)n; k++) {
            re[k] *= s;
            im[k] *= s;
        }
    }
    or_fft_plan_destroy(py);
    or_fft_plan_destroy(px);
    return 0;
}

/* 1-D convenience entry (tests): in-place, MATLAB fft/ifft convention. */
int or_fft1(int n, double* re, double* im, int inverse) {
    or_fft_plan* p = or_fft_plan_create(n);
    if (!p) return -1;
    or_fft_exec(p, re, im, 1, inverse);
    if (inverse) {
        double s = 1.0 / (double)n;
        for (int k = 0; k < n; k++) { re[k] *= s; im[k] *= s; }
    }
    or_fft_plan_destroy(p);
    return 0;
}
