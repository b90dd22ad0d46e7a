/*
 * or_ewald.c -- CPU oracle restating annabroms/FastTools2D's spectral Ewald
 * path for the 2-D Stokeslet and stresslet.  TEST INFRASTRUCTURE ONLY (see
 * or_ewald.h); the GPU library never links or calls this file.
 *
 * The restatement keeps the reference's arithmetic formulas, loop structure,
 * index conventions and OpenMP parallelisation so that it can also be timed
 * as the CPU baseline where the reference sources themselves cannot be built
 * (they use x86 SSE intrinsics and MATLAB's MEX API).  The only deliberate
 * deviations are:
 *   - the exponential integral E1 is this project's own (series + continued
 *     fraction, see or_expint_e1), not the reference's rational fits;
 *   - the fft2/ifft2 callbacks into MATLAB are replaced by or_fft.c;
 *   - the x86 SSE2/SSE3 pair arithmetic is written as scalar FP64 code.
 */
#include "or_ewald.h"

#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "or_fft.h"

#define OR_PI 3.1415926535897932385
#define OR_EULER 0.57721566490153286060651209008240243

int or_num_threads(void) { return omp_get_max_threads(); }

/* ------------------------------------------------------------------------
 * Exponential integral E1(x), x > 0.
 *   x <= 1: power series, Abramowitz & Stegun 5.1.11
 *           E1(x) = -gamma - ln x - sum_{k>=1} (-x)^k / (k k!)
 *   x >  1: continued fraction, Abramowitz & Stegun 5.1.22 in its even
 *           form e^{-x} / (x+1 - 1/(x+3 - 4/(x+5 - ...))), evaluated with the
 *           modified Lentz method (Thompson & Barnett 1986).
 * ---------------------------------------------------------------------- */
double or_expint_e1(double x) {
    if (x != x) return x;
    if (x <= 0.0) return x == 0.0 ? INFINITY : NAN;
    if (x <= 1.0) {
        double term = x, sum = x;
        for (int k = 2; k < 80; k++) {
            term *= -x / (double)k;
            double add = term / (double)k;
            sum += add;
            if (fabs(add) < 1e-19 * fabs(sum)) break;
        }
        return -OR_EULER - log(x) + sum;
    }
    if (x > 740.0) return 0.0;
    const double tiny = 1e-300;
    double b = x + 1.0;
    double c = 1.0 / tiny;
    double d = 1.0 / b;
    double h = d;
    for (int i = 1; i < 2000; i++) {
        double a = -(double)i * (double)i;
        b += 2.0;
        d = a * d + b;
        if (fabs(d) < tiny) d = tiny;
        c = b + a / c;
        if (fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        double del = c * d;
        h *= del;
        if (fabs(del - 1.0) <= 1e-16) break;
    }
    return h * exp(-x);
}

/* ------------------------------------------------------------------------
 * MATLAB rat(x) with its default tolerance 1e-6*|x|: nearest-integer
 * continued-fraction expansion (the algorithm documented for rat).
 * Used by the drivers at StokesSLP_ewald_2p.m:85 / StokesDLP_ewald_2p.m:105.
 * ---------------------------------------------------------------------- */
static double or_matlab_round(double v) { return round(v); } /* half away from zero, as MATLAB */

double or_rat(double x, int* num, int* den) {
    double tol = 1e-6 * fabs(x);
    double lastn = 1.0, lastd = 0.0;
    double n = or_matlab_round(x), d = 1.0;
    double frac = x - n;
    int guard = 0;
    while (fabs(x - n / d) >= tol && guard++ < 64) {
        double flip = 1.0 / frac;
        double step = or_matlab_round(flip);
        frac = flip - step;
        double save = n;
        n = n * step + lastn;
        lastn = save;
        save = d;
        d = d * step + lastd;
        lastd = save;
    }
    double sgn = d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0);
    *num = (int)(n * sgn);
    *den = (int)fabs(d);
    return n / d;
}

/* MATLAB mod(a, m) for m > 0, including its documented compensation that
 * returns exactly 0 when a/m is an integer to within round-off. */
static double or_matlab_mod(double a, double m) {
    double q = a / m;
    double rq = round(q);
    if (fabs(q - rq) <= DBL_EPSILON * fabs(q)) return 0.0;
    double r = a - floor(q) * m;
    return r;
}

/* ------------------------------------------------------------------------
 * Cell list: ewald_tools.cpp:7-80.  Boxes are nside_x x nside_y, numbered
 * box_y*nside_x + box_x; a counting sort keeps each box's points in input
 * order.
 * ---------------------------------------------------------------------- */
int or_assign(const double* psrc, const double* ptar, double Lx, double Ly, int nsrc, int ntar, int nside_x,
              int nside_y, int* particle_offsets_src, int* box_offsets_src, int* nsources_in_box,
              int* particle_offsets_tar, int* box_offsets_tar, int* ntargets_in_box) {
    int nb = nside_x * nside_y;
    int* in_box_src = (int*)malloc(sizeof(int) * (size_t)(nsrc > 0 ? nsrc : 1));
    int* in_box_tar = (int*)malloc(sizeof(int) * (size_t)(ntar > 0 ? ntar : 1));
    int* cur_src = (int*)malloc(sizeof(int) * (size_t)(nb + 1));
    int* cur_tar = (int*)malloc(sizeof(int) * (size_t)(nb + 1));
    if (!in_box_src || !in_box_tar || !cur_src || !cur_tar) {
        free(in_box_src); free(in_box_tar); free(cur_src); free(cur_tar);
        return -1;
    }
    for (int j = 0; j < nb; j++) nsources_in_box[j] = ntargets_in_box[j] = 0;
    for (int j = 0; j < nsrc; j++) {
        int bx = (int)floor(nside_x * (psrc[2 * j] / Lx + 0.5));
        int by = (int)floor(nside_y * (psrc[2 * j + 1] / Ly + 0.5));
        if (bx < 0) bx = 0;
        if (bx >= nside_x) bx = nside_x - 1;
        if (by < 0) by = 0;
        if (by >= nside_y) by = nside_y - 1;
        in_box_src[j] = by * nside_x + bx;
        nsources_in_box[in_box_src[j]]++;
    }
    for (int j = 0; j < ntar; j++) {
        int bx = (int)floor(nside_x * (ptar[2 * j] / Lx + 0.5));
        int by = (int)floor(nside_y * (ptar[2 * j + 1] / Ly + 0.5));
        if (bx < 0) bx = 0;
        if (bx >= nside_x) bx = nside_x - 1;
        if (by < 0) by = 0;
        if (by >= nside_y) by = nside_y - 1;
        in_box_tar[j] = by * nside_x + bx;
        ntargets_in_box[in_box_tar[j]]++;
    }
    box_offsets_src[0] = cur_src[0] = 0;
    box_offsets_tar[0] = cur_tar[0] = 0;
    for (int j = 1; j <= nb; j++) {
        box_offsets_src[j] = cur_src[j] = box_offsets_src[j - 1] + nsources_in_box[j - 1];
        box_offsets_tar[j] = cur_tar[j] = box_offsets_tar[j - 1] + ntargets_in_box[j - 1];
    }
    for (int j = 0; j < nsrc; j++) particle_offsets_src[cur_src[in_box_src[j]]++] = j;
    for (int j = 0; j < ntar; j++) particle_offsets_tar[cur_tar[in_box_tar[j]]++] = j;
    free(in_box_src);
    free(in_box_tar);
    free(cur_src);
    free(cur_tar);
    return 0;
}

/* ------------------------------------------------------------------------
 * First window node and in-cell offset: ewald_tools.cpp:86-114.
 * ---------------------------------------------------------------------- */
void or_find_closest_node(double x, double y, double Lx, double Ly, double h, int P, int* mx, int* my, double* px,
                          double* py) {
    const double TOL = 1e-13;
    *px = x - h * floor(x / h);
    *py = y - h * floor(y / h);
    double lhx = Lx / 2.0, lhy = Ly / 2.0;
    *mx = (int)(floor((x + lhx) / h) - P / 2);
    *my = (int)(floor((y + lhy) / h) - P / 2);
    if (fabs(*px) < TOL || fabs(*px - h) < TOL) *px = 0;
    if (fabs(*py) < TOL || fabs(*py - h) < TOL) *py = 0;
    if (*px == 0 && remainder((x + lhx) / h - P / 2, 1) < 0) (*mx)++;
    if (*py == 0 && remainder((y + lhy) / h - P / 2, 1) < 0) (*my)++;
}

/* ------------------------------------------------------------------------
 * Gaussian spreading with fast Gaussian gridding: ewald_tools.cpp:120-199.
 * Grid storage is column-major My x Mx: H[x*My + y].  As in the reference,
 * OpenMP threads take sources and serialise on one lock per grid column.
 * ---------------------------------------------------------------------- */
void or_spread(double* H1, double* H2, double* e1, const double* psrc, const double* f, int Nsrc, double Lx,
               double Ly, double xi, double w, double eta, int P, int Mx, int My, double h) {
    double t0 = -2 * xi * xi / eta * h * h;
    for (int j = -P / 2; j <= P / 2; j++) e1[j + P / 2] = exp(t0 * j * j);
    omp_lock_t* locks = (omp_lock_t*)malloc(sizeof(omp_lock_t) * (size_t)Mx);
    for (int j = 0; j < Mx; j++) omp_init_lock(&locks[j]);
#pragma omp parallel for
    for (int k = 0; k < Nsrc; k++) {
        double xs = psrc[2 * k], ys = psrc[2 * k + 1];
        int mx, my;
        double px, py;
        or_find_closest_node(xs, ys, Lx, Ly, h, P, &mx, &my, &px, &py);
        double t = -2 * xi * xi / eta;
        double ex = exp(t * (px * px + py * py + 2 * w * px));
        double e4y = exp(2 * t * w * py);
        double e3x = exp(-2 * t * h * px);
        double e3y = exp(-2 * t * h * py);
        for (int x = 0; x < P + 1; x++) {
            double ey = ex * e4y * e1[x];
            int col = ((x + mx) % Mx + Mx) % Mx;
            int xidx = col * My;
            omp_set_lock(&locks[col]);
            for (int y = 0; y < P + 1; y++) {
                double v = ey * e1[y];
                int idx = (((y + my) % My + My) % My) + xidx;
                H1[idx] += v * f[2 * k];
                H2[idx] += v * f[2 * k + 1];
                ey *= e3y;
            }
            omp_unset_lock(&locks[col]);
            ex *= e3x;
        }
    }
    for (int j = 0; j < Mx; j++) omp_destroy_lock(&locks[j]);
    free(locks);
}

/* ------------------------------------------------------------------------
 * Gather with quadrature: ewald_tools.cpp:206-271.  Adds into
 * output[total_components*k + component_number-1].
 * ---------------------------------------------------------------------- */
void or_gather(const double* H, int total_components, int component_number, const double* e1, const double* ptar,
               double* output, int Ntar, double Lx, double Ly, double xi, double w, double eta, int P, int Mx,
               int My, double h) {
#pragma omp parallel for
    for (int k = 0; k < Ntar; k++) {
        int ti = total_components * k + component_number - 1;
        double xt = ptar[2 * k], yt = ptar[2 * k + 1];
        int mx, my;
        double px, py;
        or_find_closest_node(xt, yt, Lx, Ly, h, P, &mx, &my, &px, &py);
        double t = -2 * xi * xi / eta;
        double ex = exp(t * (px * px + py * py + 2 * w * px));
        double e4y = exp(2 * t * w * py);
        double e3x = exp(-2 * t * h * px);
        double e3y = exp(-2 * t * h * py);
        double acc = output[ti];
        for (int x = 0; x < P + 1; x++) {
            double ey = ex * e4y * e1[x];
            int xidx = (((x + mx) % Mx + Mx) % Mx) * My;
            for (int y = 0; y < P + 1; y++) {
                double v = ey * e1[y];
                int idx = (((y + my) % My + My) % My) + xidx;
                acc += v * H[idx];
                ey *= e3y;
            }
            ex *= e3x;
        }
        double s = 4 * xi * xi / eta;
        s = s * s * h * h / OR_PI;
        output[ti] = acc * (s / (4 * OR_PI));
    }
}

/* ------------------------------------------------------------------------
 * Real-space Stokeslet sum over the cell list: mex_stokes_slp_real.cpp:58-357.
 * Own box: every pair, with the self term (-1-gamma/2-log xi) f when
 * r^2 < 1e-15.  Eight neighbour boxes (periodic, with image offsets): pairs
 * with r^2 < Lx*Ly/(nside_x*nside_y).  Result divided by 4*pi.
 * ---------------------------------------------------------------------- */
static inline void or_slp_pair(double rx, double ry, double r2, double xi2, double fx, double fy, double* ux,
                               double* uy) {
    double x = r2 * xi2;
    double e = exp(-x);
    double E = or_expint_e1(x);
    double g = e / r2;
    *ux += 0.5 * E * fx + (rx * ry * fy - ry * ry * fx) * g;
    *uy += 0.5 * E * fy + (rx * ry * fx - rx * rx * fy) * g;
}

static const int or_ilist_x[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
static const int or_ilist_y[8] = {-1, 0, 1, -1, 1, -1, 0, 1};

typedef struct {
    int *po_s, *bo_s, *ns, *po_t, *bo_t, *nt;
    double *ps, *pt;
} or_cells;

static int or_cells_build(or_cells* c, const double* psrc, int Nsrc, const double* ptar, int Ntar, int nside_x,
                          int nside_y, double Lx, double Ly) {
    int nb = nside_x * nside_y;
    memset(c, 0, sizeof(*c));
    c->po_s = (int*)malloc(sizeof(int) * (size_t)(Nsrc + 1));
    c->po_t = (int*)malloc(sizeof(int) * (size_t)(Ntar + 1));
    c->bo_s = (int*)malloc(sizeof(int) * (size_t)(nb + 1));
    c->bo_t = (int*)malloc(sizeof(int) * (size_t)(nb + 1));
    c->ns = (int*)malloc(sizeof(int) * (size_t)nb);
    c->nt = (int*)malloc(sizeof(int) * (size_t)nb);
    c->ps = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    c->pt = (double*)malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    if (!c->po_s || !c->po_t || !c->bo_s || !c->bo_t || !c->ns || !c->nt || !c->ps || !c->pt) return -1;
    if (or_assign(psrc, ptar, Lx, Ly, Nsrc, Ntar, nside_x, nside_y, c->po_s, c->bo_s, c->ns, c->po_t, c->bo_t,
                  c->nt))
        return -1;
    for (int j = 0; j < Nsrc; j++) {
        c->ps[2 * j] = psrc[2 * c->po_s[j]];
        c->ps[2 * j + 1] = psrc[2 * c->po_s[j] + 1];
    }
    for (int j = 0; j < Ntar; j++) {
        c->pt[2 * j] = ptar[2 * c->po_t[j]];
        c->pt[2 * j + 1] = ptar[2 * c->po_t[j] + 1];
    }
    return 0;
}

static void or_cells_free(or_cells* c) {
    free(c->po_s); free(c->po_t); free(c->bo_s); free(c->bo_t);
    free(c->ns); free(c->nt); free(c->ps); free(c->pt);
}

int or_slp_real(const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f, double xi,
                int nside_x, int nside_y, double Lx, double Ly, double* ur) {
    or_cells c;
    if (or_cells_build(&c, psrc, Nsrc, ptar, Ntar, nside_x, nside_y, Lx, Ly)) { or_cells_free(&c); return -1; }
    double* fs = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* us = (double*)calloc(2 * (size_t)(Ntar + 1), sizeof(double));
    for (int j = 0; j < Nsrc; j++) {
        fs[2 * j] = f[2 * c.po_s[j]];
        fs[2 * j + 1] = f[2 * c.po_s[j] + 1];
    }
    const double self = -(1.0 + 0.5 * OR_EULER) - log(xi);
    const double cutoffsq = Lx * Ly / nside_x / nside_y;
    const double xi2 = xi * xi;
    const int nb = nside_x * nside_y;
#pragma omp parallel for schedule(dynamic)
    for (int cb = 0; cb < nb; cb++) {
        if (c.nt[cb] == 0) continue;
        int tidx = c.bo_t[cb], sidx = c.bo_s[cb];
        for (int j = tidx; j < tidx + c.nt[cb]; j++) {
            double ux = 0, uy = 0;
            for (int k = sidx; k < sidx + c.ns[cb]; k++) {
                double rx = c.pt[2 * j] - c.ps[2 * k];
                double ry = c.pt[2 * j + 1] - c.ps[2 * k + 1];
                double r2 = rx * rx + ry * ry;
                if (fabs(r2) < 1e-15) {
                    ux += self * fs[2 * k];
                    uy += self * fs[2 * k + 1];
                } else {
                    or_slp_pair(rx, ry, r2, xi2, fs[2 * k], fs[2 * k + 1], &ux, &uy);
                }
            }
            us[2 * j] += ux;
            us[2 * j + 1] += uy;
        }
        for (int j = 0; j < 8; j++) {
            int psx = cb % nside_x + or_ilist_x[j];
            int psy = cb / nside_x + or_ilist_y[j];
            int tx = (psx + nside_x) % nside_x;
            int ty = (psy + nside_y) % nside_y;
            int sb = ty * nside_x + tx;
            if (c.ns[sb] <= 0) continue;
            double zre = (Lx * (psx - tx)) / nside_x;
            double zim = (Ly * (psy - ty)) / nside_y;
            for (int k = 0; k < c.nt[cb]; k++) {
                double pkx = c.pt[2 * (tidx + k)] - zre;
                double pky = c.pt[2 * (tidx + k) + 1] - zim;
                double ux = 0, uy = 0;
                int idx = c.bo_s[sb];
                for (int l = 0; l < c.ns[sb]; l++, idx++) {
                    double rx = c.ps[2 * idx] - pkx;
                    double ry = c.ps[2 * idx + 1] - pky;
                    double r2 = rx * rx + ry * ry;
                    if (r2 < cutoffsq) or_slp_pair(rx, ry, r2, xi2, fs[2 * idx], fs[2 * idx + 1], &ux, &uy);
                }
                us[2 * (tidx + k)] += ux;
                us[2 * (tidx + k) + 1] += uy;
            }
        }
    }
    for (int j = 0; j < Ntar; j++) {
        ur[2 * c.po_t[j]] = us[2 * j] / (4 * OR_PI);
        ur[2 * c.po_t[j] + 1] = us[2 * j + 1] / (4 * OR_PI);
    }
    free(fs);
    free(us);
    or_cells_free(&c);
    return 0;
}

/* ------------------------------------------------------------------------
 * Real-space stresslet sum: mex_stokes_dlp_real.cpp:15-211.  Own box skips
 * r^2 == 0 exactly and applies no cutoff; neighbours use r^2 < cutoff^2.
 * S = f (x) n per source, r = target - source.
 * ---------------------------------------------------------------------- */
static inline void or_dlp_pair(double x1, double x2, double r2, double xi2, const double* S, double* t1,
                               double* t2) {
    double e2 = exp(-xi2 * r2);
    double prefac = 2 * xi2;
    double facb = -4 * (1 + xi2 * r2) / r2 / r2;
    double T111 = x1 * x1 * x1 * facb + prefac * 3 * x1;
    double T112 = x1 * x1 * x2 * facb + prefac * x2;
    double T122 = x1 * x2 * x2 * facb + prefac * x1;
    *t1 += e2 * (T111 * S[0] + T112 * (S[1] + S[2]) + T122 * S[3]);
    double T211 = x2 * x1 * x1 * facb + prefac * x2;
    double T212 = x2 * x1 * x2 * facb + prefac * x1;
    double T222 = x2 * x2 * x2 * facb + prefac * 3 * x2;
    *t2 += e2 * (T211 * S[0] + T212 * (S[1] + S[2]) + T222 * S[3]);
}

int or_dlp_real(const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f, const double* n,
                double xi, int nside_x, int nside_y, double Lx, double Ly, double* ur) {
    or_cells c;
    if (or_cells_build(&c, psrc, Nsrc, ptar, Ntar, nside_x, nside_y, Lx, Ly)) { or_cells_free(&c); return -1; }
    double* S = (double*)malloc(sizeof(double) * 4 * (size_t)(Nsrc + 1));
    double* Ts = (double*)calloc(2 * (size_t)(Ntar + 1), sizeof(double));
    for (int j = 0; j < Nsrc; j++) {
        int o = c.po_s[j];
        S[4 * j] = f[2 * o] * n[2 * o];
        S[4 * j + 1] = f[2 * o] * n[2 * o + 1];
        S[4 * j + 2] = f[2 * o + 1] * n[2 * o];
        S[4 * j + 3] = f[2 * o + 1] * n[2 * o + 1];
    }
    const double cutoffsq = Lx * Ly / nside_x / nside_y;
    const double xi2 = xi * xi;
    const int nb = nside_x * nside_y;
#pragma omp parallel for schedule(dynamic)
    for (int cb = 0; cb < nb; cb++) {
        if (c.nt[cb] == 0) continue;
        int tidx = c.bo_t[cb], sidx = c.bo_s[cb];
        for (int j = tidx; j < tidx + c.nt[cb]; j++) {
            double t1 = 0, t2 = 0;
            for (int k = sidx; k < sidx + c.ns[cb]; k++) {
                double x1 = -(c.ps[2 * k] - c.pt[2 * j]);
                double x2 = -(c.ps[2 * k + 1] - c.pt[2 * j + 1]);
                double r2 = x1 * x1 + x2 * x2;
                if (r2 == 0) continue;
                or_dlp_pair(x1, x2, r2, xi2, &S[4 * k], &t1, &t2);
            }
            Ts[2 * j] += t1;
            Ts[2 * j + 1] += t2;
        }
        for (int j = 0; j < 8; j++) {
            int psx = cb % nside_x + or_ilist_x[j];
            int psy = cb / nside_x + or_ilist_y[j];
            int tx = (psx + nside_x) % nside_x;
            int ty = (psy + nside_y) % nside_y;
            int sb = ty * nside_x + tx;
            if (c.ns[sb] <= 0) continue;
            double zre = (Lx * (psx - tx)) / nside_x;
            double zim = (Ly * (psy - ty)) / nside_y;
            for (int k = 0; k < c.nt[cb]; k++) {
                double t1 = 0, t2 = 0;
                int idx = c.bo_s[sb];
                for (int l = 0; l < c.ns[sb]; l++, idx++) {
                    double x1 = -(c.ps[2 * idx] - c.pt[2 * (tidx + k)] + zre);
                    double x2 = -(c.ps[2 * idx + 1] - c.pt[2 * (tidx + k) + 1] + zim);
                    double r2 = x1 * x1 + x2 * x2;
                    if (r2 < cutoffsq) or_dlp_pair(x1, x2, r2, xi2, &S[4 * idx], &t1, &t2);
                }
                Ts[2 * (tidx + k)] += t1;
                Ts[2 * (tidx + k) + 1] += t2;
            }
        }
    }
    for (int j = 0; j < Ntar; j++) {
        ur[2 * c.po_t[j]] = Ts[2 * j] / 4 / OR_PI;
        ur[2 * c.po_t[j] + 1] = Ts[2 * j + 1] / 4 / OR_PI;
    }
    free(S);
    free(Ts);
    or_cells_free(&c);
    return 0;
}

/* ------------------------------------------------------------------------
 * k-space filters on full spectra.
 *   SLP: mex_stokes_slp_kspace.cpp:110-169
 *        G = (K^2 H - k (k.H)) (1/K^4 + 1/(4 xi^2 K^2)) exp(-(1-eta) K^2/(4 xi^2))
 *   DLP: mex_stokes_dlp_kspace.cpp:362-443
 *        G_i = i [2 k_i S_ii + k_j (S12+S21) + k_i (S11+S22)
 *                 - 2 k_i (k1^2 S11 + k1 k2 (S12+S21) + k2^2 S22)/K^2] E(K)
 *        E(K) = exp(-K^2 (1-eta)/(4 xi^2)) (1 + K^2/(4 xi^2)) / K^2
 * Index j <= Mx/2 is +k (Nyquist counted positive); rows 0..My/2 are +k2,
 * the remaining My/2-1 rows are -My/2+1..-1.  k = 0 is zeroed afterwards.
 * ---------------------------------------------------------------------- */
static void or_filter_point(int kind, double k1, double k2, double xi, double eta, double** re, double** im,
                            size_t p) {
    double Ksq = k1 * k1 + k2 * k2;
    if (kind == OR_KIND_SLP) {
        double e = (1.0 / (Ksq * Ksq) + 0.25 / (Ksq * xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * Ksq);
        double q1r = re[0][p], q1i = im[0][p], q2r = re[1][p], q2i = im[1][p];
        double kqr = k1 * q1r + k2 * q2r;
        double kqi = k1 * q1i + k2 * q2i;
        re[0][p] = (Ksq * q1r - k1 * kqr) * e;
        im[0][p] = (Ksq * q1i - k1 * kqi) * e;
        re[1][p] = (Ksq * q2r - k2 * kqr) * e;
        im[1][p] = (Ksq * q2i - k2 * kqi) * e;
    } else {
        double e = exp(-Ksq * (1 - eta) / (4 * xi * xi)) * (1 + Ksq / (4 * xi * xi)) / Ksq;
        /* grids: 0 = S11 (f1 n1), 1 = S21 (f2 n1), 2 = S12 (f1 n2), 3 = S22 (f2 n2) */
        double a_r = re[0][p], a_i = im[0][p];
        double s_r = re[1][p] + re[2][p], s_i = im[1][p] + im[2][p];
        double d_r = re[3][p], d_i = im[3][p];
        double qr = (k1 * k1 * a_r + k1 * k2 * s_r + k2 * k2 * d_r) / Ksq;
        double qi = (k1 * k1 * a_i + k1 * k2 * s_i + k2 * k2 * d_i) / Ksq;
        double x1r = 2 * a_r * k1 + k2 * s_r + k1 * (a_r + d_r) - 2 * k1 * qr;
        double x1i = 2 * a_i * k1 + k2 * s_i + k1 * (a_i + d_i) - 2 * k1 * qi;
        double x2r = 2 * d_r * k2 + k1 * s_r + k2 * (a_r + d_r) - 2 * k2 * qr;
        double x2i = 2 * d_i * k2 + k1 * s_i + k2 * (a_i + d_i) - 2 * k2 * qi;
        re[0][p] = -x1i * e;
        im[0][p] = x1r * e;
        re[1][p] = -x2i * e;
        im[1][p] = x2r * e;
    }
}

void or_filter(int kind, double** re, double** im, int Mx, int My, double Lx, double Ly, double xi, double eta) {
#pragma omp parallel for
    for (int j = 0; j < Mx; j++) {
        size_t ptr = (size_t)j * My;
        double k1 = (j <= Mx / 2) ? 2.0 * OR_PI / Lx * j : 2.0 * OR_PI / Lx * (j - Mx);
        for (int k = 0; k <= My / 2; k++, ptr++) or_filter_point(kind, k1, 2.0 * OR_PI / Ly * k, xi, eta, re, im, ptr);
        for (int k = 0; k < My / 2 - 1; k++, ptr++)
            or_filter_point(kind, k1, 2.0 * OR_PI / Ly * (k - My / 2 + 1), xi, eta, re, im, ptr);
    }
    re[0][0] = re[1][0] = im[0][0] = im[1][0] = 0.0;
}

static int or_kspace_common(int kind, const double* psrc, int Nsrc, const double* ptar, int Ntar, double xi,
                            double eta, const double* v1, const double* v2, int Mx, int My, double Lx, double Ly,
                            double w, int P, double* uk) {
    double h = Lx / Mx;
    int ng = kind == OR_KIND_SLP ? 2 : 4;
    size_t G = (size_t)Mx * My;
    double* re[4] = {0, 0, 0, 0};
    double* im[4] = {0, 0, 0, 0};
    for (int g = 0; g < ng; g++) {
        re[g] = (double*)calloc(G, sizeof(double));
        im[g] = (double*)calloc(G, sizeof(double));
        if (!re[g] || !im[g]) {
            for (int q = 0; q <= g; q++) { free(re[q]); free(im[q]); }
            return -1;
        }
    }
    double* e1 = (double*)malloc(sizeof(double) * (size_t)(P + 1));
    or_spread(re[0], re[1], e1, psrc, v1, Nsrc, Lx, Ly, xi, w, eta, P, Mx, My, h);
    if (kind == OR_KIND_DLP) or_spread(re[2], re[3], e1, psrc, v2, Nsrc, Lx, Ly, xi, w, eta, P, Mx, My, h);
    for (int g = 0; g < ng; g++) or_fft2(My, Mx, re[g], im[g], 0);
    or_filter(kind, re, im, Mx, My, Lx, Ly, xi, eta);
    or_fft2(My, Mx, re[0], im[0], 1);
    or_fft2(My, Mx, re[1], im[1], 1);
    for (int j = 0; j < 2 * Ntar; j++) uk[j] = 0.0;
    or_gather(re[0], 2, 1, e1, ptar, uk, Ntar, Lx, Ly, xi, w, eta, P, Mx, My, h);
    or_gather(re[1], 2, 2, e1, ptar, uk, Ntar, Lx, Ly, xi, w, eta, P, Mx, My, h);
    free(e1);
    for (int g = 0; g < ng; g++) { free(re[g]); free(im[g]); }
    return 0;
}

int or_slp_kspace(const double* psrc, int Nsrc, const double* ptar, int Ntar, double xi, double eta,
                  const double* f, int Mx, int My, double Lx, double Ly, double w, int P, double* uk) {
    return or_kspace_common(OR_KIND_SLP, psrc, Nsrc, ptar, Ntar, xi, eta, f, NULL, Mx, My, Lx, Ly, w, P, uk);
}

int or_dlp_kspace(const double* psrc, int Nsrc, const double* ptar, int Ntar, double xi, double eta,
                  const double* f, const double* n, int Mx, int My, double Lx, double Ly, double w, int P,
                  double* uk) {
    /* v1 = (f1 n1, f2 n1), v2 = (f1 n2, f2 n2): mex_stokes_dlp_kspace.cpp:290-298 */
    double* v1 = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* v2 = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    for (int i = 0; i < Nsrc; i++) {
        v1[2 * i] = f[2 * i] * n[2 * i];
        v1[2 * i + 1] = f[2 * i + 1] * n[2 * i];
        v2[2 * i] = f[2 * i] * n[2 * i + 1];
        v2[2 * i + 1] = f[2 * i + 1] * n[2 * i + 1];
    }
    int rc = or_kspace_common(OR_KIND_DLP, psrc, Nsrc, ptar, Ntar, xi, eta, v1, v2, Mx, My, Lx, Ly, w, P, uk);
    free(v1);
    free(v2);
    return rc;
}

/* ------------------------------------------------------------------------
 * Parameter selection (Palsson & Tornberg 2019 estimates, Newton solves):
 *   SLP: StokesSLP_ewald_2p.m:27-35,85-104 with find_kinfb :147-173 and
 *        find_xi :178-202.  find_kinfb receives Lx twice (:96).
 *   DLP: StokesDLP_ewald_2p.m:27-38,105-125 with find_kinfb :171-197 and
 *        find_xi :202-224.  Its find_kinfb keeps MATLAB's left-to-right
 *        evaluation of k*8*pi*Q*max(Lx,Ly)/Lx^3*Ly^3 (:379-381).
 * ---------------------------------------------------------------------- */
static double or_slp_kf(double k, double Q, double Lx, double Ly, double xi, double tol) {
    double mx = Lx > Ly ? Lx : Ly;
    return sqrt(4 * Q * OR_PI * mx / (Lx * Lx * Lx * Ly * Ly * Ly * k)) * exp(-k * k / (4 * xi * xi)) - tol;
}
static double or_slp_kfp(double k, double Q, double Lx, double Ly, double xi) {
    double mx = Lx > Ly ? Lx : Ly;
    return -sqrt(4 * Q * OR_PI * mx / (Lx * Lx * Lx * Ly * Ly * Ly)) * exp(-k * k / (4 * xi * xi)) *
           (0.5 * pow(k, -1.5) + sqrt(1 / k) * 2 * k / (4 * xi * xi));
}
static double or_dlp_kf(double k, double Q, double Lx, double Ly, double xi, double tol) {
    double mx = Lx > Ly ? Lx : Ly;
    return sqrt(k * 8 * OR_PI * Q * mx / (Lx * Lx * Lx) * (Ly * Ly * Ly)) * exp(-k * k / (4 * xi * xi)) - tol;
}
static double or_dlp_kfp(double k, double Q, double Lx, double Ly, double xi) {
    double mx = Lx > Ly ? Lx : Ly;
    return sqrt(8 * OR_PI * Q * mx / (Lx * Lx * Lx) * (Ly * Ly * Ly)) * exp(-k * k / (4 * xi * xi)) *
           (0.5 * pow(k, -0.5) - 2 * pow(k, 1.5) / (4 * xi * xi));
}
static double or_slp_xf(double x, double Q, double Lx, double Ly, double rc, double tol) {
    return sqrt(Q * OR_PI / (4 * Lx * Ly * x)) * exp(-x * x * rc * rc) - tol;
}
static double or_slp_xfp(double x, double Q, double Lx, double Ly, double rc) {
    return -sqrt(Q * OR_PI / (4 * Lx * Ly)) * exp(-x * x * rc * rc) * (0.5 * pow(x, -1.5) + 2 * rc * rc * x * sqrt(1 / x));
}
static double or_dlp_xf(double a, double Q, double Lx, double Ly, double rc, double tol) {
    return exp(-a * a * rc * rc) * a * rc * sqrt(2 * OR_PI * Q / (Lx * Ly)) - tol;
}
static double or_dlp_xfp(double a, double Q, double Lx, double Ly, double rc) {
    return (1 - 2 * a * a * rc * rc) * exp(-a * a * rc * rc) * sqrt(2 * OR_PI * Q / (Lx * Ly)) * rc;
}

static int or_matlab_length(int n) { return n == 0 ? 0 : (n > 2 ? n : 2); }

int or_choose_params(int kind, int nsrc, int ntar, const double* f1, const double* f2, double Lx, double Ly, int P,
                     double Nb, double tol, or_params* o) {
    memset(o, 0, sizeof(*o));
    if (P <= 0) P = 24;
    if (tol <= 0) tol = 1e-16;
    double npts = (double)nsrc + (double)ntar;
    if (Nb <= 0) {
        double a1 = P * round(log2(npts));
        double a2 = npts / 4;
        Nb = a1 < a2 ? a1 : a2;
    }
    o->P = P;
    o->Nb = Nb;
    o->tol = tol;
    int A, B;
    or_rat(Lx / Ly, &A, &B);
    o->A = A;
    o->B = B;
    double Q = 0;
    for (int j = 0; j < nsrc; j++) Q += f1[j] * f1[j];
    for (int j = 0; j < nsrc; j++) Q += f2[j] * f2[j];
    Q += 1;
    o->Q = Q;
    if (kind == OR_KIND_DLP) npts = (double)or_matlab_length(nsrc) + (double)or_matlab_length(ntar);
    int a = (int)ceil(sqrt(npts / (Nb * A * B)));
    o->a = a;
    o->m = 0.95 * sqrt(OR_PI * P);
    o->nside_x = a * A;
    o->nside_y = a * B;
    double rc = Lx / o->nside_x;
    o->rc = rc;
    /* find_xi */
    double x = (kind == OR_KIND_SLP) ? 4 / rc : 1 / rc;
    int it = 0;
    while (1) {
        double fx = kind == OR_KIND_SLP ? or_slp_xf(x, Q, Lx, Ly, rc, tol) : or_dlp_xf(x, Q, Lx, Ly, rc, tol);
        if (!(fabs(fx) > tol)) break;
        if (it > 100) break;
        double fp = kind == OR_KIND_SLP ? or_slp_xfp(x, Q, Lx, Ly, rc) : or_dlp_xfp(x, Q, Lx, Ly, rc);
        double d = fx / fp;
        if (0.9 * x < d) d = 0.9 * x;
        x -= d;
        it++;
    }
    o->xi = x;
    o->xi_iters = it;
    /* find_kinfb(Q, Lx, Lx, xi, tol) */
    double xi = x;
    double k = round(5 * xi);
    it = 0;
    while (1) {
        double fk = kind == OR_KIND_SLP ? or_slp_kf(k, Q, Lx, Lx, xi, tol) : or_dlp_kf(k, Q, Lx, Lx, xi, tol);
        if (!(fabs(fk) > tol)) break;
        if (it > 100) break;
        double fp = kind == OR_KIND_SLP ? or_slp_kfp(k, Q, Lx, Lx, xi) : or_dlp_kfp(k, Q, Lx, Lx, xi);
        double d = fk / fp;
        if (0.9 * k < d) d = 0.9 * k;
        k -= d;
        it++;
    }
    o->k_iters = it;
    int kinf = (int)round(Lx * k / (2 * OR_PI));
    o->kinf = kinf;
    int M = 2 * kinf < 10000 ? 2 * kinf : 10000;
    o->My = B * M;
    o->Mx = A * M;
    o->w = P * Lx / o->Mx / 2;
    o->eta = (2 * xi * o->w / o->m) * (2 * xi * o->w / o->m);
    return 0;
}

/* ------------------------------------------------------------------------
 * Drivers: StokesSLP_ewald_2p.m:74-136 and StokesDLP_ewald_2p.m:93-163.
 * The DLP driver's perturbation of n and f by 1e-60 on MATLAB releases
 * other than R2017a (:69-81) works around MATLAB returning real-valued FFT
 * arrays; it is not restated (the R2017a branch is followed).
 * ---------------------------------------------------------------------- */
static void or_wrap_pack(const double* x, const double* y, int n, double Lx, double Ly, double* p) {
    for (int j = 0; j < n; j++) {
        p[2 * j] = or_matlab_mod(x[j] + Lx / 2, Lx) - Lx / 2;
        p[2 * j + 1] = or_matlab_mod(y[j] + Ly / 2, Ly) - Ly / 2;
    }
}

int or_stokes_slp_ewald_2p(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar,
                           const double* ytar, int Ntar, const double* f1, const double* f2, double Lx, double Ly,
                           int P, double Nb, double tol, double* u1, double* u2, double* ur_out, double* uk_out,
                           or_params* prm) {
    or_params o;
    or_choose_params(OR_KIND_SLP, Nsrc, Ntar, f1, f2, Lx, Ly, P, Nb, tol, &o);
    if (prm) *prm = o;
    double* ps = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* pt = (double*)malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    double* f = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* ur = (double*)malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    double* uk = (double*)malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    or_wrap_pack(xsrc, ysrc, Nsrc, Lx, Ly, ps);
    or_wrap_pack(xtar, ytar, Ntar, Lx, Ly, pt);
    for (int j = 0; j < Nsrc; j++) { f[2 * j] = f1[j]; f[2 * j + 1] = f2[j]; }
    int rc = or_slp_real(ps, Nsrc, pt, Ntar, f, o.xi, o.nside_x, o.nside_y, Lx, Ly, ur);
    if (!rc) rc = or_slp_kspace(ps, Nsrc, pt, Ntar, o.xi, o.eta, f, o.Mx, o.My, Lx, Ly, o.w, o.P, uk);
    if (!rc) {
        for (int j = 0; j < Ntar; j++) {
            u1[j] = ur[2 * j] + uk[2 * j];
            u2[j] = ur[2 * j + 1] + uk[2 * j + 1];
        }
        if (ur_out) memcpy(ur_out, ur, sizeof(double) * 2 * (size_t)Ntar);
        if (uk_out) memcpy(uk_out, uk, sizeof(double) * 2 * (size_t)Ntar);
    }
    free(ps); free(pt); free(f); free(ur); free(uk);
    return rc;
}

int or_stokes_dlp_ewald_2p(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar,
                           const double* ytar, int Ntar, const double* n1, const double* n2, const double* f1,
                           const double* f2, double Lx, double Ly, int P, double Nb, double tol, double* u1,
                           double* u2, double* ur_out, double* uk_out, or_params* prm) {
    or_params o;
    or_choose_params(OR_KIND_DLP, Nsrc, Ntar, f1, f2, Lx, Ly, P, Nb, tol, &o);
    if (prm) *prm = o;
    double* ps = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* pt = (double*)malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    double* f = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* nn = (double*)malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* ur = (double*)malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    double* uk = (double*)malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    or_wrap_pack(xsrc, ysrc, Nsrc, Lx, Ly, ps);
    or_wrap_pack(xtar, ytar, Ntar, Lx, Ly, pt);
    for (int j = 0; j < Nsrc; j++) {
        f[2 * j] = f1[j]; f[2 * j + 1] = f2[j];
        nn[2 * j] = n1[j]; nn[2 * j + 1] = n2[j];
    }
    int rc = or_dlp_real(ps, Nsrc, pt, Ntar, f, nn, o.xi, o.nside_x, o.nside_y, Lx, Ly, ur);
    if (!rc) rc = or_dlp_kspace(ps, Nsrc, pt, Ntar, o.xi, o.eta, f, nn, o.Mx, o.My, Lx, Ly, o.w, o.P, uk);
    if (!rc) {
        /* zero mode, StokesDLP_ewald_2p.m:149-151, with the wrapped source coordinates */
        double zx = 0, zy = 0;
        for (int j = 0; j < Nsrc; j++) {
            double fn = f1[j] * n1[j] + f2[j] * n2[j];
            zx += fn * ps[2 * j];
            zy += fn * ps[2 * j + 1];
        }
        zx /= (Lx * Ly);
        zy /= (Lx * Ly);
        for (int j = 0; j < Ntar; j++) {
            uk[2 * j] += zx;
            uk[2 * j + 1] += zy;
            u1[j] = ur[2 * j] + uk[2 * j];
            u2[j] = ur[2 * j + 1] + uk[2 * j + 1];
        }
        if (ur_out) memcpy(ur_out, ur, sizeof(double) * 2 * (size_t)Ntar);
        if (uk_out) memcpy(uk_out, uk, sizeof(double) * 2 * (size_t)Ntar);
    }
    free(ps); free(pt); free(f); free(nn); free(ur); free(uk);
    return rc;
}

/* ------------------------------------------------------------------------
 * Direct sums restated from the reference's MATLAB test oracles.
 *   stokes_slp_real_ds.m:13-69   3 x 3 periodic images, no truncation,
 *                                self term when |r| < 1e-13
 *   stokes_dlp_real_ds.m:22-76   same, skipping |r| < 1e-13
 *   stokes_slp_kspace_ds.m:21-76 modes jk in [-kinf+1, kinf]^2 \ {0},
 *                                phase exp(-i k.(x_t - x_s))
 *   stokes_dlp_kspace_ds.m:20-88 same modes, phase exp(+i k.(x_t - x_s)),
 *                                plus the zero mode
 * The k-space sums are reordered through per-mode structure factors
 * (sum over sources first), which is the same finite sum.
 * ---------------------------------------------------------------------- */
static void or_real_ds(int kind, const double* xs, const double* ys, int Ns, const double* xt, const double* yt,
                       int Nt, const double* n1, const double* n2, const double* f1, const double* f2, double Lx,
                       double Ly, double xi, double* u) {
    const double selfc = -(OR_EULER / 2 + log(xi) + 1);
    const double xi2 = xi * xi;
#pragma omp parallel for schedule(dynamic, 16)
    for (int m = 0; m < Nt; m++) {
        double a1 = 0, a2 = 0;
        for (int n = 0; n < Ns; n++) {
            for (int jx = -1; jx <= 1; jx++) {
                for (int jy = -1; jy <= 1; jy++) {
                    double sx = xs[n] + jx * Lx, sy = ys[n] + jy * Ly;
                    if (kind == OR_KIND_SLP) {
                        double r1 = sx - xt[m], r2 = sy - yt[m];
                        double r = sqrt(r1 * r1 + r2 * r2);
                        if (fabs(r) < 1e-13) {
                            a1 += selfc * f1[n];
                            a2 += selfc * f2[n];
                        } else {
                            double rdf = r1 * f1[n] + r2 * f2[n];
                            double e = exp(-xi2 * r * r);
                            double E = or_expint_e1(xi2 * r * r);
                            a1 += e * (r1 * rdf / (r * r) - f1[n]) + f1[n] * E / 2;
                            a2 += e * (r2 * rdf / (r * r) - f2[n]) + f2[n] * E / 2;
                        }
                    } else {
                        double r1 = -(sx - xt[m]), r2 = -(sy - yt[m]);
                        double r = sqrt(r1 * r1 + r2 * r2);
                        if (fabs(r) < 1e-13) continue;
                        double rdf = r1 * f1[n] + r2 * f2[n];
                        double rdn = r1 * n1[n] + r2 * n2[n];
                        double ndf = n1[n] * f1[n] + n2[n] * f2[n];
                        double e = exp(-xi2 * r * r);
                        double r4 = r * r * r * r;
                        a1 += e * (-4 * r1 * rdn * rdf / r4 * (1 + xi2 * r * r) +
                                   2 * xi2 * (f1[n] * rdn + n1[n] * rdf + ndf * r1));
                        a2 += e * (-4 * r2 * rdn * rdf / r4 * (1 + xi2 * r * r) +
                                   2 * xi2 * (f2[n] * rdn + n2[n] * rdf + ndf * r2));
                    }
                }
            }
        }
        u[2 * m] = a1 / (4 * OR_PI);
        u[2 * m + 1] = a2 / (4 * OR_PI);
    }
}

void or_slp_real_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                    int Ntar, const double* f1, const double* f2, double Lx, double Ly, double xi, double* u) {
    or_real_ds(OR_KIND_SLP, xsrc, ysrc, Nsrc, xtar, ytar, Ntar, NULL, NULL, f1, f2, Lx, Ly, xi, u);
}

void or_dlp_real_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                    int Ntar, const double* n1, const double* n2, const double* f1, const double* f2, double Lx,
                    double Ly, double xi, double* u) {
    or_real_ds(OR_KIND_DLP, xsrc, ysrc, Nsrc, xtar, ytar, Ntar, n1, n2, f1, f2, Lx, Ly, xi, u);
}

/*
 * Structure-factor evaluation of the k-space sums over modes
 * jk1, jk2 in [klo, khi] (excluding 0).  For the SLP the per-mode
 * multiplier acts on F(k) = sum_s f_s exp(+i k.x_s) and the result is
 * Re sum_k M(k) F(k) exp(-i k.x_t) / (Lx Ly).  For the DLP it acts on the
 * four tensors T_ab(k) = sum_s f_a n_b exp(-i k.x_s) and the phase at the
 * target is exp(+i k.x_t).
 */
static void or_kspace_sf(int kind, const double* xs, const double* ys, int Ns, const double* xt, const double* yt,
                         int Nt, const double* n1, const double* n2, const double* f1, const double* f2, double Lx,
                         double Ly, double xi, int klo, int khi, double* u) {
    int K = khi - klo + 1;
    size_t nm = (size_t)K * K;
    int ncomp = kind == OR_KIND_SLP ? 2 : 4;
    double* Sr = (double*)calloc(nm * ncomp, sizeof(double));
    double* Si = (double*)calloc(nm * ncomp, sizeof(double));
    double sgn_s = kind == OR_KIND_SLP ? 1.0 : -1.0; /* source phase sign */
#pragma omp parallel
    {
        double* lr = (double*)calloc(nm * ncomp, sizeof(double));
        double* li = (double*)calloc(nm * ncomp, sizeof(double));
        double* cxr = (double*)malloc(sizeof(double) * K * 4);
        double* cxi = cxr + K;
        double* cyr = cxi + K;
        double* cyi = cyr + K;
#pragma omp for schedule(static)
        for (int s = 0; s < Ns; s++) {
            for (int j = 0; j < K; j++) {
                double a = sgn_s * 2 * OR_PI / Lx * (klo + j) * xs[s];
                double b = sgn_s * 2 * OR_PI / Ly * (klo + j) * ys[s];
                cxr[j] = cos(a); cxi[j] = sin(a);
                cyr[j] = cos(b); cyi[j] = sin(b);
            }
            double q[4];
            if (kind == OR_KIND_SLP) {
                q[0] = f1[s]; q[1] = f2[s];
            } else {
                q[0] = f1[s] * n1[s]; q[1] = f1[s] * n2[s]; q[2] = f2[s] * n1[s]; q[3] = f2[s] * n2[s];
            }
            for (int j1 = 0; j1 < K; j1++) {
                for (int j2 = 0; j2 < K; j2++) {
                    double pr = cxr[j1] * cyr[j2] - cxi[j1] * cyi[j2];
                    double pi = cxr[j1] * cyi[j2] + cxi[j1] * cyr[j2];
                    size_t mi = (size_t)j1 * K + j2;
                    for (int c = 0; c < ncomp; c++) {
                        lr[c * nm + mi] += q[c] * pr;
                        li[c * nm + mi] += q[c] * pi;
                    }
                }
            }
        }
#pragma omp critical
        {
            for (size_t i = 0; i < nm * ncomp; i++) { Sr[i] += lr[i]; Si[i] += li[i]; }
        }
        free(lr); free(li); free(cxr);
    }
    /* apply the per-mode multipliers */
    double* Gr = (double*)calloc(nm * 2, sizeof(double));
    double* Gi = (double*)calloc(nm * 2, sizeof(double));
    for (int j1 = 0; j1 < K; j1++) {
        for (int j2 = 0; j2 < K; j2++) {
            int jk1 = klo + j1, jk2 = klo + j2;
            if (jk1 == 0 && jk2 == 0) continue;
            double k1 = 2 * OR_PI / Lx * jk1, k2 = 2 * OR_PI / Ly * jk2;
            double kk = k1 * k1 + k2 * k2;
            double g = (1 + kk / (4 * xi * xi)) * exp(-kk / (4 * xi * xi)) / kk;
            size_t mi = (size_t)j1 * K + j2;
            if (kind == OR_KIND_SLP) {
                double Fr1 = Sr[mi], Fi1 = Si[mi], Fr2 = Sr[nm + mi], Fi2 = Si[nm + mi];
                double kfr = (k1 * Fr1 + k2 * Fr2) / kk, kfi = (k1 * Fi1 + k2 * Fi2) / kk;
                Gr[mi] = (Fr1 - k1 * kfr) * g;
                Gi[mi] = (Fi1 - k1 * kfi) * g;
                Gr[nm + mi] = (Fr2 - k2 * kfr) * g;
                Gi[nm + mi] = (Fi2 - k2 * kfi) * g;
            } else {
                /* T: 0 = f1n1, 1 = f1n2, 2 = f2n1, 3 = f2n2 */
                double r11 = Sr[mi], i11 = Si[mi], r12 = Sr[nm + mi], i12 = Si[nm + mi];
                double r21 = Sr[2 * nm + mi], i21 = Si[2 * nm + mi], r22 = Sr[3 * nm + mi], i22 = Si[3 * nm + mi];
                /* f_a (k.n) = k1 T_a1 + k2 T_a2 ; n_a (k.f) = k1 T_1a + k2 T_2a ; f.n = T11 + T22 */
                double knkf_r = k1 * k1 * r11 + k1 * k2 * (r12 + r21) + k2 * k2 * r22;
                double knkf_i = k1 * k1 * i11 + k1 * k2 * (i12 + i21) + k2 * k2 * i22;
                double x1r = (k1 * r11 + k2 * r12) + (k1 * r11 + k2 * r21) + k1 * (r11 + r22) - 2 * k1 * knkf_r / kk;
                double x1i = (k1 * i11 + k2 * i12) + (k1 * i11 + k2 * i21) + k1 * (i11 + i22) - 2 * k1 * knkf_i / kk;
                double x2r = (k1 * r21 + k2 * r22) + (k1 * r12 + k2 * r22) + k2 * (r11 + r22) - 2 * k2 * knkf_r / kk;
                double x2i = (k1 * i21 + k2 * i22) + (k1 * i12 + k2 * i22) + k2 * (i11 + i22) - 2 * k2 * knkf_i / kk;
                /* multiply by i */
                Gr[mi] = -x1i * g;
                Gi[mi] = x1r * g;
                Gr[nm + mi] = -x2i * g;
                Gi[nm + mi] = x2r * g;
            }
        }
    }
    double sgn_t = -sgn_s;
#pragma omp parallel
    {
        double* cxr = (double*)malloc(sizeof(double) * K * 4);
        double* cxi = cxr + K;
        double* cyr = cxi + K;
        double* cyi = cyr + K;
#pragma omp for schedule(static)
        for (int t = 0; t < Nt; t++) {
            for (int j = 0; j < K; j++) {
                double a = sgn_t * 2 * OR_PI / Lx * (klo + j) * xt[t];
                double b = sgn_t * 2 * OR_PI / Ly * (klo + j) * yt[t];
                cxr[j] = cos(a); cxi[j] = sin(a);
                cyr[j] = cos(b); cyi[j] = sin(b);
            }
            double a1 = 0, a2 = 0;
            for (int j1 = 0; j1 < K; j1++) {
                for (int j2 = 0; j2 < K; j2++) {
                    double pr = cxr[j1] * cyr[j2] - cxi[j1] * cyi[j2];
                    double pi = cxr[j1] * cyi[j2] + cxi[j1] * cyr[j2];
                    size_t mi = (size_t)j1 * K + j2;
                    a1 += Gr[mi] * pr - Gi[mi] * pi;
                    a2 += Gr[nm + mi] * pr - Gi[nm + mi] * pi;
                }
            }
            u[2 * t] = a1 / (Lx * Ly);
            u[2 * t + 1] = a2 / (Lx * Ly);
        }
        free(cxr);
    }
    free(Sr); free(Si); free(Gr); free(Gi);
}

void or_slp_kspace_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                      int Ntar, const double* f1, const double* f2, double Lx, double Ly, double xi, int kinf,
                      double* u) {
    or_kspace_sf(OR_KIND_SLP, xsrc, ysrc, Nsrc, xtar, ytar, Ntar, NULL, NULL, f1, f2, Lx, Ly, xi, -kinf + 1, kinf,
                 u);
}

void or_dlp_kspace_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                      int Ntar, const double* n1, const double* n2, const double* f1, const double* f2, double Lx,
                      double Ly, double xi, int kinf, double* u) {
    or_kspace_sf(OR_KIND_DLP, xsrc, ysrc, Nsrc, xtar, ytar, Ntar, n1, n2, f1, f2, Lx, Ly, xi, -kinf + 1, kinf, u);
    double zx = 0, zy = 0;
    for (int s = 0; s < Nsrc; s++) {
        double fn = f1[s] * n1[s] + f2[s] * n2[s];
        zx += fn * xsrc[s];
        zy += fn * ysrc[s];
    }
    for (int t = 0; t < Ntar; t++) {
        u[2 * t] += zx / (Lx * Ly);
        u[2 * t + 1] += zy / (Lx * Ly);
    }
}

/* ------------------------------------------------------------------------
 * Truth oracle: real part with cutoff rcut over periodic images (binned),
 * k part over the symmetric box |jk| <= kinf, SLP self term / DLP r=0 skip
 * as in the direct sums, DLP zero mode added.
 * ---------------------------------------------------------------------- */
void or_ewald_truth(int kind, const double* xs, const double* ys, int Ns, const double* xt, const double* yt,
                    int Nt, const double* n1, const double* n2, const double* f1, const double* f2, double Lx,
                    double Ly, double xi, double rcut, int kinf, double* u) {
    /* bin sources into cells no smaller than rcut */
    int ncx = (int)floor(Lx / rcut), ncy = (int)floor(Ly / rcut);
    if (ncx < 1) ncx = 1;
    if (ncy < 1) ncy = 1;
    int nc = ncx * ncy;
    int* cnt = (int*)calloc((size_t)nc + 1, sizeof(int));
    int* cell = (int*)malloc(sizeof(int) * (size_t)(Ns + 1));
    int* order = (int*)malloc(sizeof(int) * (size_t)(Ns + 1));
    for (int s = 0; s < Ns; s++) {
        int cx = (int)floor((xs[s] / Lx + 0.5) * ncx), cy = (int)floor((ys[s] / Ly + 0.5) * ncy);
        cx = cx < 0 ? 0 : (cx >= ncx ? ncx - 1 : cx);
        cy = cy < 0 ? 0 : (cy >= ncy ? ncy - 1 : cy);
        cell[s] = cy * ncx + cx;
        cnt[cell[s] + 1]++;
    }
    for (int c = 0; c < nc; c++) cnt[c + 1] += cnt[c];
    int* fill = (int*)malloc(sizeof(int) * (size_t)nc);
    memcpy(fill, cnt, sizeof(int) * (size_t)nc);
    for (int s = 0; s < Ns; s++) order[fill[cell[s]]++] = s;
    const double xi2 = xi * xi, rc2 = rcut * rcut;
    const double selfc = -(OR_EULER / 2 + log(xi) + 1);
    int span_x = ncx >= 3 ? 1 : 1, span_y = 1;
    /* number of periodic images that can lie within rcut */
    int imx = (int)ceil(rcut / Lx) + 1, imy = (int)ceil(rcut / Ly) + 1;
#pragma omp parallel for schedule(dynamic, 16)
    for (int m = 0; m < Nt; m++) {
        double a1 = 0, a2 = 0;
        int cx = (int)floor((xt[m] / Lx + 0.5) * ncx), cy = (int)floor((yt[m] / Ly + 0.5) * ncy);
        cx = cx < 0 ? 0 : (cx >= ncx ? ncx - 1 : cx);
        cy = cy < 0 ? 0 : (cy >= ncy ? ncy - 1 : cy);
        if (ncx < 3 || ncy < 3) {
            /* small domains: every source, every image */
            for (int n = 0; n < Ns; n++)
                for (int jx = -imx; jx <= imx; jx++)
                    for (int jy = -imy; jy <= imy; jy++) {
                        double r1 = xt[m] - (xs[n] + jx * Lx), r2 = yt[m] - (ys[n] + jy * Ly);
                        double rr = r1 * r1 + r2 * r2;
                        if (rr >= rc2) continue;
                        if (kind == OR_KIND_SLP) {
                            if (sqrt(rr) < 1e-13) { a1 += selfc * f1[n]; a2 += selfc * f2[n]; continue; }
                            double rdf = r1 * f1[n] + r2 * f2[n];
                            double e = exp(-xi2 * rr), E = or_expint_e1(xi2 * rr);
                            a1 += e * (r1 * rdf / rr - f1[n]) + f1[n] * E / 2;
                            a2 += e * (r2 * rdf / rr - f2[n]) + f2[n] * E / 2;
                        } else {
                            if (sqrt(rr) < 1e-13) continue;
                            double rdf = r1 * f1[n] + r2 * f2[n], rdn = r1 * n1[n] + r2 * n2[n];
                            double ndf = n1[n] * f1[n] + n2[n] * f2[n];
                            double e = exp(-xi2 * rr);
                            a1 += e * (-4 * r1 * rdn * rdf / (rr * rr) * (1 + xi2 * rr) + 2 * xi2 * (f1[n] * rdn + n1[n] * rdf + ndf * r1));
                            a2 += e * (-4 * r2 * rdn * rdf / (rr * rr) * (1 + xi2 * rr) + 2 * xi2 * (f2[n] * rdn + n2[n] * rdf + ndf * r2));
                        }
                    }
        } else {
            for (int dx = -span_x; dx <= span_x; dx++)
                for (int dy = -span_y; dy <= span_y; dy++) {
                    int qx = cx + dx, qy = cy + dy;
                    int wx = (qx + ncx) % ncx, wy = (qy + ncy) % ncy;
                    double ox = Lx * (double)((qx - wx) / ncx), oy = Ly * (double)((qy - wy) / ncy);
                    int c = wy * ncx + wx;
                    for (int q = cnt[c]; q < cnt[c + 1]; q++) {
                        int n = order[q];
                        double r1 = xt[m] - (xs[n] + ox), r2 = yt[m] - (ys[n] + oy);
                        double rr = r1 * r1 + r2 * r2;
                        if (rr >= rc2) continue;
                        if (kind == OR_KIND_SLP) {
                            if (sqrt(rr) < 1e-13) { a1 += selfc * f1[n]; a2 += selfc * f2[n]; continue; }
                            double rdf = r1 * f1[n] + r2 * f2[n];
                            double e = exp(-xi2 * rr), E = or_expint_e1(xi2 * rr);
                            a1 += e * (r1 * rdf / rr - f1[n]) + f1[n] * E / 2;
                            a2 += e * (r2 * rdf / rr - f2[n]) + f2[n] * E / 2;
                        } else {
                            if (sqrt(rr) < 1e-13) continue;
                            double rdf = r1 * f1[n] + r2 * f2[n], rdn = r1 * n1[n] + r2 * n2[n];
                            double ndf = n1[n] * f1[n] + n2[n] * f2[n];
                            double e = exp(-xi2 * rr);
                            a1 += e * (-4 * r1 * rdn * rdf / (rr * rr) * (1 + xi2 * rr) + 2 * xi2 * (f1[n] * rdn + n1[n] * rdf + ndf * r1));
                            a2 += e * (-4 * r2 * rdn * rdf / (rr * rr) * (1 + xi2 * rr) + 2 * xi2 * (f2[n] * rdn + n2[n] * rdf + ndf * r2));
                        }
                    }
                }
        }
        u[2 * m] = a1 / (4 * OR_PI);
        u[2 * m + 1] = a2 / (4 * OR_PI);
    }
    free(cnt); free(cell); free(order); free(fill);
    double* uk = (double*)malloc(sizeof(double) * 2 * (size_t)(Nt + 1));
    or_kspace_sf(kind, xs, ys, Ns, xt, yt, Nt, n1, n2, f1, f2, Lx, Ly, xi, -kinf, kinf, uk);
    double zx = 0, zy = 0;
    if (kind == OR_KIND_DLP) {
        for (int s = 0; s < Ns; s++) {
            double fn = f1[s] * n1[s] + f2[s] * n2[s];
            zx += fn * xs[s];
            zy += fn * ys[s];
        }
        zx /= Lx * Ly;
        zy /= Lx * Ly;
    }
    for (int t = 0; t < Nt; t++) {
        u[2 * t] += uk[2 * t] + zx;
        u[2 * t + 1] += uk[2 * t + 1] + zy;
    }
    free(uk);
}
