/*
 * or_quant.c -- CPU oracle of the other spectral Ewald quantities: pressure,
 * pressure gradient, velocity gradient, stress and vorticity of the 2-D
 * Stokeslet (SLP) and stresslet (DLP).
 *
 * TEST INFRASTRUCTURE ONLY (see or_ewald.h).  Restates, per quantity q and
 * kind, the reference's real-space and k-space MEX gateways (paths relative
 * to annabroms/FastTools2D, PeriodicEwald/src/mex/):
 *   real:   StokesSLP/mex_stokes_slp_{pressure,pressure_grad,gradient,stress,vorticity}_real.cpp
 *           StokesDLP/mex_stokes_dlp_{pressure,pressure_grad,gradient,stress,vorticity}_real.cpp
 *           (own box: every source except the skipped coincident one; the 8
 *            periodic neighbour boxes: r^2 < Lx Ly / (nside_x nside_y))
 *   kspace: StokesSLP/mex_stokes_slp_*_kspace.cpp, StokesDLP/mex_stokes_dlp_*_kspace.cpp
 *           (Spread of f, or of (f1 n1, f2 n1) and (f1 n2, f2 n2); fft2; the
 *            quantity's filter on the full complex spectrum with the
 *            reference's wave-number map; k = 0 zeroed; ifft2; Gather)
 * The pair formulas and filters are written term by term in the reference's
 * order of operations so that results agree to rounding.
 */
#include "or_ewald.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "or_fft.h"

#define OR_PI 3.1415926535897932385

int or_q_ncomp(int q) {
    switch (q) {
        case OR_Q_PRESSURE: return 1;
        case OR_Q_PRESSURE_GRAD: return 2;
        case OR_Q_GRADIENT: return 4;
        case OR_Q_STRESS: return 4;
        case OR_Q_VORTICITY: return 1;
        default: return 0;
    }
}

/* ---- pair terms (target - source = (r1, r2)) ----------------------------- */

/* Stokeslet quantities.  Own-box pairs at r = 0 are skipped (the gateways'
 * own-box loops; their neighbour loops have only the cutoff test). */
static int slp_pair(int q, int own, double r1, double r2, double f1, double f2, double xi, double* t) {
    const double xi2 = xi * xi;
    const double rSq = r1 * r1 + r2 * r2;
    if (own && rSq == 0) return 0;
    switch (q) {
        case OR_Q_PRESSURE: { /* mex_stokes_slp_pressure_real.cpp:98-106 */
            double rdotf = r1 * f1 + r2 * f2;
            t[0] += rdotf * exp(-xi * xi * rSq) / rSq;
            break;
        }
        case OR_Q_PRESSURE_GRAD: { /* mex_stokes_slp_pressure_grad_real.cpp:105-119 */
            double rdotf = r1 * f1 + r2 * f2;
            t[0] -= exp(-xi * xi * rSq) * ((f1 - 2 * xi * xi * rdotf * r1) / rSq - 2 * rdotf * r1 / rSq / rSq);
            t[1] -= exp(-xi * xi * rSq) * ((f2 - 2 * xi * xi * rdotf * r2) / rSq - 2 * rdotf * r2 / rSq / rSq);
            break;
        }
        case OR_Q_GRADIENT: { /* mex_stokes_slp_gradient_real.cpp (own box and neighbours) */
            double e2 = exp(-xi2 * rSq);
            double rdotf = f1 * r1 + f2 * r2;
            t[0] += e2 * (2 * xi * xi * r1 * f1 + rdotf / rSq - 2 * r1 * r1 * rdotf * (xi * xi + 1 / rSq) / rSq);
            t[1] += e2 * (2 * xi * xi * r1 * f2 + (-r1 * f2 + r2 * f1) / rSq -
                          2 * r1 * r2 * rdotf * (xi * xi + 1 / rSq) / rSq);
            t[2] += e2 * (2 * xi * xi * r2 * f1 + (r1 * f2 - r2 * f1) / rSq -
                          2 * r1 * r2 * rdotf * (xi * xi + 1 / rSq) / rSq);
            t[3] += e2 * (2 * xi * xi * r2 * f2 + rdotf / rSq - 2 * r2 * r2 * rdotf * (xi * xi + 1 / rSq) / rSq);
            break;
        }
        case OR_Q_STRESS: { /* mex_stokes_slp_stress_real.cpp */
            double e2 = exp(-xi2 * rSq);
            double rdotf = f1 * r1 + f2 * r2;
            t[0] += e2 * (2 * xi2 * (rdotf + r1 * f1 + r1 * f1) - 4 * r1 * r1 * rdotf / (rSq * rSq) * (1 + xi2 * rSq));
            t[1] += e2 * (2 * xi2 * (r2 * f1 + r1 * f2) - 4 * r1 * r2 * rdotf / (rSq * rSq) * (1 + xi2 * rSq));
            t[2] += e2 * (2 * xi2 * (r1 * f2 + r2 * f1) - 4 * r2 * r1 * rdotf / (rSq * rSq) * (1 + xi2 * rSq));
            t[3] += e2 * (2 * xi2 * (rdotf + r2 * f2 + r2 * f2) - 4 * r2 * r2 * rdotf / (rSq * rSq) * (1 + xi2 * rSq));
            break;
        }
        case OR_Q_VORTICITY: { /* mex_stokes_slp_vorticity_real.cpp */
            double e2 = exp(-xi2 * rSq);
            double fdotrperp = f1 * r2 - f2 * r1;
            t[0] += e2 * (1 / rSq - xi2) * fdotrperp;
            break;
        }
    }
    return 1;
}

/* Stresslet quantities (density f, normal n); the vorticity's own-box loop
 * skips r^2 < 1e-13, the others r = 0. */
static int dlp_pair(int q, int own, double r1, double r2, double f1, double f2, double n1, double n2, double xi,
                    double* t) {
    const double xi2 = xi * xi;
    const double rSq = r1 * r1 + r2 * r2;
    if (own && (q == OR_Q_VORTICITY ? (rSq < 1e-13) : (rSq == 0))) return 0;
    switch (q) {
        case OR_Q_PRESSURE: { /* mex_stokes_dlp_pressure_real.cpp */
            double rdotf = r1 * f1 + r2 * f2;
            double rdotn = r1 * n1 + r2 * n2;
            double fdotn = f1 * n1 + f2 * n2;
            t[0] -= exp(-xi * xi * rSq) * ((fdotn - 2 * xi * xi * rdotn * rdotf) / rSq - 2 * rdotn * rdotf / rSq / rSq);
            break;
        }
        case OR_Q_PRESSURE_GRAD: { /* mex_stokes_dlp_pressure_grad_real.cpp */
            double rdotf = r1 * f1 + r2 * f2;
            double rdotn = r1 * n1 + r2 * n2;
            double fdotn = f1 * n1 + f2 * n2;
            double e = exp(-xi2 * rSq);
            t[0] += e * (2 * xi2 * (r1 * fdotn + f1 * rdotn + n1 * rdotf - 2 * xi2 * r1 * rdotf * rdotn) / rSq +
                         2 * (r1 * fdotn + f1 * rdotn + n1 * rdotf - 4 * xi2 * r1 * rdotn * rdotf) / rSq / rSq -
                         8 * r1 * rdotn * rdotf / rSq / rSq / rSq);
            t[1] += e * (2 * xi2 * (r2 * fdotn + f2 * rdotn + n2 * rdotf - 2 * xi2 * r2 * rdotf * rdotn) / rSq +
                         2 * (r2 * fdotn + f2 * rdotn + n2 * rdotf - 4 * xi2 * r2 * rdotn * rdotf) / rSq / rSq -
                         8 * r2 * rdotn * rdotf / rSq / rSq / rSq);
            break;
        }
        case OR_Q_GRADIENT: { /* mex_stokes_dlp_gradient_real.cpp */
            double e2 = exp(-xi2 * rSq);
            double rdotf = r1 * f1 + r2 * f2;
            double rdotn = r1 * n1 + r2 * n2;
            double fdotn = f1 * n1 + f2 * n2;
            double c = (8 * xi2 * xi2 / rSq + 16 * xi2 / rSq / rSq + 16 / rSq / rSq / rSq);
            t[0] += e2 * (r1 * r1 * rdotf * rdotn * c -
                          4 * (1 + xi2 * rSq) * (rdotf * rdotn + r1 * f1 * rdotn + r1 * n1 * rdotf) / rSq / rSq +
                          2 * xi2 * (2 * f1 * n1 + fdotn - 2 * xi2 * r1 * (f1 * rdotn + n1 * rdotf + r1 * fdotn)));
            t[1] += e2 * (r1 * r2 * rdotf * rdotn * c - 4 * (1 + xi2 * rSq) * (r2 * f1 * rdotn + r2 * n1 * rdotf) / rSq / rSq +
                          2 * xi2 * (f1 * n2 + n1 * f2 - 2 * xi2 * r1 * (f2 * rdotn + n2 * rdotf + r2 * fdotn)));
            t[2] += e2 * (r1 * r2 * rdotf * rdotn * c - 4 * (1 + xi2 * rSq) * (r1 * f2 * rdotn + r1 * n2 * rdotf) / rSq / rSq +
                          2 * xi2 * (f2 * n1 + f1 * n2 - 2 * xi2 * r2 * (f1 * rdotn + n1 * rdotf + r1 * fdotn)));
            t[3] += e2 * (r2 * r2 * rdotf * rdotn * c -
                          4 * (1 + xi2 * rSq) * (rdotf * rdotn + r2 * f2 * rdotn + r2 * n2 * rdotf) / rSq / rSq +
                          2 * xi2 * (2 * f2 * n2 + fdotn - 2 * xi2 * r2 * (f2 * rdotn + n2 * rdotf + r2 * fdotn)));
            break;
        }
        case OR_Q_STRESS: { /* mex_stokes_dlp_stress_real.cpp, mu = 1 */
            const double mu = 1.0;
            double e2 = exp(-xi2 * rSq);
            double rdotf = r1 * f1 + r2 * f2;
            double rdotn = r1 * n1 + r2 * n2;
            double fdotn = f1 * n1 + f2 * n2;
            double c = ((8 * xi2 * xi2) / rSq + (16 * xi2) / (rSq * rSq) + 16 / (rSq * rSq * rSq));
            double pr = 1 / (2 * OR_PI) * ((fdotn - 2 * xi2 * rdotf * rdotn) / rSq - 2 * rdotf * rdotn / (rSq * rSq));
            t[0] += e2 * (pr + 1 / (4 * OR_PI) * 2 * mu *
                                   (r1 * r1 * rdotf * rdotn * c -
                                    2 * (1 + xi2 * rSq) *
                                        (f1 * r1 * rdotn + n1 * r1 * rdotf + r1 * f1 * rdotn + r1 * n1 * rdotf +
                                         2 * rdotf * rdotn) /
                                        (rSq * rSq) +
                                    2 * xi2 *
                                        (fdotn + n1 * f1 + f1 * n1 -
                                         xi2 * (2 * r1 * r1 * fdotn + r1 * f1 * rdotn + r1 * n1 * rdotf +
                                                f1 * r1 * rdotn + n1 * r1 * rdotf))));
            t[1] += 1 / (4 * OR_PI) * 2 * mu * e2 *
                    (r1 * r2 * rdotf * rdotn * c -
                     2 * (1 + xi2 * rSq) * (f1 * r2 * rdotn + n1 * r2 * rdotf + r1 * f2 * rdotn + r1 * n2 * rdotf) /
                         (rSq * rSq) +
                     2 * xi2 *
                         (n1 * f2 + f1 * n2 -
                          xi2 * (2 * r1 * r2 * fdotn + r1 * f2 * rdotn + r1 * n2 * rdotf + f1 * r2 * rdotn +
                                 n1 * r2 * rdotf)));
            t[2] += 1 / (4 * OR_PI) * 2 * mu * e2 *
                    (r2 * r1 * rdotf * rdotn * c -
                     2 * (1 + xi2 * rSq) * (f2 * r1 * rdotn + n2 * r1 * rdotf + r2 * f1 * rdotn + r2 * n1 * rdotf) /
                         (rSq * rSq) +
                     2 * xi2 *
                         (n2 * f1 + f2 * n1 -
                          xi2 * (2 * r2 * r1 * fdotn + r2 * f1 * rdotn + r2 * n1 * rdotf + f2 * r1 * rdotn +
                                 n2 * r1 * rdotf)));
            t[3] += e2 * (pr + 1 / (4 * OR_PI) * 2 * mu *
                                   (r2 * r2 * rdotf * rdotn * c -
                                    2 * (1 + xi2 * rSq) *
                                        (f2 * r2 * rdotn + n2 * r2 * rdotf + r2 * f2 * rdotn + r2 * n2 * rdotf +
                                         2 * rdotf * rdotn) /
                                        (rSq * rSq) +
                                    2 * xi2 *
                                        (fdotn + n2 * f2 + f2 * n2 -
                                         xi2 * (2 * r2 * r2 * fdotn + r2 * f2 * rdotn + r2 * n2 * rdotf +
                                                f2 * r2 * rdotn + n2 * r2 * rdotf))));
            break;
        }
        case OR_Q_VORTICITY: { /* mex_stokes_dlp_vorticity_real.cpp */
            double e2 = exp(-xi2 * rSq);
            double rdotn = r1 * n1 + r2 * n2;
            double rdotf = r1 * f1 + r2 * f2;
            double rdot = r1 * (n2 * rdotf + f2 * rdotn) - r2 * (n1 * rdotf + f1 * rdotn);
            double ndot = n1 * (r2 * rdotf) - n2 * (r1 * rdotf);
            double fdot = f1 * (r2 * rdotn) - f2 * (r1 * rdotn);
            t[0] += e2 * ((1 + xi2 * rSq) * rdot / (rSq * rSq) + xi2 * xi2 * (ndot + fdot));
            break;
        }
    }
    return 1;
}

/* output scaling of the gateways: SLP gradient and stress Ts/4/pi, the
 * other SLP quantities /(2 pi); DLP pressure and its gradient /(2 pi),
 * gradient /4/pi, vorticity /pi, stress unscaled (its terms carry 1/(2 pi)
 * and 1/(4 pi) themselves) */
static double real_out(int kind, int q, double v) {
    if (kind == OR_KIND_SLP) return (q == OR_Q_GRADIENT || q == OR_Q_STRESS) ? v / 4 / OR_PI : v / (2 * OR_PI);
    switch (q) {
        case OR_Q_GRADIENT: return v / 4 / OR_PI;
        case OR_Q_STRESS: return v;
        case OR_Q_VORTICITY: return v / OR_PI;
        default: return v / (2 * OR_PI);
    }
}

static const int q_ilist_x[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
static const int q_ilist_y[8] = {-1, 0, 1, -1, 1, -1, 0, 1};

int or_q_real(int kind, int q, const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f,
              const double* n, double xi, int nside_x, int nside_y, double Lx, double Ly, double* out) {
    const int nc = or_q_ncomp(q);
    if (!nc || (kind == OR_KIND_DLP && !n)) return -1;
    const int nb = nside_x * nside_y;
    int *po_s = malloc(sizeof(int) * (size_t)(Nsrc + 1)), *po_t = malloc(sizeof(int) * (size_t)(Ntar + 1));
    int *bo_s = malloc(sizeof(int) * (size_t)(nb + 1)), *bo_t = malloc(sizeof(int) * (size_t)(nb + 1));
    int *ns = malloc(sizeof(int) * (size_t)nb), *nt = malloc(sizeof(int) * (size_t)nb);
    double* ps = malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* pt = malloc(sizeof(double) * 2 * (size_t)(Ntar + 1));
    double* fs = malloc(sizeof(double) * 4 * (size_t)(Nsrc + 1));
    double* acc = calloc((size_t)nc * (size_t)(Ntar + 1), sizeof(double));
    int rc = -1;
    if (!po_s || !po_t || !bo_s || !bo_t || !ns || !nt || !ps || !pt || !fs || !acc) goto done;
    if (or_assign(psrc, ptar, Lx, Ly, Nsrc, Ntar, nside_x, nside_y, po_s, bo_s, ns, po_t, bo_t, nt)) goto done;
    for (int j = 0; j < Nsrc; j++) {
        int i = po_s[j];
        ps[2 * j] = psrc[2 * i];
        ps[2 * j + 1] = psrc[2 * i + 1];
        fs[4 * j] = f[2 * i];
        fs[4 * j + 1] = f[2 * i + 1];
        fs[4 * j + 2] = n ? n[2 * i] : 0.0;
        fs[4 * j + 3] = n ? n[2 * i + 1] : 0.0;
    }
    for (int j = 0; j < Ntar; j++) {
        pt[2 * j] = ptar[2 * po_t[j]];
        pt[2 * j + 1] = ptar[2 * po_t[j] + 1];
    }
    {
        const double cutoffsq = Lx * Ly / nside_x / nside_y;
#pragma omp parallel for schedule(dynamic)
        for (int b = 0; b < nb; b++) {
            if (nt[b] == 0) continue;
            const int t0 = bo_t[b], s0 = bo_s[b];
            for (int j = t0; j < t0 + nt[b]; j++)
                for (int k = s0; k < s0 + ns[b]; k++) {
                    double r1 = pt[2 * j] - ps[2 * k], r2 = pt[2 * j + 1] - ps[2 * k + 1];
                    if (kind == OR_KIND_SLP)
                        slp_pair(q, 1, r1, r2, fs[4 * k], fs[4 * k + 1], xi, acc + (size_t)nc * j);
                    else
                        dlp_pair(q, 1, r1, r2, fs[4 * k], fs[4 * k + 1], fs[4 * k + 2], fs[4 * k + 3], xi,
                                 acc + (size_t)nc * j);
                }
            for (int e = 0; e < 8; e++) {
                int px = b % nside_x + q_ilist_x[e], py = b / nside_x + q_ilist_y[e];
                int tx = (px + nside_x) % nside_x, ty = (py + nside_y) % nside_y;
                int sb = ty * nside_x + tx;
                if (ns[sb] <= 0) continue;
                double zx = (Lx * (px - tx)) / nside_x, zy = (Ly * (py - ty)) / nside_y;
                for (int j = t0; j < t0 + nt[b]; j++)
                    for (int k = bo_s[sb]; k < bo_s[sb] + ns[sb]; k++) {
                        double r1 = pt[2 * j] - (ps[2 * k] + zx), r2 = pt[2 * j + 1] - (ps[2 * k + 1] + zy);
                        if (!(r1 * r1 + r2 * r2 < cutoffsq)) continue;
                        if (kind == OR_KIND_SLP)
                            slp_pair(q, 0, r1, r2, fs[4 * k], fs[4 * k + 1], xi, acc + (size_t)nc * j);
                        else
                            dlp_pair(q, 0, r1, r2, fs[4 * k], fs[4 * k + 1], fs[4 * k + 2], fs[4 * k + 3], xi,
                                     acc + (size_t)nc * j);
                    }
            }
        }
    }
    for (int j = 0; j < Ntar; j++)
        for (int c = 0; c < nc; c++) out[(size_t)nc * po_t[j] + c] = real_out(kind, q, acc[(size_t)nc * j + c]);
    rc = 0;
done:
    free(po_s); free(po_t); free(bo_s); free(bo_t); free(ns); free(nt);
    free(ps); free(pt); free(fs); free(acc);
    return rc;
}

/* ---- k-space ------------------------------------------------------------ */

/* The quantity filter at one mode.  in[g] / out[o] hold (re, im) of the
 * spread spectra and of the outputs; all are read before any is written. */
static void q_filter(int kind, int q, double k1, double k2, double xi, double eta, const double* inr,
                     const double* ini, double* outr, double* outi) {
    const double Ksq = k1 * k1 + k2 * k2;
    const double xi2 = xi * xi;
    if (kind == OR_KIND_SLP) {
        const double q1r = inr[0], q1i = ini[0], q2r = inr[1], q2i = ini[1];
        switch (q) {
            case OR_Q_PRESSURE: { /* mex_stokes_slp_pressure_kspace.cpp */
                double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
                double kr = k1 * q1r + k2 * q2r, ki = k1 * q1i + k2 * q2i;
                outr[0] = ki * e / Ksq;
                outi[0] = -kr * e / Ksq;
                break;
            }
            case OR_Q_PRESSURE_GRAD: { /* mex_stokes_slp_pressure_grad_kspace.cpp */
                double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
                double kr = k1 * q1r + k2 * q2r, ki = k1 * q1i + k2 * q2i;
                outr[0] = -k1 * kr * e / Ksq;
                outi[0] = -k1 * ki * e / Ksq;
                outr[1] = -k2 * kr * e / Ksq;
                outi[1] = -k2 * ki * e / Ksq;
                break;
            }
            case OR_Q_GRADIENT: { /* mex_stokes_slp_gradient_kspace.cpp */
                double e = (1.0 / (Ksq * Ksq) + 0.25 / (Ksq * xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * Ksq);
                double kr = k1 * q1r + k2 * q2r, ki = k1 * q1i + k2 * q2i;
                outi[0] = k1 * (Ksq * q1r - k1 * kr) * e;
                outr[0] = -k1 * (Ksq * q1i - k1 * ki) * e;
                outi[1] = k1 * (Ksq * q2r - k2 * kr) * e;
                outr[1] = -k1 * (Ksq * q2i - k2 * ki) * e;
                outi[2] = k2 * (Ksq * q1r - k1 * kr) * e;
                outr[2] = -k2 * (Ksq * q1i - k1 * ki) * e;
                outi[3] = k2 * (Ksq * q2r - k2 * kr) * e;
                outr[3] = -k2 * (Ksq * q2i - k2 * ki) * e;
                break;
            }
            case OR_Q_STRESS: { /* mex_stokes_slp_stress_kspace.cpp */
                double e = exp(-0.25 * (1 - eta) / xi2 * Ksq) * (1.0 + Ksq / (4 * xi2)) / Ksq;
                double kr = k1 * q1r + k2 * q2r, ki = k1 * q1i + k2 * q2i;
                outr[0] = -(ki + q1i * k1 + q1i * k1 - 2 * (k1 * k1 * ki) / Ksq) * e;
                outi[0] = (kr + q1r * k1 + q1r * k1 - 2 * (k1 * k1 * kr) / Ksq) * e;
                outr[1] = -(q2i * k1 + q1i * k2 - 2 * (k2 * k1 * ki) / Ksq) * e;
                outi[1] = (q2r * k1 + q1r * k2 - 2 * (k2 * k1 * kr) / Ksq) * e;
                outr[2] = -(q1i * k2 + q2i * k1 - 2 * (k1 * k2 * ki) / Ksq) * e;
                outi[2] = (q1r * k2 + q2r * k1 - 2 * (k1 * k2 * kr) / Ksq) * e;
                outr[3] = -(ki + q2i * k2 + q2i * k2 - 2 * (k2 * k2 * ki) / Ksq) * e;
                outi[3] = (kr + q2r * k2 + q2r * k2 - 2 * (k2 * k2 * kr) / Ksq) * e;
                break;
            }
            case OR_Q_VORTICITY: { /* mex_stokes_slp_vorticity_kspace.cpp */
                double e = (1.0 / Ksq + 0.25 / (xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * Ksq);
                double fr = q1r * k2 - q2r * k1, fi = q1i * k2 - q2i * k1;
                outr[0] = fi * e;
                outi[0] = -fr * e;
                break;
            }
        }
        return;
    }
    /* stresslet: grids 0..3 hold the spectra of f1 n1, f2 n1, f1 n2, f2 n2.
     * The reference names grid 1 "f1n2" and grid 2 "f2n1"; the formulas below
     * keep its names (a = f1n1, b = its "f1n2", c = its "f2n1", d = f2n2). */
    for (int part = 0; part < 2; part++) {
        const double* in = part ? ini : inr;
        double* out = part ? outi : outr;
        const double a = in[0], b = in[1], c = in[2], d = in[3];
        switch (q) {
            case OR_Q_PRESSURE: { /* mex_stokes_dlp_pressure_kspace.cpp */
                double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
                out[0] = -(k1 * k1 * a + k1 * k2 * (b + c) + k2 * k2 * d) * e / Ksq;
                break;
            }
            case OR_Q_GRADIENT: { /* mex_stokes_dlp_gradient_kspace.cpp */
                double e = exp(-Ksq * (1 - eta) / (4 * xi * xi)) * (1 + Ksq / (4 * xi * xi)) / Ksq;
                double S = (k1 * k1 * a + k1 * k2 * (b + c) + k2 * k2 * d);
                out[0] = -k1 * (2 * a * k1 + k2 * (b + c) + k1 * (a + d) - 2 * k1 * S / Ksq) * e;
                out[1] = -k1 * (2 * d * k2 + k1 * (b + c) + k2 * (a + d) - 2 * k2 * S / Ksq) * e;
                out[2] = -k2 * (2 * a * k1 + k2 * (b + c) + k1 * (a + d) - 2 * k1 * S / Ksq) * e;
                out[3] = -k2 * (2 * d * k2 + k1 * (b + c) + k2 * (a + d) - 2 * k2 * S / Ksq) * e;
                break;
            }
            case OR_Q_STRESS: { /* mex_stokes_dlp_stress_kspace.cpp, mu = 1 */
                const double mu = 1.0;
                double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
                double S = (k1 * k1 * a + k1 * k2 * b + k2 * k1 * c + k2 * k2 * d);
                double m = mu * (1 / Ksq + 0.25 / (xi * xi));
                out[0] = e * (S / Ksq - m * (2 * k1 * k1 * (a + d) + k1 * (k1 * a + k2 * b) + k1 * (k1 * a + k2 * c) +
                                             k1 * (k1 * a + k2 * b) + k1 * (k1 * a + k2 * c) - 4 * k1 * k1 * S / Ksq));
                out[1] = -e * m * (2 * k2 * k1 * (a + d) + k2 * (k1 * a + k2 * b) + k2 * (k1 * a + k2 * c) +
                                   k1 * (k1 * c + k2 * d) + k1 * (k1 * b + k2 * d) - 4 * k2 * k1 * S / Ksq);
                out[2] = -e * m * (2 * k1 * k2 * (a + d) + k1 * (k1 * c + k2 * d) + k1 * (k1 * b + k2 * d) +
                                   k2 * (k1 * a + k2 * b) + k2 * (k1 * a + k2 * c) - 4 * k1 * k2 * S / Ksq);
                out[3] = e * (S / Ksq - m * (2 * k2 * k2 * (a + d) + k2 * (k1 * c + k2 * d) + k2 * (k1 * b + k2 * d) +
                                             k2 * (k1 * c + k2 * d) + k2 * (k1 * b + k2 * d) - 4 * k2 * k2 * S / Ksq));
                break;
            }
            case OR_Q_VORTICITY: { /* mex_stokes_dlp_vorticity_kspace.cpp */
                double e = (1.0 / Ksq + 1 / (4 * xi2)) * exp(-Ksq * (1 - eta) / (4 * xi2));
                double t1 = k1 * k2 * a + k2 * k2 * b - (k1 * k1 * c + k1 * k2 * d);
                double t2 = k1 * k2 * a + k2 * k2 * c - (k1 * k1 * b + k1 * k2 * d);
                out[0] = (t1 + t2) * e;
                break;
            }
            default: break;
        }
    }
    if (q == OR_Q_PRESSURE_GRAD) { /* mex_stokes_dlp_pressure_grad_kspace.cpp: i k times the pressure part */
        double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
        double Sr = k1 * k1 * inr[0] + k1 * k2 * (inr[1] + inr[2]) + k2 * k2 * inr[3];
        double Si = k1 * k1 * ini[0] + k1 * k2 * (ini[1] + ini[2]) + k2 * k2 * ini[3];
        outi[0] = -k1 * Sr * e / Ksq;
        outr[0] = k1 * Si * e / Ksq;
        outi[1] = -k2 * Sr * e / Ksq;
        outr[1] = k2 * Si * e / Ksq;
    }
}

int or_q_kspace(int kind, int q, const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f,
                const double* n, double xi, double eta, int Mx, int My, double Lx, double Ly, double w, int P,
                double* out) {
    const int nc = or_q_ncomp(q);
    if (!nc || (kind == OR_KIND_DLP && !n)) return -1;
    const int ng = kind == OR_KIND_SLP ? 2 : 4;
    const double h = Lx / Mx;
    const size_t G = (size_t)Mx * My;
    double *re[4] = {0, 0, 0, 0}, *im[4] = {0, 0, 0, 0}, *ore[4] = {0, 0, 0, 0}, *oim[4] = {0, 0, 0, 0};
    double* e1 = malloc(sizeof(double) * (size_t)(P + 1));
    double* v1 = malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    double* v2 = malloc(sizeof(double) * 2 * (size_t)(Nsrc + 1));
    int rc = -1;
    for (int g = 0; g < 4; g++) {
        re[g] = calloc(G, sizeof(double));
        im[g] = calloc(G, sizeof(double));
        ore[g] = calloc(G, sizeof(double));
        oim[g] = calloc(G, sizeof(double));
        if (!re[g] || !im[g] || !ore[g] || !oim[g]) goto done;
    }
    if (!e1 || !v1 || !v2) goto done;
    for (int i = 0; i < Nsrc; i++) {
        if (kind == OR_KIND_SLP) {
            v1[2 * i] = f[2 * i];
            v1[2 * i + 1] = f[2 * i + 1];
        } else {
            v1[2 * i] = f[2 * i] * n[2 * i];
            v1[2 * i + 1] = f[2 * i + 1] * n[2 * i];
            v2[2 * i] = f[2 * i] * n[2 * i + 1];
            v2[2 * i + 1] = f[2 * i + 1] * n[2 * i + 1];
        }
    }
    or_spread(re[0], re[1], e1, psrc, v1, Nsrc, Lx, Ly, xi, w, eta, P, Mx, My, h);
    if (kind == OR_KIND_DLP) or_spread(re[2], re[3], e1, psrc, v2, Nsrc, Lx, Ly, xi, w, eta, P, Mx, My, h);
    for (int g = 0; g < ng; g++) or_fft2(My, Mx, re[g], im[g], 0);
    for (int j = 0; j < Mx; j++) {
        double k1 = j <= Mx / 2 ? 2.0 * OR_PI / Lx * j : 2.0 * OR_PI / Lx * (j - Mx);
        for (int k = 0; k < My; k++) {
            /* rows 0..My/2 carry k2 >= 0 (Nyquist positive), the rest negative */
            double k2 = k <= My / 2 ? 2.0 * OR_PI / Ly * k : 2.0 * OR_PI / Ly * (k - My);
            size_t p = (size_t)j * My + k;
            double ir[4], ii[4], orr[4], oii[4];
            for (int g = 0; g < 4; g++) {
                ir[g] = g < ng ? re[g][p] : 0.0;
                ii[g] = g < ng ? im[g][p] : 0.0;
            }
            q_filter(kind, q, k1, k2, xi, eta, ir, ii, orr, oii);
            for (int o = 0; o < nc; o++) {
                ore[o][p] = orr[o];
                oim[o][p] = oii[o];
            }
        }
    }
    for (int o = 0; o < nc; o++) {
        ore[o][0] = 0;
        oim[o][0] = 0;
        or_fft2(My, Mx, ore[o], oim[o], 1);
    }
    for (size_t j = 0; j < (size_t)nc * Ntar; j++) out[j] = 0.0;
    for (int o = 0; o < nc; o++) or_gather(ore[o], nc, o + 1, e1, ptar, out, Ntar, Lx, Ly, xi, w, eta, P, Mx, My, h);
    rc = 0;
done:
    for (int g = 0; g < 4; g++) { free(re[g]); free(im[g]); free(ore[g]); free(oim[g]); }
    free(e1); free(v1); free(v2);
    return rc;
}
