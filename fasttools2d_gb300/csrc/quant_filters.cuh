// quant_filters.cuh -- k-space multipliers of the other spectral Ewald
// quantities (pressure, pressure gradient, velocity gradient, stress,
// vorticity), restating the filter loops of the reference's k-space gateways
// (paths relative to annabroms/FastTools2D, PeriodicEwald/src/mex/):
//   StokesSLP/mex_stokes_slp_{pressure,pressure_grad,gradient,stress,vorticity}_kspace.cpp
//   StokesDLP/mex_stokes_dlp_{pressure,pressure_grad,gradient,stress,vorticity}_kspace.cpp
// Inputs: the spread spectra at wave vector (k1, k2) -- SLP: f1, f2; DLP:
// f1 n1, f2 n1, f1 n2, f2 n2 (the reference names the middle two "f1n2" and
// "f2n1"; the formulas keep its names: a = f1n1, b = its f1n2, c = its f2n1,
// d = f2n2).  Outputs: fte_q_ncomp(q) spectra, in the gateways' order.
#pragma once

#include "fte_internal.cuh"

__host__ __device__ constexpr int fte_q_nout(int q) {
    return q == FTE_Q_PRESSURE ? 1
           : q == FTE_Q_PRESSURE_GRAD ? 2
           : (q == FTE_Q_GRADIENT || q == FTE_Q_STRESS) ? 4
           : q == FTE_Q_VORTICITY ? 1
                                  : 2;
}

// stresslet filters act on real and imaginary parts alike (real coefficients)
template <int Q>
__device__ __forceinline__ void dlp_q_part(double k1, double k2, double xi, double eta, double a, double b, double c,
                                           double d, double* out) {
    const double Ksq = k1 * k1 + k2 * k2;
    const double xi2 = xi * xi;
    if constexpr (Q == FTE_Q_PRESSURE) {
        const double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
        out[0] = -(k1 * k1 * a + k1 * k2 * (b + c) + k2 * k2 * d) * e / Ksq;
    } else if constexpr (Q == FTE_Q_GRADIENT) {
        const double e = exp(-Ksq * (1 - eta) / (4 * xi * xi)) * (1 + Ksq / (4 * xi * xi)) / Ksq;
        const double S = (k1 * k1 * a + k1 * k2 * (b + c) + k2 * k2 * d);
        out[0] = -k1 * (2 * a * k1 + k2 * (b + c) + k1 * (a + d) - 2 * k1 * S / Ksq) * e;
        out[1] = -k1 * (2 * d * k2 + k1 * (b + c) + k2 * (a + d) - 2 * k2 * S / Ksq) * e;
        out[2] = -k2 * (2 * a * k1 + k2 * (b + c) + k1 * (a + d) - 2 * k1 * S / Ksq) * e;
        out[3] = -k2 * (2 * d * k2 + k1 * (b + c) + k2 * (a + d) - 2 * k2 * S / Ksq) * e;
    } else if constexpr (Q == FTE_Q_STRESS) {
        const double mu = 1.0;
        const double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
        const double S = (k1 * k1 * a + k1 * k2 * b + k2 * k1 * c + k2 * k2 * d);
        const double m = mu * (1 / Ksq + 0.25 / (xi * xi));
        out[0] = e * (S / Ksq - m * (2 * k1 * k1 * (a + d) + k1 * (k1 * a + k2 * b) + k1 * (k1 * a + k2 * c) +
                                     k1 * (k1 * a + k2 * b) + k1 * (k1 * a + k2 * c) - 4 * k1 * k1 * S / Ksq));
        out[1] = -e * m * (2 * k2 * k1 * (a + d) + k2 * (k1 * a + k2 * b) + k2 * (k1 * a + k2 * c) +
                           k1 * (k1 * c + k2 * d) + k1 * (k1 * b + k2 * d) - 4 * k2 * k1 * S / Ksq);
        out[2] = -e * m * (2 * k1 * k2 * (a + d) + k1 * (k1 * c + k2 * d) + k1 * (k1 * b + k2 * d) +
                           k2 * (k1 * a + k2 * b) + k2 * (k1 * a + k2 * c) - 4 * k1 * k2 * S / Ksq);
        out[3] = e * (S / Ksq - m * (2 * k2 * k2 * (a + d) + k2 * (k1 * c + k2 * d) + k2 * (k1 * b + k2 * d) +
                                     k2 * (k1 * c + k2 * d) + k2 * (k1 * b + k2 * d) - 4 * k2 * k2 * S / Ksq));
    } else if constexpr (Q == FTE_Q_VORTICITY) {
        const double e = (1.0 / Ksq + 1 / (4 * xi2)) * exp(-Ksq * (1 - eta) / (4 * xi2));
        const double t1 = k1 * k2 * a + k2 * k2 * b - (k1 * k1 * c + k1 * k2 * d);
        const double t2 = k1 * k2 * a + k2 * k2 * c - (k1 * k1 * b + k1 * k2 * d);
        out[0] = (t1 + t2) * e;
    }
}

// One mode: in[g] -> out[o] (complex), as the gateways compute it.
template <int KIND, int Q>
__device__ __forceinline__ void fte_q_apply(double k1, double k2, double xi, double eta, const double2* in,
                                            double2* out) {
    const double Ksq = k1 * k1 + k2 * k2;
    const double xi2 = xi * xi;
    if constexpr (KIND == FTE_KIND_SLP) {
        const double q1r = in[0].x, q1i = in[0].y, q2r = in[1].x, q2i = in[1].y;
        const double kr = k1 * q1r + k2 * q2r, ki = k1 * q1i + k2 * q2i;
        if constexpr (Q == FTE_Q_PRESSURE) {
            const double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
            out[0] = make_double2(ki * e / Ksq, -kr * e / Ksq);
        } else if constexpr (Q == FTE_Q_PRESSURE_GRAD) {
            const double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
            out[0] = make_double2(-k1 * kr * e / Ksq, -k1 * ki * e / Ksq);
            out[1] = make_double2(-k2 * kr * e / Ksq, -k2 * ki * e / Ksq);
        } else if constexpr (Q == FTE_Q_GRADIENT) {
            const double e = (1.0 / (Ksq * Ksq) + 0.25 / (Ksq * xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * Ksq);
            out[0] = make_double2(-k1 * (Ksq * q1i - k1 * ki) * e, k1 * (Ksq * q1r - k1 * kr) * e);
            out[1] = make_double2(-k1 * (Ksq * q2i - k2 * ki) * e, k1 * (Ksq * q2r - k2 * kr) * e);
            out[2] = make_double2(-k2 * (Ksq * q1i - k1 * ki) * e, k2 * (Ksq * q1r - k1 * kr) * e);
            out[3] = make_double2(-k2 * (Ksq * q2i - k2 * ki) * e, k2 * (Ksq * q2r - k2 * kr) * e);
        } else if constexpr (Q == FTE_Q_STRESS) {
            const double e = exp(-0.25 * (1 - eta) / xi2 * Ksq) * (1.0 + Ksq / (4 * xi2)) / Ksq;
            out[0] = make_double2(-(ki + q1i * k1 + q1i * k1 - 2 * (k1 * k1 * ki) / Ksq) * e,
                                  (kr + q1r * k1 + q1r * k1 - 2 * (k1 * k1 * kr) / Ksq) * e);
            out[1] = make_double2(-(q2i * k1 + q1i * k2 - 2 * (k2 * k1 * ki) / Ksq) * e,
                                  (q2r * k1 + q1r * k2 - 2 * (k2 * k1 * kr) / Ksq) * e);
            out[2] = make_double2(-(q1i * k2 + q2i * k1 - 2 * (k1 * k2 * ki) / Ksq) * e,
                                  (q1r * k2 + q2r * k1 - 2 * (k1 * k2 * kr) / Ksq) * e);
            out[3] = make_double2(-(ki + q2i * k2 + q2i * k2 - 2 * (k2 * k2 * ki) / Ksq) * e,
                                  (kr + q2r * k2 + q2r * k2 - 2 * (k2 * k2 * kr) / Ksq) * e);
        } else if constexpr (Q == FTE_Q_VORTICITY) {
            const double e = (1.0 / Ksq + 0.25 / (xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * Ksq);
            const double fr = q1r * k2 - q2r * k1, fi = q1i * k2 - q2i * k1;
            out[0] = make_double2(fi * e, -fr * e);
        }
    } else {
        if constexpr (Q == FTE_Q_PRESSURE_GRAD) {
            // i k times the stresslet pressure's sum
            const double e = exp(-Ksq * (1 - eta) / (4 * xi * xi));
            const double Sr = k1 * k1 * in[0].x + k1 * k2 * (in[1].x + in[2].x) + k2 * k2 * in[3].x;
            const double Si = k1 * k1 * in[0].y + k1 * k2 * (in[1].y + in[2].y) + k2 * k2 * in[3].y;
            out[0] = make_double2(k1 * Si * e / Ksq, -k1 * Sr * e / Ksq);
            out[1] = make_double2(k2 * Si * e / Ksq, -k2 * Sr * e / Ksq);
        } else {
            constexpr int NO = fte_q_nout(Q);
            double orr[NO], oii[NO];
            dlp_q_part<Q>(k1, k2, xi, eta, in[0].x, in[1].x, in[2].x, in[3].x, orr);
            dlp_q_part<Q>(k1, k2, xi, eta, in[0].y, in[1].y, in[2].y, in[3].y, oii);
#pragma unroll
            for (int o = 0; o < NO; o++) out[o] = make_double2(orr[o], oii[o]);
        }
    }
}
