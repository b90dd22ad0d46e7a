/*
 * or_ewald.h -- CPU oracle for the doubly-periodic spectral Ewald (SE) sums of
 * the 2-D Stokeslet (single layer, SLP) and stresslet (double layer, DLP).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests, the smoke check and the CPU-baseline
 * leg of the benchmark load this library, and only as a checker or as the
 * timed CPU restatement of the reference; the shipped GPU library never
 * calls it.
 *
 * Every function restates a piece of annabroms/FastTools2D (paths relative
 * to that project):
 *   or_assign               PeriodicEwald/src/mex/common/ewald_tools.cpp:7-80
 *   or_find_closest_node    PeriodicEwald/src/mex/common/ewald_tools.cpp:86-114
 *   or_spread               PeriodicEwald/src/mex/common/ewald_tools.cpp:120-199
 *   or_gather               PeriodicEwald/src/mex/common/ewald_tools.cpp:206-271
 *   or_slp_real             PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:58-357
 *   or_slp_kspace           PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:7-215
 *   or_dlp_real             PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:15-211
 *   or_dlp_kspace           PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:10-282
 *   or_choose_params        PeriodicEwald/src/matlab/StokesSLP_ewald_2p.m:27-104,147-202
 *                           PeriodicEwald/src/matlab/StokesDLP_ewald_2p.m:27-61,105-125,171-225
 *   or_stokes_*_ewald_2p    the two MATLAB drivers end to end
 *   or_*_ds                 PeriodicEwald/tests/direct_sums/matlab_sums/stokes_{slp,dlp}_{real,kspace}_ds.m
 *
 * Conventions follow the reference MEX gateways: point and density arrays are
 * 2 x N column-major (x/y interleaved), counts are int, output arrays are
 * 2 x N_trg interleaved and written in the caller's target order.
 */
#ifndef OR_EWALD_H
#define OR_EWALD_H
#ifdef __cplusplus
extern "C" {
#endif

#define OR_KIND_SLP 0
#define OR_KIND_DLP 1

/* parameter set chosen by the MATLAB drivers */
typedef struct {
    int P;          /* window support (nodes per direction minus one) */
    double Nb;      /* requested average points per cell */
    double tol;     /* requested tolerance */
    double Q;       /* sum |f|^2 + 1 */
    int A, B;       /* rat(Lx/Ly) */
    int a;          /* cell multiplier */
    int nside_x, nside_y;
    double rc;      /* real-space cutoff = Lx/nside_x */
    double xi;      /* Ewald parameter */
    int kinf;       /* find_kinfb result */
    int Mx, My;     /* grid size */
    double w;       /* window half width P*h/2 */
    double eta;     /* window shape parameter */
    double m;       /* 0.95*sqrt(pi*P) */
    int xi_iters, k_iters; /* Newton iterations taken (101 = gave up) */
} or_params;

double or_expint_e1(double x);
double or_rat(double x, int* num, int* den);

int or_assign(const double* psrc, const double* ptar, double Lx, double Ly, int nsrc, int ntar, int nside_x,
              int nside_y, int* particle_offsets_src, int* box_offsets_src, int* nsources_in_box,
              int* particle_offsets_tar, int* box_offsets_tar, int* ntargets_in_box);
void or_find_closest_node(double x, double y, double Lx, double Ly, double h, int P, int* mx, int* my, double* px,
                          double* py);
void or_spread(double* H1, double* H2, double* e1, const double* psrc, const double* f, int Nsrc, double Lx,
               double Ly, double xi, double w, double eta, int P, int Mx, int My, double h);
void or_gather(const double* H, int total_components, int component_number, const double* e1, const double* ptar,
               double* output, int Ntar, double Lx, double Ly, double xi, double w, double eta, int P, int Mx,
               int My, double h);

int or_slp_real(const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f, double xi,
                int nside_x, int nside_y, double Lx, double Ly, double* ur);
int or_dlp_real(const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f, const double* n,
                double xi, int nside_x, int nside_y, double Lx, double Ly, double* ur);
int or_slp_kspace(const double* psrc, int Nsrc, const double* ptar, int Ntar, double xi, double eta,
                  const double* f, int Mx, int My, double Lx, double Ly, double w, int P, double* uk);
int or_dlp_kspace(const double* psrc, int Nsrc, const double* ptar, int Ntar, double xi, double eta,
                  const double* f, const double* n, int Mx, int My, double Lx, double Ly, double w, int P,
                  double* uk);
/* Filter stage alone, on full complex spectra (re/im separate, column-major
 * My x Mx), in place on the first two grids. kind = OR_KIND_SLP uses grids
 * 0..1, OR_KIND_DLP grids 0..3 = spectra of (f1n1, f2n1, f1n2, f2n2). */
void or_filter(int kind, double** re, double** im, int Mx, int My, double Lx, double Ly, double xi, double eta);

int or_choose_params(int kind, int nsrc, int ntar, const double* f1, const double* f2, double Lx, double Ly, int P,
                     double Nb, double tol, or_params* out);

/* Drivers.  Nb <= 0 selects the default, P <= 0 selects 24, tol <= 0 selects 1e-16.
 * ur/uk (2 x Ntar interleaved) may be NULL. */
int or_stokes_slp_ewald_2p(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar,
                           const double* ytar, int Ntar, const double* f1, const double* f2, double Lx, double Ly,
                           int P, double Nb, double tol, double* u1, double* u2, double* ur, double* uk,
                           or_params* prm);
int or_stokes_dlp_ewald_2p(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar,
                           const double* ytar, int Ntar, const double* n1, const double* n2, const double* f1,
                           const double* f2, double Lx, double Ly, int P, double Nb, double tol, double* u1,
                           double* u2, double* ur, double* uk, or_params* prm);

/* Direct sums restated from the reference's test oracles.  Separate x/y arrays,
 * output u (2 x Ntar interleaved). */
void or_slp_real_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                    int Ntar, const double* f1, const double* f2, double Lx, double Ly, double xi, double* u);
void or_dlp_real_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                    int Ntar, const double* n1, const double* n2, const double* f1, const double* f2, double Lx,
                    double Ly, double xi, double* u);
void or_slp_kspace_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                      int Ntar, const double* f1, const double* f2, double Lx, double Ly, double xi, int kinf,
                      double* u);
void or_dlp_kspace_ds(const double* xsrc, const double* ysrc, int Nsrc, const double* xtar, const double* ytar,
                      int Ntar, const double* n1, const double* n2, const double* f1, const double* f2, double Lx,
                      double Ly, double xi, int kinf, double* u);

/* Other quantities (or_quant.c): pressure, pressure gradient, velocity
 * gradient, stress, vorticity.  Outputs have or_q_ncomp(q) components per
 * target (interleaved, caller's target order): pressure 1; pressure gradient
 * 2; velocity gradient and stress 4, in the gateways' order; vorticity 1.
 * n is required for the DLP and ignored for the SLP. */
#define OR_Q_PRESSURE 1
#define OR_Q_PRESSURE_GRAD 2
#define OR_Q_GRADIENT 3
#define OR_Q_STRESS 4
#define OR_Q_VORTICITY 5
int or_q_ncomp(int q);
int or_q_real(int kind, int q, const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f,
              const double* n, double xi, int nside_x, int nside_y, double Lx, double Ly, double* out);
int or_q_kspace(int kind, int q, const double* psrc, int Nsrc, const double* ptar, int Ntar, const double* f,
                const double* n, double xi, double eta, int Mx, int My, double Lx, double Ly, double w, int P,
                double* out);

/* Truth oracle: a converged Ewald sum with its own xi_o, real-space cutoff
 * rcut (periodic images, cell binned) and Fourier box |jk| <= kinf.  Includes
 * the SLP self term and, for the DLP, the zero mode.  Points must already be
 * wrapped into [-L/2, L/2).  n1/n2 are ignored for the SLP. */
void or_ewald_truth(int kind, const double* xsrc, const double* ysrc, int Nsrc, const double* xtar,
                    const double* ytar, int Ntar, const double* n1, const double* n2, const double* f1,
                    const double* f2, double Lx, double Ly, double xi, double rcut, int kinf, double* u);

/* number of OpenMP threads the oracle uses (for reporting) */
int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
