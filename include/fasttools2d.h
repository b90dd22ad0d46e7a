/*
 * fasttools2d.h -- C ABI of the GB300 implementation of the doubly-periodic
 * spectral Ewald (SE) summation for the 2-D Stokeslet (single layer, SLP)
 * and stresslet (double layer, DLP).
 *
 * The entry points replace annabroms/FastTools2D's spectral Ewald path
 * (paths relative to that project):
 *
 *   fte_slp_real      <- mex_stokes_slp_real     PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:58-83,340-346
 *   fte_slp_kspace    <- mex_stokes_slp_kspace   PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:7-48,205-209
 *   fte_dlp_real      <- mex_stokes_dlp_real     PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:15-52,193-200
 *   fte_dlp_kspace    <- mex_stokes_dlp_kspace   PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:10-53,272-276
 *   fte_stokes_slp_ewald_2p <- StokesSLP_ewald_2p PeriodicEwald/src/matlab/StokesSLP_ewald_2p.m:1-138
 *   fte_stokes_dlp_ewald_2p <- StokesDLP_ewald_2p PeriodicEwald/src/matlab/StokesDLP_ewald_2p.m:1-163
 *   fte_choose_params       <- the drivers' parameter selection and find_xi/find_kinfb
 *                              (StokesSLP_ewald_2p.m:27-35,85-104,147-202;
 *                               StokesDLP_ewald_2p.m:27-38,105-125,171-224)
 *
 * Conventions (as the MEX gateways): point, density and normal arrays given
 * as one pointer are 2 x N column-major doubles, i.e. x/y interleaved
 * (p[2*j], p[2*j+1]); the driver-level entries take separate x and y arrays
 * like the MATLAB functions.  Outputs are caller-allocated and written in the
 * caller's target order.  Quadrature weights are not a separate argument in
 * the reference (callers fold them into f); fte_options.weights offers the
 * same folding as a convenience.
 *
 * Pointers are host pointers unless FTE_DEVICE_POINTERS is set in `flags`,
 * in which case every array argument of that call is device memory of the
 * context's device.  Every entry returns FTE_OK or an FTE_ERR_* status; the
 * message of the last failure on the calling thread is fte_last_error().
 * A context owns one CUDA stream and its workspace; calls on one context
 * must not overlap, calls on different contexts are independent.
 */
#ifndef FASTTOOLS2D_H
#define FASTTOOLS2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FTE_VERSION 100

/* status codes */
#define FTE_OK 0
#define FTE_ERR_INVALID 1     /* argument rejected by validation */
#define FTE_ERR_CUDA 2        /* a CUDA runtime call failed */
#define FTE_ERR_ALLOC 3       /* device or host allocation failed */
#define FTE_ERR_UNSUPPORTED 4 /* valid input outside what this build implements */
#define FTE_ERR_DEVICE 5      /* a kernel reported an error status */

/* flags */
#define FTE_DEVICE_POINTERS 1u /* all array arguments are device pointers */
/* fte_batch_set_density / fte_batch_get_velocity: the host arrays are
 * page-locked (pinned); the copies are queued on the context's stream and the
 * call returns without synchronising -- the caller synchronises the stream
 * before reusing the density arrays or reading the velocities.  Many plans'
 * copies then cost one synchronisation instead of one each. */
#define FTE_HOST_ASYNC 2u

/* arithmetic forms */
/* fte_options.form: FTE_FORM_PLAIN = the drivers' parameters, FP64
 * everywhere (the drop-in); FTE_FORM_MIXED = the tuned parameter choice with
 * the cheapest arithmetic per stage that meets the tolerance (the precision
 * form).  fte_params.form reports the k-space arithmetic of an evaluation:
 *   FTE_FORM_PLAIN  FP64 spread, transforms, multiplier and gather;
 *   FTE_FORM_MIXED  FP32 spread (Kahan-compensated), transforms and gather,
 *                   the multiplier in FP64 (tol >= 1e-6 SLP, 2e-7 DLP);
 *   FTE_FORM_FF     float-float (pairs of FP32 numbers, ~48 bits) spread,
 *                   transforms, multiplier and gather (tol >= 1e-11);
 *   FTE_FORM_FF32   float-float window factors, transforms and multiplier,
 *                   FP32 products with Kahan-compensated sums in the spread
 *                   and gather (tol >= 1e-6 SLP, 2e-7 DLP; window supports
 *                   P <= 30, FTE_ERR_UNSUPPORTED when forced beyond).
 * The real-space pairs of the mixed form are FP32 for pairs whose terms lie
 * far below the tolerance, float-float for the others from tol 1e-11, and
 * FP64 below (fte_options.near). */
#define FTE_FORM_PLAIN 0
#define FTE_FORM_MIXED 1
#define FTE_FORM_FF 2
#define FTE_FORM_FF32 3

/* fte_options.kspace (FTE_FORM_MIXED): the k-space arithmetic of the tuned
 * choice; AUTO lets the chooser pick by tolerance and cost */
#define FTE_KSPACE_AUTO 0
#define FTE_KSPACE_FP64 1
#define FTE_KSPACE_FP32 2
#define FTE_KSPACE_FF 3
#define FTE_KSPACE_FF32 4

/* fte_options.near (FTE_FORM_MIXED): the arithmetic of the real-space pairs;
 * AUTO: FP32 for pairs whose terms are below the tolerance's reach of FP32
 * rounding, float-float for the others where the tolerance allows (>= 1e-11),
 * else FP64 */
#define FTE_NEAR_AUTO 0
#define FTE_NEAR_FP64 1 /* every pair in FP64 */
#define FTE_NEAR_FF 2   /* float-float pairs (stresslet pairs with xi^2 r^2 < 1e-8 in FP64), no FP32 class */

/* kinds */
#define FTE_KIND_SLP 0
#define FTE_KIND_DLP 1

typedef struct fte_context fte_context;

/* Parameters of one SE evaluation (what the MATLAB drivers compute). */
typedef struct {
    int P;          /* window support: P+1 grid nodes per direction */
    double Nb;      /* average points per cell used to size the cell list */
    double tol;     /* requested tolerance */
    double Q;       /* sum |f|^2 + 1 */
    int A, B;       /* rat(Lx/Ly) */
    int nside_x, nside_y;
    double rc;      /* real-space cutoff Lx/nside_x */
    double xi;      /* Ewald parameter */
    int kinf;       /* Fourier truncation from find_kinfb */
    int Mx, My;     /* grid size */
    double w;       /* window half-width P*h/2 */
    double eta;     /* window shape (2 xi w / m)^2, m = 0.95 sqrt(pi P) */
    int form;       /* arithmetic of the k-space part: FTE_FORM_PLAIN (FP64), FTE_FORM_MIXED (FP32),
                       FTE_FORM_FF (float-float spread, transforms, multiplier and gather) or
                       FTE_FORM_FF32 (float-float transforms, FP32 spread and gather products) */
    int ts_spread;  /* k-space spread / gather tile sizes in grid nodes (plans; 0: the default rule) */
    int ts_gather;
} fte_params;

/* Options of the driver-level entries; zero-initialise for the reference
 * defaults (P = 24, Nb = min(P round(log2 npts), npts/4), tol = 1e-16). */
typedef struct {
    int P;
    double Nb;
    double tol;
    double xi;             /* > 0: override xi */
    int Mx, My;            /* > 0: override the grid */
    int nside_x, nside_y;  /* > 0: override the cell list (cutoff = sqrt(Lx Ly/(nside_x nside_y))) */
    const double* weights; /* optional quadrature weights, multiplied into f (length nsrc) */
    int form;              /* FTE_FORM_PLAIN or FTE_FORM_MIXED */
    int tune;              /* plans: 1 = time the k-space tile sizes on the plan's points at creation */
    double slack;          /* FTE_FORM_MIXED: error-estimate slack of the tuned choice (0: calibrated) */
    int kspace;            /* FTE_FORM_MIXED: FTE_KSPACE_* (0: the chooser's pick) */
    int near;              /* FTE_FORM_MIXED: FTE_NEAR_* (0: by tolerance) */
} fte_options;

/* Per-call diagnostics (optional output of the driver entries). */
typedef struct {
    fte_params params;
    double ms_total;       /* device time of the whole evaluation (CUDA events) */
    double ms_cells;       /* cell list */
    double ms_near;        /* real-space sum */
    double ms_spread;
    double ms_fft;         /* forward + inverse FFTs and the filter */
    double ms_gather;
    long long near_pairs;  /* pairs evaluated in the real-space sum (when counted) */
    int kernels_launched;
} fte_info;

const char* fte_last_error(void);
int fte_version(void);

int fte_create(fte_context** ctx, int device);
int fte_destroy(fte_context* ctx);
/* Use an existing cudaStream_t for subsequent calls (NULL restores the
 * context's own stream). */
int fte_set_stream(fte_context* ctx, void* stream);
/* Collect per-stage CUDA-event timings into fte_info (adds syncs). */
int fte_set_timing(fte_context* ctx, int enable);
/* Number of kernels this context launched so far. */
long long fte_kernel_count(const fte_context* ctx);

/* ---- gateway-level entries (2 x N interleaved arrays) -------------------- */
int fte_slp_real(fte_context* ctx, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                 const double* f, double xi, int nside_x, int nside_y, double Lx, double Ly, double* ur,
                 unsigned flags);
int fte_dlp_real(fte_context* ctx, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar,
                 const double* f, const double* n, double xi, int nside_x, int nside_y, double Lx, double Ly,
                 double* ur, unsigned flags);
int fte_slp_kspace(fte_context* ctx, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar, double xi,
                   double eta, const double* f, int Mx, int My, double Lx, double Ly, double w, int P, double* uk,
                   unsigned flags);
int fte_dlp_kspace(fte_context* ctx, const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar, double xi,
                   double eta, const double* f, const double* n, int Mx, int My, double Lx, double Ly, double w,
                   int P, double* uk, unsigned flags);

/* ---- driver-level entries (separate x/y arrays) ------------------------- */
/* u1, u2: length ntar; ur, uk: 2 x ntar interleaved or NULL; info may be NULL. */
int fte_stokes_slp_ewald_2p(fte_context* ctx, const double* xsrc, const double* ysrc, int64_t nsrc,
                            const double* xtar, const double* ytar, int64_t ntar, const double* f1,
                            const double* f2, double Lx, double Ly, const fte_options* opt, double* u1, double* u2,
                            double* ur, double* uk, fte_info* info, unsigned flags);
int fte_stokes_dlp_ewald_2p(fte_context* ctx, const double* xsrc, const double* ysrc, int64_t nsrc,
                            const double* xtar, const double* ytar, int64_t ntar, const double* n1,
                            const double* n2, const double* f1, const double* f2, double Lx, double Ly,
                            const fte_options* opt, double* u1, double* u2, double* ur, double* uk, fte_info* info,
                            unsigned flags);

/* Parameter selection alone (host arrays f1, f2 of length nsrc; Q is
 * computed from them). */
int fte_choose_params(int kind, int64_t nsrc, int64_t ntar, const double* f1, const double* f2, double Lx,
                      double Ly, const fte_options* opt, fte_params* out);

/* ---- plans: geometry reused across density vectors ------------------------ */
/* No single counterpart in the reference, which recomputes the cell list
 * (PeriodicEwald/src/mex/common/ewald_tools.cpp:7-80) and the parameters
 * (PeriodicEwald/src/matlab/StokesSLP_ewald_2p.m:85-104) on every call.  A
 * plan does the density-independent work of a driver call once: wrapping,
 * the parameter choice (from f1, f2, a representative density, and opt; the
 * mixed form's tuned choice when opt->form == FTE_FORM_MIXED), the cell list,
 * the k-space tile bins and all scratch.  fte_plan_execute then evaluates
 * u = SLP[f] (kind FTE_KIND_SLP) or DLP[f] (FTE_KIND_DLP, normals fixed at
 * creation) for nv <= nvmax density vectors, stored as nv consecutive blocks
 * of nsrc (f1s, f2s) and ntar (u1s, u2s) values; the real-space pair geometry
 * and special functions are shared by the nv vectors.  Results equal the
 * driver entries' with the same parameters. */
typedef struct fte_plan fte_plan;
int fte_plan_create(fte_context* ctx, int kind, const double* xsrc, const double* ysrc, int64_t nsrc,
                    const double* xtar, const double* ytar, int64_t ntar, const double* n1, const double* n2,
                    const double* f1, const double* f2, double Lx, double Ly, const fte_options* opt, int nvmax,
                    fte_plan** plan, unsigned flags);
int fte_plan_params(const fte_plan* plan, fte_params* out);
int fte_plan_execute(fte_plan* plan, int nv, const double* f1s, const double* f2s, double* u1s, double* u2s,
                     unsigned flags);
int fte_plan_destroy(fte_plan* plan);

/* ---- batches: many plans in one graph launch ------------------------------ */
/* No counterpart in the reference.  A batch binds plans of one context (any
 * sizes, both kinds) and nv density vectors each to device buffers
 * (fte_batch_buffers: plan i's f1s, f2s, u1s, u2s, laid out as in
 * fte_plan_execute).  fte_batch_launch evaluates all of them, every stage as
 * one launch over a work list of all plans: densities, the real-space sum
 * (per kind, over every plan's cells), and the float-float k-space stages of
 * every (plan, vector) (plans with another k-space form run theirs on forked
 * streams beside them); with use_graph = 1 it replays the CUDA graph captured
 * at creation (one graph launch per step of an iterative solver).
 * Asynchronous on the context's stream. */
typedef struct fte_batch fte_batch;
int fte_batch_create(fte_context* ctx, fte_plan* const* plans, int nplans, int nv, fte_batch** batch);
int fte_batch_buffers(const fte_batch* batch, int i, double** f1s, double** f2s, double** u1s, double** u2s);
int fte_batch_launch(fte_batch* batch, int use_graph);
int fte_batch_destroy(fte_batch* batch);
/* copy plan i's nv density vectors in / velocities out (host or, with
 * FTE_DEVICE_POINTERS, device arrays; host copies synchronise unless
 * FTE_HOST_ASYNC) */
int fte_batch_set_density(fte_batch* batch, int i, const double* f1s, const double* f2s, unsigned flags);
int fte_batch_get_velocity(fte_batch* batch, int i, double* u1s, double* u2s, unsigned flags);

/* ---- other quantities: gateway level ------------------------------------- */
/* Replace the reference's quantity gateways (PeriodicEwald/src/mex/):
 *   StokesSLP/mex_stokes_slp_<q>_real.cpp, StokesSLP/mex_stokes_slp_<q>_kspace.cpp,
 *   StokesDLP/mex_stokes_dlp_<q>_real.cpp, StokesDLP/mex_stokes_dlp_<q>_kspace.cpp
 * for q = pressure, pressure_grad, gradient, stress, vorticity.  Arguments
 * carry the same meaning as there (the gateways differ only in argument
 * order); n (normals) is used by the stresslet (FTE_KIND_DLP) only.  out
 * receives fte_q_ncomp(q) values per target (interleaved, the caller's target
 * order): pressure and vorticity 1, pressure gradient 2, velocity gradient
 * and stress 4, each in the gateway's component order and scaling.  FP64. */
#define FTE_Q_VELOCITY 0
#define FTE_Q_PRESSURE 1
#define FTE_Q_PRESSURE_GRAD 2
#define FTE_Q_GRADIENT 3
#define FTE_Q_STRESS 4
#define FTE_Q_VORTICITY 5
int fte_q_ncomp(int quantity);
int fte_q_real(fte_context* ctx, int kind, int quantity, const double* psrc, int64_t nsrc, const double* ptar,
               int64_t ntar, const double* f, const double* n, double xi, int nside_x, int nside_y, double Lx,
               double Ly, double* out, unsigned flags);
int fte_q_kspace(fte_context* ctx, int kind, int quantity, const double* psrc, int64_t nsrc, const double* ptar,
                 int64_t ntar, const double* f, const double* n, double xi, double eta, int Mx, int My, double Lx,
                 double Ly, double w, int P, double* out, unsigned flags);

/* Driver level: replace PeriodicEwald/src/matlab/StokesSLP_<q>_ewald_2p.m and
 * StokesDLP_<q>_ewald_2p.m (wrapping, the analytic parameter choice, the two
 * gateways, zero modes, the self terms of sources that coincide with
 * targets, and for the gradient and the stress the contraction with the
 * vector b = (b1, b2) at each target).  out receives the driver's result: 1
 * value per target for the pressure and the vorticity, 2 (interleaved) for
 * the pressure gradient, gradient.b and stress.b; out_real / out_k (may be
 * NULL) the driver's real and k parts, same layout.  n1/n2: stresslet only;
 * b1/b2: gradient and stress only.  opt as for the velocity drivers (FP64
 * plain form; opt->form is ignored).  info->params.xi is the driver's xi. */
int fte_stokes_q_ewald_2p(fte_context* ctx, int kind, int quantity, const double* xsrc, const double* ysrc,
                          int64_t nsrc, const double* xtar, const double* ytar, int64_t ntar, const double* n1,
                          const double* n2, const double* f1, const double* f2, const double* b1, const double* b2,
                          double Lx, double Ly, const fte_options* opt, double* out, double* out_real,
                          double* out_k, fte_info* info, unsigned flags);

/* ---- learned parameter selector: the network ------------------------------ */
/* No counterpart in the reference.  An FP32 multilayer perceptron
 * 8 -> 64 -> 64 -> 4 (tanh hidden units) that maps features of a
 * configuration to corrections of the tuned parameter choice (cell list,
 * xi, grid, window support).  Parameters are one FP32 vector of
 * FTE_MLP_PARAMS values: W1[64x8], b1[64], W2[64x64], b2[64], W3[4x64], b3[4]
 * (row-major, y = W x + b).  All pointers are device pointers; `stream` is a
 * cudaStream_t (NULL: default stream); calls are asynchronous. */
#define FTE_MLP_IN 8
#define FTE_MLP_HIDDEN 64
#define FTE_MLP_OUT 4
#define FTE_MLP_PARAMS (FTE_MLP_HIDDEN * FTE_MLP_IN + FTE_MLP_HIDDEN + FTE_MLP_HIDDEN * FTE_MLP_HIDDEN + \
                        FTE_MLP_HIDDEN + FTE_MLP_OUT * FTE_MLP_HIDDEN + FTE_MLP_OUT)
int fte_mlp_param_count(void);
/* scratch (floats) of fte_mlp_loss_grad for n samples */
size_t fte_mlp_scratch_floats(int n);
/* Y[n x 4] = network(X[n x 8]) */
int fte_mlp_forward(const float* params, const float* X, int n, float* Y, void* stream);
/* loss = (1/n) sum_i w_i |y_i - t_i|^2 (w null: 1) and its gradient (FTE_MLP_PARAMS floats) */
int fte_mlp_loss_grad(const float* params, const float* X, const float* T, const float* weights, int n,
                      float* scratch, float* grad, float* loss, void* stream);
/* one Adam step (step = 1, 2, ...; m, v: moment vectors, zero at step 1) */
int fte_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                 float beta2, float eps, void* stream);

/* Layout statistics for the selector's features (no counterpart in the
 * reference): for a sample of the sources -- every stride-th one, stride =
 * max(1, nsrc / nsample) -- the distance to the nearest other source in the
 * periodic Lx x Ly box, from a device cell list.  out receives
 * min(nsample, ceil(nsrc / stride)) distances in sample order (host array, or
 * device with FTE_DEVICE_POINTERS, like xsrc and ysrc).  Synchronises. */
int fte_nn_sample(fte_context* ctx, const double* xsrc, const double* ysrc, int64_t nsrc, double Lx, double Ly,
                  int nsample, double* out, unsigned flags);

/* ---- allocation-free variant --------------------------------------------- */
/* No counterpart in the reference.  The Stokeslet k-space sum of
 * fte_slp_kspace (same arguments and results) for callers that may not
 * allocate device memory: an application that hands all GPU memory to its own
 * pool, a real-time loop that must not allocate (or risk the implicit
 * synchronisation of cudaMalloc/cudaFree) after start-up, a plugin host that
 * forbids allocation outside initialisation.  It needs no context: every
 * pointer is a device pointer, `stream` is a cudaStream_t (NULL = default
 * stream), and all scratch (grids, spectra, FFT tables) lives in one fixed
 * device array of about 8.5 MB that the library holds on each GPU that loads
 * it until the process exits.  The grid is limited to
 * Mx, My <= FTE_NOALLOC_MAX_SIDE and Mx*My <= FTE_NOALLOC_MAX_NODES; larger
 * grids return FTE_ERR_UNSUPPORTED.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress), so make that first call
 * before any stream capture.  Calls share the array: calls that overlap on the
 * GPU (other streams, other threads on the same device) race and must be
 * serialised by the caller.  The call is asynchronous on `stream`. */
#define FTE_NOALLOC_MAX_SIDE 512
#define FTE_NOALLOC_MAX_NODES (512 * 512)
int fte_slp_kspace_noalloc(const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar, double xi,
                           double eta, const double* f, int Mx, int My, double Lx, double Ly, double w, int P,
                           double* uk, void* stream);

#ifdef __cplusplus
}
#endif
#endif
