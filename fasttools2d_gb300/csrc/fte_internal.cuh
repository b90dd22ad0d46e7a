// fte_internal.cuh -- shared declarations of the GB300 spectral Ewald library.
#pragma once

#include <cuda_runtime.h>
#include <cmath>
#include <stdint.h>

#include <map>
#include <vector>

#include "../../include/fasttools2d.h"

// the k-space forms with float-float window factors and transforms
__host__ __device__ inline bool fte_form_ff(int form) { return form == FTE_FORM_FF || form == FTE_FORM_FF32; }

#define FTE_PI 3.14159265358979323846
#define FTE_EULER 0.57721566490153286060651209008240243

// ---------------------------------------------------------------------------
// Errors: every internal routine returns an FTE_* status and records a message
// in a thread-local buffer read by fte_last_error().
// ---------------------------------------------------------------------------
void fte_set_error(const char* fmt, ...);

#define FTE_CUDA_TRY(expr)                                                                         \
    do {                                                                                           \
        cudaError_t e_ = (expr);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            fte_set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return FTE_ERR_CUDA;                                                                   \
        }                                                                                          \
    } while (0)

// Dynamic shared-memory ceiling of a kernel.  The ceiling
// (cudaFuncAttributeMaxDynamicSharedMemorySize) belongs to the kernel -- one
// value per device for the whole process -- not to a context or a stream, so
// setting it per call to that call's own need would let a concurrent call on
// another thread lower it between a raise and the matching launch.  Instead it
// is raised once per (device, kernel), under a lock, to the most the device
// allows that kernel (the opt-in maximum minus the kernel's static shared
// memory), and never lowered.  Returns cudaErrorInvalidValue when `bytes`
// exceeds that ceiling (the launch would fail).
cudaError_t fte_smem_ceiling_raw(const void* kernel, size_t bytes);
template <typename K>
inline cudaError_t fte_smem_ceiling(K* kernel, size_t bytes) {
    return fte_smem_ceiling_raw(reinterpret_cast<const void*>(kernel), bytes);
}

#define FTE_TRY(expr)          \
    do {                       \
        int s_ = (expr);       \
        if (s_ != FTE_OK) return s_; \
    } while (0)

// launch a kernel on ctx->stream and count it
#define FTE_LAUNCH(ctx, kernel, grid, block, smem, ...)                                       \
    do {                                                                                      \
        kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                      \
        cudaError_t e_ = cudaGetLastError();                                                  \
        if (e_ != cudaSuccess) {                                                              \
            fte_set_error("launch of %s failed: %s (%s:%d)", #kernel, cudaGetErrorString(e_), \
                          __FILE__, __LINE__);                                                \
            return FTE_ERR_CUDA;                                                              \
        }                                                                                     \
        (ctx)->kernels++;                                                                     \
    } while (0)

// ---------------------------------------------------------------------------
// FFT plan for one transform length (device tables are owned by the plan).
// ---------------------------------------------------------------------------
struct FftPlan {
    int n = 0;           // transform length
    int nrad = 0;        // Stockham passes of the inner transform
    int rad[24] = {0};   // radices (2, 3, 4, 5, 7, 8)
    int bluestein = 0;   // 1: chirp-z over the 7-smooth length m
    int m = 0;           // inner transform length (n, or m >= 2n-1 for Bluestein)
    double2* tw = nullptr;     // W_m^t = exp(-2 pi i t / m), t < m   (device, FP64)
    double2* chirp = nullptr;  // exp(-i pi k^2 / n), k < n           (Bluestein)
    double2* bhat = nullptr;   // DFT_m of the conjugate chirp / m    (Bluestein)
    float2* tw32 = nullptr;    // FP32 copies for the mixed form
    float2* chirp32 = nullptr;
    float2* bhat32 = nullptr;
    float4* twff = nullptr;    // float-float copies (re hi, re lo, im hi, im lo)
    float4* chirpff = nullptr;
    float4* bhatff = nullptr;
};

// Device view of a plan passed by value to kernels.
struct FftDev {
    int n, m, nrad, bluestein;
    int rad[24];
    const double2* tw;
    const double2* chirp;
    const double2* bhat;
    const float2* tw32;
    const float2* chirp32;
    const float2* bhat32;
    const float4* twff;
    const float4* chirpff;
    const float4* bhatff;
};

// Long 1-D transforms: lines whose block transform does not fit one block's
// shared memory.  Four-step (Bailey 1990) over L = n1 * n2 with block
// transforms of n1 and n2 -- on L = n directly (mode 1), or (mode 2), when n
// has no such factorisation, as Bluestein's chirp-z convolution in global
// memory over a factorable 7-smooth L >= 2n - 1.
struct LongFft {
    int n = 0;
    int mode = 0;  // 1: four-step on n; 2: Bluestein over L
    int L = 0, n1 = 0, n2 = 0;
    FftDev d1, d2;                   // block plans of n1 and n2
    const double2* tw = nullptr;     // W_L^t, t < L
    const double2* chirp = nullptr;  // mode 2: exp(-i pi k^2 / n), k < n
    const double2* bhat = nullptr;   // mode 2: DFT_L of the conjugate chirp, / L
};
struct LongPlan {
    LongFft dev;
    double2* tw = nullptr;
    double2* chirp = nullptr;
    double2* bhat = nullptr;
};
// Lines of a batch: element j of line l sits at
//   (l / lpg) * gs + (l % lpg) * ls + j * es   (complex elements)
struct LineMap {
    long long gs, ls, es;
    int lpg;
};
// opt-in shared memory per block on sm_100 / sm_103 (227 KB)
constexpr int kFftSmemCap = 232448;

struct fte_context {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int timing = 0;
    long long kernels = 0;
    // workspace (grown on demand, reused across calls)
    char* ws = nullptr;   // point data staged for one call
    size_t ws_size = 0;
    char* ws2 = nullptr;  // cell list, grids and outputs
    size_t ws2_size = 0;
    // small pinned host buffer for scalar read-backs
    double* host_scalars = nullptr;
    std::map<int, FftPlan*> plans;
    std::map<int, LongPlan*> lplans;
    cudaEvent_t ev[8] = {nullptr};
    cudaEvent_t ev_q = nullptr;  // the drivers' Q read-back (no timing)
    int max_smem_optin = 0;
    int num_sms = 0;
    unsigned int* dev_flags = nullptr;  // device counters of the input checks
};

// ---------------------------------------------------------------------------
// Input checks.  Every array value of an entry's points, densities, normals
// and weights must be finite: a NaN or infinite coordinate has no cell, grid
// node or periodic image.  The check is one launch over the staged device
// arrays; its count is read back with the entry's first synchronisation, and
// the entry then fails with FTE_ERR_INVALID before any other kernel runs.
// ---------------------------------------------------------------------------
struct FiniteSet {
    enum { kMax = 12 };
    const double* p[kMax] = {nullptr};
    int64_t n[kMax] = {0};
    int k = 0;
    void add(const double* a, int64_t count) {
        if (a && count > 0 && k < kMax) {
            p[k] = a;
            n[k] = count;
            k++;
        }
    }
};
// queue the check and the read-back of its count (no synchronisation)
int fte_finite_launch(fte_context* c, const FiniteSet& s);
// after a synchronisation of c->stream: FTE_ERR_INVALID if a value was not finite
int fte_finite_result(fte_context* c, const char* entry);
// both, with a synchronisation between them
int fte_check_finite(fte_context* c, const FiniteSet& s, const char* entry);

// Host-side fault injection for tests (fasttools2d_debug.h): true when the
// device allocation about to be made must fail as if the device were out of
// memory.
bool fte_alloc_should_fail();

// Bump allocator over the context workspace.  Sizes are rounded to 256 B.
struct WsCarver {
    char* base;
    size_t off = 0;
    size_t cap;
    template <typename T>
    T* take(size_t count) {
        size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        T* p = reinterpret_cast<T*>(base + off);
        off += bytes;
        return p;
    }
    bool ok() const { return off <= cap; }
};
// Fails the call (before any kernel touches the carved memory) when the
// workspace estimate was too small.
#define FTE_WS_CHECK(wc)                                                                        \
    do {                                                                                        \
        if (!(wc).ok()) {                                                                       \
            fte_set_error("internal: workspace estimate too small (%zu > %zu) at %s:%d",        \
                          (size_t)(wc).off, (size_t)(wc).cap, __FILE__, __LINE__);              \
            return FTE_ERR_ALLOC;                                                               \
        }                                                                                       \
    } while (0)
inline size_t ws_bytes(size_t count, size_t elem) { return (count * elem + 255) & ~size_t(255); }

int fte_ws_reserve(fte_context* ctx, size_t bytes);

// FFT lengths: does one block transform a line of n complex values of
// `complex_bytes` each (two buffers of the inner length in shared memory)?
bool fte_fft_fits_block(int n, int complex_bytes);
// shape of the long transform of length n (FP64); false when none exists
bool fte_long_shape(int n, int* mode, int* L, int* n1, int* n2);
int fte_get_long_plan(fte_context* c, int n, LongFft* out);
// scratch (complex elements) of fte_long_fft for nl lines of length n
size_t fte_long_scratch(int n, long long nl);
// in-place FP64 transform of nl lines (unnormalised; inv: exp(+i...))
int fte_long_fft(fte_context* c, const LongFft& f, double2* X, LineMap mx, long long nl, bool inv, double2* scratch);
// block plan or long plan of length n, whichever the FP64 kernels will use
int fte_fft_prepare(fte_context* c, int n);
int fte_ws2_reserve(fte_context* ctx, size_t bytes);
int fte_get_plan(fte_context* ctx, int n, FftDev* out);
int fte_record(fte_context* ctx, int slot);
double fte_elapsed(fte_context* ctx, int a, int b);

// ---------------------------------------------------------------------------
// Device helpers shared by the kernels.
// ---------------------------------------------------------------------------

// x / d rounded to nearest from rd = RN(1/d): q = RN(x rd), the remainder
// x - q d exactly by one FMA, and RN(q + (x - q d) rd), which is the IEEE
// quotient for normal operands (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Develop. 34,
// 1990).  One multiply and two FMAs instead of a division: the per-point
// kernels divide by a grid step, a cell side or a box length that is fixed
// for the launch, and GB300 issues FP64 at 1/64 of its FP32 rate.
__device__ __forceinline__ double fte_div_rcp(double x, double d, double rd) {
    const double q = __dmul_rn(x, rd);
    const double r = __fma_rn(-q, d, x);
    return __fma_rn(r, rd, q);
}

// First window node (mx, my) and in-cell offsets (px, py) of a point: the
// reference's FindClosestNode (PeriodicEwald/src/mex/common/ewald_tools.cpp:86-114),
// with a grid step per axis (hx = Lx/Mx, hy = Ly/My; the reference has one h,
// and hx = hy reproduces it exactly).  Written with explicitly rounded
// operations so that no multiply-add is fused: the tie-break below depends on
// the exact rounding of each step (the quotients by h are the IEEE quotients,
// formed from rh = RN(1/h); halving is exact).
__device__ __forceinline__ void fte_closest_node(double x, double y, double Lx, double Ly, double hx, double rhx,
                                                 double hy, double rhy, int P, int* mx, int* my, double* px,
                                                 double* py) {
    const double TOL = 1e-13;
    double qx = fte_div_rcp(x, hx, rhx), qy = fte_div_rcp(y, hy, rhy);
    double ppx = __dsub_rn(x, __dmul_rn(hx, floor(qx)));
    double ppy = __dsub_rn(y, __dmul_rn(hy, floor(qy)));
    double lhx = __dmul_rn(Lx, 0.5), lhy = __dmul_rn(Ly, 0.5);
    double ax = fte_div_rcp(__dadd_rn(x, lhx), hx, rhx), ay = fte_div_rcp(__dadd_rn(y, lhy), hy, rhy);
    int half = P / 2;
    int ix = (int)__dsub_rn(floor(ax), (double)half);
    int iy = (int)__dsub_rn(floor(ay), (double)half);
    if (fabs(ppx) < TOL || fabs(__dsub_rn(ppx, hx)) < TOL) ppx = 0;
    if (fabs(ppy) < TOL || fabs(__dsub_rn(ppy, hy)) < TOL) ppy = 0;
    if (ppx == 0 && remainder(__dsub_rn(ax, (double)half), 1.0) < 0) ix++;
    if (ppy == 0 && remainder(__dsub_rn(ay, (double)half), 1.0) < 0) iy++;
    *mx = ix;
    *my = iy;
    *px = ppx;
    *py = ppy;
}

// MATLAB mod(v + L/2, L) - L/2 with mod's round-off compensation
// (StokesSLP_ewald_2p.m:75-78): exactly 0 when a/L is an integer to within
// eps; rL = RN(1/L).
__device__ __forceinline__ double fte_wrap_coord(double v, double L, double rL) {
    const double hl = __dmul_rn(L, 0.5);
    const double a = __dadd_rn(v, hl);
    const double q = fte_div_rcp(a, L, rL);
    double r;
    if (fabs(__dsub_rn(q, round(q))) <= 2.220446049250313e-16 * fabs(q))
        r = 0.0;
    else
        r = __dsub_rn(a, __dmul_rn(floor(q), L));
    return __dsub_rn(r, hl);
}

__device__ __forceinline__ int fte_wrap_index(int i, int M) {
    int r = i % M;
    return r < 0 ? r + M : r;
}

// Cell of a point: floor(nside (x/L + 0.5)) clamped to [0, nside-1]
// (PeriodicEwald/src/mex/common/ewald_tools.cpp:27-34).
// rL = RN(1/L).
__device__ __forceinline__ int fte_cell_1d(double x, double L, double rL, int nside) {
    int b = (int)floor(__dmul_rn((double)nside, __dadd_rn(fte_div_rcp(x, L, rL), 0.5)));
    if (b < 0) b = 0;
    if (b >= nside) b = nside - 1;
    return b;
}

// Host launchers (one translation unit each).
struct CellList {
    int nsx, nsy, nb;
    // sources sorted by cell
    int* src_off;   // nb + 1
    double2* spos;  // sorted source positions
    double* q0;     // SLP: f1 ; DLP: S11 = f1 n1
    double* q1;     // SLP: f2 ; DLP: S12 + S21
    double* q2;     // DLP: S22
    // targets sorted by cell
    int* tar_off;   // nb + 1
    double2* tpos;
    int* tidx;      // original index of each sorted target
    int max_neigh;  // upper bound of sources in a 3x3 neighbourhood (0 = unknown)
    long long qstride;  // distance between density vectors in q0..q2 (0: one vector)
    int* sidx;          // original index of each sorted source (plans only; may be null)
    int64_t nsrc = 0;   // sources
    // real-space cutoff squared; 0: the reference's Lx Ly / (nsx nsy) (the
    // square of the side of square cells).  The tuned choice of a box with an
    // irrational aspect ratio has nearly square cells and sets the square of
    // the shorter side, so that the 3 x 3 neighbourhood covers the cutoff disc.
    double cutoffsq = 0.0;
};

// Cutoff squared of a tuned parameter choice whose cells have unequal sides
// (boxes with an irrational aspect ratio): the square of the shorter side; 0
// (the reference's Lx Ly / (nsx nsy)) for square cells.
inline double fte_tuned_cutoffsq(const fte_params& p, double Lx, double Ly) {
    const double bx = Lx / p.nside_x, by = Ly / p.nside_y;
    if (std::fabs(bx - by) <= 1e-12 * std::fmax(bx, by)) return 0.0;
    const double r = std::fmin(bx, by);
    return r * r;
}

size_t fte_cells_ws(int64_t nsrc, int64_t ntar, int nb);
int fte_cells_build(fte_context* ctx, WsCarver& wc, int kind, const double* psrc, int64_t nsrc, const double* ptar,
                    int64_t ntar, const double* f, const double* nrm, const double* wts, int nsx, int nsy, double Lx,
                    double Ly, CellList* cl);
int fte_scan_exclusive(fte_context* ctx, WsCarver& wc, const int* in, int* out, int n);

// points binned by k-space grid tile (ts x ts nodes)
struct TileBins {
    int ntx, nty, ts;
    int* off;   // ntx*nty + 1
    int* perm;  // original index of the k-th point in tile order
};
size_t fte_tiles_ws(int64_t n, int ntiles);
// region_w > 0: order each tile's points for the tiled gathers (staged
// region rows of region_w nodes; see k_tile_assign)
int fte_tiles_build(fte_context* ctx, WsCarver& wc, const double* p, int64_t n, double Lx, double Ly, double hx,
                    double hy,
                    int ts, int ntx, int nty, TileBins* out, int region_w = 0);

// ff: float-float pairs, with ffmem scratch of fte_near_ff_ws(kind, 1, nsrc)
int fte_near_launch(fte_context* ctx, int kind, const CellList& cl, double xi, double Lx, double Ly, double2* ur,
                    double x32 = HUGE_VAL, bool ff = false, void* ffmem = nullptr);
// xi^2 r^2 above which a pair's terms are small enough for FP32 at tolerance
// tol (mixed form); HUGE_VAL: every pair in FP64
double fte_near_fp32_threshold(double tol);
// mixed form: may the FP64 pairs with xi^2 r^2 >= 1 be evaluated in
// float-float at tolerance tol
bool fte_near_ff_ok(double tol);
// the near-pair classes of the options (x32 = HUGE_VAL: no FP32 class)
int fte_near_classes(const fte_options* opt, double tol, double* x32, bool* ff);
// Near-field launch description, opaque outside near.cu.
struct NearParamsHost {
    alignas(16) unsigned char raw[320];
};
void fte_near_fill_params(int kind, const CellList& cl, double xi, double Lx, double Ly, NearParamsHost* hp,
                          double x32 = HUGE_VAL, bool ff = false);
size_t fte_near_params_size();
bool fte_near_uses_ff(const NearParamsHost& hp);
// float-float pairs read per-source float-float data (own-box-relative
// positions, densities of nv vectors) prepared once per evaluation:
// scratch bytes, attaching the scratch to a description, and the preparation
// (after the densities are in place)
size_t fte_near_ff_ws(int kind, int nv, int64_t nsrc);
void fte_near_ff_attach(NearParamsHost* hp, int kind, int nv, int64_t nsrc, void* mem);
int fte_near_ff_prep(fte_context* ctx, int kind, int nv, const NearParamsHost& hp);
// the same for many descriptions (device array plist_dev, a warp per (description, box) item)
int fte_near_ff_prep_batch(fte_context* ctx, int kind, int nv, const void* plist_dev, const int2* items, int nitems);
// sources staged per chunk (ff: the description uses the float-float class)
int fte_near_cap(const fte_context* ctx, int kind, int nv, bool ff);
// nv (1..4) density vectors at q* + v*cl.qstride; outputs at ur + v*ustride
int fte_near_launch_nv(fte_context* ctx, int kind, int nv, const NearParamsHost& hp, double2* ur, long long ustride);
// many problems in one launch: plist_dev = device array of the filled
// descriptions (ur/ustride/cap set), items = (problem, box) pairs
int fte_near_launch_batch(fte_context* ctx, int kind, int nv, bool ff, const void* plist_dev, const int2* items,
                          int nitems);
void fte_near_set_output(NearParamsHost* hp, double2* ur, long long ustride, int cap);

struct KspaceArgs {
    int kind;
    int form;
    int64_t nsrc, ntar;
    const double* psrc;  // interleaved
    const double* ptar;
    const double* f;     // interleaved
    const double* nrm;   // interleaved (DLP)
    const double* wts;   // optional weights (driver option)
    double xi, eta, w, Lx, Ly;
    int Mx, My, P;
    double2* uk;         // output, interleaved
    // tile bins built beforehand (plans); null: built by the call
    const TileBins* pre_src = nullptr;
    const TileBins* pre_tar = nullptr;
    // spread / gather tile sizes (grid nodes a side); 0: the default rule
    int ts_spread = 0, ts_gather = 0;
};
// Work lists of many float-float k-space evaluations (batches): each added
// evaluation (scratch carved from wc as fte_kspace_run carves it, tile bins
// prebuilt) becomes an item of one launch per stage; *taken = false when its
// form or shape needs the per-call path (FP64/FP32 k-space, long
// transforms, untiled spread/gather, the FP64 multiplier).
// Tile sizes of an evaluation inside a batch's work lists: the default rule
// without the small-grid shrink and without a plan's tuned sizes (many plans
// share each launch, so the GPU is filled by the batch; tiles timed on one
// plan alone, or shrunk to fill the GPU with one grid, only add halo work).
int fte_kspace_batch_tiles(const fte_context* ctx, const KspaceArgs& a, int* ts_s, int* ts_g);
struct KMulti;
int fte_kmulti_create(KMulti** out);
int fte_kmulti_add(KMulti* km, fte_context* ctx, WsCarver& wc, const KspaceArgs& a, bool* taken);
int fte_kmulti_finalize(KMulti* km, fte_context* ctx);
int fte_kmulti_run(KMulti* km, fte_context* ctx);
int fte_kmulti_items(const KMulti* km);
void fte_kmulti_destroy(KMulti* km);
size_t fte_kspace_ws(int kind, int form, int Mx, int My, int64_t nsrc, int64_t ntar);
// float-float form: bytes of the sources' window records (0 for the other forms)
size_t fte_kspace_rec_ws(int form, int64_t nsrc);
// build the spread/gather tile bins that fte_kspace_run would build for `a`
int fte_kspace_tiles(fte_context* ctx, WsCarver& wc, const KspaceArgs& a, TileBins* src, TileBins* tar);
int fte_kspace_run(fte_context* ctx, WsCarver& wc, const KspaceArgs& a, fte_info* info);
// time every fitting spread and gather tile size on a's points; sets
// a.ts_spread / a.ts_gather to the fastest (grid: ng grids of scratch; bins:
// scratch for one candidate's tile bins, fte_tiles_ws(max(nsrc, ntar), tiles
// of 8 nodes))
int fte_kspace_tune(fte_context* ctx, void* grid, WsCarver bins, KspaceArgs& a, float* ms_spread, float* ms_gather);

// other quantities (quant.cu, kspace.cu): real-space sums from a cell list
// (f, nrm: input order, interleaved) and k-space sums; out holds
// fte_q_ncomp(q) values per target
int fte_q_near_launch(fte_context* ctx, int kind, int q, const CellList& cl, const double* f, const double* nrm,
                      double xi, double Lx, double Ly, double* out);
size_t fte_q_kspace_ws(int Mx, int My, int64_t nsrc, int64_t ntar);
int fte_q_kspace_run(fte_context* ctx, WsCarver& wc, int q, const KspaceArgs& a, double* out);
