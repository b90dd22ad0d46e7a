// plan.cu -- geometry plans reused across density vectors, and batches of
// plans replayed as one CUDA graph.
//
// The reference recomputes everything on every call (cell list,
// ewald_tools.cpp:7-80; windows, ewald_tools.cpp:120-199), which in an
// iterative solver (GMRES on a boundary integral equation) repeats all the
// geometry work for every new density.  A plan does the density-independent
// work once: wrapping, the parameter choice, the real-space cell list and the
// k-space tile bins, the FFT tables and all scratch memory.  Executing a plan
// for nv density vectors (1..4) then runs only the density-dependent kernels;
// the real-space pair geometry and special functions are evaluated once per
// pair for all nv vectors.
//
// A batch holds many plans (uneven sizes, both kernels).  Its launch runs one
// persistent near-field kernel over the (plan, box) work list of all its
// Stokeslet plans and one over its stresslet plans, then each plan's k-space
// part on one of several forked streams, and is captured once into a CUDA
// graph so that a step of the iterative solver is a single graph launch.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "fte_internal.cuh"

namespace {

// sorted (cell-ordered) densities for nv vectors and packed f per vector:
// sorted source d
template <int KIND>
__device__ __forceinline__ void plan_dens_one(const double* __restrict__ f1s, const double* __restrict__ f2s, int nv,
                                              int64_t n, const double* __restrict__ nrm,
                                              const double* __restrict__ wts, const int* __restrict__ sidx,
                                              double* __restrict__ q0, double* __restrict__ q1,
                                              double* __restrict__ q2, double* __restrict__ fv, int64_t d) {
    {
        const int i = sidx[d];
        const double w = wts ? wts[i] : 1.0;
        for (int v = 0; v < nv; v++) {
            const double a = f1s[v * n + i], b = f2s[v * n + i];
            // packed, unweighted f in input order for the k-space part
            fv[(v * n + d) * 2] = f1s[v * n + d];
            fv[(v * n + d) * 2 + 1] = f2s[v * n + d];
            const double f1 = a * w, f2 = b * w;
            if (KIND == FTE_KIND_SLP) {
                q0[v * n + d] = f1;
                q1[v * n + d] = f2;
            } else {
                const double n1 = nrm[2 * i], n2 = nrm[2 * i + 1];
                q0[v * n + d] = f1 * n1;
                q1[v * n + d] = f1 * n2 + f2 * n1;
                q2[v * n + d] = f2 * n2;
            }
        }
    }
}

template <int KIND>
__global__ void k_plan_dens(const double* __restrict__ f1s, const double* __restrict__ f2s, int nv, int64_t n,
                            const double* __restrict__ nrm, const double* __restrict__ wts,
                            const int* __restrict__ sidx, double* __restrict__ q0, double* __restrict__ q1,
                            double* __restrict__ q2, double* __restrict__ fv) {
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < n; d += (int64_t)gridDim.x * blockDim.x)
        plan_dens_one<KIND>(f1s, f2s, nv, n, nrm, wts, sidx, q0, q1, q2, fv, d);
}

// zero mode sum_s (f.n) x_s of vector v (stresslet): block c of 256 threads
// sums sources [c kZeroChunk, (c + 1) kZeroChunk) and adds its part to
// zero[2v..2v+1] (zeroed before) with FP64 atomics, as the drivers' density
// reduction does (one block per vector took 2 ms at 1e6 sources)
constexpr int kZeroChunk = 8192;
__host__ __device__ inline int zero_chunks(int64_t n) { return (int)((n + kZeroChunk - 1) / kZeroChunk); }

__device__ __forceinline__ void plan_zero_part(const double* __restrict__ ps, const double* __restrict__ fv,
                                               const double* __restrict__ nrm, const double* __restrict__ wts,
                                               int64_t n, double* __restrict__ zero, int v, int c) {
    double zx = 0, zy = 0;
    const int64_t i1 = (int64_t)(c + 1) * kZeroChunk < n ? (int64_t)(c + 1) * kZeroChunk : n;
    for (int64_t i = (int64_t)c * kZeroChunk + threadIdx.x; i < i1; i += blockDim.x) {
        const double w = wts ? wts[i] : 1.0;
        const double fn = (fv[(v * n + i) * 2] * nrm[2 * i] + fv[(v * n + i) * 2 + 1] * nrm[2 * i + 1]) * w;
        zx += fn * ps[2 * i];
        zy += fn * ps[2 * i + 1];
    }
    __shared__ double sx[256], sy[256];
    sx[threadIdx.x] = zx;
    sy[threadIdx.x] = zy;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sx[threadIdx.x] += sx[threadIdx.x + o];
            sy[threadIdx.x] += sy[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(&zero[2 * v], sx[0]);
        atomicAdd(&zero[2 * v + 1], sy[0]);
    }
}

// grid (chunks, vectors)
__global__ void k_plan_zero(const double* __restrict__ ps, const double* __restrict__ fv,
                            const double* __restrict__ nrm, const double* __restrict__ wts, int64_t n,
                            double* __restrict__ zero) {
    plan_zero_part(ps, fv, nrm, wts, n, zero, blockIdx.y, blockIdx.x);
}

// u = ur + uk (+ the zero mode) of target i for nv vectors
__device__ __forceinline__ void plan_combine_one(const double2* __restrict__ ur, const double2* __restrict__ uk,
                                                 int nv, int64_t n, const double* __restrict__ zero, double inv_area,
                                                 double* __restrict__ u1s, double* __restrict__ u2s, int64_t i) {
    for (int v = 0; v < nv; v++) {
        double2 r = ur[v * n + i], k = uk[v * n + i];
        double zx = zero ? zero[2 * v] * inv_area : 0.0, zy = zero ? zero[2 * v + 1] * inv_area : 0.0;
        u1s[v * n + i] = r.x + k.x + zx;
        u2s[v * n + i] = r.y + k.y + zy;
    }
}

__global__ void k_plan_combine(const double2* __restrict__ ur, const double2* __restrict__ uk, int nv, int64_t n,
                               const double* __restrict__ zero, double inv_area, double* __restrict__ u1s,
                               double* __restrict__ u2s) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        plan_combine_one(ur, uk, nv, n, zero, inv_area, u1s, u2s, i);
}

// ---- a batch's per-plan work as work lists (one launch for all plans) -----
struct PItem {
    int kind, nv;
    int64_t nsrc, ntar;
    const double *f1s, *f2s, *nrm, *wts, *ps;
    const int* sidx;
    double *q0, *q1, *q2, *fv, *zero;
    const double2 *ur, *uk;
    double *u1s, *u2s;
    double inv_area;
};

// work items (plan, block of 256 sorted sources)
__global__ void k_plan_dens_multi(const PItem* __restrict__ items, const int2* __restrict__ wl) {
    const int2 w = wl[blockIdx.x];
    const PItem& it = items[w.x];
    // the zero-mode sums start from zero (their kernel runs after this one)
    if (w.y == 0 && it.zero && threadIdx.x < 2 * it.nv) it.zero[threadIdx.x] = 0.0;
    const int64_t d = (int64_t)w.y * blockDim.x + threadIdx.x;
    if (d >= it.nsrc) return;
    if (it.kind == FTE_KIND_SLP)
        plan_dens_one<FTE_KIND_SLP>(it.f1s, it.f2s, it.nv, it.nsrc, it.nrm, it.wts, it.sidx, it.q0, it.q1, it.q2,
                                    it.fv, d);
    else
        plan_dens_one<FTE_KIND_DLP>(it.f1s, it.f2s, it.nv, it.nsrc, it.nrm, it.wts, it.sidx, it.q0, it.q1, it.q2,
                                    it.fv, d);
}

// work items (stresslet plan, vector x chunks + chunk)
__global__ void k_plan_zero_multi(const PItem* __restrict__ items, const int2* __restrict__ wl) {
    const int2 w = wl[blockIdx.x];
    const PItem& it = items[w.x];
    const int nch = zero_chunks(it.nsrc);
    plan_zero_part(it.ps, it.fv, it.nrm, it.wts, it.nsrc, it.zero, w.y / nch, w.y % nch);
}

// work items (plan, block of 256 targets)
__global__ void k_plan_combine_multi(const PItem* __restrict__ items, const int2* __restrict__ wl) {
    const int2 w = wl[blockIdx.x];
    const PItem& it = items[w.x];
    const int64_t i = (int64_t)w.y * blockDim.x + threadIdx.x;
    if (i < it.ntar) plan_combine_one(it.ur, it.uk, it.nv, it.ntar, it.zero, it.inv_area, it.u1s, it.u2s, i);
}

__global__ void k_plan_wrap(const double* __restrict__ x, const double* __restrict__ y, int64_t n, double Lx,
                            double Ly, double* __restrict__ p) {
    const double rLx = __drcp_rn(Lx), rLy = __drcp_rn(Ly);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        p[2 * i] = fte_wrap_coord(x[i], Lx, rLx);
        p[2 * i + 1] = fte_wrap_coord(y[i], Ly, rLy);
    }
}

__global__ void k_plan_pack(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                            double* __restrict__ p) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        p[2 * i] = a[i];
        p[2 * i + 1] = b[i];
    }
}

__global__ void k_plan_sumsq(const double* __restrict__ f1, const double* __restrict__ f2,
                             const double* __restrict__ wts, int64_t n, double* __restrict__ acc) {
    double q = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double w = wts ? wts[i] : 1.0;
        q += f1[i] * f1[i] * w * w + f2[i] * f2[i] * w * w;
    }
    for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, q);
}

int grid_of(const fte_context* c, int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > c->num_sms * 8) b = c->num_sms * 8;
    return (int)b;
}

}  // namespace

int fte_choose_params_ex(int kind, int64_t nsrc, int64_t ntar, double Q, double Lx, double Ly, const fte_options* opt,
                         fte_params* out);

struct fte_plan {
    fte_context* ctx = nullptr;
    int kind = 0;
    int nvmax = 1;
    int64_t nsrc = 0, ntar = 0;
    double Lx = 1, Ly = 1;
    fte_params prm;
    char* mem = nullptr;  // geometry + scratch, owned
    size_t mem_size = 0;
    double *ps = nullptr, *pt = nullptr, *nrm = nullptr, *wts = nullptr;
    CellList cl;
    TileBins tb_src, tb_tar;
    NearParamsHost near;
    double *q0 = nullptr, *q1 = nullptr, *q2 = nullptr, *fv = nullptr, *zero = nullptr;
    double2 *ur = nullptr, *uk = nullptr;
    char* kscratch = nullptr;  // grids and spectra of one vector
    size_t kscratch_size = 0;
    bool ffnear = false;       // float-float near pairs (per-source data in ffmem)
    char* ffmem = nullptr;
};

struct fte_batch {
    fte_context* ctx = nullptr;
    std::vector<fte_plan*> plans;
    int nv = 1;
    char* mem = nullptr;
    std::vector<double*> f1, f2, u1, u2;
    // batched near-field work lists (device): per kind and near-pair form
    // (list kind * 2 + ff), plist + items
    void* plist[4] = {nullptr, nullptr, nullptr, nullptr};
    int2* items[4] = {nullptr, nullptr, nullptr, nullptr};
    int nitems[4] = {0, 0, 0, 0};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    // work lists: every plan's densities (dens); the k-space parts of the
    // plans whose float-float k-space the work lists take (km, multi[i] = 1),
    // their stresslet zero modes (zero) and combinations (comb); the other
    // plans run their k-space per call on the forked streams
    KMulti* km = nullptr;
    std::vector<char> multi;
    char* mem2 = nullptr;
    // the work lists' tile sizes and bins per plan (the plan's own bins where
    // the sizes agree, else bins built into mem3)
    std::vector<int2> wl_ts;
    std::vector<TileBins> wl_src, wl_tar;
    char* mem3 = nullptr;
    PItem* pitems = nullptr;
    int2 *wl_dens = nullptr, *wl_zero = nullptr, *wl_comb = nullptr;
    int n_dens = 0, n_zero = 0, n_comb = 0;
};

// the k-space arguments of plan p's vector v in a batch
// multi: arguments for the batch work lists, which evaluate an FP32-product
// plan with the float-float kernels (the same parameters, window records and
// grids; the result is the float-float one, within the FP32 products'
// rounding of the plan's own), so that it joins the work lists instead of
// running per plan.  A plan the work lists do not take keeps its own form.
static KspaceArgs batch_kspace_args(const fte_plan* p, int v, bool multi = false) {
    KspaceArgs a;
    a.kind = p->kind;
    a.form = multi && p->prm.form == FTE_FORM_FF32 ? FTE_FORM_FF : p->prm.form;
    a.nsrc = p->nsrc;
    a.ntar = p->ntar;
    a.psrc = p->ps;
    a.ptar = p->pt;
    a.f = p->fv + 2 * v * p->nsrc;
    a.nrm = p->nrm;
    a.wts = p->wts;
    a.xi = p->prm.xi;
    a.eta = p->prm.eta;
    a.w = p->prm.w;
    a.Lx = p->Lx;
    a.Ly = p->Ly;
    a.Mx = p->prm.Mx;
    a.My = p->prm.My;
    a.P = p->prm.P;
    a.uk = p->uk + v * p->ntar;
    a.pre_src = &p->tb_src;
    a.pre_tar = &p->tb_tar;
    a.ts_spread = p->prm.ts_spread;
    a.ts_gather = p->prm.ts_gather;
    return a;
}

// density-dependent work of one plan (device pointers; nv vectors)
static int plan_exec_body(fte_plan* p, int nv, const double* f1s, const double* f2s, double* u1s, double* u2s,
                          bool skip_near) {
    fte_context* c = p->ctx;
    const int64_t ns = p->nsrc, nt = p->ntar;
    if (ns > 0) {
        if (p->kind == FTE_KIND_SLP)
            FTE_LAUNCH(c, k_plan_dens<FTE_KIND_SLP>, grid_of(c, ns), 256, 0, f1s, f2s, nv, ns, (const double*)p->nrm,
                       (const double*)p->wts, (const int*)p->cl.sidx, p->q0, p->q1, p->q2, p->fv);
        else
            FTE_LAUNCH(c, k_plan_dens<FTE_KIND_DLP>, grid_of(c, ns), 256, 0, f1s, f2s, nv, ns, (const double*)p->nrm,
                       (const double*)p->wts, (const int*)p->cl.sidx, p->q0, p->q1, p->q2, p->fv);
    }
    if (nt == 0) return FTE_OK;
    if (!skip_near) {
        if (p->ffnear && ns > 0) FTE_TRY(fte_near_ff_prep(c, p->kind, nv, p->near));
        FTE_TRY(fte_near_launch_nv(c, p->kind, nv, p->near, p->ur, nt));
    }
    for (int v = 0; v < nv; v++) {
        WsCarver wc{p->kscratch, 0, p->kscratch_size};
        KspaceArgs a;
        a.kind = p->kind;
        a.form = p->prm.form;
        a.nsrc = ns;
        a.ntar = nt;
        a.psrc = p->ps;
        a.ptar = p->pt;
        a.f = p->fv + 2 * v * ns;
        a.nrm = p->nrm;
        a.wts = p->wts;
        a.xi = p->prm.xi;
        a.eta = p->prm.eta;
        a.w = p->prm.w;
        a.Lx = p->Lx;
        a.Ly = p->Ly;
        a.Mx = p->prm.Mx;
        a.My = p->prm.My;
        a.P = p->prm.P;
        a.uk = p->uk + v * nt;
        a.pre_src = &p->tb_src;
        a.pre_tar = &p->tb_tar;
        a.ts_spread = p->prm.ts_spread;
        a.ts_gather = p->prm.ts_gather;
        FTE_TRY(fte_kspace_run(c, wc, a, nullptr));
    }
    if (p->kind == FTE_KIND_DLP && ns > 0) {
        FTE_CUDA_TRY(cudaMemsetAsync(p->zero, 0, 2 * nv * sizeof(double), c->stream));
        FTE_LAUNCH(c, k_plan_zero, dim3(zero_chunks(ns), nv), 256, 0, (const double*)p->ps, (const double*)p->fv,
                   (const double*)p->nrm, (const double*)p->wts, ns, p->zero);
    }
    FTE_LAUNCH(c, k_plan_combine, grid_of(c, nt), 256, 0, (const double2*)p->ur, (const double2*)p->uk, nv, nt,
               p->kind == FTE_KIND_DLP ? (const double*)p->zero : nullptr, 1.0 / (p->Lx * p->Ly), u1s, u2s);
    return FTE_OK;
}

extern "C" int fte_plan_create(fte_context* c, int kind, const double* xsrc, const double* ysrc, int64_t nsrc,
                               const double* xtar, const double* ytar, int64_t ntar, const double* n1,
                               const double* n2, const double* f1, const double* f2, double Lx, double Ly,
                               const fte_options* opt, int nvmax, fte_plan** out, unsigned flags) {
    if (!c || !out) {
        fte_set_error("fte_plan_create: null argument");
        return FTE_ERR_INVALID;
    }
    *out = nullptr;
    if (kind != FTE_KIND_SLP && kind != FTE_KIND_DLP) {
        fte_set_error("fte_plan_create: unknown kind %d", kind);
        return FTE_ERR_INVALID;
    }
    if (nvmax < 1 || nvmax > 4) {
        fte_set_error("fte_plan_create: 1 to 4 density vectors per execution (nvmax=%d)", nvmax);
        return FTE_ERR_INVALID;
    }
    if (nsrc < 0 || ntar < 0 || nsrc > 2000000000LL || ntar > 2000000000LL || !(Lx > 0) || !(Ly > 0) ||
        !std::isfinite(Lx) || !std::isfinite(Ly)) {
        fte_set_error("fte_plan_create: bad sizes or box");
        return FTE_ERR_INVALID;
    }
    if ((nsrc > 0 && (!xsrc || !ysrc || !f1 || !f2 || (kind == FTE_KIND_DLP && (!n1 || !n2)))) ||
        (ntar > 0 && (!xtar || !ytar))) {
        fte_set_error("fte_plan_create: null array argument");
        return FTE_ERR_INVALID;
    }
    fte_options defaults;
    std::memset(&defaults, 0, sizeof(defaults));
    if (!opt) opt = &defaults;
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    fte_plan* p = new (std::nothrow) fte_plan();
    if (!p) {
        fte_set_error("fte_plan_create: out of host memory");
        return FTE_ERR_ALLOC;
    }
    p->ctx = c;
    p->kind = kind;
    p->nvmax = nvmax;
    p->nsrc = nsrc;
    p->ntar = ntar;
    p->Lx = Lx;
    p->Ly = Ly;
    // stage the inputs (context workspace) to reduce Q and build the geometry
    size_t stage = 8 * ws_bytes(nsrc + 1, 8) + 2 * ws_bytes(ntar + 1, 8) + 4096;
    int st = fte_ws_reserve(c, stage);
    if (st) {
        delete p;
        return st;
    }
    WsCarver wc{c->ws, 0, c->ws_size};
    auto put = [&](const double* src, int64_t n) -> const double* {
        if (!host || !src) return src;
        double* d = wc.take<double>(n + 1);
        if (n) cudaMemcpyAsync(d, src, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
        return d;
    };
    const double *dxs = put(xsrc, nsrc), *dys = put(ysrc, nsrc), *dxt = put(xtar, ntar), *dyt = put(ytar, ntar);
    const double *df1 = put(f1, nsrc), *df2 = put(f2, nsrc), *dn1 = put(n1, nsrc), *dn2 = put(n2, nsrc);
    const double* dw = put(opt->weights, nsrc);
    double* acc = wc.take<double>(8);
    if (!wc.ok()) {
        delete p;
        fte_set_error("fte_plan_create: staging workspace too small");
        return FTE_ERR_ALLOC;
    }
    FiniteSet fin;
    for (const double* a : {dxs, dys, df1, df2, dn1, dn2, dw}) fin.add(a, nsrc);
    fin.add(dxt, ntar);
    fin.add(dyt, ntar);
    st = fte_finite_launch(c, fin);
    if (st) {
        delete p;
        return st;
    }
    cudaMemsetAsync(acc, 0, 8 * sizeof(double), c->stream);
    if (nsrc > 0) k_plan_sumsq<<<grid_of(c, nsrc), 256, 0, c->stream>>>(df1, df2, dw, nsrc, acc);
    cudaMemcpyAsync(c->host_scalars, acc, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
        delete p;
        fte_set_error("fte_plan_create: %s", cudaGetErrorString(cudaGetLastError()));
        return FTE_ERR_CUDA;
    }
    st = fte_finite_result(c, "fte_plan_create");
    if (st) {
        delete p;
        return st;
    }
    double Q = c->host_scalars[0] + 1.0;
    st = fte_choose_params_ex(kind, nsrc, ntar, Q, Lx, Ly, opt, &p->prm);
    if (st) {
        delete p;
        return st;
    }
    const fte_params& prm = p->prm;
    // plan memory: geometry, cell list, tiles, densities, outputs, k-space scratch
    const int nv = nvmax;
    KspaceArgs ka;
    ka.kind = kind;
    ka.form = prm.form;
    ka.nsrc = nsrc;
    ka.ntar = ntar;
    ka.Lx = Lx;
    ka.Ly = Ly;
    ka.Mx = prm.Mx;
    ka.My = prm.My;
    ka.P = prm.P;
    p->kscratch_size = fte_kspace_ws(kind, prm.form, prm.Mx, prm.My, 0, 0) + fte_kspace_rec_ws(prm.form, nsrc) + (1 << 16);
    double x32;
    bool ffn;
    FTE_TRY(fte_near_classes(opt, prm.tol, &x32, &ffn));
    const size_t ffws = ffn ? fte_near_ff_ws(kind, nv, nsrc) : 0;
    size_t need = 3 * ws_bytes(2 * (nsrc + 1), 8) + ws_bytes(2 * (ntar + 1), 8) + ws_bytes(nsrc + 1, 8) +
                  fte_cells_ws(nsrc, ntar, prm.nside_x * prm.nside_y) +
                  fte_kspace_ws(kind, prm.form, prm.Mx, prm.My, nsrc, ntar) + 3 * ws_bytes(nv * (nsrc + 1), 8) +
                  ws_bytes(2 * nv * (nsrc + 1), 8) + ws_bytes(16 * nv, 8) + 2 * ws_bytes(nv * (ntar + 1), 16) +
                  p->kscratch_size + ffws + (1 << 16);
    if (fte_alloc_should_fail() || cudaMalloc(&p->mem, need) != cudaSuccess) {
        cudaGetLastError();
        delete p;
        fte_set_error("fte_plan_create: %zu bytes of device memory not available", need);
        return FTE_ERR_ALLOC;
    }
    p->mem_size = need;
    // frees the plan on every early return below
    struct Guard {
        fte_plan* p;
        ~Guard() {
            if (p) {
                cudaStreamSynchronize(p->ctx->stream);
                cudaFree(p->mem);
                delete p;
            }
        }
    } guard{p};
    WsCarver pm{p->mem, 0, need};
    p->ps = pm.take<double>(2 * (nsrc + 1));
    p->pt = pm.take<double>(2 * (ntar + 1));
    double* pf = pm.take<double>(2 * (nsrc + 1));
    p->nrm = kind == FTE_KIND_DLP ? pm.take<double>(2 * (nsrc + 1)) : nullptr;
    p->wts = dw ? pm.take<double>(nsrc + 1) : nullptr;
    p->q0 = pm.take<double>(nv * (nsrc + 1));
    p->q1 = pm.take<double>(nv * (nsrc + 1));
    p->q2 = pm.take<double>(nv * (nsrc + 1));
    p->fv = pm.take<double>(2 * nv * (nsrc + 1));
    p->zero = pm.take<double>(16 * nv);
    p->ur = pm.take<double2>(nv * (ntar + 1));
    p->uk = pm.take<double2>(nv * (ntar + 1));
    p->kscratch = pm.take<char>(p->kscratch_size);
    p->ffmem = ffn ? pm.take<char>(ffws) : nullptr;
    FTE_WS_CHECK(pm);
    if (nsrc > 0) {
        FTE_LAUNCH(c, k_plan_wrap, grid_of(c, nsrc), 256, 0, dxs, dys, nsrc, Lx, Ly, p->ps);
        FTE_LAUNCH(c, k_plan_pack, grid_of(c, nsrc), 256, 0, df1, df2, nsrc, pf);
        if (p->nrm) FTE_LAUNCH(c, k_plan_pack, grid_of(c, nsrc), 256, 0, dn1, dn2, nsrc, p->nrm);
        if (p->wts) FTE_CUDA_TRY(cudaMemcpyAsync(p->wts, dw, nsrc * 8, cudaMemcpyDeviceToDevice, c->stream));
    }
    if (ntar > 0) FTE_LAUNCH(c, k_plan_wrap, grid_of(c, ntar), 256, 0, dxt, dyt, ntar, Lx, Ly, p->pt);
    FTE_TRY(fte_cells_build(c, pm, kind, p->ps, nsrc, p->pt, ntar, pf, p->nrm, p->wts, prm.nside_x, prm.nside_y, Lx,
                            Ly, &p->cl));
    if (opt->form == FTE_FORM_MIXED) p->cl.cutoffsq = fte_tuned_cutoffsq(prm, Lx, Ly);
    FTE_WS_CHECK(pm);
    ka.psrc = p->ps;
    ka.ptar = p->pt;
    ka.f = pf;
    ka.nrm = p->nrm;
    ka.wts = p->wts;
    ka.xi = prm.xi;
    ka.eta = prm.eta;
    ka.w = prm.w;
    ka.uk = p->uk;
    if (opt->tune && (nsrc > 0 || ntar > 0)) {
        // the staged inputs are no longer needed: the context workspace holds
        // one candidate's tile bins at a time
        const int ntiles8 = ((prm.Mx + 7) / 8) * ((prm.My + 7) / 8);
        const size_t bins = fte_tiles_ws(nsrc > ntar ? nsrc : ntar, ntiles8) + fte_kspace_rec_ws(prm.form, nsrc) + 4096;
        FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
        FTE_TRY(fte_ws_reserve(c, bins));
        WsCarver bw{c->ws, 0, c->ws_size};
        FTE_TRY(fte_kspace_tune(c, p->kscratch, bw, ka, nullptr, nullptr));
    }
    FTE_TRY(fte_kspace_tiles(c, pm, ka, &p->tb_src, &p->tb_tar));
    FTE_WS_CHECK(pm);
    p->prm.ts_spread = nsrc > 0 ? p->tb_src.ts : ka.ts_spread;
    p->prm.ts_gather = ntar > 0 ? p->tb_tar.ts : ka.ts_gather;
    CellList cl = p->cl;
    cl.q0 = p->q0;
    cl.q1 = p->q1;
    cl.q2 = p->q2;
    cl.qstride = nsrc;
    fte_near_fill_params(kind, cl, prm.xi, Lx, Ly, &p->near, x32, ffn);
    p->ffnear = ffn;
    if (ffn) fte_near_ff_attach(&p->near, kind, nv, nsrc, p->ffmem);
    fte_near_set_output(&p->near, p->ur, ntar, fte_near_cap(c, kind, nv, fte_near_uses_ff(p->near)));
    // warm the FFT tables so that executions (and graph capture) allocate nothing
    FTE_TRY(fte_fft_prepare(c, prm.Mx));
    FTE_TRY(fte_fft_prepare(c, prm.My));
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    guard.p = nullptr;
    *out = p;
    return FTE_OK;
}

extern "C" int fte_plan_params(const fte_plan* p, fte_params* out) {
    if (!p || !out) {
        fte_set_error("fte_plan_params: null argument");
        return FTE_ERR_INVALID;
    }
    *out = p->prm;
    return FTE_OK;
}

extern "C" int fte_plan_execute(fte_plan* p, int nv, const double* f1s, const double* f2s, double* u1s, double* u2s,
                                unsigned flags) {
    if (!p) {
        fte_set_error("fte_plan_execute: null plan");
        return FTE_ERR_INVALID;
    }
    if (nv < 1 || nv > p->nvmax) {
        fte_set_error("fte_plan_execute: nv=%d outside 1..%d", nv, p->nvmax);
        return FTE_ERR_INVALID;
    }
    if ((p->nsrc > 0 && (!f1s || !f2s)) || (p->ntar > 0 && (!u1s || !u2s))) {
        fte_set_error("fte_plan_execute: null array argument");
        return FTE_ERR_INVALID;
    }
    fte_context* c = p->ctx;
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    const bool host = !(flags & FTE_DEVICE_POINTERS);
    const double *d1 = f1s, *d2 = f2s;
    double *o1 = u1s, *o2 = u2s;
    if (host) {
        size_t need = 2 * ws_bytes(nv * (p->nsrc + 1), 8) + 2 * ws_bytes(nv * (p->ntar + 1), 8) + 4096;
        FTE_TRY(fte_ws_reserve(c, need));
        WsCarver wc{c->ws, 0, c->ws_size};
        double* a = wc.take<double>(nv * (p->nsrc + 1));
        double* b = wc.take<double>(nv * (p->nsrc + 1));
        o1 = wc.take<double>(nv * (p->ntar + 1));
        o2 = wc.take<double>(nv * (p->ntar + 1));
        FTE_WS_CHECK(wc);
        FTE_CUDA_TRY(cudaMemcpyAsync(a, f1s, nv * p->nsrc * 8, cudaMemcpyHostToDevice, c->stream));
        FTE_CUDA_TRY(cudaMemcpyAsync(b, f2s, nv * p->nsrc * 8, cudaMemcpyHostToDevice, c->stream));
        d1 = a;
        d2 = b;
    }
    FTE_TRY(plan_exec_body(p, nv, d1, d2, o1, o2, false));
    if (host && p->ntar > 0) {
        FTE_CUDA_TRY(cudaMemcpyAsync(u1s, o1, nv * p->ntar * 8, cudaMemcpyDeviceToHost, c->stream));
        FTE_CUDA_TRY(cudaMemcpyAsync(u2s, o2, nv * p->ntar * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}

extern "C" int fte_plan_destroy(fte_plan* p) {
    if (!p) return FTE_OK;
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->ctx->stream);
    cudaFree(p->mem);
    delete p;
    return FTE_OK;
}

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
static int batch_run(fte_batch* b) {
    fte_context* c = b->ctx;
    cudaStream_t main = c->stream;
    // densities into cell order, every plan in one launch; the float-float
    // near data per kind
    if (b->n_dens > 0)
        FTE_LAUNCH(c, k_plan_dens_multi, b->n_dens, 256, 0, (const PItem*)b->pitems, (const int2*)b->wl_dens);
    for (int kind = 0; kind < 2; kind++)
        FTE_TRY(fte_near_ff_prep_batch(c, kind, b->nv, b->plist[kind * 2 + 1], b->items[kind * 2 + 1],
                                       b->nitems[kind * 2 + 1]));
    // one persistent near-field launch per kind over all (plan, box) items
    for (int l = 0; l < 4; l++)
        if (b->nitems[l] > 0)
            FTE_TRY(fte_near_launch_batch(c, l / 2, b->nv, l % 2 == 1, b->plist[l], b->items[l], b->nitems[l]));
    // the k-space parts the work lists do not take: per plan on forked streams
    bool percall = false;
    for (size_t i = 0; i < b->plans.size(); i++) percall = percall || (!b->multi[i] && b->plans[i]->ntar > 0);
    int rc = FTE_OK;
    if (percall) {
        const int S = (int)b->streams.size();
        FTE_CUDA_TRY(cudaEventRecord(b->events[0], main));
        for (int s = 0; s < S; s++) FTE_CUDA_TRY(cudaStreamWaitEvent(b->streams[s], b->events[0], 0));
        for (size_t i = 0; i < b->plans.size() && rc == FTE_OK; i++) {
            fte_plan* p = b->plans[i];
            if (b->multi[i] || p->ntar == 0) continue;
            c->stream = b->streams[i % S];
            for (int v = 0; v < b->nv && rc == FTE_OK; v++) {
                WsCarver wc{p->kscratch, 0, p->kscratch_size};
                const KspaceArgs a = batch_kspace_args(p, v);
                rc = fte_kspace_run(c, wc, a, nullptr);
            }
            if (rc == FTE_OK && p->kind == FTE_KIND_DLP && p->nsrc > 0) {
                const cudaError_t em = cudaMemsetAsync(p->zero, 0, 2 * b->nv * sizeof(double), c->stream);
                if (em != cudaSuccess) {
                    fte_set_error("batch: memset failed: %s", cudaGetErrorString(em));
                    rc = FTE_ERR_CUDA;
                    break;
                }
                k_plan_zero<<<dim3(zero_chunks(p->nsrc), b->nv), 256, 0, c->stream>>>(p->ps, p->fv, p->nrm, p->wts,
                                                                                      p->nsrc, p->zero);
                c->kernels++;
            }
            if (rc == FTE_OK) {
                k_plan_combine<<<grid_of(c, p->ntar), 256, 0, c->stream>>>(
                    p->ur, p->uk, b->nv, p->ntar, p->kind == FTE_KIND_DLP ? p->zero : nullptr, 1.0 / (p->Lx * p->Ly),
                    b->u1[i], b->u2[i]);
                c->kernels++;
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) {
                    fte_set_error("batch: launch failed: %s", cudaGetErrorString(e));
                    rc = FTE_ERR_CUDA;
                }
            }
        }
        c->stream = main;
        for (int s = 0; s < S; s++) {
            FTE_CUDA_TRY(cudaEventRecord(b->events[1 + s], b->streams[s]));
            FTE_CUDA_TRY(cudaStreamWaitEvent(main, b->events[1 + s], 0));
        }
        FTE_TRY(rc);
    }
    // the work lists' k-space parts, zero modes and combinations
    FTE_TRY(fte_kmulti_run(b->km, c));
    if (b->n_zero > 0)
        FTE_LAUNCH(c, k_plan_zero_multi, b->n_zero, 256, 0, (const PItem*)b->pitems, (const int2*)b->wl_zero);
    if (b->n_comb > 0)
        FTE_LAUNCH(c, k_plan_combine_multi, b->n_comb, 256, 0, (const PItem*)b->pitems, (const int2*)b->wl_comb);
    return FTE_OK;
}

// Work lists of a batch: the k-space items of every plan whose float-float
// k-space they take (vector 0 in the plan's own scratch, the others in the
// batch's), and the per-plan items of the densities, zero modes and
// combinations.
static int batch_build_lists(fte_batch* b) {
    fte_context* c = b->ctx;
    const int nv = b->nv;
    const size_t np = b->plans.size();
    b->multi.assign(np, 0);
    FTE_TRY(fte_kmulti_create(&b->km));
    // tile sizes for the work lists (fte_kspace_batch_tiles); bins where a
    // plan's own differ (tuned or shrunk for its grid alone)
    b->wl_ts.assign(np, make_int2(0, 0));
    b->wl_src.resize(np);
    b->wl_tar.resize(np);
    std::vector<char> rebuild(np, 0);
    size_t need3 = 4096;
    for (size_t i = 0; i < np; i++) {
        fte_plan* p = b->plans[i];
        b->wl_src[i] = p->tb_src;
        b->wl_tar[i] = p->tb_tar;
        if (!fte_form_ff(p->prm.form) || p->ntar == 0) continue;
        int ts_s = 0, ts_g = 0;
        FTE_TRY(fte_kspace_batch_tiles(c, batch_kspace_args(p, 0, true), &ts_s, &ts_g));
        b->wl_ts[i] = make_int2(ts_s, ts_g);
        if ((p->nsrc > 0 && ts_s != p->tb_src.ts) || ts_g != p->tb_tar.ts) {
            rebuild[i] = 1;
            const int M = p->prm.Mx, Mb = p->prm.My;
            if (ts_s > 0) need3 += fte_tiles_ws(p->nsrc, ((M + ts_s - 1) / ts_s) * ((Mb + ts_s - 1) / ts_s));
            if (ts_g > 0) need3 += fte_tiles_ws(p->ntar, ((M + ts_g - 1) / ts_g) * ((Mb + ts_g - 1) / ts_g));
        }
    }
    if (need3 > 4096) {
        if (fte_alloc_should_fail() || cudaMalloc(&b->mem3, need3) != cudaSuccess) {
            cudaGetLastError();
            b->mem3 = nullptr;
            fte_set_error("fte_batch_create: %zu bytes of device memory for tile bins not available", need3);
            return FTE_ERR_ALLOC;
        }
        WsCarver tb{b->mem3, 0, need3};
        for (size_t i = 0; i < np; i++) {
            if (!rebuild[i]) continue;
            KspaceArgs a = batch_kspace_args(b->plans[i], 0, true);
            a.ts_spread = b->wl_ts[i].x;
            a.ts_gather = b->wl_ts[i].y;
            FTE_TRY(fte_kspace_tiles(c, tb, a, &b->wl_src[i], &b->wl_tar[i]));
            FTE_WS_CHECK(tb);
        }
    }
    // scratch of vectors 1..nv-1 of the float-float plans
    size_t need = ws_bytes(np * sizeof(PItem), 1) + 4096;
    for (size_t i = 0; i < np; i++) {
        const fte_plan* p = b->plans[i];
        if (fte_form_ff(p->prm.form) && p->ntar > 0) need += (size_t)(nv - 1) * ws_bytes(p->kscratch_size, 1);
    }
    std::vector<int2> dens, zero, comb;
    for (size_t i = 0; i < np; i++) {
        const fte_plan* p = b->plans[i];
        if (p->nsrc > 0)
            for (int j = 0; j < (int)((p->nsrc + 255) / 256); j++) dens.push_back(make_int2((int)i, j));
    }
    need += 3 * ws_bytes((dens.size() + np * (nv + 1) + 1) * sizeof(int2), 1);
    for (size_t i = 0; i < np; i++) need += ws_bytes((size_t)(b->plans[i]->ntar + 255) / 256 * sizeof(int2), 1);
    if (fte_alloc_should_fail() || cudaMalloc(&b->mem2, need) != cudaSuccess) {
        cudaGetLastError();
        b->mem2 = nullptr;
        fte_set_error("fte_batch_create: %zu bytes of device memory not available", need);
        return FTE_ERR_ALLOC;
    }
    WsCarver m{b->mem2, 0, need};
    b->pitems = m.take<PItem>(np);
    std::vector<PItem> hp(np);
    for (size_t i = 0; i < np; i++) {
        fte_plan* p = b->plans[i];
        PItem& it = hp[i];
        std::memset(&it, 0, sizeof(it));
        it.kind = p->kind;
        it.nv = nv;
        it.nsrc = p->nsrc;
        it.ntar = p->ntar;
        it.f1s = b->f1[i];
        it.f2s = b->f2[i];
        it.nrm = p->nrm;
        it.wts = p->wts;
        it.ps = p->ps;
        it.sidx = p->cl.sidx;
        it.q0 = p->q0;
        it.q1 = p->q1;
        it.q2 = p->q2;
        it.fv = p->fv;
        // the stresslet's zero mode (none without sources)
        it.zero = p->kind == FTE_KIND_DLP && p->nsrc > 0 ? p->zero : nullptr;
        it.ur = p->ur;
        it.uk = p->uk;
        it.u1s = b->u1[i];
        it.u2s = b->u2[i];
        it.inv_area = 1.0 / (p->Lx * p->Ly);
        if (p->ntar == 0) continue;
        // the k-space items: all vectors of a plan or none
        for (int v = 0; v < nv; v++) {
            char* scr = v == 0 ? p->kscratch : m.take<char>(p->kscratch_size);
            FTE_WS_CHECK(m);
            WsCarver wc{scr, 0, p->kscratch_size};
            bool taken = false;
            KspaceArgs a = batch_kspace_args(p, v, true);
            if (b->wl_ts[i].y > 0) {
                a.ts_spread = b->wl_ts[i].x;
                a.ts_gather = b->wl_ts[i].y;
                a.pre_src = &b->wl_src[i];
                a.pre_tar = &b->wl_tar[i];
            }
            FTE_TRY(fte_kmulti_add(b->km, c, wc, a, &taken));
            if (!taken) {
                if (v > 0) {
                    fte_set_error("internal: batch work list took vector 0 of plan %zu but not vector %d", i, v);
                    return FTE_ERR_INVALID;
                }
                break;
            }
            b->multi[i] = 1;
        }
        if (!b->multi[i]) continue;
        if (p->kind == FTE_KIND_DLP && p->nsrc > 0)
            for (int v = 0; v < nv * zero_chunks(p->nsrc); v++) zero.push_back(make_int2((int)i, v));
        for (int j = 0; j < (int)((p->ntar + 255) / 256); j++) comb.push_back(make_int2((int)i, j));
    }
    FTE_TRY(fte_kmulti_finalize(b->km, c));
    b->n_dens = (int)dens.size();
    b->n_zero = (int)zero.size();
    b->n_comb = (int)comb.size();
    b->wl_dens = m.take<int2>(dens.size() + 1);
    b->wl_zero = m.take<int2>(zero.size() + 1);
    b->wl_comb = m.take<int2>(comb.size() + 1);
    FTE_WS_CHECK(m);
    FTE_CUDA_TRY(cudaMemcpyAsync(b->pitems, hp.data(), np * sizeof(PItem), cudaMemcpyHostToDevice, c->stream));
    if (!dens.empty())
        FTE_CUDA_TRY(cudaMemcpyAsync(b->wl_dens, dens.data(), dens.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                     c->stream));
    if (!zero.empty())
        FTE_CUDA_TRY(cudaMemcpyAsync(b->wl_zero, zero.data(), zero.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                     c->stream));
    if (!comb.empty())
        FTE_CUDA_TRY(cudaMemcpyAsync(b->wl_comb, comb.data(), comb.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                     c->stream));
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}

extern "C" int fte_batch_create(fte_context* c, fte_plan* const* plans, int nplans, int nv, fte_batch** out) {
    if (!c || !out || (nplans > 0 && !plans) || nplans < 0) {
        fte_set_error("fte_batch_create: bad arguments");
        return FTE_ERR_INVALID;
    }
    *out = nullptr;
    for (int i = 0; i < nplans; i++) {
        if (!plans[i] || plans[i]->ctx != c || nv < 1 || nv > plans[i]->nvmax) {
            fte_set_error("fte_batch_create: plan %d is null, of another context, or allows fewer than %d vectors", i,
                          nv);
            return FTE_ERR_INVALID;
        }
    }
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    fte_batch* b = new (std::nothrow) fte_batch();
    if (!b) {
        fte_set_error("fte_batch_create: out of host memory");
        return FTE_ERR_ALLOC;
    }
    b->ctx = c;
    b->nv = nv;
    b->plans.assign(plans, plans + nplans);
    // device buffers of densities and velocities, and the near-field work lists
    size_t need = 0;
    std::vector<int2> its[4];
    std::vector<NearParamsHost> pls[4];
    for (int i = 0; i < nplans; i++) {
        fte_plan* p = plans[i];
        need += 2 * ws_bytes(nv * (p->nsrc + 1), 8) + 2 * ws_bytes(nv * (p->ntar + 1), 8);
        if (p->ntar > 0) {
            NearParamsHost h = p->near;
            const bool ff = fte_near_uses_ff(h);
            const int k = p->kind * 2 + (ff ? 1 : 0);
            fte_near_set_output(&h, p->ur, p->ntar, fte_near_cap(c, p->kind, nv, ff));
            int idx = (int)pls[k].size();
            pls[k].push_back(h);
            int nb = p->prm.nside_x * p->prm.nside_y;
            for (int box = 0; box < nb; box++) its[k].push_back(make_int2(idx, box));
        }
    }
    for (int k = 0; k < 4; k++)
        need += ws_bytes(pls[k].size() * sizeof(NearParamsHost), 1) + ws_bytes(its[k].size() * sizeof(int2), 1);
    need += 4096;
    if (cudaMalloc(&b->mem, need) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        fte_set_error("fte_batch_create: %zu bytes of device memory not available", need);
        return FTE_ERR_ALLOC;
    }
    WsCarver bm{b->mem, 0, need};
    for (int i = 0; i < nplans; i++) {
        fte_plan* p = plans[i];
        b->f1.push_back(bm.take<double>(nv * (p->nsrc + 1)));
        b->f2.push_back(bm.take<double>(nv * (p->nsrc + 1)));
        b->u1.push_back(bm.take<double>(nv * (p->ntar + 1)));
        b->u2.push_back(bm.take<double>(nv * (p->ntar + 1)));
    }
    for (int k = 0; k < 4; k++) {
        b->nitems[k] = (int)its[k].size();
        if (b->nitems[k] == 0) continue;
        b->plist[k] = bm.take<NearParamsHost>(pls[k].size());
        b->items[k] = bm.take<int2>(its[k].size());
    }
    if (!bm.ok()) {
        fte_batch_destroy(b);
        fte_set_error("internal: batch buffer estimate too small");
        return FTE_ERR_ALLOC;
    }
    // zero the density/velocity buffers, then upload the work lists (in that
    // order, on the context's stream, finished before the host vectors go)
    FTE_CUDA_TRY(cudaMemsetAsync(b->mem, 0, bm.off, c->stream));
    for (int k = 0; k < 4; k++) {
        if (b->nitems[k] == 0) continue;
        FTE_CUDA_TRY(cudaMemcpyAsync(b->plist[k], pls[k].data(), pls[k].size() * sizeof(NearParamsHost),
                                     cudaMemcpyHostToDevice, c->stream));
        FTE_CUDA_TRY(cudaMemcpyAsync(b->items[k], its[k].data(), its[k].size() * sizeof(int2),
                                     cudaMemcpyHostToDevice, c->stream));
    }
    FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    {
        const int st = batch_build_lists(b);
        if (st != FTE_OK) {
            fte_batch_destroy(b);
            return st;
        }
    }
    const int S = nplans < 8 ? (nplans > 0 ? nplans : 1) : 8;
    b->streams.resize(S);
    b->events.resize(S + 1);
    for (int s = 0; s < S; s++) FTE_CUDA_TRY(cudaStreamCreateWithFlags(&b->streams[s], cudaStreamNonBlocking));
    for (int s = 0; s <= S; s++) FTE_CUDA_TRY(cudaEventCreateWithFlags(&b->events[s], cudaEventDisableTiming));
    // one eager run (sets kernel attributes), then capture the whole batch
    int timing = c->timing;
    c->timing = 0;
    int rc = batch_run(b);
    if (rc == FTE_OK) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            fte_set_error("fte_batch_create: first run failed: %s", cudaGetErrorString(e));
            rc = FTE_ERR_CUDA;
        }
    }
    if (rc == FTE_OK) {
        cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            rc = batch_run(b);
            cudaError_t e2 = cudaStreamEndCapture(c->stream, &b->graph);
            if (rc == FTE_OK && e2 == cudaSuccess)
                e2 = cudaGraphInstantiate(&b->exec, b->graph, 0);
            if (e2 != cudaSuccess && rc == FTE_OK) {
                fte_set_error("fte_batch_create: graph capture failed: %s", cudaGetErrorString(e2));
                rc = FTE_ERR_CUDA;
            }
        } else {
            fte_set_error("fte_batch_create: %s", cudaGetErrorString(e));
            rc = FTE_ERR_CUDA;
        }
    }
    c->timing = timing;
    if (rc != FTE_OK) {
        cudaGetLastError();
        fte_batch_destroy(b);
        return rc;
    }
    *out = b;
    return FTE_OK;
}

extern "C" int fte_batch_buffers(const fte_batch* b, int i, double** f1s, double** f2s, double** u1s, double** u2s) {
    if (!b || i < 0 || i >= (int)b->plans.size()) {
        fte_set_error("fte_batch_buffers: bad arguments");
        return FTE_ERR_INVALID;
    }
    if (f1s) *f1s = b->f1[i];
    if (f2s) *f2s = b->f2[i];
    if (u1s) *u1s = b->u1[i];
    if (u2s) *u2s = b->u2[i];
    return FTE_OK;
}

extern "C" int fte_batch_launch(fte_batch* b, int use_graph) {
    if (!b) {
        fte_set_error("fte_batch_launch: null batch");
        return FTE_ERR_INVALID;
    }
    fte_context* c = b->ctx;
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    if (use_graph && b->exec) {
        FTE_CUDA_TRY(cudaGraphLaunch(b->exec, c->stream));
        return FTE_OK;
    }
    int timing = c->timing;
    c->timing = 0;
    int rc = batch_run(b);
    c->timing = timing;
    return rc;
}

extern "C" int fte_batch_destroy(fte_batch* b) {
    if (!b) return FTE_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto s : b->streams) cudaStreamDestroy(s);
    for (auto e : b->events) cudaEventDestroy(e);
    cudaFree(b->mem);
    if (b->mem2) cudaFree(b->mem2);
    if (b->mem3) cudaFree(b->mem3);
    fte_kmulti_destroy(b->km);
    delete b;
    return FTE_OK;
}

extern "C" int fte_batch_set_density(fte_batch* b, int i, const double* f1s, const double* f2s, unsigned flags) {
    if (!b || i < 0 || i >= (int)b->plans.size() || (b->plans[i]->nsrc > 0 && (!f1s || !f2s))) {
        fte_set_error("fte_batch_set_density: bad arguments");
        return FTE_ERR_INVALID;
    }
    fte_context* c = b->ctx;
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    size_t bytes = (size_t)b->nv * b->plans[i]->nsrc * sizeof(double);
    cudaMemcpyKind k = (flags & FTE_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (bytes) {
        FTE_CUDA_TRY(cudaMemcpyAsync(b->f1[i], f1s, bytes, k, c->stream));
        FTE_CUDA_TRY(cudaMemcpyAsync(b->f2[i], f2s, bytes, k, c->stream));
    }
    if (!(flags & (FTE_DEVICE_POINTERS | FTE_HOST_ASYNC))) FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}

extern "C" int fte_batch_get_velocity(fte_batch* b, int i, double* u1s, double* u2s, unsigned flags) {
    if (!b || i < 0 || i >= (int)b->plans.size() || (b->plans[i]->ntar > 0 && (!u1s || !u2s))) {
        fte_set_error("fte_batch_get_velocity: bad arguments");
        return FTE_ERR_INVALID;
    }
    fte_context* c = b->ctx;
    FTE_CUDA_TRY(cudaSetDevice(c->device));
    size_t bytes = (size_t)b->nv * b->plans[i]->ntar * sizeof(double);
    cudaMemcpyKind k = (flags & FTE_DEVICE_POINTERS) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (bytes) {
        FTE_CUDA_TRY(cudaMemcpyAsync(u1s, b->u1[i], bytes, k, c->stream));
        FTE_CUDA_TRY(cudaMemcpyAsync(u2s, b->u2[i], bytes, k, c->stream));
    }
    if (!(flags & (FTE_DEVICE_POINTERS | FTE_HOST_ASYNC))) FTE_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return FTE_OK;
}
