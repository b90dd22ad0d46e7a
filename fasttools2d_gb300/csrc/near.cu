// near.cu -- real-space (near-field) sums of the Stokeslet and stresslet in FP64.
//
// Restates the reference's real-space gateways
//   SLP: PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:124-333
//   DLP: PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:97-187
// Per target box: every source of the own box (no cutoff; Stokeslet self term
// (-1 - gamma/2 - log xi) f when r^2 < 1e-15, stresslet skips r^2 == 0) plus
// the sources of the 8 periodic neighbour boxes (image-shifted) with
// r^2 < Lx Ly / (nside_x nside_y).  Result / (4 pi).
//
// GPU design: one CTA per target box stages the 3x3 neighbourhood's sources
// (image shift applied, FP64 positions and densities, FP32 box-relative
// positions) in shared memory, in chunks when the neighbourhood is large.  A
// warp owns one target at a time: its lanes sweep the staged sources 32 at a
// time with a conservative FP32 distance test, compact the survivors into a
// per-warp ring queue (ballot + popc), and every full queue of 32 candidate
// pairs is evaluated with all lanes busy in FP64 (exact cutoff test, exp, E1).
// GB300's FP64 pipe issues a warp instruction every ~16 cycles per SM, so the
// compaction is what keeps the FP64 work proportional to pairs inside the
// cutoff instead of to candidate pairs.
#include "fte_internal.cuh"

#define FTE_E1_STORAGE_R static __constant__
#define FTE_E1_STORAGE_G static __device__ const
#include "fte_e1_coeffs.h"

namespace {

constexpr int kNearThreads = 256;
constexpr int kNearWarps = kNearThreads / 32;
constexpr int kQueue = 64;
constexpr int kGtab = FTE_E1_NPIECE_G * (FTE_E1_DEG_G + 1);

struct NearParams {
    int nsx, nsy, nb;
    const int* __restrict__ src_off;
    const double2* __restrict__ spos;
    const double* __restrict__ q0;
    const double* __restrict__ q1;
    const double* __restrict__ q2;
    const int* __restrict__ tar_off;
    const double2* __restrict__ tpos;
    const int* __restrict__ tidx;
    double Lx, Ly, xi, xi2, inv_xi2, selfc, cutoffsq;
    float cut32;
    int cap;
    double2* __restrict__ ur;
};

// E1(x) for x > 0 from the piecewise polynomials of gen_e1_coeffs.py:
//   x < 1:     -gamma - ln x + x R(2x - 1)
//   1 <= x:    exp(-x) G(x) / x  (quarter-octave piece from the exponent and
//              the top two mantissa bits), 0 beyond 1024.
// emx = exp(-x) and inv_x = 1/x are supplied by the caller, which needs them
// anyway.
__device__ __forceinline__ double fte_e1(double x, double emx, double inv_x, const double* __restrict__ gtab) {
    if (x < 1.0) {
        double t = fma(2.0, x, -1.0);
        double r = fte_e1_coef_r[FTE_E1_DEG_R];
#pragma unroll
        for (int k = FTE_E1_DEG_R - 1; k >= 0; k--) r = fma(r, t, fte_e1_coef_r[k]);
        return fma(x, r, -FTE_EULER - log(x));
    }
    if (x >= 1024.0) return 0.0;
    long long bits = __double_as_longlong(x);
    int k = (int)((bits >> 52) & 0x7ff) - 1023;
    int q = (int)((bits >> 50) & 3);
    double mant = __longlong_as_double((bits & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
    double t = (mant - (1.125 + 0.25 * q)) * 8.0;
    const double* c = gtab + (4 * k + q) * (FTE_E1_DEG_G + 1);
    double g = c[FTE_E1_DEG_G];
#pragma unroll
    for (int j = FTE_E1_DEG_G - 1; j >= 0; j--) g = fma(g, t, c[j]);
    return emx * g * inv_x;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int KIND>
__global__ void __launch_bounds__(kNearThreads) k_near(const NearParams prm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int cap = prm.cap;
    double* gtab = reinterpret_cast<double*>(smem_raw);
    double* sx = gtab + kGtab;
    double* sy = sx + cap;
    double* a0 = sy + cap;
    double* a1 = a0 + cap;
    double* a2 = a1 + cap;  // DLP only (allocated for both)
    float2* s32 = reinterpret_cast<float2*>(a2 + (KIND == FTE_KIND_DLP ? cap : 0));
    int* qbuf = reinterpret_cast<int*>(s32 + cap);
    __shared__ int nb_box[9];
    __shared__ int nb_start[10];
    __shared__ double nb_shx[9], nb_shy[9];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int* myq = qbuf + warp * kQueue;
    const unsigned lt_mask = (1u << lane) - 1u;
    const double inv4pi = 1.0 / (4.0 * FTE_PI);

    for (int i = tid; i < kGtab; i += kNearThreads) gtab[i] = (&fte_e1_coef_g[0][0])[i];

    for (int b = blockIdx.x; b < prm.nb; b += gridDim.x) {
        const int t0 = prm.tar_off[b];
        const int nt = prm.tar_off[b + 1] - t0;
        if (nt == 0) continue;
        const int bx = b % prm.nsx, by = b / prm.nsx;
        __syncthreads();  // previous box finished with the staging buffers
        if (tid < 9) {
            // own box first, then the reference's neighbour order (ilist_x/ilist_y)
            const int ox_tab[9] = {0, -1, -1, -1, 0, 0, 1, 1, 1};
            const int oy_tab[9] = {0, -1, 0, 1, -1, 1, -1, 0, 1};
            int psx = bx + ox_tab[tid], psy = by + oy_tab[tid];
            int tx = (psx + prm.nsx) % prm.nsx, ty = (psy + prm.nsy) % prm.nsy;
            int sb = ty * prm.nsx + tx;
            nb_box[tid] = sb;
            nb_shx[tid] = (prm.Lx * (psx - tx)) / prm.nsx;
            nb_shy[tid] = (prm.Ly * (psy - ty)) / prm.nsy;
        }
        __syncthreads();
        if (tid == 0) {
            int s = 0;
            for (int e = 0; e < 9; e++) {
                nb_start[e] = s;
                s += prm.src_off[nb_box[e] + 1] - prm.src_off[nb_box[e]];
            }
            nb_start[9] = s;
        }
        __syncthreads();
        const int S = nb_start[9];
        const int n_own = nb_start[1];
        const double cx = -prm.Lx / 2 + (bx + 0.5) * prm.Lx / prm.nsx;
        const double cy = -prm.Ly / 2 + (by + 0.5) * prm.Ly / prm.nsy;

        if (S == 0) {
            for (int t = tid; t < nt; t += kNearThreads) prm.ur[prm.tidx[t0 + t]] = make_double2(0.0, 0.0);
            continue;
        }

        for (int chunk = 0; chunk < S; chunk += cap) {
            const int clen = min(cap, S - chunk);
            if (chunk > 0) __syncthreads();
            for (int i = tid; i < clen; i += kNearThreads) {
                int g = chunk + i;
                int e = 0;
#pragma unroll
                for (int k = 1; k < 9; k++) e += (g >= nb_start[k]);
                int si = prm.src_off[nb_box[e]] + (g - nb_start[e]);
                double2 p = prm.spos[si];
                double xs = p.x + nb_shx[e], ys = p.y + nb_shy[e];
                sx[i] = xs;
                sy[i] = ys;
                a0[i] = prm.q0[si];
                a1[i] = prm.q1[si];
                if (KIND == FTE_KIND_DLP) a2[i] = prm.q2[si];
                s32[i] = make_float2((float)(xs - cx), (float)(ys - cy));
            }
            __syncthreads();
            const int own_lim = n_own - chunk;  // local index < own_lim: own box

            for (int t = warp; t < nt; t += kNearWarps) {
                const double2 tp = prm.tpos[t0 + t];
                const float tx32 = (float)(tp.x - cx), ty32 = (float)(tp.y - cy);
                double acc0 = 0.0, acc1 = 0.0;
                int qhead = 0, qcount = 0;

                auto eval = [&](int s) {
                    double dx = tp.x - sx[s], dy = tp.y - sy[s];
                    double r2 = dx * dx + dy * dy;
                    bool own = s < own_lim;
                    if (KIND == FTE_KIND_SLP) {
                        double fx = a0[s], fy = a1[s];
                        if (own && fabs(r2) < 1e-15) {
                            acc0 += prm.selfc * fx;
                            acc1 += prm.selfc * fy;
                        } else if (own || r2 < prm.cutoffsq) {
                            double x = r2 * prm.xi2;
                            double emx = exp(-x);
                            double ir2 = 1.0 / r2;
                            double E = fte_e1(x, emx, ir2 * prm.inv_xi2, gtab);
                            double g2 = emx * ir2;
                            double hE = 0.5 * E;
                            double dxy = dx * dy;
                            acc0 += hE * fx + (dxy * fy - dy * dy * fx) * g2;
                            acc1 += hE * fy + (dxy * fx - dx * dx * fy) * g2;
                        }
                    } else {
                        if ((own && r2 != 0.0) || (!own && r2 < prm.cutoffsq)) {
                            double s11 = a0[s], ssym = a1[s], s22 = a2[s];
                            double e2 = exp(-prm.xi2 * r2);
                            double ir2 = 1.0 / r2;
                            double facb = -4.0 * (1.0 + prm.xi2 * r2) * ir2 * ir2;
                            double Q = dx * dx * s11 + dx * dy * ssym + dy * dy * s22;
                            double pf = 2.0 * prm.xi2;
                            acc0 += e2 * (facb * dx * Q + pf * (3.0 * dx * s11 + dy * ssym + dx * s22));
                            acc1 += e2 * (facb * dy * Q + pf * (dx * ssym + 3.0 * dy * s22 + dy * s11));
                        }
                    }
                };

                for (int base = 0; base < clen; base += 32) {
                    int s = base + lane;
                    bool pass = false;
                    if (s < clen) {
                        if (s < own_lim) {
                            pass = true;
                        } else {
                            float2 q = s32[s];
                            float dx = q.x - tx32, dy = q.y - ty32;
                            pass = dx * dx + dy * dy < prm.cut32;
                        }
                    }
                    unsigned m = __ballot_sync(0xffffffffu, pass);
                    if (pass) myq[(qhead + qcount + __popc(m & lt_mask)) & (kQueue - 1)] = s;
                    qcount += __popc(m);
                    __syncwarp();
                    if (qcount >= 32) {
                        eval(myq[(qhead + lane) & (kQueue - 1)]);
                        qhead = (qhead + 32) & (kQueue - 1);
                        qcount -= 32;
                        __syncwarp();
                    }
                }
                if (lane < qcount) eval(myq[(qhead + lane) & (kQueue - 1)]);
                __syncwarp();
                acc0 = warp_sum(acc0);
                acc1 = warp_sum(acc1);
                if (lane == 0) {
                    int oi = prm.tidx[t0 + t];
                    double2 v = make_double2(acc0 * inv4pi, acc1 * inv4pi);
                    if (chunk == 0) {
                        prm.ur[oi] = v;
                    } else {
                        double2 o = prm.ur[oi];
                        prm.ur[oi] = make_double2(o.x + v.x, o.y + v.y);
                    }
                }
            }
        }
    }
}

size_t near_smem_bytes(int kind, int cap) {
    size_t per = (kind == FTE_KIND_DLP ? 5 : 4) * sizeof(double) + sizeof(float2);
    return kGtab * sizeof(double) + (size_t)cap * per + kNearWarps * kQueue * sizeof(int) + 64;
}

}  // namespace

int fte_near_launch(fte_context* ctx, int kind, const CellList& cl, double xi, double Lx, double Ly, double2* ur) {
    NearParams p;
    p.nsx = cl.nsx;
    p.nsy = cl.nsy;
    p.nb = cl.nb;
    p.src_off = cl.src_off;
    p.spos = cl.spos;
    p.q0 = cl.q0;
    p.q1 = cl.q1;
    p.q2 = cl.q2;
    p.tar_off = cl.tar_off;
    p.tpos = cl.tpos;
    p.tidx = cl.tidx;
    p.Lx = Lx;
    p.Ly = Ly;
    p.xi = xi;
    p.xi2 = xi * xi;
    p.inv_xi2 = 1.0 / (xi * xi);
    p.selfc = -(1.0 + 0.5 * FTE_EULER) - log(xi);
    p.cutoffsq = Lx * Ly / cl.nsx / cl.nsy;
    double bsx = Lx / cl.nsx, bsy = Ly / cl.nsy;
    double bmax = bsx > bsy ? bsx : bsy;
    p.cut32 = (float)(p.cutoffsq + 1e-4 * bmax * bmax);
    p.ur = ur;
    int cap = kind == FTE_KIND_DLP ? 1792 : 2048;
    size_t smem = near_smem_bytes(kind, cap);
    while (smem > (size_t)ctx->max_smem_optin && cap > 256) {
        cap -= 256;
        smem = near_smem_bytes(kind, cap);
    }
    p.cap = cap;
    int grid = cl.nb;
    int maxgrid = ctx->num_sms * 16;
    if (grid > maxgrid) grid = maxgrid;
    if (grid < 1) grid = 1;
    if (kind == FTE_KIND_SLP) {
        FTE_CUDA_TRY(cudaFuncSetAttribute(k_near<FTE_KIND_SLP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FTE_LAUNCH(ctx, k_near<FTE_KIND_SLP>, grid, kNearThreads, smem, p);
    } else {
        FTE_CUDA_TRY(cudaFuncSetAttribute(k_near<FTE_KIND_DLP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        FTE_LAUNCH(ctx, k_near<FTE_KIND_DLP>, grid, kNearThreads, smem, p);
    }
    return FTE_OK;
}

// ---- diagnostics: E1 on the device (test hook) ------------------------------
namespace {
__global__ void k_e1_probe(const double* __restrict__ x, double* __restrict__ out, int n) {
    __shared__ double gtab[kGtab];
    for (int i = threadIdx.x; i < kGtab; i += blockDim.x) gtab[i] = (&fte_e1_coef_g[0][0])[i];
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        double v = x[i];
        out[i] = fte_e1(v, exp(-v), 1.0 / v, gtab);
    }
}
}  // namespace

int fte_e1_device(fte_context* ctx, const double* x_dev, double* out_dev, int n) {
    if (n <= 0) return FTE_OK;
    FTE_LAUNCH(ctx, k_e1_probe, (n + 255) / 256, 256, 0, x_dev, out_dev, n);
    return FTE_OK;
}
