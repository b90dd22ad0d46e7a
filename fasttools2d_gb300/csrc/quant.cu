// quant.cu -- real-space sums of the other spectral Ewald quantities
// (pressure, pressure gradient, velocity gradient, stress, vorticity) of the
// 2-D Stokeslet and stresslet, in FP64.
//
// Restates the reference's real-space gateways (paths relative to
// annabroms/FastTools2D, PeriodicEwald/src/mex/):
//   StokesSLP/mex_stokes_slp_{pressure,pressure_grad,gradient,stress,vorticity}_real.cpp
//   StokesDLP/mex_stokes_dlp_{pressure,pressure_grad,gradient,stress,vorticity}_real.cpp
// Per target box: the own box's sources (the coincident one skipped: r = 0,
// for the stresslet vorticity r^2 < 1e-13) and the 8 periodic neighbour
// boxes' sources with r^2 < Lx Ly / (nside_x nside_y); the sum is scaled as
// each gateway scales it.
//
// GPU design as in near.cu: one CTA per target box stages the 3x3
// neighbourhood (image shift applied, densities gathered by the cell list's
// source index) in shared memory; a warp owns a target; lanes test 32 staged
// sources at a time (exact FP64 cutoff), compact the survivors into a per-warp
// ring and evaluate full batches of 32 pairs with all lanes busy.
#include "fte_internal.cuh"
#include "quant_filters.cuh"

namespace {

constexpr int kQThreads = 256;
constexpr int kQWarps = kQThreads / 32;
constexpr int kQRing = 64;
constexpr double kPi = 3.1415926535897932385;

struct QNearParams {
    int nsx, nsy, nb;
    const int* __restrict__ src_off;
    const double2* __restrict__ spos;
    const int* __restrict__ sidx;
    const int* __restrict__ tar_off;
    const double2* __restrict__ tpos;
    const int* __restrict__ tidx;
    const double* __restrict__ f;    // input order, interleaved
    const double* __restrict__ nrm;  // input order, interleaved (DLP)
    double Lx, Ly, xi, cutoffsq;
    int cap;
    double* __restrict__ out;  // ncomp per target, caller's order
};

// pair terms, target - source = (r1, r2); t[] accumulates the gateway's sums
template <int KIND, int Q>
__device__ __forceinline__ void q_pair(bool own, double r1, double r2, double f1, double f2, double n1, double n2,
                                       double xi, double* t) {
    const double xi2 = xi * xi;
    const double rSq = r1 * r1 + r2 * r2;
    if constexpr (KIND == FTE_KIND_SLP) {
        if (own && rSq == 0) return;
        if constexpr (Q == FTE_Q_PRESSURE) {
            const double rdotf = r1 * f1 + r2 * f2;
            t[0] += rdotf * exp(-xi * xi * rSq) / rSq;
        } else if constexpr (Q == FTE_Q_PRESSURE_GRAD) {
            const double rdotf = r1 * f1 + r2 * f2;
            const double e = exp(-xi * xi * rSq);
            t[0] -= e * ((f1 - 2 * xi * xi * rdotf * r1) / rSq - 2 * rdotf * r1 / rSq / rSq);
            t[1] -= e * ((f2 - 2 * xi * xi * rdotf * r2) / rSq - 2 * rdotf * r2 / rSq / rSq);
        } else if constexpr (Q == FTE_Q_GRADIENT) {
            const double e2 = exp(-xi2 * rSq);
            const double rdotf = f1 * r1 + f2 * r2;
            const double g = (xi * xi + 1 / rSq) / rSq;
            t[0] += e2 * (2 * xi * xi * r1 * f1 + rdotf / rSq - 2 * r1 * r1 * rdotf * g);
            t[1] += e2 * (2 * xi * xi * r1 * f2 + (-r1 * f2 + r2 * f1) / rSq - 2 * r1 * r2 * rdotf * g);
            t[2] += e2 * (2 * xi * xi * r2 * f1 + (r1 * f2 - r2 * f1) / rSq - 2 * r1 * r2 * rdotf * g);
            t[3] += e2 * (2 * xi * xi * r2 * f2 + rdotf / rSq - 2 * r2 * r2 * rdotf * g);
        } else if constexpr (Q == FTE_Q_STRESS) {
            const double e2 = exp(-xi2 * rSq);
            const double rdotf = f1 * r1 + f2 * r2;
            const double g = rdotf / (rSq * rSq) * (1 + xi2 * rSq);
            t[0] += e2 * (2 * xi2 * (rdotf + r1 * f1 + r1 * f1) - 4 * r1 * r1 * g);
            t[1] += e2 * (2 * xi2 * (r2 * f1 + r1 * f2) - 4 * r1 * r2 * g);
            t[2] += e2 * (2 * xi2 * (r1 * f2 + r2 * f1) - 4 * r2 * r1 * g);
            t[3] += e2 * (2 * xi2 * (rdotf + r2 * f2 + r2 * f2) - 4 * r2 * r2 * g);
        } else if constexpr (Q == FTE_Q_VORTICITY) {
            const double e2 = exp(-xi2 * rSq);
            t[0] += e2 * (1 / rSq - xi2) * (f1 * r2 - f2 * r1);
        }
    } else {
        if (own && (Q == FTE_Q_VORTICITY ? (rSq < 1e-13) : (rSq == 0))) return;
        const double rdotf = r1 * f1 + r2 * f2;
        const double rdotn = r1 * n1 + r2 * n2;
        const double fdotn = f1 * n1 + f2 * n2;
        const double e2 = exp(-xi2 * rSq);
        if constexpr (Q == FTE_Q_PRESSURE) {
            t[0] -= e2 * ((fdotn - 2 * xi * xi * rdotn * rdotf) / rSq - 2 * rdotn * rdotf / rSq / rSq);
        } else if constexpr (Q == FTE_Q_PRESSURE_GRAD) {
            const double a1 = r1 * fdotn + f1 * rdotn + n1 * rdotf, a2 = r2 * fdotn + f2 * rdotn + n2 * rdotf;
            t[0] += e2 * (2 * xi2 * (a1 - 2 * xi2 * r1 * rdotf * rdotn) / rSq +
                          2 * (a1 - 4 * xi2 * r1 * rdotn * rdotf) / rSq / rSq - 8 * r1 * rdotn * rdotf / rSq / rSq / rSq);
            t[1] += e2 * (2 * xi2 * (a2 - 2 * xi2 * r2 * rdotf * rdotn) / rSq +
                          2 * (a2 - 4 * xi2 * r2 * rdotn * rdotf) / rSq / rSq - 8 * r2 * rdotn * rdotf / rSq / rSq / rSq);
        } else if constexpr (Q == FTE_Q_GRADIENT) {
            const double c = (8 * xi2 * xi2 / rSq + 16 * xi2 / rSq / rSq + 16 / rSq / rSq / rSq) * rdotf * rdotn;
            const double h = 4 * (1 + xi2 * rSq) / rSq / rSq;
            t[0] += e2 * (r1 * r1 * c - h * (rdotf * rdotn + r1 * f1 * rdotn + r1 * n1 * rdotf) +
                          2 * xi2 * (2 * f1 * n1 + fdotn - 2 * xi2 * r1 * (f1 * rdotn + n1 * rdotf + r1 * fdotn)));
            t[1] += e2 * (r1 * r2 * c - h * (r2 * f1 * rdotn + r2 * n1 * rdotf) +
                          2 * xi2 * (f1 * n2 + n1 * f2 - 2 * xi2 * r1 * (f2 * rdotn + n2 * rdotf + r2 * fdotn)));
            t[2] += e2 * (r1 * r2 * c - h * (r1 * f2 * rdotn + r1 * n2 * rdotf) +
                          2 * xi2 * (f2 * n1 + f1 * n2 - 2 * xi2 * r2 * (f1 * rdotn + n1 * rdotf + r1 * fdotn)));
            t[3] += e2 * (r2 * r2 * c - h * (rdotf * rdotn + r2 * f2 * rdotn + r2 * n2 * rdotf) +
                          2 * xi2 * (2 * f2 * n2 + fdotn - 2 * xi2 * r2 * (f2 * rdotn + n2 * rdotf + r2 * fdotn)));
        } else if constexpr (Q == FTE_Q_STRESS) {
            const double mu = 1.0;
            const double c = ((8 * xi2 * xi2) / rSq + (16 * xi2) / (rSq * rSq) + 16 / (rSq * rSq * rSq)) * rdotf * rdotn;
            const double h = 2 * (1 + xi2 * rSq) / (rSq * rSq);
            const double pr = 1 / (2 * kPi) * ((fdotn - 2 * xi2 * rdotf * rdotn) / rSq - 2 * rdotf * rdotn / (rSq * rSq));
            const double s = 1 / (4 * kPi) * 2 * mu;
            t[0] += e2 * (pr + s * (r1 * r1 * c -
                                    h * (f1 * r1 * rdotn + n1 * r1 * rdotf + r1 * f1 * rdotn + r1 * n1 * rdotf +
                                         2 * rdotf * rdotn) +
                                    2 * xi2 * (fdotn + n1 * f1 + f1 * n1 -
                                               xi2 * (2 * r1 * r1 * fdotn + r1 * f1 * rdotn + r1 * n1 * rdotf +
                                                      f1 * r1 * rdotn + n1 * r1 * rdotf))));
            t[1] += s * e2 *
                    (r1 * r2 * c - h * (f1 * r2 * rdotn + n1 * r2 * rdotf + r1 * f2 * rdotn + r1 * n2 * rdotf) +
                     2 * xi2 * (n1 * f2 + f1 * n2 -
                                xi2 * (2 * r1 * r2 * fdotn + r1 * f2 * rdotn + r1 * n2 * rdotf + f1 * r2 * rdotn +
                                       n1 * r2 * rdotf)));
            t[2] += s * e2 *
                    (r2 * r1 * c - h * (f2 * r1 * rdotn + n2 * r1 * rdotf + r2 * f1 * rdotn + r2 * n1 * rdotf) +
                     2 * xi2 * (n2 * f1 + f2 * n1 -
                                xi2 * (2 * r2 * r1 * fdotn + r2 * f1 * rdotn + r2 * n1 * rdotf + f2 * r1 * rdotn +
                                       n2 * r1 * rdotf)));
            t[3] += e2 * (pr + s * (r2 * r2 * c -
                                    h * (f2 * r2 * rdotn + n2 * r2 * rdotf + r2 * f2 * rdotn + r2 * n2 * rdotf +
                                         2 * rdotf * rdotn) +
                                    2 * xi2 * (fdotn + n2 * f2 + f2 * n2 -
                                               xi2 * (2 * r2 * r2 * fdotn + r2 * f2 * rdotn + r2 * n2 * rdotf +
                                                      f2 * r2 * rdotn + n2 * r2 * rdotf))));
        } else if constexpr (Q == FTE_Q_VORTICITY) {
            const double rdot = r1 * (n2 * rdotf + f2 * rdotn) - r2 * (n1 * rdotf + f1 * rdotn);
            const double ndot = n1 * (r2 * rdotf) - n2 * (r1 * rdotf);
            const double fdot = f1 * (r2 * rdotn) - f2 * (r1 * rdotn);
            t[0] += e2 * ((1 + xi2 * rSq) * rdot / (rSq * rSq) + xi2 * xi2 * (ndot + fdot));
        }
    }
}

// the gateways' final scaling
template <int KIND, int Q>
__device__ __forceinline__ double q_scale(double v) {
    if constexpr (KIND == FTE_KIND_SLP) {
        if constexpr (Q == FTE_Q_GRADIENT || Q == FTE_Q_STRESS)
            return v / 4 / kPi;
        else
            return v / (2 * kPi);
    } else {
        if constexpr (Q == FTE_Q_GRADIENT)
            return v / 4 / kPi;
        else if constexpr (Q == FTE_Q_STRESS)
            return v;
        else if constexpr (Q == FTE_Q_VORTICITY)
            return v / kPi;
        else
            return v / (2 * kPi);
    }
}

__device__ __forceinline__ double q_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int KIND>
constexpr int q_stage_doubles() {
    return KIND == FTE_KIND_SLP ? 4 : 6;  // x, y, f1, f2 (, n1, n2)
}

template <int KIND>
size_t q_smem(int cap) {
    return (size_t)cap * q_stage_doubles<KIND>() * sizeof(double) + kQWarps * kQRing * sizeof(int) + 64;
}

template <int KIND, int Q>
__global__ void __launch_bounds__(kQThreads, 2) k_near_q(const QNearParams p) {
    constexpr int NO = fte_q_nout(Q);
    constexpr int SD = q_stage_doubles<KIND>();
    extern __shared__ __align__(16) unsigned char q_smem_raw[];
    __shared__ int nb_box[9], nb_start[10];
    __shared__ double nb_shx[9], nb_shy[9];
    const int cap = p.cap;
    double* st = reinterpret_cast<double*>(q_smem_raw);  // st[c * cap + i], c = x, y, f1, f2, (n1, n2)
    int* ring_all = reinterpret_cast<int*>(st + (size_t)SD * cap);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int* ring = ring_all + warp * kQRing;
    const unsigned lt_mask = (1u << lane) - 1u;

    for (int b = blockIdx.x; b < p.nb; b += gridDim.x) {
        const int t0 = p.tar_off[b];
        const int nt = p.tar_off[b + 1] - t0;
        if (nt == 0) continue;
        const int bx = b % p.nsx, by = b / p.nsx;
        __syncthreads();  // the previous box is done with the staging buffers
        if (tid < 9) {
            // own box first, then the reference's neighbour order
            const int ox = tid == 0 ? 0 : (tid <= 3 ? -1 : (tid <= 5 ? 0 : 1));
            const int oy = tid == 0 ? 0 : ((tid == 1 || tid == 4 || tid == 6) ? -1 : ((tid == 2 || tid == 7) ? 0 : 1));
            const int psx = bx + ox, psy = by + oy;
            const int tx = (psx + p.nsx) % p.nsx, ty = (psy + p.nsy) % p.nsy;
            nb_box[tid] = ty * p.nsx + tx;
            nb_shx[tid] = (p.Lx * (psx - tx)) / p.nsx;
            nb_shy[tid] = (p.Ly * (psy - ty)) / p.nsy;
        }
        __syncthreads();
        if (tid == 0) {
            int s = 0;
            for (int e = 0; e < 9; e++) {
                nb_start[e] = s;
                s += p.src_off[nb_box[e] + 1] - p.src_off[nb_box[e]];
            }
            nb_start[9] = s;
        }
        __syncthreads();
        const int S = nb_start[9];
        const int n_own = nb_start[1];
        if (S == 0) {
            for (int t = tid; t < nt; t += kQThreads)
                for (int c = 0; c < NO; c++) p.out[(size_t)p.tidx[t0 + t] * NO + c] = 0.0;
            continue;
        }
        for (int chunk = 0; chunk < S; chunk += cap) {
            const int clen = min(cap, S - chunk);
            if (chunk > 0) __syncthreads();
            for (int i = tid; i < clen; i += kQThreads) {
                const int g = chunk + i;
                int e = 0;
#pragma unroll
                for (int k = 1; k < 9; k++) e += (g >= nb_start[k]);
                const int si = p.src_off[nb_box[e]] + (g - nb_start[e]);
                const double2 ps = p.spos[si];
                const int ii = p.sidx[si];
                st[i] = ps.x + nb_shx[e];
                st[cap + i] = ps.y + nb_shy[e];
                st[2 * cap + i] = p.f[2 * (size_t)ii];
                st[3 * cap + i] = p.f[2 * (size_t)ii + 1];
                if constexpr (KIND == FTE_KIND_DLP) {
                    st[4 * cap + i] = p.nrm[2 * (size_t)ii];
                    st[5 * cap + i] = p.nrm[2 * (size_t)ii + 1];
                }
            }
            __syncthreads();
            const int own_lim = n_own - chunk;
            for (int t = warp; t < nt; t += kQWarps) {
                const double2 tp = p.tpos[t0 + t];
                double acc[NO];
#pragma unroll
                for (int c = 0; c < NO; c++) acc[c] = 0.0;
                auto eval = [&](int s) {
                    const double r1 = tp.x - st[s], r2 = tp.y - st[cap + s];
                    double n1 = 0.0, n2 = 0.0;
                    if constexpr (KIND == FTE_KIND_DLP) {
                        n1 = st[4 * cap + s];
                        n2 = st[5 * cap + s];
                    }
                    q_pair<KIND, Q>(s < own_lim, r1, r2, st[2 * cap + s], st[3 * cap + s], n1, n2, p.xi, acc);
                };
                int head = 0, cnt = 0;
                for (int base = 0; base < clen; base += 32) {
                    const int s = base + lane;
                    bool pass = false;
                    if (s < clen) {
                        const double dx = tp.x - st[s], dy = tp.y - st[cap + s];
                        pass = (s < own_lim) || (dx * dx + dy * dy < p.cutoffsq);
                    }
                    const unsigned m = __ballot_sync(0xffffffffu, pass);
                    if (pass) ring[(head + cnt + __popc(m & lt_mask)) & (kQRing - 1)] = s;
                    cnt += __popc(m);
                    __syncwarp();
                    if (cnt >= 32) {
                        eval(ring[(head + lane) & (kQRing - 1)]);
                        head = (head + 32) & (kQRing - 1);
                        cnt -= 32;
                        __syncwarp();
                    }
                }
                if (lane < cnt) eval(ring[(head + lane) & (kQRing - 1)]);
                __syncwarp();
#pragma unroll
                for (int c = 0; c < NO; c++) {
                    const double a = q_warp_sum(acc[c]);
                    if (lane == 0) {
                        double* o = p.out + (size_t)p.tidx[t0 + t] * NO + c;
                        *o = chunk == 0 ? a : *o + a;
                    }
                }
            }
        }
        // all chunks summed: scale once (own targets only, after the last chunk)
        __syncthreads();
        for (int t = tid; t < nt; t += kQThreads)
            for (int c = 0; c < NO; c++) {
                double* o = p.out + (size_t)p.tidx[t0 + t] * NO + c;
                *o = q_scale<KIND, Q>(*o);
            }
    }
}

template <int KIND, int Q>
int q_near_launch(fte_context* ctx, QNearParams p) {
    const size_t budget = 110 * 1024 < (size_t)ctx->max_smem_optin ? 110 * 1024 : (size_t)ctx->max_smem_optin;
    int cap = 2048;
    while (cap > 128 && q_smem<KIND>(cap) > budget) cap -= 64;
    p.cap = cap;
    const size_t smem = q_smem<KIND>(cap);
    int grid = p.nb < ctx->num_sms * 16 ? p.nb : ctx->num_sms * 16;
    if (grid < 1) grid = 1;
    FTE_CUDA_TRY(fte_smem_ceiling(k_near_q<KIND, Q>, (int)smem));
    FTE_LAUNCH(ctx, (k_near_q<KIND, Q>), grid, kQThreads, smem, p);
    return FTE_OK;
}

template <int KIND>
int q_near_dispatch(fte_context* ctx, int q, const QNearParams& p) {
    switch (q) {
        case FTE_Q_PRESSURE: return q_near_launch<KIND, FTE_Q_PRESSURE>(ctx, p);
        case FTE_Q_PRESSURE_GRAD: return q_near_launch<KIND, FTE_Q_PRESSURE_GRAD>(ctx, p);
        case FTE_Q_GRADIENT: return q_near_launch<KIND, FTE_Q_GRADIENT>(ctx, p);
        case FTE_Q_STRESS: return q_near_launch<KIND, FTE_Q_STRESS>(ctx, p);
        case FTE_Q_VORTICITY: return q_near_launch<KIND, FTE_Q_VORTICITY>(ctx, p);
        default: break;
    }
    fte_set_error("unknown quantity %d", q);
    return FTE_ERR_INVALID;
}

}  // namespace

int fte_q_near_launch(fte_context* ctx, int kind, int q, const CellList& cl, const double* f, const double* nrm,
                      double xi, double Lx, double Ly, double* out) {
    if (!cl.sidx) {
        fte_set_error("internal: cell list without source index");
        return FTE_ERR_INVALID;
    }
    QNearParams p;
    p.nsx = cl.nsx;
    p.nsy = cl.nsy;
    p.nb = cl.nb;
    p.src_off = cl.src_off;
    p.spos = cl.spos;
    p.sidx = cl.sidx;
    p.tar_off = cl.tar_off;
    p.tpos = cl.tpos;
    p.tidx = cl.tidx;
    p.f = f;
    p.nrm = nrm;
    p.Lx = Lx;
    p.Ly = Ly;
    p.xi = xi;
    p.cutoffsq = Lx * Ly / cl.nsx / cl.nsy;
    p.cap = 0;
    p.out = out;
    return kind == FTE_KIND_SLP ? q_near_dispatch<FTE_KIND_SLP>(ctx, q, p) : q_near_dispatch<FTE_KIND_DLP>(ctx, q, p);
}
