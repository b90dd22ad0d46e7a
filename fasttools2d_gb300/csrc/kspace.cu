// kspace.cu -- Fourier-space part of the spectral Ewald sums (FP64 form).
//
// Restates the reference's k-space gateways
//   SLP: PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:47-209
//   DLP: PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_kspace.cpp:266-487
// and the shared Spread/Gather (PeriodicEwald/src/mex/common/ewald_tools.cpp:120-271):
//
//   1. spread: every source adds omega(node) q_c to (P+1)^2 nodes of each
//      grid, omega the fast-Gaussian-gridding window of the reference
//      (e1[j] = exp(-2 xi^2 h^2 j^2 / eta) and four exps per point);
//   2. forward 2-D FFT of each real grid;
//   3. the Stokeslet / stresslet multiplier with the reference's index ->
//      wave-number map (index <= M/2 counted positive) and k = 0 set to 0;
//   4. inverse FFT, real part;
//   5. gather with the same window, scaled by (4 xi^2/eta)^2 h^2/pi/(4 pi).
//
// Layout in HBM: real grids [g][x][y] (y fastest, the reference's column-major
// My x Mx); half spectra [g][x][ky], ky = 0..My/2.  The 2-D transform is a
// real-to-complex FFT along y (two real columns packed in one complex FFT),
// complex FFTs along x, the multiplier, inverse FFTs along x and a
// complex-to-real FFT along y.  Because the reference multiplies the Nyquist
// column/row with +k on both the k and -k copies and then keeps only the real
// part of the inverse transform, the half-spectrum multiplier is the average
// of the multiplier at (k1, k2) and at the Nyquist-mirrored wave vector
// (k1', k2') (k' = -k on a Nyquist index, k' = k elsewhere); this reproduces
// real(ifft2(.)) of the full-grid reference exactly.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "ff.cuh"
#include "fft.cuh"
#include "fte_internal.cuh"
#include "quant_filters.cuh"

namespace {

constexpr int kPtThreads = 128;

// Window geometry.  h, rh, w belong to the x axis (h = Lx / Mx, w = P h / 2
// as the drivers choose it), hy, rhy, wy to the y axis.  The reference has
// one step (hx = hy, checked by its drivers); the tuned choice for boxes whose
// aspect ratio is not a small rational gives each axis its own step, and then
// aniso = 1: the window keeps one Gaussian shape eta (isotropic in physical
// space, the filter deconvolves it) and each axis its own table e1 of
// exp(-2 xi^2/eta h^2 j^2) and its support half-width P h / 2.
struct WinParams {
    double Lx, Ly, h, xi, eta, w;
    double rh;  // RN(1 / h)
    int P, Mx, My;
    double hy, rhy, wy;
    int aniso;
};

// doubles (or float2) of the e1 table(s) in shared memory: one table padded
// to an even length, two when the axes' steps differ
__host__ __device__ inline int e1_len(int P, int aniso) { return (aniso ? 2 : 1) * ((P + 2) & ~1); }

// per-point window factors, as in ewald_tools.cpp:152-160 / 226-232
struct Win {
    int mx, my;
    double ex, e4y, e3x, e3y;
};

__device__ __forceinline__ Win window_of(double x, double y, const WinParams& wp) {
    Win o;
    double px, py;
    fte_closest_node(x, y, wp.Lx, wp.Ly, wp.h, wp.rh, wp.hy, wp.rhy, wp.P, &o.mx, &o.my, &px, &py);
    double t = -2 * wp.xi * wp.xi / wp.eta;
    o.ex = exp(t * (px * px + py * py + 2 * wp.w * px));
    o.e4y = exp(2 * t * wp.wy * py);
    o.e3x = exp(-2 * t * wp.h * px);
    o.e3y = exp(-2 * t * wp.hy * py);
    return o;
}

// e1[j] = exp(-2 xi^2/eta h^2 (j - P/2)^2)   (ewald_tools.cpp:125-127); with
// aniso the y axis's table follows at e1 + (P + 2 & ~1)
__device__ __forceinline__ void load_e1(double* e1, const WinParams& wp) {
    double t0 = -2 * wp.xi * wp.xi / wp.eta * wp.h * wp.h;
    double t0y = -2 * wp.xi * wp.xi / wp.eta * wp.hy * wp.hy;
    const int P1e = (wp.P + 2) & ~1;
    for (int j = threadIdx.x; j <= wp.P; j += blockDim.x) {
        int jj = j - wp.P / 2;
        e1[j] = exp(t0 * jj * jj);
        if (wp.aniso) e1[P1e + j] = exp(t0y * jj * jj);
    }
}
template <typename T>
__device__ __forceinline__ const T* e1y_of(const T* e1, const WinParams& wp) {
    return wp.aniso ? e1 + ((wp.P + 2) & ~1) : e1;
}

// ---- spread: one thread per source, FP64 atomics into the global grids ------
template <int NG>
__global__ void __launch_bounds__(kPtThreads) k_spread(const double* __restrict__ p, const double* __restrict__ f,
                                                      const double* __restrict__ nrm, const double* __restrict__ wts,
                                                      int64_t n, WinParams wp, double* __restrict__ H) {
    extern __shared__ double sh[];
    double* e1 = sh;
    const int P1 = wp.P + 1;
    double* wyb = e1 + e1_len(wp.P, wp.aniso) + threadIdx.x * P1;
    load_e1(e1, wp);
    const double* e1y = e1y_of(e1, wp);
    __syncthreads();
    const size_t G = (size_t)wp.Mx * wp.My;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x = p[2 * i], y = p[2 * i + 1];
        Win wn = window_of(x, y, wp);
        double q[4];
        double f1 = f[2 * i], f2 = f[2 * i + 1];
        if (wts) {
            f1 *= wts[i];
            f2 *= wts[i];
        }
        if (NG == 2) {
            q[0] = f1;
            q[1] = f2;
        } else {
            // (f1 n1, f2 n1, f1 n2, f2 n2): mex_stokes_dlp_kspace.cpp:290-298
            double n1 = nrm[2 * i], n2 = nrm[2 * i + 1];
            q[0] = f1 * n1;
            q[1] = f2 * n1;
            q[2] = f1 * n2;
            q[3] = f2 * n2;
        }
        // y factors e1[y] e3y^y
        double ey = 1.0;
        for (int j = 0; j < P1; j++) {
            wyb[j] = ey * e1y[j];
            ey *= wn.e3y;
        }
        bool ywrap = !(wn.my >= 0 && wn.my + wp.P < wp.My);
        double ex = wn.ex * wn.e4y;
        for (int a = 0; a < P1; a++) {
            double wxa = ex * e1[a];
            ex *= wn.e3x;
            int col = fte_wrap_index(wn.mx + a, wp.Mx);
            size_t base = (size_t)col * wp.My;
            double fw[NG];
#pragma unroll
            for (int g = 0; g < NG; g++) fw[g] = q[g] * wxa;
            for (int j = 0; j < P1; j++) {
                int row = ywrap ? fte_wrap_index(wn.my + j, wp.My) : wn.my + j;
                double wyj = wyb[j];
#pragma unroll
                for (int g = 0; g < NG; g++) atomicAdd(&H[g * G + base + row], fw[g] * wyj);
            }
        }
    }
}

// ---- gather: one thread per target -------------------------------------------
__global__ void __launch_bounds__(kPtThreads) k_gather(const double* __restrict__ p, int64_t n, WinParams wp,
                                                       const double* __restrict__ G0, const double* __restrict__ G1,
                                                       double scale, double2* __restrict__ out) {
    extern __shared__ double sh[];
    double* e1 = sh;
    const int P1 = wp.P + 1;
    double* wyb = e1 + e1_len(wp.P, wp.aniso) + threadIdx.x * P1;
    load_e1(e1, wp);
    const double* e1y = e1y_of(e1, wp);
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double x = p[2 * i], y = p[2 * i + 1];
        Win wn = window_of(x, y, wp);
        double ey = 1.0;
        for (int j = 0; j < P1; j++) {
            wyb[j] = ey * e1y[j];
            ey *= wn.e3y;
        }
        bool ywrap = !(wn.my >= 0 && wn.my + wp.P < wp.My);
        double ex = wn.ex * wn.e4y;
        double acc0 = 0.0, acc1 = 0.0;
        for (int a = 0; a < P1; a++) {
            double wxa = ex * e1[a];
            ex *= wn.e3x;
            int col = fte_wrap_index(wn.mx + a, wp.Mx);
            const double* c0 = G0 + (size_t)col * wp.My;
            const double* c1 = G1 + (size_t)col * wp.My;
            double s0 = 0.0, s1 = 0.0;
            if (!ywrap) {
                for (int j = 0; j < P1; j++) {
                    double wyj = wyb[j];
                    s0 = fma(wyj, __ldg(c0 + wn.my + j), s0);
                    s1 = fma(wyj, __ldg(c1 + wn.my + j), s1);
                }
            } else {
                for (int j = 0; j < P1; j++) {
                    int row = fte_wrap_index(wn.my + j, wp.My);
                    double wyj = wyb[j];
                    s0 = fma(wyj, __ldg(c0 + row), s0);
                    s1 = fma(wyj, __ldg(c1 + row), s1);
                }
            }
            acc0 = fma(wxa, s0, acc0);
            acc1 = fma(wxa, s1, acc1);
        }
        out[i] = make_double2(acc0 * scale, acc1 * scale);
    }
}

// ---- tiled spread / gather ------------------------------------------------------
// Points are binned by grid tile (ts x ts nodes).  A CTA owns one tile and a
// shared-memory region of W x W nodes per grid, W = ts + P + 4, starting at
// node (tx ts - P/2 - 2, ty ts - P/2 - 2): every window of a point binned in
// the tile lies inside it.  The spread accumulates with shared-memory atomics
// and flushes the region to the global grids (wrapped, atomics only where
// regions of neighbouring tiles overlap); the gather stages the region once
// and reads every target's window from shared memory.  A point whose window
// is not inside the region (a caller passing points outside [-L/2, L/2))
// takes the global, wrapped path.
constexpr int kTileThreads = 128;

__host__ __device__ inline int tile_region(int ts, int P) { return ts + P + 4; }

template <int NG>
__global__ void __launch_bounds__(kTileThreads) k_spread_tiled(const double* __restrict__ p, const double* __restrict__ f,
                                                              const double* __restrict__ nrm,
                                                              const double* __restrict__ wts,
                                                              const int* __restrict__ toff, const int* __restrict__ perm,
                                                              int ts, int ntx, int nty, WinParams wp,
                                                              double* __restrict__ H) {
    extern __shared__ double sh[];
    const int P1 = wp.P + 1, W = tile_region(ts, wp.P), WW = W * W;
    double* buf = sh;
    double* e1 = buf + NG * WW;
    double* wyb = e1 + e1_len(wp.P, wp.aniso) + threadIdx.x * P1;
    load_e1(e1, wp);
    const double* e1y = e1y_of(e1, wp);
    const size_t G = (size_t)wp.Mx * wp.My;
    for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
        const int k0 = toff[tile], k1 = toff[tile + 1];
        if (k0 == k1) continue;
        const int ox = (tile % ntx) * ts - wp.P / 2 - 2, oy = (tile / ntx) * ts - wp.P / 2 - 2;
        __syncthreads();
        for (int i = threadIdx.x; i < NG * WW; i += blockDim.x) buf[i] = 0.0;
        __syncthreads();
        for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
            const int i = perm[k];
            Win wn = window_of(p[2 * i], p[2 * i + 1], wp);
            double q[4];
            double f1 = f[2 * i], f2 = f[2 * i + 1];
            if (wts) {
                f1 *= wts[i];
                f2 *= wts[i];
            }
            if (NG == 2) {
                q[0] = f1;
                q[1] = f2;
            } else {
                double n1 = nrm[2 * i], n2 = nrm[2 * i + 1];
                q[0] = f1 * n1;
                q[1] = f2 * n1;
                q[2] = f1 * n2;
                q[3] = f2 * n2;
            }
            double ey = 1.0;
            for (int j = 0; j < P1; j++) {
                wyb[j] = ey * e1y[j];
                ey *= wn.e3y;
            }
            const int lx = wn.mx - ox, ly = wn.my - oy;
            double ex = wn.ex * wn.e4y;
            if (lx >= 0 && ly >= 0 && lx + wp.P < W && ly + wp.P < W) {
                for (int a = 0; a < P1; a++) {
                    double wxa = ex * e1[a];
                    ex *= wn.e3x;
                    double* row = buf + (lx + a) * W + ly;
                    double fw[NG];
#pragma unroll
                    for (int g = 0; g < NG; g++) fw[g] = q[g] * wxa;
                    for (int j = 0; j < P1; j++) {
                        double wyj = wyb[j];
#pragma unroll
                        for (int g = 0; g < NG; g++) atomicAdd(row + g * WW + j, fw[g] * wyj);
                    }
                }
            } else {
                for (int a = 0; a < P1; a++) {
                    double wxa = ex * e1[a];
                    ex *= wn.e3x;
                    size_t base = (size_t)fte_wrap_index(wn.mx + a, wp.Mx) * wp.My;
                    for (int j = 0; j < P1; j++) {
                        size_t at = base + fte_wrap_index(wn.my + j, wp.My);
#pragma unroll
                        for (int g = 0; g < NG; g++) atomicAdd(&H[g * G + at], q[g] * wxa * wyb[j]);
                    }
                }
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < NG * WW; idx += blockDim.x) {
            double v = buf[idx];
            if (v == 0.0) continue;
            int g = idx / WW, r = idx - g * WW;
            int xx = r / W, yy = r - xx * W;
            size_t at = (size_t)fte_wrap_index(ox + xx, wp.Mx) * wp.My + fte_wrap_index(oy + yy, wp.My);
            atomicAdd(&H[g * G + at], v);
        }
    }
}

// Column-owned spread of two grids without atomics.  For a chunk of the
// tile's sources, threads first compute each source's window origin and its
// factors fw_g[a] = q_g ex e4y e1[a] e3x^a and wy[j] = e1[j] e3y^j into
// shared memory; then warp w adds the products for every region column
// c = w (mod warps) of every source of the chunk, lane j owning window row j,
// so every update is one FMA on an address no other thread touches.
// mode 0: (f1, f2) [Stokeslet]; 1: (f1 n1, f2 n1); 2: (f1 n2, f2 n2) [stresslet].
constexpr int kColThreads = 256;
constexpr int kColWarps = kColThreads / 32;  // a power of two (column owner = column mod warps)
static_assert((kColWarps & (kColWarps - 1)) == 0, "column ownership needs a power-of-two warp count");
constexpr int kColChunk = 32;

__global__ void __launch_bounds__(kColThreads) k_spread_cols(int mode, const double* __restrict__ p,
                                                            const double* __restrict__ f,
                                                            const double* __restrict__ nrm,
                                                            const double* __restrict__ wts,
                                                            const int* __restrict__ toff,
                                                            const int* __restrict__ perm, int ts, int ntx, int nty,
                                                            WinParams wp, double* __restrict__ H0,
                                                            double* __restrict__ H1) {
    extern __shared__ double sh[];
    const int P1 = wp.P + 1, W = tile_region(ts, wp.P), WW = W * W;
    double* buf = sh;                     // 2 * WW
    double* e1 = buf + 2 * WW;            // e1_len (P1e, or 2 P1e with aniso)
    double* fw = e1 + e1_len(wp.P, wp.aniso);  // kColChunk * 2 * P1
    double* wy = fw + kColChunk * 2 * P1; // kColChunk * P1
    int* org = reinterpret_cast<int*>(wy + kColChunk * P1);  // kColChunk * 2 (lx, ly; lx < 0: global path)
    load_e1(e1, wp);
    const double* e1y = e1y_of(e1, wp);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int nw = kColWarps;
    for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
        const int k0 = toff[tile], k1 = toff[tile + 1];
        if (k0 == k1) continue;
        const int ox = (tile % ntx) * ts - wp.P / 2 - 2, oy = (tile / ntx) * ts - wp.P / 2 - 2;
        __syncthreads();
        for (int i = threadIdx.x; i < 2 * WW; i += blockDim.x) buf[i] = 0.0;
        for (int c0 = k0; c0 < k1; c0 += kColChunk) {
            const int cn = min(kColChunk, k1 - c0);
            __syncthreads();
            if (threadIdx.x < cn) {
                const int s = threadIdx.x;
                const int i = perm[c0 + s];
                Win wn = window_of(p[2 * i], p[2 * i + 1], wp);
                double f1 = f[2 * i], f2 = f[2 * i + 1];
                if (wts) {
                    f1 *= wts[i];
                    f2 *= wts[i];
                }
                double q0 = f1, q1 = f2;
                if (mode == 1) {
                    q0 = f1 * nrm[2 * i];
                    q1 = f2 * nrm[2 * i];
                } else if (mode == 2) {
                    q0 = f1 * nrm[2 * i + 1];
                    q1 = f2 * nrm[2 * i + 1];
                }
                double ey = 1.0;
                for (int j = 0; j < P1; j++) {
                    wy[s * P1 + j] = ey * e1y[j];
                    ey *= wn.e3y;
                }
                double ex = wn.ex * wn.e4y;
                for (int a = 0; a < P1; a++) {
                    double wxa = ex * e1[a];
                    ex *= wn.e3x;
                    fw[(s * 2 + 0) * P1 + a] = q0 * wxa;
                    fw[(s * 2 + 1) * P1 + a] = q1 * wxa;
                }
                const int lx = wn.mx - ox, ly = wn.my - oy;
                if (lx >= 0 && ly >= 0 && lx + wp.P < W && ly + wp.P < W) {
                    org[2 * s] = lx;
                    org[2 * s + 1] = ly;
                } else {
                    // window outside the region: add straight into the global grids
                    org[2 * s] = -1;
                    for (int a = 0; a < P1; a++) {
                        size_t base = (size_t)fte_wrap_index(wn.mx + a, wp.Mx) * wp.My;
                        for (int j = 0; j < P1; j++) {
                            size_t at = base + fte_wrap_index(wn.my + j, wp.My);
                            atomicAdd(&H0[at], fw[(s * 2 + 0) * P1 + a] * wy[s * P1 + j]);
                            atomicAdd(&H1[at], fw[(s * 2 + 1) * P1 + a] * wy[s * P1 + j]);
                        }
                    }
                }
            }
            __syncthreads();
            for (int s = 0; s < cn; s++) {
                const int lx = org[2 * s];
                if (lx < 0) continue;
                const int ly = org[2 * s + 1];
                // first column >= lx owned by this warp; window rows in
                // blocks of 32 (P up to 64)
                const int cfirst = lx + ((warp - lx) & (nw - 1));
                for (int j = lane; j < P1; j += 32) {
                    const double wyj = wy[s * P1 + j];
                    const double* fa = fw + (s * 2) * P1;
                    const double* fb = fa + P1;
                    for (int c = cfirst; c <= lx + wp.P; c += nw) {
                        double* b0 = buf + c * W + ly + j;
                        b0[0] = fma(fa[c - lx], wyj, b0[0]);
                        b0[WW] = fma(fb[c - lx], wyj, b0[WW]);
                    }
                }
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < 2 * WW; idx += blockDim.x) {
            double v = buf[idx];
            if (v == 0.0) continue;
            int g = idx >= WW, r = idx - g * WW;
            int xx = r / W, yy = r - xx * W;
            size_t at = (size_t)fte_wrap_index(ox + xx, wp.Mx) * wp.My + fte_wrap_index(oy + yy, wp.My);
            atomicAdd(g ? &H1[at] : &H0[at], v);
        }
    }
}

size_t spread_cols_smem(int ts, int P, int aniso = 0) {
    const int P1 = P + 1, W = tile_region(ts, P);
    return (size_t)(2 * W * W + e1_len(P, aniso) + kColChunk * 3 * P1) * sizeof(double) + kColChunk * 2 * sizeof(int);
}

__global__ void __launch_bounds__(kTileThreads) k_gather_tiled(const double* __restrict__ p,
                                                              const int* __restrict__ toff,
                                                              const int* __restrict__ perm, int ts, int ntx, int nty,
                                                              WinParams wp, const double* __restrict__ G0,
                                                              const double* __restrict__ G1, double scale,
                                                              double2* __restrict__ out) {
    extern __shared__ double sh[];
    const int P1 = wp.P + 1, W = tile_region(ts, wp.P), WW = W * W;
    double* r0 = sh;
    double* r1 = r0 + WW;
    double* e1 = r1 + WW;
    double* wyb = e1 + e1_len(wp.P, wp.aniso) + threadIdx.x * P1;
    load_e1(e1, wp);
    const double* e1y = e1y_of(e1, wp);
    for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
        const int k0 = toff[tile], k1 = toff[tile + 1];
        if (k0 == k1) continue;
        const int ox = (tile % ntx) * ts - wp.P / 2 - 2, oy = (tile / ntx) * ts - wp.P / 2 - 2;
        __syncthreads();
        for (int idx = threadIdx.x; idx < WW; idx += blockDim.x) {
            int xx = idx / W, yy = idx - xx * W;
            size_t at = (size_t)fte_wrap_index(ox + xx, wp.Mx) * wp.My + fte_wrap_index(oy + yy, wp.My);
            r0[idx] = __ldg(G0 + at);
            r1[idx] = __ldg(G1 + at);
        }
        __syncthreads();
        for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
            const int i = perm[k];
            Win wn = window_of(p[2 * i], p[2 * i + 1], wp);
            double ey = 1.0;
            for (int j = 0; j < P1; j++) {
                wyb[j] = ey * e1y[j];
                ey *= wn.e3y;
            }
            const int lx = wn.mx - ox, ly = wn.my - oy;
            double ex = wn.ex * wn.e4y;
            double acc0 = 0.0, acc1 = 0.0;
            if (lx >= 0 && ly >= 0 && lx + wp.P < W && ly + wp.P < W) {
                for (int a = 0; a < P1; a++) {
                    double wxa = ex * e1[a];
                    ex *= wn.e3x;
                    const double* c0 = r0 + (lx + a) * W + ly;
                    const double* c1 = r1 + (lx + a) * W + ly;
                    double s0 = 0.0, s1 = 0.0;
                    for (int j = 0; j < P1; j++) {
                        double wyj = wyb[j];
                        s0 = fma(wyj, c0[j], s0);
                        s1 = fma(wyj, c1[j], s1);
                    }
                    acc0 = fma(wxa, s0, acc0);
                    acc1 = fma(wxa, s1, acc1);
                }
            } else {
                for (int a = 0; a < P1; a++) {
                    double wxa = ex * e1[a];
                    ex *= wn.e3x;
                    size_t base = (size_t)fte_wrap_index(wn.mx + a, wp.Mx) * wp.My;
                    double s0 = 0.0, s1 = 0.0;
                    for (int j = 0; j < P1; j++) {
                        size_t at = base + fte_wrap_index(wn.my + j, wp.My);
                        s0 = fma(wyb[j], __ldg(G0 + at), s0);
                        s1 = fma(wyb[j], __ldg(G1 + at), s1);
                    }
                    acc0 = fma(wxa, s0, acc0);
                    acc1 = fma(wxa, s1, acc1);
                }
            }
            out[i] = make_double2(acc0 * scale, acc1 * scale);
        }
    }
}

// ---- FFT along y: real -> half spectrum (two columns per complex FFT) -------
__global__ void k_fft_y_r2c(const double* __restrict__ H, double2* __restrict__ Hh, int Mx, int My, FftDev plan) {
    extern __shared__ double2 shc[];
    double2* A = shc;
    double2* B = shc + plan.m;
    const int c = blockIdx.x, g = blockIdx.y;
    const int Kh = My / 2 + 1;
    const double* h0 = H + ((size_t)g * Mx + 2 * c) * My;
    const double* h1 = h0 + My;
    for (int y = threadIdx.x; y < My; y += blockDim.x) A[y] = make_double2(h0[y], h1[y]);
    double2* R = fft_block<double>(A, B, plan, false);
    double2* o0 = Hh + ((size_t)g * Mx + 2 * c) * Kh;
    double2* o1 = o0 + Kh;
    for (int k = threadIdx.x; k < Kh; k += blockDim.x) {
        double2 zk = R[k], zm = R[(My - k) % My];
        // A_k = (Z_k + conj Z_{-k})/2,  B_k = (Z_k - conj Z_{-k})/(2i)
        o0[k] = make_double2(0.5 * (zk.x + zm.x), 0.5 * (zk.y - zm.y));
        o1[k] = make_double2(0.5 * (zk.y + zm.y), -0.5 * (zk.x - zm.x));
    }
}

// ---- FFT along x of half spectra, in place: one block per (ky, grid) ---------
__global__ void k_fft_x(double2* __restrict__ Hh, int Mx, int Kh, FftDev plan, int inv) {
    extern __shared__ double2 shc[];
    double2* A = shc;
    double2* B = shc + plan.m;
    const int k = blockIdx.x, g = blockIdx.y;
    double2* base = Hh + (size_t)g * Mx * Kh + k;
    for (int x = threadIdx.x; x < Mx; x += blockDim.x) A[x] = base[(size_t)x * Kh];
    double2* R = fft_block<double>(A, B, plan, inv != 0);
    for (int x = threadIdx.x; x < Mx; x += blockDim.x) base[(size_t)x * Kh] = R[x];
}

// ---- FFT along y: half spectrum -> real, two columns per complex FFT --------
__global__ void k_fft_y_c2r(const double2* __restrict__ Hh, double* __restrict__ H, int Mx, int My, FftDev plan) {
    extern __shared__ double2 shc[];
    double2* A = shc;
    double2* B = shc + plan.m;
    const int c = blockIdx.x, g = blockIdx.y;
    const int Kh = My / 2 + 1;
    const double2* i0 = Hh + ((size_t)g * Mx + 2 * c) * Kh;
    const double2* i1 = i0 + Kh;
    for (int k = threadIdx.x; k < Kh; k += blockDim.x) {
        double2 a = i0[k], b = i1[k];
        if (k == 0 || 2 * k == My) {
            a.y = 0.0;
            b.y = 0.0;
        }
        // Z_k = a + i b ; Z_{My-k} = conj(a) + i conj(b)
        A[k] = make_double2(a.x - b.y, a.y + b.x);
        if (k > 0 && 2 * k < My) A[My - k] = make_double2(a.x + b.y, -a.y + b.x);
    }
    double2* R = fft_block<double>(A, B, plan, true);
    double* o0 = H + ((size_t)g * Mx + 2 * c) * My;
    double* o1 = o0 + My;
    for (int y = threadIdx.x; y < My; y += blockDim.x) {
        double2 z = R[y];
        o0[y] = z.x;
        o1[y] = z.y;
    }
}

// ---- the same three transforms in float-float (FFT lines of FfCx) --------------
// (two CTAs of up to 512 threads per SM: registers capped at 64 so that a
// second line's transform hides the first's barrier and load latency)
// column pair c of grid g (the kernels: one pair per CTA; the work-list
// kernels of batches read the evaluation's parameters first)
__device__ __forceinline__ void fft_y_r2c_ff_line(const double* __restrict__ H, float4* __restrict__ Hh, int Mx,
                                                  int My, const FftDev& plan, int c, int g, unsigned char* shff) {
    float4* A = reinterpret_cast<float4*>(shff);
    float4* B = A + plan.m;
    const int Kh = My / 2 + 1;
    const double* h0 = H + ((size_t)g * Mx + 2 * c) * My;
    const double* h1 = h0 + My;
    for (int y = threadIdx.x; y < My; y += blockDim.x) A[y] = ffc_mk(ff_split(h0[y]), ff_split(h1[y]));
    float4* R = fft_block<FfCx>(A, B, plan, false);
    // half spectra stored ky-major ([g][ky][x]): the x transforms then read
    // and write contiguous lines; columns 2c and 2c + 1 are adjacent
    float4* o0 = Hh + (size_t)g * Mx * Kh + 2 * c;
    const float2 half = make_float2(0.5f, 0.0f);
    for (int k = threadIdx.x; k < Kh; k += blockDim.x) {
        const float4 zk = R[k], zm = R[(My - k) % My];
        // A_k = (Z_k + conj Z_{-k})/2,  B_k = (Z_k - conj Z_{-k})/(2i)
        o0[(size_t)k * Mx] = cscale(ffc_mk(ff_add(ffc_re(zk), ffc_re(zm)), ff_add(ffc_im(zk), ff_neg(ffc_im(zm)))), half);
        o0[(size_t)k * Mx + 1] = cscale(ffc_mk(ff_add(ffc_im(zk), ffc_im(zm)), ff_add(ffc_re(zm), ff_neg(ffc_re(zk)))), half);
    }
}

__global__ void __launch_bounds__(512, 2) k_fft_y_r2c_ff(const double* __restrict__ H, float4* __restrict__ Hh, int Mx, int My, FftDev plan) {
    extern __shared__ __align__(16) unsigned char shff[];
    fft_y_r2c_ff_line(H, Hh, Mx, My, plan, blockIdx.x, blockIdx.y, shff);
}

// line ky = k of grid g
__device__ __forceinline__ void fft_x_ff_line(float4* __restrict__ Hh, int Mx, int Kh, const FftDev& plan, int inv,
                                              int k, int g, unsigned char* shff) {
    float4* A = reinterpret_cast<float4*>(shff);
    float4* B = A + plan.m;
    float4* base = Hh + ((size_t)g * Kh + k) * Mx;  // ky-major half spectra: line k is contiguous
    for (int x = threadIdx.x; x < Mx; x += blockDim.x) A[x] = base[x];
    float4* R = fft_block<FfCx>(A, B, plan, inv != 0);
    for (int x = threadIdx.x; x < Mx; x += blockDim.x) base[x] = R[x];
}

__global__ void __launch_bounds__(512, 2) k_fft_x_ff(float4* __restrict__ Hh, int Mx, int Kh, FftDev plan, int inv) {
    extern __shared__ __align__(16) unsigned char shff[];
    fft_x_ff_line(Hh, Mx, Kh, plan, inv, blockIdx.x, blockIdx.y, shff);
}

// half spectra -> real grids as float-float pairs (the gather's input):
// column pair c of grid g
__device__ __forceinline__ void fft_y_c2r_ff_line(const float4* __restrict__ Hh, float2* __restrict__ H, int Mx,
                                                  int My, const FftDev& plan, int c, int g, unsigned char* shff) {
    float4* A = reinterpret_cast<float4*>(shff);
    float4* B = A + plan.m;
    const int Kh = My / 2 + 1;
    const float4* i0 = Hh + (size_t)g * Mx * Kh + 2 * c;  // ky-major: columns 2c, 2c + 1 adjacent
    for (int k = threadIdx.x; k < Kh; k += blockDim.x) {
        float4 a = i0[(size_t)k * Mx], b = i0[(size_t)k * Mx + 1];
        if (k == 0 || 2 * k == My) {
            a.z = a.w = 0.f;
            b.z = b.w = 0.f;
        }
        // Z_k = a + i b ; Z_{My-k} = conj(a) + i conj(b)
        A[k] = ffc_mk(ff_add(ffc_re(a), ff_neg(ffc_im(b))), ff_add(ffc_im(a), ffc_re(b)));
        if (k > 0 && 2 * k < My) A[My - k] = ffc_mk(ff_add(ffc_re(a), ffc_im(b)), ff_add(ffc_re(b), ff_neg(ffc_im(a))));
    }
    float4* R = fft_block<FfCx>(A, B, plan, true);
    float2* o0 = H + ((size_t)g * Mx + 2 * c) * My;
    float2* o1 = o0 + My;
    for (int y = threadIdx.x; y < My; y += blockDim.x) {
        const float4 z = R[y];
        o0[y] = ffc_re(z);
        o1[y] = ffc_im(z);
    }
}

__global__ void __launch_bounds__(512, 2) k_fft_y_c2r_ff(const float4* __restrict__ Hh, float2* __restrict__ H, int Mx, int My, FftDev plan) {
    extern __shared__ __align__(16) unsigned char shff[];
    fft_y_c2r_ff_line(Hh, H, Mx, My, plan, blockIdx.x, blockIdx.y, shff);
}

// ---- k-space multipliers ------------------------------------------------------
// SLP (mex_stokes_slp_kspace.cpp:128-139): G = (K^2 H - k (k.H)) (1/K^4 + 1/(4 xi^2 K^2)) e^{-(1-eta)K^2/(4xi^2)}
__device__ __forceinline__ void slp_mult(double k1, double k2, double xi, double eta, double2 q1, double2 q2,
                                         double2& g1, double2& g2) {
    double K = k1 * k1 + k2 * k2;
    double e = (1.0 / (K * K) + 0.25 / (K * xi * xi)) * exp(-0.25 * (1 - eta) / (xi * xi) * K);
    double kqr = k1 * q1.x + k2 * q2.x, kqi = k1 * q1.y + k2 * q2.y;
    g1 = make_double2((K * q1.x - k1 * kqr) * e, (K * q1.y - k1 * kqi) * e);
    g2 = make_double2((K * q2.x - k2 * kqr) * e, (K * q2.y - k2 * kqi) * e);
}

// DLP (mex_stokes_dlp_kspace.cpp:372-402) on the spectra of S11, S21, S12, S22
__device__ __forceinline__ void dlp_mult(double k1, double k2, double xi, double eta, double2 a, double2 s21,
                                         double2 s12, double2 d, double2& g1, double2& g2) {
    double K = k1 * k1 + k2 * k2;
    double e = exp(-K * (1 - eta) / (4 * xi * xi)) * (1 + K / (4 * xi * xi)) / K;
    double sr = s21.x + s12.x, si = s21.y + s12.y;
    double qr = (k1 * k1 * a.x + k1 * k2 * sr + k2 * k2 * d.x) / K;
    double qi = (k1 * k1 * a.y + k1 * k2 * si + k2 * k2 * d.y) / K;
    double x1r = 2 * a.x * k1 + k2 * sr + k1 * (a.x + d.x) - 2 * k1 * qr;
    double x1i = 2 * a.y * k1 + k2 * si + k1 * (a.y + d.y) - 2 * k1 * qi;
    double x2r = 2 * d.x * k2 + k1 * sr + k2 * (a.x + d.x) - 2 * k2 * qr;
    double x2i = 2 * d.y * k2 + k1 * si + k2 * (a.y + d.y) - 2 * k2 * qi;
    g1 = make_double2(-x1i * e, x1r * e);
    g2 = make_double2(-x2i * e, x2r * e);
}

// spectra in FP64 (double2) or float-float (float4), read and written in FP64
__device__ __forceinline__ double2 spec_ld(const double2* p) { return *p; }
__device__ __forceinline__ double2 spec_ld(const float4* p) {
    const float4 v = *p;
    return make_double2(ff_join(v.x, v.y), ff_join(v.z, v.w));
}
__device__ __forceinline__ void spec_st(double2* p, double2 v) { *p = v; }
__device__ __forceinline__ void spec_st(float4* p, double2 v) {
    const float2 r = ff_split(v.x), i = ff_split(v.y);
    *p = make_float4(r.x, r.y, i.x, i.y);
}

// DLP spectra: ng = 4 (S11, S21, S12, S22) or 3 (S11, S12 + S21, S22).
// KYMAJOR: half spectra stored [g][ky][x] (the float-float block transforms)
// instead of [g][x][ky].
template <int KIND, typename S, bool KYMAJOR = false>
__global__ void k_filter(S* __restrict__ Hh, int Mx, int My, double Lx, double Ly, double xi, double eta, int ng) {
    const int Kh = My / 2 + 1;
    const size_t GS = (size_t)Mx * Kh;
    const size_t tot = GS;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
        const int j = KYMAJOR ? (int)(idx % Mx) : (int)(idx / Kh), k = KYMAJOR ? (int)(idx / Mx) : (int)(idx % Kh);
        S* p0 = Hh + idx;
        if (j == 0 && k == 0) {
            spec_st(p0, make_double2(0, 0));
            spec_st(p0 + GS, make_double2(0, 0));
            continue;
        }
        double k1 = (j <= Mx / 2) ? 2.0 * FTE_PI / Lx * j : 2.0 * FTE_PI / Lx * (j - Mx);
        double k2 = 2.0 * FTE_PI / Ly * k;
        bool nyq_x = (2 * j == Mx), nyq_y = (2 * k == My);
        double2 g1, g2;
        if (KIND == FTE_KIND_SLP) {
            double2 q1 = spec_ld(p0), q2 = spec_ld(p0 + GS);
            slp_mult(k1, k2, xi, eta, q1, q2, g1, g2);
            if (nyq_x || nyq_y) {
                double2 h1, h2;
                slp_mult(nyq_x ? -k1 : k1, nyq_y ? -k2 : k2, xi, eta, q1, q2, h1, h2);
                g1 = make_double2(0.5 * (g1.x + h1.x), 0.5 * (g1.y + h1.y));
                g2 = make_double2(0.5 * (g2.x + h2.x), 0.5 * (g2.y + h2.y));
            }
        } else {
            const double2 a = spec_ld(p0), s21 = spec_ld(p0 + GS), d = spec_ld(p0 + (ng - 1) * GS);
            const double2 s12 = ng == 4 ? spec_ld(p0 + 2 * GS) : make_double2(0, 0);
            dlp_mult(k1, k2, xi, eta, a, s21, s12, d, g1, g2);
            if (nyq_x || nyq_y) {
                double2 h1, h2;
                dlp_mult(nyq_x ? -k1 : k1, nyq_y ? -k2 : k2, xi, eta, a, s21, s12, d, h1, h2);
                g1 = make_double2(0.5 * (g1.x + h1.x), 0.5 * (g1.y + h1.y));
                g2 = make_double2(0.5 * (g2.x + h2.x), 0.5 * (g2.y + h2.y));
            }
        }
        spec_st(p0, g1);
        spec_st(p0 + GS, g2);
    }
}

// ---- the multipliers in float-float (float-float spectra) ---------------------
// The same formulas as slp_mult / dlp_mult and k_filter, on the FP32 pipe:
// wave numbers k = (2 pi / L) index from a float-float 2 pi / L, the Gaussian
// factor by fte_expm_ff, 1/K by ff_rcp.  Relative error ~1e-13.
struct FfFilt {
    float2 c1, c2;  // 2 pi / Lx, 2 pi / Ly
    float2 c4, cq;  // 1 / (4 xi^2), (1 - eta) / (4 xi^2)
};

__device__ __forceinline__ float2 ff_scale2(float2 a, float c) { return make_float2(a.x * c, a.y * c); }

// SLP: G = (K q - k (k.q)) (1/K^2 + 1/(4 xi^2 K)) e^{-(1-eta) K/(4 xi^2)}
__device__ __forceinline__ void slp_mult_ff(float2 k1, float2 k2, const FfFilt& f, const float2* etab, float4 q1,
                                            float4 q2, float4& g1, float4& g2) {
    const float2 K = ff_add(ff_sqr(k1), ff_sqr(k2));
    const float2 iK = ff_rcp(K);
    const float2 e = ff_mul(ff_add(ff_sqr(iK), ff_mul(iK, f.c4)), fte_expm_ff(ff_mul(K, f.cq), etab));
    const float2 kqr = ff_add(ff_mul(k1, ffc_re(q1)), ff_mul(k2, ffc_re(q2)));
    const float2 kqi = ff_add(ff_mul(k1, ffc_im(q1)), ff_mul(k2, ffc_im(q2)));
    g1 = ffc_mk(ff_mul(ff_add(ff_mul(K, ffc_re(q1)), ff_neg(ff_mul(k1, kqr))), e),
                ff_mul(ff_add(ff_mul(K, ffc_im(q1)), ff_neg(ff_mul(k1, kqi))), e));
    g2 = ffc_mk(ff_mul(ff_add(ff_mul(K, ffc_re(q2)), ff_neg(ff_mul(k2, kqr))), e),
                ff_mul(ff_add(ff_mul(K, ffc_im(q2)), ff_neg(ff_mul(k2, kqi))), e));
}

// DLP on the spectra of S11, S21, S12, S22 (as dlp_mult)
__device__ __forceinline__ void dlp_mult_ff(float2 k1, float2 k2, const FfFilt& f, const float2* etab, float4 a,
                                            float4 s21, float4 s12, float4 d, float4& g1, float4& g2) {
    const float2 K = ff_add(ff_sqr(k1), ff_sqr(k2));
    const float2 iK = ff_rcp(K);
    const float2 e = ff_mul(ff_mul(fte_expm_ff(ff_mul(K, f.cq), etab), ff_add(make_float2(1.0f, 0.0f), ff_mul(K, f.c4))),
                            iK);
    const float2 k11 = ff_sqr(k1), k12 = ff_mul(k1, k2), k22 = ff_sqr(k2);
    float2 x1[2], x2[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {  // real, imaginary parts (real multipliers)
        const float2 av = c ? ffc_im(a) : ffc_re(a), dv = c ? ffc_im(d) : ffc_re(d);
        const float2 sv = ff_add(c ? ffc_im(s21) : ffc_re(s21), c ? ffc_im(s12) : ffc_re(s12));
        const float2 q = ff_mul(ff_add(ff_add(ff_mul(k11, av), ff_mul(k12, sv)), ff_mul(k22, dv)), iK);
        const float2 ad = ff_add(av, dv);
        x1[c] = ff_add(ff_add(ff_add(ff_scale2(ff_mul(av, k1), 2.0f), ff_mul(k2, sv)), ff_mul(k1, ad)),
                       ff_neg(ff_scale2(ff_mul(k1, q), 2.0f)));
        x2[c] = ff_add(ff_add(ff_add(ff_scale2(ff_mul(dv, k2), 2.0f), ff_mul(k1, sv)), ff_mul(k2, ad)),
                       ff_neg(ff_scale2(ff_mul(k2, q), 2.0f)));
    }
    // g = i x e
    g1 = ffc_mk(ff_neg(ff_mul(x1[1], e)), ff_mul(x1[0], e));
    g2 = ffc_mk(ff_neg(ff_mul(x2[1], e)), ff_mul(x2[0], e));
}

__device__ __forceinline__ float4 ffc_avg(float4 a, float4 b) {
    return ffc_mk(ff_scale2(ff_add(ffc_re(a), ffc_re(b)), 0.5f), ff_scale2(ff_add(ffc_im(a), ffc_im(b)), 0.5f));
}

// modes idx0, idx0 + stride, ... of the half spectra (etab loaded)
template <int KIND>
__device__ __forceinline__ void filter_ff_run(float4* __restrict__ Hh, int Mx, int My, const FfFilt& f, int ng,
                                              size_t idx0, size_t stride, const float2* etab) {
    const int Kh = My / 2 + 1;
    const size_t GS = (size_t)Mx * Kh;
    for (size_t idx = idx0; idx < GS; idx += stride) {
        const int k = (int)(idx / Mx), j = (int)(idx % Mx);  // ky-major half spectra
        float4* p0 = Hh + idx;
        if (j == 0 && k == 0) {
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            p0[0] = z;
            p0[GS] = z;
            continue;
        }
        const float2 k1 = ff_mulf(f.c1, (float)((j <= Mx / 2) ? j : j - Mx));
        const float2 k2 = ff_mulf(f.c2, (float)k);
        const bool nyq_x = (2 * j == Mx), nyq_y = (2 * k == My);
        const float2 k1m = nyq_x ? ff_neg(k1) : k1, k2m = nyq_y ? ff_neg(k2) : k2;
        float4 g1, g2;
        if (KIND == FTE_KIND_SLP) {
            const float4 q1 = p0[0], q2 = p0[GS];
            slp_mult_ff(k1, k2, f, etab, q1, q2, g1, g2);
            if (nyq_x || nyq_y) {
                float4 h1, h2;
                slp_mult_ff(k1m, k2m, f, etab, q1, q2, h1, h2);
                g1 = ffc_avg(g1, h1);
                g2 = ffc_avg(g2, h2);
            }
        } else {
            const float4 a = p0[0], s21 = p0[GS], d = p0[(ng - 1) * GS];
            const float4 s12 = ng == 4 ? p0[2 * GS] : make_float4(0.f, 0.f, 0.f, 0.f);
            dlp_mult_ff(k1, k2, f, etab, a, s21, s12, d, g1, g2);
            if (nyq_x || nyq_y) {
                float4 h1, h2;
                dlp_mult_ff(k1m, k2m, f, etab, a, s21, s12, d, h1, h2);
                g1 = ffc_avg(g1, h1);
                g2 = ffc_avg(g2, h2);
            }
        }
        p0[0] = g1;
        p0[GS] = g2;
    }
}

template <int KIND>
__global__ void k_filter_ff(float4* __restrict__ Hh, int Mx, int My, FfFilt f, int ng) {
    __shared__ float2 etab[64];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) etab[i] = ff_split(exp2(-i / 64.0));
    __syncthreads();
    filter_ff_run<KIND>(Hh, Mx, My, f, ng, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                        (size_t)gridDim.x * blockDim.x, etab);
}

FfFilt ff_filter_consts(double Lx, double Ly, double xi, double eta) {
    auto sp = [](double v) {
        const float h = (float)v;
        return make_float2(h, (float)(v - (double)h));
    };
    FfFilt f;
    f.c1 = sp(2.0 * FTE_PI / Lx);
    f.c2 = sp(2.0 * FTE_PI / Ly);
    f.c4 = sp(0.25 / (xi * xi));
    f.cq = sp((1.0 - eta) / (4.0 * xi * xi));
    return f;
}

inline int pt_grid(fte_context* ctx, int64_t n) {
    int64_t b = (n + kPtThreads - 1) / kPtThreads;
    int64_t maxb = (int64_t)ctx->num_sms * 16;
    if (b > maxb) b = maxb;
    if (b < 1) b = 1;
    return (int)b;
}

int fft_threads(int m) {
    int t = 64;
    while (t < 512 && t * 8 < m) t *= 2;
    return t;
}

}  // namespace

// ===========================================================================
// Long FP64 transforms (grids whose lines do not fit one block's shared
// memory: the drivers' analytic grids reach A * 10000 nodes along x).
//
// Four-step (Bailey 1990) over L = n1 n2, x_j = x[j1 + n1 j2]:
//   pass 1, per (line, j1):  v[k2] = W_L^{j1 k2} * DFT_{n2}(x[j1 + n1 j2])[k2]
//                            stored at Y[line][j1 + n1 k2]
//   pass 2, per (line, k2):  X[k2 + n2 k1] = DFT_{n1}(Y[line][j1 + n1 k2])[k1]
// The inverse uses the conjugate roots throughout.  Lengths without a
// block-sized factorisation run Bluestein's convolution in global memory
// over a factorable L >= 2n - 1 (chirp, forward four-step, multiply by the
// transformed conjugate chirp, inverse four-step, chirp).
// ===========================================================================
namespace {
__device__ __forceinline__ size_t lm_off(const LineMap& m, long long l) {
    return (size_t)(l / m.lpg) * m.gs + (size_t)(l % m.lpg) * m.ls;
}

__global__ void k_lf_pass1(const double2* __restrict__ X, LineMap mx, int L, int n1, int n2, FftDev d2,
                           const double2* __restrict__ tw, double2* __restrict__ Y, int inv) {
    extern __shared__ double2 shc[];
    double2* A = shc;
    double2* B = shc + d2.m;
    const long long line = blockIdx.x;
    const int j1 = blockIdx.y;
    const double2* x = X + lm_off(mx, line);
    for (int j2 = threadIdx.x; j2 < n2; j2 += blockDim.x) A[j2] = x[(size_t)(j1 + (long long)n1 * j2) * mx.es];
    double2* R = fft_block<double>(A, B, d2, inv != 0);
    double2* y = Y + (size_t)line * L;
    for (int k2 = threadIdx.x; k2 < n2; k2 += blockDim.x) {
        double2 w = __ldg(tw + (long long)j1 * k2 % L);
        if (inv) w.y = -w.y;
        y[j1 + (size_t)n1 * k2] = cmul(R[k2], w);
    }
}

__global__ void k_lf_pass2(const double2* __restrict__ Y, int L, int n1, int n2, FftDev d1, double2* __restrict__ X,
                           LineMap mx, int inv) {
    extern __shared__ double2 shc[];
    double2* A = shc;
    double2* B = shc + d1.m;
    const long long line = blockIdx.x;
    const int k2 = blockIdx.y;
    const double2* y = Y + (size_t)line * L + (size_t)n1 * k2;
    for (int j1 = threadIdx.x; j1 < n1; j1 += blockDim.x) A[j1] = y[j1];
    double2* R = fft_block<double>(A, B, d1, inv != 0);
    double2* x = X + lm_off(mx, line);
    for (int k1 = threadIdx.x; k1 < n1; k1 += blockDim.x) x[(size_t)(k2 + (long long)n2 * k1) * mx.es] = R[k1];
}

__global__ void k_lb_pre(const double2* __restrict__ X, LineMap mx, int n, int L, const double2* __restrict__ chirp,
                         double2* __restrict__ Z, long long nl, int inv) {
    const long long total = nl * L;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long l = i / L;
        const int k = (int)(i - l * L);
        double2 v = make_double2(0.0, 0.0);
        if (k < n) {
            double2 x = X[lm_off(mx, l) + (size_t)k * mx.es];
            if (inv) x.y = -x.y;
            v = cmul(x, __ldg(chirp + k));
        }
        Z[i] = v;
    }
}

__global__ void k_lb_mul(double2* __restrict__ Z, const double2* __restrict__ bhat, int L, long long total) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x)
        Z[i] = cmul(Z[i], __ldg(bhat + i % L));
}

__global__ void k_lb_post(const double2* __restrict__ Z, int n, int L, const double2* __restrict__ chirp,
                          double2* __restrict__ X, LineMap mx, long long nl, int inv) {
    const long long total = nl * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long l = i / n;
        const int k = (int)(i - l * n);
        double2 y = cmul(Z[(size_t)l * L + k], __ldg(chirp + k));
        if (inv) y.y = -y.y;
        X[lm_off(mx, l) + (size_t)k * mx.es] = y;
    }
}

// y direction through a staging buffer S of complex lines (two real rows each)
__global__ void k_ly_pack_r2c(const double* __restrict__ H, double2* __restrict__ S, int Mx, int My, int ng) {
    const long long total = (long long)ng * (Mx / 2) * My;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long line = i / My;
        const int y = (int)(i - line * My);
        const long long g = line / (Mx / 2), c = line - g * (Mx / 2);
        const double* h0 = H + ((size_t)g * Mx + 2 * c) * My;
        S[i] = make_double2(h0[y], h0[My + y]);
    }
}

__global__ void k_ly_unpack_r2c(const double2* __restrict__ S, double2* __restrict__ Hh, int Mx, int My, int ng) {
    const int Kh = My / 2 + 1;
    const long long total = (long long)ng * (Mx / 2) * Kh;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long line = i / Kh;
        const int k = (int)(i - line * Kh);
        const long long g = line / (Mx / 2), c = line - g * (Mx / 2);
        const double2* R = S + (size_t)line * My;
        double2 zk = R[k], zm = R[(My - k) % My];
        double2* o0 = Hh + ((size_t)g * Mx + 2 * c) * Kh;
        o0[k] = make_double2(0.5 * (zk.x + zm.x), 0.5 * (zk.y - zm.y));
        o0[Kh + k] = make_double2(0.5 * (zk.y + zm.y), -0.5 * (zk.x - zm.x));
    }
}

__global__ void k_ly_pack_c2r(const double2* __restrict__ Hh, double2* __restrict__ S, int Mx, int My, int ng) {
    const int Kh = My / 2 + 1;
    const long long total = (long long)ng * (Mx / 2) * Kh;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long line = i / Kh;
        const int k = (int)(i - line * Kh);
        const long long g = line / (Mx / 2), c = line - g * (Mx / 2);
        const double2* i0 = Hh + ((size_t)g * Mx + 2 * c) * Kh;
        double2 a = i0[k], b = i0[Kh + k];
        if (k == 0 || 2 * k == My) {
            a.y = 0.0;
            b.y = 0.0;
        }
        double2* A = S + (size_t)line * My;
        A[k] = make_double2(a.x - b.y, a.y + b.x);
        if (k > 0 && 2 * k < My) A[My - k] = make_double2(a.x + b.y, -a.y + b.x);
    }
}

__global__ void k_ly_unpack_c2r(const double2* __restrict__ S, double* __restrict__ H, int Mx, int My, int ng) {
    const long long total = (long long)ng * (Mx / 2) * My;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long line = i / My;
        const int y = (int)(i - line * My);
        const long long g = line / (Mx / 2), c = line - g * (Mx / 2);
        double* o0 = H + ((size_t)g * Mx + 2 * c) * My;
        double2 z = S[i];
        o0[y] = z.x;
        o0[My + y] = z.y;
    }
}

int ew_grid(const fte_context* c, long long total) {
    long long b = (total + 255) / 256;
    if (b < 1) b = 1;
    if (b > c->num_sms * 16) b = c->num_sms * 16;
    return (int)b;
}
}  // namespace

int fte_long_fft(fte_context* c, const LongFft& f, double2* X, LineMap mx, long long nl, bool inv, double2* scratch) {
    if (nl <= 0) return FTE_OK;
    if (nl > 0x7fffffffLL || f.n1 > 65535 || f.n2 > 65535) {
        fte_set_error("long FFT: %lld lines of %d beyond the launch limits", nl, f.n);
        return FTE_ERR_UNSUPPORTED;
    }
    const size_t sm1 = 2 * (size_t)f.d2.m * sizeof(double2), sm2 = 2 * (size_t)f.d1.m * sizeof(double2);
    if (sm1 > (size_t)c->max_smem_optin || sm2 > (size_t)c->max_smem_optin) {
        fte_set_error("long FFT: block transforms of %d / %d exceed shared memory", f.n2, f.n1);
        return FTE_ERR_UNSUPPORTED;
    }
    FTE_CUDA_TRY(fte_smem_ceiling(k_lf_pass1, (int)sm1));
    FTE_CUDA_TRY(fte_smem_ceiling(k_lf_pass2, (int)sm2));
    const LineMap flat{(long long)f.L, 0, 1, 1};
    auto four_step = [&](double2* data, LineMap m, double2* Y, bool iv) -> int {
        FTE_LAUNCH(c, k_lf_pass1, dim3((unsigned)nl, f.n1), fft_threads(f.d2.m), sm1, (const double2*)data, m, f.L,
                   f.n1, f.n2, f.d2, f.tw, Y, iv ? 1 : 0);
        FTE_LAUNCH(c, k_lf_pass2, dim3((unsigned)nl, f.n2), fft_threads(f.d1.m), sm2, (const double2*)Y, f.L, f.n1,
                   f.n2, f.d1, data, m, iv ? 1 : 0);
        return FTE_OK;
    };
    if (f.mode == 1) return four_step(X, mx, scratch, inv);
    // Bluestein over L: Z = chirp * x (zero padded), Z <- IDFT(DFT(Z) * bhat), x = chirp * Z
    double2* Z = scratch;
    double2* Y = scratch + (size_t)nl * f.L;
    const long long total = nl * (long long)f.L;
    FTE_LAUNCH(c, k_lb_pre, ew_grid(c, total), 256, 0, (const double2*)X, mx, f.n, f.L, f.chirp, Z, nl, inv ? 1 : 0);
    FTE_TRY(four_step(Z, flat, Y, false));
    FTE_LAUNCH(c, k_lb_mul, ew_grid(c, total), 256, 0, Z, f.bhat, f.L, total);
    FTE_TRY(four_step(Z, flat, Y, true));
    FTE_LAUNCH(c, k_lb_post, ew_grid(c, nl * (long long)f.n), 256, 0, (const double2*)Z, f.n, f.L, f.chirp, X, mx, nl,
               inv ? 1 : 0);
    return FTE_OK;
}

namespace {
size_t tile_budget(const fte_context* ctx) {
    size_t b = 110 * 1024;  // two CTAs per SM
    return b < (size_t)ctx->max_smem_optin ? b : (size_t)ctx->max_smem_optin;
}

// ===========================================================================
// Mixed form: grids, spectra and window weights in FP32.
//
// Window weights: for node offset a the window is exp(t ((a - P/2) h - px)^2),
// t = -2 xi^2/eta (the fast-Gaussian-gridding product with w = P h / 2, which
// the drivers always use); the argument is formed in FP64 and the
// exponential taken in FP32, so no error accumulates along the window (the
// FP32 recurrence would lose ~P ulps).  The spread accumulates with Kahan
// compensation (sum and carry per node); the gather sums a window column in
// FP32 and the columns in FP64.  Filter multipliers are evaluated in FP64 and
// applied to the FP32 spectra.
// ===========================================================================
// h: the axis's grid step (wp.h along x, wp.hy along y)
__device__ __forceinline__ void win32(double pp, double h, const WinParams& wp, float* out) {
    const double t = -2 * wp.xi * wp.xi / wp.eta;
    const int P1 = wp.P + 1;
    for (int a = 0; a < P1; a++) {
        double d = fma((double)(a - wp.P / 2), h, -pp);
        out[a] = expf((float)(t * d * d));
    }
}

__device__ __forceinline__ void closest32(double x, double y, const WinParams& wp, int* mx, int* my, double* px,
                                          double* py) {
    fte_closest_node(x, y, wp.Lx, wp.Ly, wp.h, wp.rh, wp.hy, wp.rhy, wp.P, mx, my, px, py);
}

constexpr int kColChunk32 = 64;

__global__ void __launch_bounds__(kColThreads) k_spread_cols32(int mode, const double* __restrict__ p,
                                                              const double* __restrict__ f,
                                                              const double* __restrict__ nrm,
                                                              const double* __restrict__ wts,
                                                              const int* __restrict__ toff,
                                                              const int* __restrict__ perm, int ts, int ntx, int nty,
                                                              WinParams wp, float* __restrict__ H0,
                                                              float* __restrict__ H1) {
    extern __shared__ float shf[];
    const int P1 = wp.P + 1, W = tile_region(ts, wp.P), WW = W * W;
    float* sum = shf;                       // 2 * WW
    float* car = sum + 2 * WW;              // 2 * WW (Kahan carries)
    float* fw = car + 2 * WW;               // kColChunk32 * 2 * P1
    float* wy = fw + kColChunk32 * 2 * P1;  // kColChunk32 * P1
    int* org = reinterpret_cast<int*>(wy + kColChunk32 * P1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int nw = kColWarps;
    for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
        const int k0 = toff[tile], k1 = toff[tile + 1];
        if (k0 == k1) continue;
        const int ox = (tile % ntx) * ts - wp.P / 2 - 2, oy = (tile / ntx) * ts - wp.P / 2 - 2;
        __syncthreads();
        for (int i = threadIdx.x; i < 4 * WW; i += blockDim.x) sum[i] = 0.f;
        for (int c0 = k0; c0 < k1; c0 += kColChunk32) {
            const int cn = min(kColChunk32, k1 - c0);
            __syncthreads();
            if (threadIdx.x < cn) {
                const int s = threadIdx.x;
                const int i = perm[c0 + s];
                int mx, my;
                double px, py;
                closest32(p[2 * i], p[2 * i + 1], wp, &mx, &my, &px, &py);
                double f1 = f[2 * i], f2 = f[2 * i + 1];
                if (wts) {
                    f1 *= wts[i];
                    f2 *= wts[i];
                }
                double q0 = f1, q1 = f2;
                if (mode == 1) {
                    q0 = f1 * nrm[2 * i];
                    q1 = f2 * nrm[2 * i];
                } else if (mode == 2) {
                    q0 = f1 * nrm[2 * i + 1];
                    q1 = f2 * nrm[2 * i + 1];
                }
                float* wyx = wy + s * P1;
                win32(py, wp.hy, wp, wyx);
                float* fa = fw + (s * 2) * P1;
                win32(px, wp.h, wp, fa);
                const float q0f = (float)q0, q1f = (float)q1;
                for (int a = 0; a < P1; a++) {
                    float wxa = fa[a];
                    fa[a] = q0f * wxa;
                    fa[P1 + a] = q1f * wxa;
                }
                const int lx = mx - ox, ly = my - oy;
                if (lx >= 0 && ly >= 0 && lx + wp.P < W && ly + wp.P < W) {
                    org[2 * s] = lx;
                    org[2 * s + 1] = ly;
                } else {
                    org[2 * s] = -1;
                    for (int a = 0; a < P1; a++) {
                        size_t base = (size_t)fte_wrap_index(mx + a, wp.Mx) * wp.My;
                        for (int j = 0; j < P1; j++) {
                            size_t at = base + fte_wrap_index(my + j, wp.My);
                            atomicAdd(&H0[at], fa[a] * wyx[j]);
                            atomicAdd(&H1[at], fa[P1 + a] * wyx[j]);
                        }
                    }
                }
            }
            __syncthreads();
            for (int s = 0; s < cn; s++) {
                const int lx = org[2 * s];
                if (lx < 0) continue;
                const int ly = org[2 * s + 1];
                // window rows in blocks of 32 (P up to 64)
                const int cfirst = lx + ((warp - lx) & (nw - 1));
                for (int j = lane; j < P1; j += 32) {
                    const float wyj = wy[s * P1 + j];
                    const float* fa = fw + (s * 2) * P1;
                    for (int c = cfirst; c <= lx + wp.P; c += nw) {
                        const int at = c * W + ly + j;
#pragma unroll
                        for (int g = 0; g < 2; g++) {
                            // Kahan: sum += v with carry
                            float v = fa[g * P1 + c - lx] * wyj - car[g * WW + at];
                            float s0 = sum[g * WW + at];
                            float t = s0 + v;
                            car[g * WW + at] = (t - s0) - v;
                            sum[g * WW + at] = t;
                        }
                    }
                }
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < 2 * WW; idx += blockDim.x) {
            float v = sum[idx] - car[idx];
            if (v == 0.f) continue;
            int g = idx >= WW, r = idx - g * WW;
            int xx = r / W, yy = r - xx * W;
            size_t at = (size_t)fte_wrap_index(ox + xx, wp.Mx) * wp.My + fte_wrap_index(oy + yy, wp.My);
            atomicAdd(g ? &H1[at] : &H0[at], v);
        }
    }
}

size_t spread_cols32_smem(int ts, int P) {
    const int P1 = P + 1, W = tile_region(ts, P);
    return (size_t)(4 * W * W + kColChunk32 * 3 * P1) * sizeof(float) + kColChunk32 * 2 * sizeof(int);
}

__global__ void __launch_bounds__(kTileThreads) k_gather_tiled32(const double* __restrict__ p,
                                                                const int* __restrict__ toff,
                                                                const int* __restrict__ perm, int ts, int ntx,
                                                                int nty, WinParams wp, const float* __restrict__ G0,
                                                                const float* __restrict__ G1, double scale,
                                                                double2* __restrict__ out) {
    extern __shared__ float shf[];
    const int P1 = wp.P + 1, W = tile_region(ts, wp.P), WW = W * W;
    float* r0 = shf;
    float* r1 = r0 + WW;
    float* wxb = r1 + WW + threadIdx.x * 2 * P1;
    float* wyb = wxb + P1;
    for (int tile = blockIdx.x; tile < ntx * nty; tile += gridDim.x) {
        const int k0 = toff[tile], k1 = toff[tile + 1];
        if (k0 == k1) continue;
        const int ox = (tile % ntx) * ts - wp.P / 2 - 2, oy = (tile / ntx) * ts - wp.P / 2 - 2;
        __syncthreads();
        for (int idx = threadIdx.x; idx < WW; idx += blockDim.x) {
            int xx = idx / W, yy = idx - xx * W;
            size_t at = (size_t)fte_wrap_index(ox + xx, wp.Mx) * wp.My + fte_wrap_index(oy + yy, wp.My);
            r0[idx] = __ldg(G0 + at);
            r1[idx] = __ldg(G1 + at);
        }
        __syncthreads();
        for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
            const int i = perm[k];
            int mx, my;
            double px, py;
            closest32(p[2 * i], p[2 * i + 1], wp, &mx, &my, &px, &py);
            win32(px, wp.h, wp, wxb);
            win32(py, wp.hy, wp, wyb);
            const int lx = mx - ox, ly = my - oy;
            const bool inside = lx >= 0 && ly >= 0 && lx + wp.P < W && ly + wp.P < W;
            double acc0 = 0.0, acc1 = 0.0;
            for (int a = 0; a < P1; a++) {
                float s0 = 0.f, s1 = 0.f;
                if (inside) {
                    const float* c0 = r0 + (lx + a) * W + ly;
                    const float* c1 = r1 + (lx + a) * W + ly;
                    for (int j = 0; j < P1; j++) {
                        s0 = fmaf(wyb[j], c0[j], s0);
                        s1 = fmaf(wyb[j], c1[j], s1);
                    }
                } else {
                    size_t base = (size_t)fte_wrap_index(mx + a, wp.Mx) * wp.My;
                    for (int j = 0; j < P1; j++) {
                        size_t at = base + fte_wrap_index(my + j, wp.My);
                        s0 = fmaf(wyb[j], __ldg(G0 + at), s0);
                        s1 = fmaf(wyb[j], __ldg(G1 + at), s1);
                    }
                }
                acc0 = fma((double)wxb[a], (double)s0, acc0);
                acc1 = fma((double)wxb[a], (double)s1, acc1);
            }
            out[i] = make_double2(acc0 * scale, acc1 * scale);
        }
    }
}

size_t gather32_smem(int ts, int P) {
    const int W = tile_region(ts, P);
    return (size_t)(2 * W * W + kTileThreads * 2 * (P + 1)) * sizeof(float);
}

// FP32 FFT passes (same structure as the FP64 kernels)
__global__ void k_fft_y_r2c32(const float* __restrict__ H, float2* __restrict__ Hh, int Mx, int My, FftDev plan) {
    extern __shared__ float2 shc32[];
    float2* A = shc32;
    float2* B = shc32 + plan.m;
    const int c = blockIdx.x, g = blockIdx.y;
    const int Kh = My / 2 + 1;
    const float* h0 = H + ((size_t)g * Mx + 2 * c) * My;
    const float* h1 = h0 + My;
    for (int y = threadIdx.x; y < My; y += blockDim.x) A[y] = make_float2(h0[y], h1[y]);
    float2* R = fft_block<float>(A, B, plan, false);
    float2* o0 = Hh + ((size_t)g * Mx + 2 * c) * Kh;
    float2* o1 = o0 + Kh;
    for (int k = threadIdx.x; k < Kh; k += blockDim.x) {
        float2 zk = R[k], zm = R[(My - k) % My];
        o0[k] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        o1[k] = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
    }
}

__global__ void k_fft_x32(float2* __restrict__ Hh, int Mx, int Kh, FftDev plan, int inv) {
    extern __shared__ float2 shc32[];
    float2* A = shc32;
    float2* B = shc32 + plan.m;
    const int k = blockIdx.x, g = blockIdx.y;
    float2* base = Hh + (size_t)g * Mx * Kh + k;
    for (int x = threadIdx.x; x < Mx; x += blockDim.x) A[x] = base[(size_t)x * Kh];
    float2* R = fft_block<float>(A, B, plan, inv != 0);
    for (int x = threadIdx.x; x < Mx; x += blockDim.x) base[(size_t)x * Kh] = R[x];
}

__global__ void k_fft_y_c2r32(const float2* __restrict__ Hh, float* __restrict__ H, int Mx, int My, FftDev plan) {
    extern __shared__ float2 shc32[];
    float2* A = shc32;
    float2* B = shc32 + plan.m;
    const int c = blockIdx.x, g = blockIdx.y;
    const int Kh = My / 2 + 1;
    const float2* i0 = Hh + ((size_t)g * Mx + 2 * c) * Kh;
    const float2* i1 = i0 + Kh;
    for (int k = threadIdx.x; k < Kh; k += blockDim.x) {
        float2 a = i0[k], b = i1[k];
        if (k == 0 || 2 * k == My) {
            a.y = 0.f;
            b.y = 0.f;
        }
        A[k] = make_float2(a.x - b.y, a.y + b.x);
        if (k > 0 && 2 * k < My) A[My - k] = make_float2(a.x + b.y, -a.y + b.x);
    }
    float2* R = fft_block<float>(A, B, plan, true);
    float* o0 = H + ((size_t)g * Mx + 2 * c) * My;
    float* o1 = o0 + My;
    for (int y = threadIdx.x; y < My; y += blockDim.x) {
        float2 z = R[y];
        o0[y] = z.x;
        o1[y] = z.y;
    }
}

// multipliers in FP64 applied to FP32 spectra (same Nyquist averaging)
template <int KIND>
__global__ void k_filter32(float2* __restrict__ Hh, int Mx, int My, double Lx, double Ly, double xi, double eta) {
    const int Kh = My / 2 + 1;
    const size_t GS = (size_t)Mx * Kh;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < GS; idx += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(idx / Kh), k = (int)(idx % Kh);
        float2* p0 = Hh + idx;
        if (j == 0 && k == 0) {
            p0[0] = make_float2(0.f, 0.f);
            p0[GS] = make_float2(0.f, 0.f);
            continue;
        }
        double k1 = (j <= Mx / 2) ? 2.0 * FTE_PI / Lx * j : 2.0 * FTE_PI / Lx * (j - Mx);
        double k2 = 2.0 * FTE_PI / Ly * k;
        bool nyq_x = (2 * j == Mx), nyq_y = (2 * k == My);
        double2 g1, g2;
        auto d2 = [](float2 v) { return make_double2(v.x, v.y); };
        if (KIND == FTE_KIND_SLP) {
            double2 q1 = d2(p0[0]), q2 = d2(p0[GS]);
            slp_mult(k1, k2, xi, eta, q1, q2, g1, g2);
            if (nyq_x || nyq_y) {
                double2 h1, h2;
                slp_mult(nyq_x ? -k1 : k1, nyq_y ? -k2 : k2, xi, eta, q1, q2, h1, h2);
                g1 = make_double2(0.5 * (g1.x + h1.x), 0.5 * (g1.y + h1.y));
                g2 = make_double2(0.5 * (g2.x + h2.x), 0.5 * (g2.y + h2.y));
            }
        } else {
            double2 a = d2(p0[0]), s21 = d2(p0[GS]), s12 = d2(p0[2 * GS]), d = d2(p0[3 * GS]);
            dlp_mult(k1, k2, xi, eta, a, s21, s12, d, g1, g2);
            if (nyq_x || nyq_y) {
                double2 h1, h2;
                dlp_mult(nyq_x ? -k1 : k1, nyq_y ? -k2 : k2, xi, eta, a, s21, s12, d, h1, h2);
                g1 = make_double2(0.5 * (g1.x + h1.x), 0.5 * (g1.y + h1.y));
                g2 = make_double2(0.5 * (g2.x + h2.x), 0.5 * (g2.y + h2.y));
            }
        }
        p0[0] = make_float2((float)g1.x, (float)g1.y);
        p0[GS] = make_float2((float)g2.x, (float)g2.y);
    }
}

// ===========================================================================
// Float-float k-space (FTE_FORM_FF): the spread and the gather carry every
// window weight, density and grid value as an unevaluated sum hi + lo of two
// FP32 numbers (about 48 significant bits) and do their arithmetic on the
// FP32 pipe, which GB300 runs at 64 times its FP64 rate: products by the
// FMA-based exact product (Dekker 1971, "A floating-point technique for
// extending the available precision"), sums by Knuth's two-sum.  The
// transforms and the filter stay FP64.  Per-point window factors are formed
// once in FP64 (the reference's closest node and four exponentials,
// ewald_tools.cpp:86-114, 152-160), rounded to float-float, and the window
// rows by float-float recurrences; relative error ~1e-13 against FP64.
// ===========================================================================
// per-source window record in tile order (64 bytes)
struct FfWin {
    int mx, my;            // first window node
    float2 e0, ex3, ey3;   // ex e4y, e3x, e3y (float-float)
    float2 q[4];           // densities of the grids (SLP: f1, f2; DLP: f1 n1, f2 n1 + f1 n2, f2 n2), weights folded in
};
static_assert(sizeof(FfWin) == 64, "FfWin layout");

__device__ __forceinline__ void load_e1_ff(float2* e1, const WinParams& wp) {
    double t0 = -2 * wp.xi * wp.xi / wp.eta * wp.h * wp.h;
    double t0y = -2 * wp.xi * wp.xi / wp.eta * wp.hy * wp.hy;
    const int P1e = (wp.P + 2) & ~1;
    for (int j = threadIdx.x; j <= wp.P; j += blockDim.x) {
        int jj = j - wp.P / 2;
        e1[j] = ff_split(exp(t0 * jj * jj));
        if (wp.aniso) e1[P1e + j] = ff_split(exp(t0y * jj * jj));
    }
}

// exponent of e0 = ex e4y: px^2 + py^2 + 2 (w px + wy py), formed as the
// reference forms it (2 w (px + py)) when the axes share their step
__device__ __forceinline__ double e0_arg(double px, double py, const WinParams& wp) {
    return wp.aniso ? px * px + py * py + 2 * (wp.w * px + wp.wy * py) : px * px + py * py + 2 * wp.w * (px + py);
}

// the window record of the k-th source in tile order: the three window
// factors as float-float exponentials of FP64 arguments, e0 = ex e4y =
// exp(t (px^2 + py^2 + 2 w (px + py))), e3x = exp(-2 t h px), e3y =
// exp(-2 t h py), t = -2 xi^2 / eta (the factors of window_of), and the
// densities; etab = 2^(-j/64), j < 64, in float-float
__device__ __forceinline__ void ff_win_rec(int kind, const double* __restrict__ p, const double* __restrict__ f,
                                           const double* __restrict__ nrm, const double* __restrict__ wts,
                                           const int* __restrict__ perm, int64_t k, const WinParams& wp,
                                           const float2* etab, FfWin* __restrict__ out) {
    const double t = -2 * wp.xi * wp.xi / wp.eta;
    {
        const int i = perm[k];
        int mx, my;
        double px, py;
        fte_closest_node(p[2 * i], p[2 * i + 1], wp.Lx, wp.Ly, wp.h, wp.rh, wp.hy, wp.rhy, wp.P, &mx, &my, &px, &py);
        FfWin r;
        r.mx = mx;
        r.my = my;
        r.e0 = fte_expm_ff(ff_split(-t * e0_arg(px, py, wp)), etab);
        r.ex3 = fte_expm_ff(ff_split(2 * t * wp.h * px), etab);
        r.ey3 = fte_expm_ff(ff_split(2 * t * wp.hy * py), etab);
        double f1 = f[2 * i], f2 = f[2 * i + 1];
        if (wts) {
            f1 *= wts[i];
            f2 *= wts[i];
        }
        if (kind == FTE_KIND_SLP) {
            r.q[0] = ff_split(f1);
            r.q[1] = ff_split(f2);
            r.q[2] = r.q[3] = make_float2(0.f, 0.f);
        } else {
            // the stresslet's three symmetric products (the multiplier takes
            // f2 n1 and f1 n2 only through their sum)
            const double n1 = nrm[2 * i], n2 = nrm[2 * i + 1];
            r.q[0] = ff_split(f1 * n1);
            r.q[1] = ff_split(f2 * n1 + f1 * n2);
            r.q[2] = ff_split(f2 * n2);
            r.q[3] = make_float2(0.f, 0.f);
        }
        out[k] = r;
    }
}

__device__ __forceinline__ void load_etab(float2* etab) {
    for (int j = threadIdx.x; j < 64; j += blockDim.x) etab[j] = ff_split(exp2(-j / 64.0));
}

// window records of the sources in tile order (k indexes perm)
__global__ void k_ff_win(int kind, const double* __restrict__ p, const double* __restrict__ f,
                         const double* __restrict__ nrm, const double* __restrict__ wts, const int* __restrict__ perm,
                         int64_t n, WinParams wp, FfWin* __restrict__ out) {
    __shared__ float2 etab[64];
    load_etab(etab);
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        ff_win_rec(kind, p, f, nrm, wts, perm, k, wp, etab, out);
}

// Column-owned spread of grids (2 pass, 2 pass + 1) in float-float: the
// scheme of k_spread_cols (warp w adds every region column c = w mod warps,
// lane j window row j) with the first two grids' (sum, low parts) interleaved
// in one float4 per region node (a third grid's pair in a float2 array); the
// region is flushed to the FP64 grids.  NG = 2 (Stokeslet: f1, f2) or 3
// (stresslet: the symmetric products f1 n1, f1 n2 + f2 n1, f2 n2 -- the
// stresslet multiplier sees the two mixed products only through their sum).
// tiles tile0, tile0 + tstep, ... of one grid (the kernels below: a grid-
// stride loop over one evaluation's tiles, or one tile of a work list).
// C32 (FTE_FORM_FF32, loose tolerances): the window factors as above, but
// the products in FP32 (high parts of the float-float rows and columns) and
// the region's sums Kahan-compensated (fs_mac): four FP32 operations per node
// and grid instead of eleven; the region keeps its (sum, compensation) pairs
// and is flushed as for float-float.
template <int NG, bool C32 = false>
__device__ __forceinline__ void spread_ff_run(const FfWin* __restrict__ recs, const int* __restrict__ toff, int ts,
                                              int ntx, int nty, const WinParams& wp, double* __restrict__ H0,
                                              double* __restrict__ H1, double* __restrict__ H2, int tile0, int tstep,
                                              unsigned char* shraw) {
    const int P1 = wp.P + 1, W = tile_region(ts, wp.P), WW = W * W;
    float4* buf = reinterpret_cast<float4*>(shraw);  // WW: (grid 0 sum, low, grid 1 sum, low)
    float4* fw = buf + WW;                            // kColChunk * P1: q0 wx, q1 wx (float-float each)
    float2* e1 = reinterpret_cast<float2*>(fw + kColChunk * P1);  // e1_len (P1e, 2 P1e with aniso)
    float2* wy = e1 + e1_len(wp.P, wp.aniso);                      // kColChunk * P1
    float2* buf2 = wy + kColChunk * P1;                            // NG == 3: WW (grid 2 sum, low)
    float2* fw2 = buf2 + (NG == 3 ? WW : 0);                       // NG == 3: kColChunk * P1 (q2 wx)
    int* org = reinterpret_cast<int*>(fw2 + (NG == 3 ? kColChunk * P1 : 0));  // kColChunk * 2 (lx, ly)
    // C32: the same arrays hold FP32 values (q0 wx, q1 wx pairs; wy; q2 wx)
    float2* fwc = reinterpret_cast<float2*>(fw);
    float* wyc = reinterpret_cast<float*>(wy);
    float* fw2c = reinterpret_cast<float*>(fw2);
    load_e1_ff(e1, wp);
    const float2* e1y = e1y_of(e1, wp);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int nw = kColWarps;
    for (int tile = tile0; tile < ntx * nty; tile += tstep) {
        const int k0 = toff[tile], k1 = toff[tile + 1];
        if (k0 == k1) continue;
        const int ox = (tile % ntx) * ts - wp.P / 2 - 2, oy = (tile / ntx) * ts - wp.P / 2 - 2;
        __syncthreads();
        for (int i = threadIdx.x; i < WW; i += blockDim.x) {
            buf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            if constexpr (NG == 3) buf2[i] = make_float2(0.f, 0.f);
        }
        for (int c0 = k0; c0 < k1; c0 += kColChunk) {
            const int cn = min(kColChunk, k1 - c0);
            __syncthreads();
            // window rows (warps 0-3) and density-weighted columns (warps
            // 4-7) of the chunk's sources, a quarter of the support per warp
            // (each quarter's recurrence starts from a power of the ratio)
            {
                const int seg = warp & 3, L = (P1 + 3) >> 2;
                const int j0 = seg * L, j1 = min(P1, j0 + L);
                if (lane < cn && j0 < j1) {
                    const FfWin& r = recs[c0 + lane];
                    if (warp < 4) {
                        const float2 e3 = r.ey3;
                        float2 ey = ff_powi(e3, j0);
                        for (int j = j0; j < j1; j++) {
                            const float2 w = ff_mul(e1y[j], ey);
                            if constexpr (C32)
                                wyc[lane * P1 + j] = w.x;
                            else
                                wy[lane * P1 + j] = w;
                            ey = ff_mul(ey, e3);
                        }
                        if (seg == 0) {
                            org[2 * lane] = r.mx - ox;
                            org[2 * lane + 1] = r.my - oy;
                        }
                    } else {
                        const float2 e3 = r.ex3, q0 = r.q[0], q1 = r.q[1], q2 = r.q[2];
                        float2 ex = j0 ? ff_mul(r.e0, ff_powi(e3, j0)) : r.e0;
                        float4* fa = fw + lane * P1;
                        for (int a = j0; a < j1; a++) {
                            const float2 wxa = ff_mul(ex, e1[a]);
                            const float2 u = ff_mul(q0, wxa), v = ff_mul(q1, wxa);
                            if constexpr (C32) {
                                fwc[lane * P1 + a] = make_float2(u.x, v.x);
                                if constexpr (NG == 3) fw2c[lane * P1 + a] = ff_mul(q2, wxa).x;
                            } else {
                                fa[a] = make_float4(u.x, u.y, v.x, v.y);
                                if constexpr (NG == 3) fw2[lane * P1 + a] = ff_mul(q2, wxa);
                            }
                            ex = ff_mul(ex, e3);
                        }
                    }
                }
            }
            __syncthreads();
            // supports of at most 16 nodes: the warp's two halves take
            // alternate owned columns of a window (row j = lane mod 16), one
            // pass per two columns instead of half the lanes idle
            const bool split = P1 <= 16;
            const int cstep = split ? 2 * nw : nw;
            // window rows in blocks of 32 (P up to 64; one block when split)
            for (int jb = 0; jb < P1; jb += 32) {
                const int j = split ? (lane & 15) : jb + lane;
                if (j >= P1) continue;
                for (int s = 0; s < cn; s++) {
                    const int2 o = *reinterpret_cast<const int2*>(org + 2 * s);
                    const int lx = o.x, ly = o.y;
                    const float2 wyj = C32 ? make_float2(wyc[s * P1 + j], 0.f) : wy[s * P1 + j];
                    const float4* fa = fw + s * P1;
                    const float2* fa2 = fw2 + s * P1;
                    const float2* fac = fwc + s * P1;
                    const float* fa2c = fw2c + s * P1;
                    // first column >= lx owned by this warp (by this half)
                    int c = lx + ((warp - lx) & (nw - 1)) + (split ? (lane >> 4) * nw : 0);
                    if (lx >= 0 && ly >= 0 && lx + wp.P < W && ly + wp.P < W) {
                        float4* b = buf + ly + j;
                        float2* b2 = buf2 + ly + j;
                        if constexpr (C32) {
                            for (; c <= lx + wp.P; c += cstep) {
                                const float2 f = fac[c - lx];
                                float4 v = b[c * W];
                                fs_mac(f.x, wyj.x, v.x, v.y);
                                fs_mac(f.y, wyj.x, v.z, v.w);
                                b[c * W] = v;
                                if constexpr (NG == 3) {
                                    float2 v2 = b2[c * W];
                                    fs_mac(fa2c[c - lx], wyj.x, v2.x, v2.y);
                                    b2[c * W] = v2;
                                }
                            }
                        } else {
                            for (; c <= lx + wp.P; c += cstep) {
                                const float4 f = fa[c - lx];
                                float4 v = b[c * W];
                                ff_mac(make_float2(f.x, f.y), wyj, v.x, v.y);
                                ff_mac(make_float2(f.z, f.w), wyj, v.z, v.w);
                                b[c * W] = v;
                                if constexpr (NG == 3) {
                                    float2 v2 = b2[c * W];
                                    ff_mac(fa2[c - lx], wyj, v2.x, v2.y);
                                    b2[c * W] = v2;
                                }
                            }
                        }
                    } else {
                        // window outside the region: straight into the global grids
                        const size_t row = fte_wrap_index(oy + ly + j, wp.My);
                        if constexpr (C32) {
                            for (; c <= lx + wp.P; c += cstep) {
                                const size_t at = (size_t)fte_wrap_index(ox + c, wp.Mx) * wp.My + row;
                                const float2 f = fac[c - lx];
                                atomicAdd(&H0[at], (double)__fmul_rn(f.x, wyj.x));
                                atomicAdd(&H1[at], (double)__fmul_rn(f.y, wyj.x));
                                if constexpr (NG == 3) atomicAdd(&H2[at], (double)__fmul_rn(fa2c[c - lx], wyj.x));
                            }
                        } else {
                            for (; c <= lx + wp.P; c += cstep) {
                                const size_t at = (size_t)fte_wrap_index(ox + c, wp.Mx) * wp.My + row;
                                const float4 f = fa[c - lx];
                                const float2 p0 = ff_mul(make_float2(f.x, f.y), wyj);
                                const float2 p1 = ff_mul(make_float2(f.z, f.w), wyj);
                                atomicAdd(&H0[at], ff_join(p0.x, p0.y));
                                atomicAdd(&H1[at], ff_join(p1.x, p1.y));
                                if constexpr (NG == 3) {
                                    const float2 p2 = ff_mul(fa2[c - lx], wyj);
                                    atomicAdd(&H2[at], ff_join(p2.x, p2.y));
                                }
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
        // flush: warp per region column, lanes along it (wrapped indices formed
        // incrementally)
        for (int xx = warp; xx < W; xx += nw) {
            const size_t col = (size_t)fte_wrap_index(ox + xx, wp.Mx) * wp.My;
            int gy = fte_wrap_index(oy + lane, wp.My);
            for (int yy = lane; yy < W; yy += 32) {
                const float4 v = buf[xx * W + yy];
                if (v.x != 0.f || v.y != 0.f) atomicAdd(&H0[col + gy], ff_join(v.x, v.y));
                if (v.z != 0.f || v.w != 0.f) atomicAdd(&H1[col + gy], ff_join(v.z, v.w));
                if constexpr (NG == 3) {
                    const float2 v2 = buf2[xx * W + yy];
                    if (v2.x != 0.f || v2.y != 0.f) atomicAdd(&H2[col + gy], ff_join(v2.x, v2.y));
                }
                gy += 32;
                while (gy >= wp.My) gy -= wp.My;
            }
        }
    }
}

template <int NG, bool C32>
__global__ void __launch_bounds__(kColThreads) k_spread_ff(const FfWin* __restrict__ recs,
                                                          const int* __restrict__ toff, int ts, int ntx, int nty,
                                                          WinParams wp, double* __restrict__ H0,
                                                          double* __restrict__ H1, double* __restrict__ H2) {
    extern __shared__ __align__(16) unsigned char shraw[];
    spread_ff_run<NG, C32>(recs, toff, ts, ntx, nty, wp, H0, H1, H2, blockIdx.x, gridDim.x, shraw);
}

size_t spread_ff_smem(int ts, int P, int ng, int aniso = 0) {
    const int P1 = P + 1, W = tile_region(ts, P);
    const size_t third = ng == 3 ? ((size_t)W * W + (size_t)kColChunk * P1) * sizeof(float2) : 0;
    return (size_t)W * W * sizeof(float4) + (size_t)kColChunk * P1 * sizeof(float4) +
           (size_t)(e1_len(P, aniso) + kColChunk * P1) * sizeof(float2) + third + kColChunk * 2 * sizeof(int);
}

// FP64 grid values -> float-float pairs, in place
__global__ void k_ff_split(double* __restrict__ H, int64_t n) {
    float2* o = reinterpret_cast<float2*>(H);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = H[i];
        o[i] = ff_split(v);
    }
}

// float-float pairs -> FP64 grid values, in place
__global__ void k_ff_join(double* __restrict__ H, int64_t n) {
    const float2* o = reinterpret_cast<const float2*>(H);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = o[i];
        H[i] = ff_join(v);
    }
}

// Tiled gather in float-float from grids of pairs: a thread per target, the
// tile's region of both grids staged once in shared memory.  PM > 0: window
// supports of at most PM nodes, the target's window column held in registers
// and the node loops unrolled to PM (independent products in flight, no
// shared-memory traffic for the weights); PM == 0: any support, the window
// column in a per-thread shared-memory row.  C32 (FTE_FORM_FF32, loose
// tolerances): the region holds the grids' high parts only (FP32), each
// window column is summed with FP32 FMAs and the column sums are added with
// Kahan's compensation (fs_mac); the window factors are the float-float ones.
template <int PM, bool C32 = false>
__device__ __forceinline__ void gather_ff_run(const double* __restrict__ p, const int* __restrict__ toff,
                                              const int* __restrict__ perm, int ts, int ntx, int nty,
                                              const WinParams& wp, const float2* __restrict__ G0,
                                              const float2* __restrict__ G1, double scale, double2* __restrict__ out,
                                              int tile0, int tstep, unsigned char* shraw, float2* etab) {
    float2* shf = reinterpret_cast<float2*>(shraw);
    const int P1 = wp.P + 1, W = tile_region(ts, wp.P), WW = W * W;
    float2* r0 = shf;
    float2* r1 = r0 + WW;
    float2* e1 = C32 ? shf + WW : r1 + WW;  // C32: one pair region (below)
    float2* wyb = e1 + e1_len(wp.P, wp.aniso) + threadIdx.x * P1;  // PM == 0 only
    // C32: the grids' high parts interleaved per node (one 8-byte read gives
    // both grids' values; the tile bins' order of the targets keeps a half
    // warp's rows on distinct banks for 8-byte values) and FP32 window rows
    float2* rc = shf;
    float* wybf = reinterpret_cast<float*>(e1 + e1_len(wp.P, wp.aniso)) + threadIdx.x * P1;
    load_etab(etab);  // 2^(-j/64) for the window factors (as in k_ff_win)
    load_e1_ff(e1, wp);
    const float2* e1y = e1y_of(e1, wp);
    const double tw = -2 * wp.xi * wp.xi / wp.eta;
    constexpr int NW = PM > 0 ? PM : 1;
    for (int tile = tile0; tile < ntx * nty; tile += tstep) {
        const int k0 = toff[tile], k1 = toff[tile + 1];
        if (k0 == k1) continue;
        const int ox = (tile % ntx) * ts - wp.P / 2 - 2, oy = (tile / ntx) * ts - wp.P / 2 - 2;
        __syncthreads();
        for (int idx = threadIdx.x; idx < WW; idx += blockDim.x) {
            int xx = idx / W, yy = idx - xx * W;
            size_t at = (size_t)fte_wrap_index(ox + xx, wp.Mx) * wp.My + fte_wrap_index(oy + yy, wp.My);
            if constexpr (C32) {
                rc[idx] = make_float2(G0[at].x, G1[at].x);
            } else {
                r0[idx] = G0[at];
                r1[idx] = G1[at];
            }
        }
        __syncthreads();
        for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
            const int i = perm[k];
            int mx, my;
            double px, py;
            fte_closest_node(p[2 * i], p[2 * i + 1], wp.Lx, wp.Ly, wp.h, wp.rh, wp.hy, wp.rhy, wp.P, &mx, &my, &px,
                             &py);
            float2 wy[C32 ? 1 : NW];
            float wyf[C32 ? NW : 1];
            {
                const float2 e3 = fte_expm_ff(ff_split(2 * tw * wp.hy * py), etab);
                float2 ey = make_float2(1.f, 0.f);
                if constexpr (PM > 0) {
#pragma unroll
                    for (int j = 0; j < PM; j++) {
                        const float2 w = j < P1 ? ff_mul(e1y[j], ey) : make_float2(0.f, 0.f);
                        if constexpr (C32)
                            wyf[j] = w.x;
                        else
                            wy[j] = w;
                        ey = ff_mul(ey, e3);
                    }
                } else {
                    for (int j = 0; j < P1; j++) {
                        const float2 w = ff_mul(e1y[j], ey);
                        if constexpr (C32)
                            wybf[j] = w.x;
                        else
                            wyb[j] = w;
                        ey = ff_mul(ey, e3);
                    }
                }
            }
            const float2 e3x = fte_expm_ff(ff_split(2 * tw * wp.h * px), etab);
            float2 ex = fte_expm_ff(ff_split(-tw * e0_arg(px, py, wp)), etab);
            const int lx = mx - ox, ly = my - oy;
            float a0 = 0.f, c0 = 0.f, a1 = 0.f, c1 = 0.f;
            const bool inside = lx >= 0 && ly >= 0 && lx + wp.P < W && ly + wp.P < W;
            for (int a = 0; a < P1; a++) {
                const float2 wxa = ff_mul(ex, e1[a]);
                ex = ff_mul(ex, e3x);
                if constexpr (C32) {
                    float s0 = 0.f, s1 = 0.f;
                    if (inside) {
                        const float2* g = rc + (lx + a) * W + ly;
                        if constexpr (PM > 0) {
#pragma unroll
                            for (int j = 0; j < PM; j++) {
                                if (j < P1) {
                                    const float2 v = g[j];
                                    s0 = __fmaf_rn(wyf[j], v.x, s0);
                                    s1 = __fmaf_rn(wyf[j], v.y, s1);
                                }
                            }
                        } else {
                            for (int j = 0; j < P1; j++) {
                                const float w = wybf[j];
                                const float2 v = g[j];
                                s0 = __fmaf_rn(w, v.x, s0);
                                s1 = __fmaf_rn(w, v.y, s1);
                            }
                        }
                    } else {
                        const size_t base = (size_t)fte_wrap_index(mx + a, wp.Mx) * wp.My;
                        if constexpr (PM > 0) {
#pragma unroll
                            for (int j = 0; j < PM; j++) {
                                if (j < P1) {
                                    const size_t at = base + fte_wrap_index(my + j, wp.My);
                                    s0 = __fmaf_rn(wyf[j], G0[at].x, s0);
                                    s1 = __fmaf_rn(wyf[j], G1[at].x, s1);
                                }
                            }
                        } else {
                            for (int j = 0; j < P1; j++) {
                                const size_t at = base + fte_wrap_index(my + j, wp.My);
                                const float w = wybf[j];
                                s0 = __fmaf_rn(w, G0[at].x, s0);
                                s1 = __fmaf_rn(w, G1[at].x, s1);
                            }
                        }
                    }
                    fs_mac(wxa.x, s0, a0, c0);
                    fs_mac(wxa.x, s1, a1, c1);
                } else {
                    float s0 = 0.f, t0 = 0.f, s1 = 0.f, t1 = 0.f;
                    if (inside) {
                        const float2* g0 = r0 + (lx + a) * W + ly;
                        const float2* g1 = r1 + (lx + a) * W + ly;
                        if constexpr (PM > 0) {
#pragma unroll
                            for (int j = 0; j < PM; j++) {
                                if (j < P1) {
                                    ff_mac(wy[j], g0[j], s0, t0);
                                    ff_mac(wy[j], g1[j], s1, t1);
                                }
                            }
                        } else {
                            for (int j = 0; j < P1; j++) {
                                const float2 w = wyb[j];
                                ff_mac(w, g0[j], s0, t0);
                                ff_mac(w, g1[j], s1, t1);
                            }
                        }
                    } else {
                        const size_t base = (size_t)fte_wrap_index(mx + a, wp.Mx) * wp.My;
                        if constexpr (PM > 0) {
#pragma unroll
                            for (int j = 0; j < PM; j++) {
                                if (j < P1) {
                                    const size_t at = base + fte_wrap_index(my + j, wp.My);
                                    ff_mac(wy[j], G0[at], s0, t0);
                                    ff_mac(wy[j], G1[at], s1, t1);
                                }
                            }
                        } else {
                            for (int j = 0; j < P1; j++) {
                                const size_t at = base + fte_wrap_index(my + j, wp.My);
                                const float2 w = wyb[j];
                                ff_mac(w, G0[at], s0, t0);
                                ff_mac(w, G1[at], s1, t1);
                            }
                        }
                    }
                    ff_mac(wxa, ff_norm(s0, t0), a0, c0);
                    ff_mac(wxa, ff_norm(s1, t1), a1, c1);
                }
            }
            out[i] = make_double2(ff_join(a0, c0) * scale, ff_join(a1, c1) * scale);
        }
    }
}

template <int PM, bool C32>
__global__ void __launch_bounds__(kTileThreads, C32 ? 8 : 5) k_gather_ff(const double* __restrict__ p, const int* __restrict__ toff,
                                                           const int* __restrict__ perm, int ts, int ntx, int nty,
                                                           WinParams wp, const float2* __restrict__ G0,
                                                           const float2* __restrict__ G1, double scale,
                                                           double2* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char shraw[];
    __shared__ float2 etab[64];
    gather_ff_run<PM, C32>(p, toff, perm, ts, ntx, nty, wp, G0, G1, scale, out, blockIdx.x, gridDim.x, shraw, etab);
}

// the register form's support bound for window support P1 (0: none fits)
// (the supports P1 = 17 .. 25 have their own instance: the unrolled loops
// carry no products beyond the support; 1e6 points, stresslet gather at tol
// 1e-10 / 1e-8: 0.905 -> 0.883 / 0.696 -> 0.666 ms; at P1 = 15 the instance
// for 16 was as fast)
__host__ __device__ inline int gather_ff_pm(int P1) {
    if (P1 >= 17 && P1 <= 25 && (P1 & 1)) return P1;
    return P1 <= 16 ? 16 : (P1 <= 24 ? 24 : (P1 <= 32 ? 32 : 0));
}
// the register form's instances, in the order of the batches' work lists
constexpr int kGatherPms[] = {16, 17, 19, 21, 23, 24, 25, 32};
constexpr int kGatherPmClasses = sizeof(kGatherPms) / sizeof(kGatherPms[0]);
inline int gather_pm_class(int PM) {
    for (int i = 0; i < kGatherPmClasses; i++)
        if (kGatherPms[i] == PM) return i;
    return -1;
}

// c32: the FP32-product gather's region holds one (grid 0, grid 1) pair of
// high parts per node and its window rows are FP32
size_t gather_ff_smem(int ts, int P, int aniso = 0, bool c32 = false) {
    const int P1 = P + 1, W = tile_region(ts, P);
    const size_t rows = gather_ff_pm(P1) ? 0 : (size_t)kTileThreads * P1;  // per-thread window columns
    if (c32)
        return (size_t)W * W * sizeof(float2) + (size_t)e1_len(P, aniso) * sizeof(float2) + rows * sizeof(float);
    return 2 * (size_t)W * W * sizeof(float2) + (size_t)(e1_len(P, aniso) + rows) * sizeof(float2);
}

// ---- tile sizes -------------------------------------------------------------
// Spread and gather tiles are ts x ts grid nodes (ts >= 8); a tile's shared-
// memory region (ts + P + 4 nodes a side) must fit the two-CTAs-per-SM budget.
// The default is the largest fitting multiple of 4 up to 64; a plan may carry
// a tuned size instead (fte_kspace_tune).
size_t gather64_smem(int ts, int P, int aniso = 0) {
    const int P1 = P + 1, W = tile_region(ts, P);
    return 2 * (size_t)W * W * sizeof(double) + (size_t)(e1_len(P, aniso) + kPtThreads * P1) * sizeof(double);
}
// do the axes' grid steps differ (beyond rounding)?
int kspace_aniso(double Lx, int Mx, double Ly, int My) {
    const double hx = Lx / Mx, hy = Ly / My;
    return std::fabs(hx - hy) > 1e-12 * std::fmax(hx, hy) ? 1 : 0;
}
int kspace_aniso(const KspaceArgs& a) { return kspace_aniso(a.Lx, a.Mx, a.Ly, a.My); }
bool spread_fits(const fte_context* ctx, int form, int kind, int ts, int P, int aniso = 0) {
    if (ts < 8 || ts > 256) return false;
    size_t sm = form == FTE_FORM_MIXED ? spread_cols32_smem(ts, P)
                : (fte_form_ff(form) ? spread_ff_smem(ts, P, kind == FTE_KIND_SLP ? 2 : 3, aniso)
                                       : spread_cols_smem(ts, P, aniso));
    return sm <= tile_budget(ctx);
}
bool gather_fits(const fte_context* ctx, int form, int ts, int P, int aniso = 0) {
    if (ts < 8 || ts > 256) return false;
    size_t sm = form == FTE_FORM_MIXED ? gather32_smem(ts, P)
                : (fte_form_ff(form) ? gather_ff_smem(ts, P, aniso, form == FTE_FORM_FF32)
                                       : gather64_smem(ts, P, aniso));
    return sm <= tile_budget(ctx);
}
int resolve_tiles(const fte_context* ctx, const KspaceArgs& a, int* ts_s, int* ts_g, bool fill = true) {
    *ts_s = 0;
    *ts_g = 0;
    const int an = kspace_aniso(a);
    if (a.ts_spread > 0) {
        if (!spread_fits(ctx, a.form, a.kind, a.ts_spread, a.P, an)) {
            fte_set_error("spread tile %d does not fit shared memory at P=%d", a.ts_spread, a.P);
            return FTE_ERR_INVALID;
        }
        *ts_s = a.ts_spread;
    } else {
        // float-float: three CTAs per SM where that still leaves tiles of at
        // least 28 nodes a side (else the halo flushes cost more than the
        // occupancy gains: measured at 1e6 points, P 14..22)
        // FP32 products (four operations per node instead of eleven): four
        // CTAs per SM, tiles down to 16 nodes (1e6 points, tol 1e-6: the
        // tuner's picks, 32 / 16 nodes for the two / three grids, were 2 %
        // faster than the three-CTA tiles)
        if (fte_form_ff(a.form)) {
            const int ngf = a.kind == FTE_KIND_SLP ? 2 : 3;
            const bool c32 = a.form == FTE_FORM_FF32;
            const size_t cap = c32 ? tile_budget(ctx) / 2 : tile_budget(ctx) * 2 / 3;
            for (int ts = 64; ts >= (c32 ? 16 : 28) && !*ts_s; ts -= 4)
                if (spread_ff_smem(ts, a.P, ngf, an) <= cap) *ts_s = ts;
        }
        for (int ts = 64; ts >= 8 && !*ts_s; ts -= 4)
            if (spread_fits(ctx, a.form, a.kind, ts, a.P, an)) *ts_s = ts;
    }
    if (a.ts_gather > 0) {
        if (!gather_fits(ctx, a.form, a.ts_gather, a.P, an)) {
            fte_set_error("gather tile %d does not fit shared memory at P=%d", a.ts_gather, a.P);
            return FTE_ERR_INVALID;
        }
        *ts_g = a.ts_gather;
    } else if (fte_form_ff(a.form) && gather_ff_pm(a.P + 1)) {
        // register form: tiles small enough for four CTAs per SM (more warps
        // to hide the products' latency; the region re-reads cost little),
        // at most 28 nodes a side (fewer idle threads in a tile's last round
        // of targets; 28 was the fastest of 24..48 at 1e6 points)
        // (FP32 products: up to 32 nodes, the tuner's pick at tol 1e-6, and
        // a half-size region: eight CTAs per SM, registers capped at 64)
        const bool c32 = a.form == FTE_FORM_FF32;
        for (int ts = c32 ? 32 : 28; ts >= 8 && !*ts_g; ts -= 4)
            if (gather_ff_smem(ts, a.P, an, c32) <= tile_budget(ctx) / (c32 ? 4 : 2)) *ts_g = ts;
        if (!*ts_g) *ts_g = 8;
    } else {
        for (int ts = 64; ts >= 8 && !*ts_g; ts -= 4)
            if (gather_fits(ctx, a.form, ts, a.P, an)) *ts_g = ts;
    }
    // Small grids: a tile is one CTA, so that a grid of a few tiles leaves
    // most SMs idle while each CTA walks its tile's points alone (48 x 108
    // nodes at tile 64: two CTAs).  Default sizes shrink (by 4, not below 8)
    // until the grid has two tiles per SM; the halo a smaller tile adds is
    // small in absolute terms on such grids.
    if (!fill) return FTE_OK;
    auto tiles = [&](int ts) { return (int64_t)((a.Mx + ts - 1) / ts) * ((a.My + ts - 1) / ts); };
    const int64_t want = 2 * (int64_t)(ctx->num_sms > 0 ? ctx->num_sms : 1);
    if (a.ts_spread <= 0)
        while (*ts_s > 8 && tiles(*ts_s) < want) *ts_s -= 4;
    if (a.ts_gather <= 0)
        while (*ts_g > 8 && tiles(*ts_g) < want) *ts_g -= 4;
    return FTE_OK;
}

// Window parameters of an evaluation.  With equal steps (the reference's
// case) the y axis takes the x axis's values, so that every result is the
// reference's; otherwise hy = Ly / My and the y support keeps the x axis's
// ratio w / h (w = P h / 2 when the chooser set it).
WinParams win_params(const KspaceArgs& a) {
    WinParams wp;
    wp.Lx = a.Lx;
    wp.Ly = a.Ly;
    wp.h = a.Lx / a.Mx;
    wp.rh = 1.0 / wp.h;
    wp.xi = a.xi;
    wp.eta = a.eta;
    wp.w = a.w;
    wp.P = a.P;
    wp.Mx = a.Mx;
    wp.My = a.My;
    wp.aniso = kspace_aniso(a);
    if (wp.aniso) {
        wp.hy = a.Ly / a.My;
        wp.rhy = 1.0 / wp.hy;
        wp.wy = a.w * (wp.hy / wp.h);
    } else {
        wp.hy = wp.h;
        wp.rhy = wp.rh;
        wp.wy = wp.w;
    }
    return wp;
}

// tiled spread of all source grids (H holds ng grids of G nodes, FP64 or
// FP32); the float-float form first writes the sources' window records to
// recs (nsrc entries)
int launch_spread_tiled(fte_context* ctx, const KspaceArgs& a, const TileBins& tb, const WinParams& wp, void* H,
                        FfWin* recs) {
    const int ng = a.kind == FTE_KIND_SLP ? 2 : 4;
    const size_t G = (size_t)a.Mx * a.My;
    const bool f32 = a.form == FTE_FORM_MIXED;
    const size_t sm = f32 ? spread_cols32_smem(tb.ts, a.P) : spread_cols_smem(tb.ts, a.P, wp.aniso);
    const int nt = tb.ntx * tb.nty;
    const int grid = nt < ctx->num_sms * 8 ? nt : ctx->num_sms * 8;
    if (fte_form_ff(a.form)) {
        if (!recs) {
            fte_set_error("internal: float-float spread without window records");
            return FTE_ERR_INVALID;
        }
        // one pass over the sources: the Stokeslet's two grids or the
        // stresslet's three symmetric ones
        double* Hd = static_cast<double*>(H);
        const int ngf = a.kind == FTE_KIND_SLP ? 2 : 3;
        const size_t smf = spread_ff_smem(tb.ts, a.P, ngf, wp.aniso);
        FTE_LAUNCH(ctx, k_ff_win, ew_grid(ctx, a.nsrc), 256, 0, a.kind, a.psrc, a.f, a.nrm, a.wts, (const int*)tb.perm,
                   a.nsrc, wp, recs);
        auto go = [&](auto kern) -> int {
            FTE_CUDA_TRY(fte_smem_ceiling(kern, (int)smf));
            FTE_LAUNCH(ctx, kern, grid, kColThreads, smf, (const FfWin*)recs, (const int*)tb.off, tb.ts, tb.ntx,
                       tb.nty, wp, Hd, Hd + G, ngf == 3 ? Hd + 2 * G : nullptr);
            return FTE_OK;
        };
        if (a.form == FTE_FORM_FF32)
            FTE_TRY(ngf == 2 ? go(k_spread_ff<2, true>) : go(k_spread_ff<3, true>));
        else
            FTE_TRY(ngf == 2 ? go(k_spread_ff<2, false>) : go(k_spread_ff<3, false>));
    } else if (f32) {
        float* Hf = static_cast<float*>(H);
        FTE_CUDA_TRY(fte_smem_ceiling(k_spread_cols32, (int)sm));
        for (int pass = 0; pass < ng / 2; pass++) {
            int mode = ng == 2 ? 0 : 1 + pass;
            FTE_LAUNCH(ctx, k_spread_cols32, grid, kColThreads, sm, mode, a.psrc, a.f, a.nrm, a.wts,
                       (const int*)tb.off, (const int*)tb.perm, tb.ts, tb.ntx, tb.nty, wp, Hf + 2 * pass * G,
                       Hf + (2 * pass + 1) * G);
        }
    } else {
        double* Hd = static_cast<double*>(H);
        FTE_CUDA_TRY(fte_smem_ceiling(k_spread_cols, (int)sm));
        for (int pass = 0; pass < ng / 2; pass++) {
            int mode = ng == 2 ? 0 : 1 + pass;
            FTE_LAUNCH(ctx, k_spread_cols, grid, kColThreads, sm, mode, a.psrc, a.f, a.nrm, a.wts,
                       (const int*)tb.off, (const int*)tb.perm, tb.ts, tb.ntx, tb.nty, wp, Hd + 2 * pass * G,
                       Hd + (2 * pass + 1) * G);
        }
    }
    return FTE_OK;
}

// tiled gather of the two velocity grids at the targets (the float-float
// form reads grids already split into pairs)
int launch_gather_tiled(fte_context* ctx, const KspaceArgs& a, const TileBins& tb, const WinParams& wp,
                        const void* H, double scale) {
    const size_t G = (size_t)a.Mx * a.My;
    const int nt = tb.ntx * tb.nty;
    const int grid = nt < ctx->num_sms * 8 ? nt : ctx->num_sms * 8;
    if (fte_form_ff(a.form)) {
        const float2* Hf = static_cast<const float2*>(H);
        size_t sm = gather_ff_smem(tb.ts, a.P, wp.aniso, a.form == FTE_FORM_FF32);
        auto go = [&](auto kern) -> int {
            FTE_CUDA_TRY(fte_smem_ceiling(kern, (int)sm));
            FTE_LAUNCH(ctx, kern, grid, kTileThreads, sm, a.ptar, (const int*)tb.off, (const int*)tb.perm, tb.ts,
                       tb.ntx, tb.nty, wp, Hf, Hf + G, scale, a.uk);
            return FTE_OK;
        };
        if (a.form == FTE_FORM_FF32) {
            // FP32 products: the instances for 16, 24 and 32 nodes (the
            // form is confined to P <= 30)
            const int pm = gather_ff_pm(a.P + 1);
            if (pm == 0) {
                fte_set_error("internal: FP32-product gather with a support of %d nodes", a.P + 1);
                return FTE_ERR_INVALID;
            } else if (pm <= 16)
                FTE_TRY(go(k_gather_ff<16, true>));
            else if (pm <= 24)
                FTE_TRY(go(k_gather_ff<24, true>));
            else
                FTE_TRY(go(k_gather_ff<32, true>));
        } else {
            switch (gather_ff_pm(a.P + 1)) {
                case 16: FTE_TRY(go(k_gather_ff<16, false>)); break;
                case 17: FTE_TRY(go(k_gather_ff<17, false>)); break;
                case 19: FTE_TRY(go(k_gather_ff<19, false>)); break;
                case 21: FTE_TRY(go(k_gather_ff<21, false>)); break;
                case 23: FTE_TRY(go(k_gather_ff<23, false>)); break;
                case 24: FTE_TRY(go(k_gather_ff<24, false>)); break;
                case 25: FTE_TRY(go(k_gather_ff<25, false>)); break;
                case 32: FTE_TRY(go(k_gather_ff<32, false>)); break;
                default: FTE_TRY(go(k_gather_ff<0, false>)); break;
            }
        }
    } else if (a.form == FTE_FORM_MIXED) {
        const float* Hf = static_cast<const float*>(H);
        size_t sm = gather32_smem(tb.ts, a.P);
        FTE_CUDA_TRY(fte_smem_ceiling(k_gather_tiled32, (int)sm));
        FTE_LAUNCH(ctx, k_gather_tiled32, grid, kTileThreads, sm, a.ptar, (const int*)tb.off, (const int*)tb.perm,
                   tb.ts, tb.ntx, tb.nty, wp, Hf, Hf + G, scale, a.uk);
    } else {
        const double* Hd = static_cast<const double*>(H);
        size_t sm = gather64_smem(tb.ts, a.P, wp.aniso);
        FTE_CUDA_TRY(fte_smem_ceiling(k_gather_tiled, (int)sm));
        FTE_LAUNCH(ctx, k_gather_tiled, grid, kTileThreads, sm, a.ptar, (const int*)tb.off, (const int*)tb.perm,
                   tb.ts, tb.ntx, tb.nty, wp, Hd, Hd + G, scale, a.uk);
    }
    return FTE_OK;
}

// (4 xi^2/eta)^2 hx hy / pi / (4 pi) / (Mx My): the reference's
// (4 xi^2/eta)^2 h^2 / pi scale (ewald_tools.cpp:267-269) with the cell area
// hx hy of the grid, and the inverse transform's normalisation
double gather_scale(const KspaceArgs& a) {
    const WinParams wp = win_params(a);
    double s = 4 * a.xi * a.xi / a.eta;
    s = s * s * wp.h * wp.hy / FTE_PI;
    return s / (4 * FTE_PI) / ((double)a.Mx * (double)a.My);
}

int kspace_run_mixed(fte_context* ctx, WsCarver& wc, const KspaceArgs& a) {
    const int ng = a.kind == FTE_KIND_SLP ? 2 : 4;
    const int Mx = a.Mx, My = a.My;
    const size_t G = (size_t)Mx * My;
    const int Kh = My / 2 + 1;
    float* H = wc.take<float>(ng * G);
    float2* Hh = wc.take<float2>(ng * (size_t)Mx * Kh);
    FTE_WS_CHECK(wc);
    const WinParams wp = win_params(a);
    FftDev py, px;
    FTE_TRY(fte_get_plan(ctx, My, &py));
    FTE_TRY(fte_get_plan(ctx, Mx, &px));
    size_t sm_y = 2 * (size_t)py.m * sizeof(float2), sm_x = 2 * (size_t)px.m * sizeof(float2);
    if (sm_y > (size_t)ctx->max_smem_optin || sm_x > (size_t)ctx->max_smem_optin) {
        fte_set_error("grid %d x %d beyond this build's shared-memory transform", Mx, My);
        return FTE_ERR_UNSUPPORTED;
    }
    int ts_s = 0, ts_g = 0;
    FTE_TRY(resolve_tiles(ctx, a, &ts_s, &ts_g));
    if (!ts_s || !ts_g) {
        fte_set_error("window support P=%d too large for the mixed form's tiles", a.P);
        return FTE_ERR_UNSUPPORTED;
    }
    TileBins tb_s, tb_g;
    if (a.pre_src && a.nsrc > 0)
        tb_s = *a.pre_src;
    else if (a.nsrc > 0)
        FTE_TRY(fte_tiles_build(ctx, wc, a.psrc, a.nsrc, a.Lx, a.Ly, wp.h, wp.hy, ts_s, (Mx + ts_s - 1) / ts_s,
                                (My + ts_s - 1) / ts_s, &tb_s));
    if (a.pre_tar && a.ntar > 0)
        tb_g = *a.pre_tar;
    else if (a.ntar > 0)
        FTE_TRY(fte_tiles_build(ctx, wc, a.ptar, a.ntar, a.Lx, a.Ly, wp.h, wp.hy, ts_g, (Mx + ts_g - 1) / ts_g,
                                (My + ts_g - 1) / ts_g, &tb_g, tile_region(ts_g, a.P)));
    if ((a.nsrc > 0 && tb_s.ts != ts_s) || (a.ntar > 0 && tb_g.ts != ts_g)) {
        fte_set_error("internal: prebuilt tiles do not match the mixed-form tile sizes");
        return FTE_ERR_INVALID;
    }
    FTE_TRY(fte_record(ctx, 2));
    FTE_CUDA_TRY(cudaMemsetAsync(H, 0, sizeof(float) * ng * G, ctx->stream));
    if (a.nsrc > 0) FTE_TRY(launch_spread_tiled(ctx, a, tb_s, wp, H, nullptr));
    FTE_TRY(fte_record(ctx, 3));
    FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_r2c32, (int)sm_y));
    FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_c2r32, (int)sm_y));
    FTE_CUDA_TRY(fte_smem_ceiling(k_fft_x32, (int)sm_x));
    FTE_LAUNCH(ctx, k_fft_y_r2c32, dim3(Mx / 2, ng), fft_threads(py.m), sm_y, (const float*)H, Hh, Mx, My, py);
    FTE_LAUNCH(ctx, k_fft_x32, dim3(Kh, ng), fft_threads(px.m), sm_x, Hh, Mx, Kh, px, 0);
    int fb = (int)(((size_t)Mx * Kh + 255) / 256);
    if (fb > ctx->num_sms * 32) fb = ctx->num_sms * 32;
    if (a.kind == FTE_KIND_SLP)
        FTE_LAUNCH(ctx, k_filter32<FTE_KIND_SLP>, fb, 256, 0, Hh, Mx, My, a.Lx, a.Ly, a.xi, a.eta);
    else
        FTE_LAUNCH(ctx, k_filter32<FTE_KIND_DLP>, fb, 256, 0, Hh, Mx, My, a.Lx, a.Ly, a.xi, a.eta);
    FTE_LAUNCH(ctx, k_fft_x32, dim3(Kh, 2), fft_threads(px.m), sm_x, Hh, Mx, Kh, px, 1);
    FTE_LAUNCH(ctx, k_fft_y_c2r32, dim3(Mx / 2, 2), fft_threads(py.m), sm_y, (const float2*)Hh, H, Mx, My, py);
    FTE_TRY(fte_record(ctx, 4));
    if (a.ntar > 0) FTE_TRY(launch_gather_tiled(ctx, a, tb_g, wp, H, gather_scale(a)));
    FTE_TRY(fte_record(ctx, 5));
    return FTE_OK;
}
}  // namespace

int fte_kspace_batch_tiles(const fte_context* ctx, const KspaceArgs& a, int* ts_s, int* ts_g) {
    KspaceArgs d = a;
    d.ts_spread = d.ts_gather = 0;
    return resolve_tiles(ctx, d, ts_s, ts_g, false);
}

int fte_kspace_tiles(fte_context* ctx, WsCarver& wc, const KspaceArgs& a, TileBins* src, TileBins* tar) {
    int ts_s = 0, ts_g = 0;
    FTE_TRY(resolve_tiles(ctx, a, &ts_s, &ts_g));
    src->ts = tar->ts = 0;
    src->ntx = tar->ntx = 0;
    const WinParams wp = win_params(a);
    if (ts_s > 0 && a.nsrc > 0)
        FTE_TRY(fte_tiles_build(ctx, wc, a.psrc, a.nsrc, a.Lx, a.Ly, wp.h, wp.hy, ts_s, (a.Mx + ts_s - 1) / ts_s,
                                (a.My + ts_s - 1) / ts_s, src));
    if (ts_g > 0 && a.ntar > 0)
        FTE_TRY(fte_tiles_build(ctx, wc, a.ptar, a.ntar, a.Lx, a.Ly, wp.h, wp.hy, ts_g, (a.Mx + ts_g - 1) / ts_g,
                                (a.My + ts_g - 1) / ts_g, tar, tile_region(ts_g, a.P)));
    return FTE_OK;
}

// Autotuner of the spread and gather tiles.  Small tiles give more CTAs (a
// 256 x 256 grid has only 16 tiles of 64 x 64 for 152 SMs) but re-read more
// halo nodes per grid node; the best size depends on the grid, the window
// support and how the points cluster, so it is measured: every candidate size
// that fits shared memory is timed (bins built, one warm-up, then the median
// of three launches, CUDA events on the context's stream) on the plan's own
// points and densities.  `grid` holds the plan's grids (ng grids of Mx*My
// nodes, FP64 or FP32 by form) and `bins` scratch for one candidate's tile
// bins; a.uk receives junk velocities.
int fte_kspace_tune(fte_context* ctx, void* grid, WsCarver bins, KspaceArgs& a, float* ms_spread,
                    float* ms_gather) {
    static const int cand[] = {8, 12, 16, 20, 24, 32, 40, 48, 56, 64};
    const WinParams wp = win_params(a);
    const int ng = a.kind == FTE_KIND_SLP ? 2 : 4;
    const size_t gbytes = (size_t)ng * a.Mx * a.My * (a.form == FTE_FORM_MIXED ? sizeof(float) : sizeof(double));
    cudaEvent_t e[4];
    for (int i = 0; i < 4; i++) FTE_CUDA_TRY(cudaEventCreate(&e[i]));
    auto time3 = [&](auto&& launch, float* out) -> int {
        FTE_TRY(launch());  // warm-up
        float t[3];
        for (int r = 0; r < 3; r++) {
            FTE_CUDA_TRY(cudaEventRecord(e[0], ctx->stream));
            FTE_TRY(launch());
            FTE_CUDA_TRY(cudaEventRecord(e[1], ctx->stream));
            FTE_CUDA_TRY(cudaEventSynchronize(e[1]));
            FTE_CUDA_TRY(cudaEventElapsedTime(&t[r], e[0], e[1]));
        }
        float lo = fminf(t[0], fminf(t[1], t[2])), hi = fmaxf(t[0], fmaxf(t[1], t[2]));
        *out = t[0] + t[1] + t[2] - lo - hi;
        return FTE_OK;
    };
    int rc = FTE_OK;
    float best_s = 1e30f, best_g = 1e30f;
    int ts_s = 0, ts_g = 0;
    for (int ts : cand) {
        if (rc || a.nsrc == 0 || !spread_fits(ctx, a.form, a.kind, ts, a.P, kspace_aniso(a))) continue;
        WsCarver w = bins;
        TileBins tb;
        rc = fte_tiles_build(ctx, w, a.psrc, a.nsrc, a.Lx, a.Ly, wp.h, wp.hy, ts, (a.Mx + ts - 1) / ts,
                             (a.My + ts - 1) / ts, &tb);
        FfWin* recs = fte_form_ff(a.form) ? w.take<FfWin>(a.nsrc) : nullptr;
        if (!rc && !w.ok()) {
            fte_set_error("internal: tuner bin scratch too small");
            rc = FTE_ERR_ALLOC;
        }
        float ms = 0;
        if (!rc)
            rc = time3(
                [&]() -> int {
                    FTE_CUDA_TRY(cudaMemsetAsync(grid, 0, gbytes, ctx->stream));
                    return launch_spread_tiled(ctx, a, tb, wp, grid, recs);
                },
                &ms);
        if (!rc && ms < best_s) {
            best_s = ms;
            ts_s = ts;
        }
    }
    const double scale = gather_scale(a);
    for (int ts : cand) {
        if (rc || a.ntar == 0 || !gather_fits(ctx, a.form, ts, a.P, kspace_aniso(a))) continue;
        WsCarver w = bins;
        TileBins tb;
        rc = fte_tiles_build(ctx, w, a.ptar, a.ntar, a.Lx, a.Ly, wp.h, wp.hy, ts, (a.Mx + ts - 1) / ts,
                             (a.My + ts - 1) / ts, &tb, tile_region(ts, a.P));
        if (!rc && !w.ok()) {
            fte_set_error("internal: tuner bin scratch too small");
            rc = FTE_ERR_ALLOC;
        }
        float ms = 0;
        if (!rc) rc = time3([&]() -> int { return launch_gather_tiled(ctx, a, tb, wp, grid, scale); }, &ms);
        if (!rc && ms < best_g) {
            best_g = ms;
            ts_g = ts;
        }
    }
    for (int i = 0; i < 4; i++) cudaEventDestroy(e[i]);
    if (rc) return rc;
    a.ts_spread = ts_s;
    a.ts_gather = ts_g;
    if (ms_spread) *ms_spread = ts_s ? best_s : 0.f;
    if (ms_gather) *ms_gather = ts_g ? best_g : 0.f;
    return FTE_OK;
}

size_t fte_kspace_rec_ws(int form, int64_t nsrc) {
    return fte_form_ff(form) ? ws_bytes((size_t)nsrc + 1, sizeof(FfWin)) : 0;
}

size_t fte_kspace_ws(int kind, int form, int Mx, int My, int64_t nsrc, int64_t ntar) {
    int ng = kind == FTE_KIND_SLP ? 2 : 4;
    size_t G = (size_t)Mx * My;
    size_t Gh = (size_t)Mx * (My / 2 + 1);
    // tiles no smaller than 8 nodes
    int ntiles = ((Mx + 7) / 8) * ((My + 7) / 8);
    size_t s = ws_bytes(ng * G, sizeof(double)) + ws_bytes(ng * Gh, sizeof(double2)) + fte_tiles_ws(nsrc, ntiles) +
               fte_tiles_ws(ntar, ntiles) + fte_kspace_rec_ws(form, nsrc) + 4096;
    if (form != FTE_FORM_MIXED) {
        // long FP64 transforms: staging lines along y and the four-step scratch
        const bool ly = !fte_fft_fits_block(My, sizeof(double2)), lx = !fte_fft_fits_block(Mx, sizeof(double2));
        if (ly) s += ws_bytes((size_t)ng * (Mx / 2) * My, sizeof(double2));
        size_t a = ly ? fte_long_scratch(My, (long long)ng * (Mx / 2)) : 0;
        size_t b = lx ? fte_long_scratch(Mx, (long long)ng * (My / 2 + 1)) : 0;
        if (a || b) s += ws_bytes(a > b ? a : b, sizeof(double2));
    }
    return s;
}

int fte_kspace_run(fte_context* ctx, WsCarver& wc, const KspaceArgs& a, fte_info* info) {
    if (a.form == FTE_FORM_MIXED) return kspace_run_mixed(ctx, wc, a);
    const int ng = a.kind == FTE_KIND_SLP ? 2 : 4;
    const int Mx = a.Mx, My = a.My;
    const size_t G = (size_t)Mx * My;
    const int Kh = My / 2 + 1;
    double* H = wc.take<double>(ng * G);
    double2* Hh = wc.take<double2>(ng * (size_t)Mx * Kh);
    FTE_WS_CHECK(wc);
    const WinParams wp = win_params(a);
    // block transforms where a line fits shared memory, long ones elsewhere
    const bool long_y = !fte_fft_fits_block(My, sizeof(double2));
    const bool long_x = !fte_fft_fits_block(Mx, sizeof(double2));
    FftDev py{}, px{};
    LongFft ly, lx;
    if (long_y)
        FTE_TRY(fte_get_long_plan(ctx, My, &ly));
    else
        FTE_TRY(fte_get_plan(ctx, My, &py));
    if (long_x)
        FTE_TRY(fte_get_long_plan(ctx, Mx, &lx));
    else
        FTE_TRY(fte_get_plan(ctx, Mx, &px));
    size_t sm_y = 2 * (size_t)py.m * sizeof(double2);
    size_t sm_x = 2 * (size_t)px.m * sizeof(double2);
    if (sm_y > (size_t)ctx->max_smem_optin || sm_x > (size_t)ctx->max_smem_optin) {
        fte_set_error("grid %d x %d needs FFT lengths (%d, %d) beyond this device's shared memory", Mx, My, px.m,
                      py.m);
        return FTE_ERR_UNSUPPORTED;
    }
    double2* S = long_y ? wc.take<double2>((size_t)ng * (Mx / 2) * My) : nullptr;
    const size_t lsy = long_y ? fte_long_scratch(My, (long long)ng * (Mx / 2)) : 0;
    const size_t lsx = long_x ? fte_long_scratch(Mx, (long long)ng * Kh) : 0;
    double2* LS = (lsy || lsx) ? wc.take<double2>(lsy > lsx ? lsy : lsx) : nullptr;
    FTE_WS_CHECK(wc);
    const LineMap rows{(long long)My, 0, 1, 1};
    const LineMap cols{(long long)Mx * Kh, 1, (long long)Kh, Kh};
    const int P1 = a.P + 1;
    size_t sm_pt = (size_t)(e1_len(a.P, wp.aniso) + kPtThreads * P1) * sizeof(double);

    // tile the grid for the shared-memory spread and gather (0: window too
    // wide for any tile; the per-point kernels with global atomics are used)
    int ts_s = 0, ts_g = 0;
    FTE_TRY(resolve_tiles(ctx, a, &ts_s, &ts_g));
    TileBins tb_s, tb_g;
    tb_s.ntx = tb_g.ntx = 0;
    tb_s.ts = tb_g.ts = 0;
    if (a.pre_src && ts_s > 0 && a.nsrc > 0)
        tb_s = *a.pre_src;
    else if (ts_s > 0 && a.nsrc > 0)
        FTE_TRY(fte_tiles_build(ctx, wc, a.psrc, a.nsrc, a.Lx, a.Ly, wp.h, wp.hy, ts_s, (Mx + ts_s - 1) / ts_s,
                                (My + ts_s - 1) / ts_s, &tb_s));
    if (a.pre_tar && ts_g > 0 && a.ntar > 0)
        tb_g = *a.pre_tar;
    else if (ts_g > 0 && a.ntar > 0)
        FTE_TRY(fte_tiles_build(ctx, wc, a.ptar, a.ntar, a.Lx, a.Ly, wp.h, wp.hy, ts_g, (Mx + ts_g - 1) / ts_g,
                                (My + ts_g - 1) / ts_g, &tb_g, tile_region(ts_g, a.P)));
    if ((a.nsrc > 0 && tb_s.ts != ts_s) || (a.ntar > 0 && tb_g.ts != ts_g)) {
        fte_set_error("internal: prebuilt tiles do not match the FP64 tile sizes");
        return FTE_ERR_INVALID;
    }
    // float-float form: window records of the sources (tiled spread only)
    const bool ff = fte_form_ff(a.form);
    FfWin* recs = ff && a.nsrc > 0 && ts_s > 0 ? wc.take<FfWin>(a.nsrc) : nullptr;
    FTE_WS_CHECK(wc);

    // grids spread: the stresslet's tiled float-float spread writes its
    // three symmetric products (S12 + S21 as one grid)
    const int ngs = ff && a.kind == FTE_KIND_DLP && ts_s > 0 ? 3 : ng;
    FTE_TRY(fte_record(ctx, 2));
    FTE_CUDA_TRY(cudaMemsetAsync(H, 0, sizeof(double) * ngs * G, ctx->stream));
    if (a.nsrc > 0 && ts_s > 0) {
        FTE_TRY(launch_spread_tiled(ctx, a, tb_s, wp, H, recs));
    } else if (a.nsrc > 0) {
        if (ng == 2) {
            FTE_CUDA_TRY(fte_smem_ceiling(k_spread<2>, (int)sm_pt));
            FTE_LAUNCH(ctx, k_spread<2>, pt_grid(ctx, a.nsrc), kPtThreads, sm_pt, a.psrc, a.f, a.nrm, a.wts, a.nsrc,
                       wp, H);
        } else {
            FTE_CUDA_TRY(fte_smem_ceiling(k_spread<4>, (int)sm_pt));
            FTE_LAUNCH(ctx, k_spread<4>, pt_grid(ctx, a.nsrc), kPtThreads, sm_pt, a.psrc, a.f, a.nrm, a.wts, a.nsrc,
                       wp, H);
        }
    }
    FTE_TRY(fte_record(ctx, 3));
    // float-float form with block transforms: the transforms in float-float
    // too, the last one writing the float-float grids the gather reads
    const bool fft_ff = ff && !long_x && !long_y;
    if (fft_ff) {
        float4* Hf = reinterpret_cast<float4*>(Hh);
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_r2c_ff, (int)sm_y));
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_c2r_ff, (int)sm_y));
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_x_ff, (int)sm_x));
        FTE_LAUNCH(ctx, k_fft_y_r2c_ff, dim3(Mx / 2, ngs), fft_threads(py.m), sm_y, (const double*)H, Hf, Mx, My, py);
        FTE_LAUNCH(ctx, k_fft_x_ff, dim3(Kh, ngs), fft_threads(px.m), sm_x, Hf, Mx, Kh, px, 0);
        int fb = (int)(((size_t)Mx * Kh + 255) / 256);
        if (fb > ctx->num_sms * 32) fb = ctx->num_sms * 32;
        // the multipliers in float-float while (1 - eta) K / (4 xi^2) stays
        // inside the float-float exponential's range (it reaches K ~ (pi M / L)^2)
        const double kmax = FTE_PI * (Mx / a.Lx > My / a.Ly ? Mx / a.Lx : My / a.Ly);
        const double xext = fabs(1.0 - a.eta) * 2.0 * kmax * kmax / (4.0 * a.xi * a.xi);
        if (xext < 75.0) {
            const FfFilt ffc = ff_filter_consts(a.Lx, a.Ly, a.xi, a.eta);
            if (a.kind == FTE_KIND_SLP)
                FTE_LAUNCH(ctx, k_filter_ff<FTE_KIND_SLP>, fb, 256, 0, Hf, Mx, My, ffc, ngs);
            else
                FTE_LAUNCH(ctx, k_filter_ff<FTE_KIND_DLP>, fb, 256, 0, Hf, Mx, My, ffc, ngs);
        } else if (a.kind == FTE_KIND_SLP) {
            FTE_LAUNCH(ctx, (k_filter<FTE_KIND_SLP, float4, true>), fb, 256, 0, Hf, Mx, My, a.Lx, a.Ly, a.xi, a.eta, ngs);
        } else {
            FTE_LAUNCH(ctx, (k_filter<FTE_KIND_DLP, float4, true>), fb, 256, 0, Hf, Mx, My, a.Lx, a.Ly, a.xi, a.eta, ngs);
        }
        FTE_LAUNCH(ctx, k_fft_x_ff, dim3(Kh, 2), fft_threads(px.m), sm_x, Hf, Mx, Kh, px, 1);
        FTE_LAUNCH(ctx, k_fft_y_c2r_ff, dim3(Mx / 2, 2), fft_threads(py.m), sm_y, (const float4*)Hf,
                   reinterpret_cast<float2*>(H), Mx, My, py);
        FTE_TRY(fte_record(ctx, 4));
        const double scale = gather_scale(a);
        if (a.ntar > 0 && ts_g > 0) {
            FTE_TRY(launch_gather_tiled(ctx, a, tb_g, wp, H, scale));
        } else if (a.ntar > 0) {
            // the per-point gather reads FP64 grids
            FTE_LAUNCH(ctx, k_ff_join, ew_grid(ctx, 2LL * (long long)G), 256, 0, H, 2LL * (long long)G);
            FTE_CUDA_TRY(fte_smem_ceiling(k_gather, (int)sm_pt));
            FTE_LAUNCH(ctx, k_gather, pt_grid(ctx, a.ntar), kPtThreads, sm_pt, a.ptar, a.ntar, wp, (const double*)H,
                       (const double*)(H + G), scale, a.uk);
        }
        FTE_TRY(fte_record(ctx, 5));
        (void)info;
        return FTE_OK;
    }
    if (!long_y) {
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_r2c, (int)sm_y));
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_c2r, (int)sm_y));
        FTE_LAUNCH(ctx, k_fft_y_r2c, dim3(Mx / 2, ngs), fft_threads(py.m), sm_y, (const double*)H, Hh, Mx, My, py);
    } else {
        const long long tot = (long long)ngs * (Mx / 2) * My;
        FTE_LAUNCH(ctx, k_ly_pack_r2c, ew_grid(ctx, tot), 256, 0, (const double*)H, S, Mx, My, ngs);
        FTE_TRY(fte_long_fft(ctx, ly, S, rows, (long long)ngs * (Mx / 2), false, LS));
        FTE_LAUNCH(ctx, k_ly_unpack_r2c, ew_grid(ctx, (long long)ngs * (Mx / 2) * Kh), 256, 0, (const double2*)S, Hh,
                   Mx, My, ngs);
    }
    if (!long_x) {
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_x, (int)sm_x));
        FTE_LAUNCH(ctx, k_fft_x, dim3(Kh, ngs), fft_threads(px.m), sm_x, Hh, Mx, Kh, px, 0);
    } else {
        FTE_TRY(fte_long_fft(ctx, lx, Hh, cols, (long long)ngs * Kh, false, LS));
    }
    int fb = (int)(((size_t)Mx * Kh + 255) / 256);
    if (fb > ctx->num_sms * 32) fb = ctx->num_sms * 32;
    if (a.kind == FTE_KIND_SLP)
        FTE_LAUNCH(ctx, (k_filter<FTE_KIND_SLP, double2>), fb, 256, 0, Hh, Mx, My, a.Lx, a.Ly, a.xi, a.eta, ngs);
    else
        FTE_LAUNCH(ctx, (k_filter<FTE_KIND_DLP, double2>), fb, 256, 0, Hh, Mx, My, a.Lx, a.Ly, a.xi, a.eta, ngs);
    if (!long_x)
        FTE_LAUNCH(ctx, k_fft_x, dim3(Kh, 2), fft_threads(px.m), sm_x, Hh, Mx, Kh, px, 1);
    else
        FTE_TRY(fte_long_fft(ctx, lx, Hh, cols, 2LL * Kh, true, LS));
    if (!long_y) {
        FTE_LAUNCH(ctx, k_fft_y_c2r, dim3(Mx / 2, 2), fft_threads(py.m), sm_y, (const double2*)Hh, H, Mx, My, py);
    } else {
        FTE_LAUNCH(ctx, k_ly_pack_c2r, ew_grid(ctx, 2LL * (Mx / 2) * Kh), 256, 0, (const double2*)Hh, S, Mx, My, 2);
        FTE_TRY(fte_long_fft(ctx, ly, S, rows, 2LL * (Mx / 2), true, LS));
        FTE_LAUNCH(ctx, k_ly_unpack_c2r, ew_grid(ctx, 2LL * (Mx / 2) * My), 256, 0, (const double2*)S, H, Mx, My, 2);
    }
    FTE_TRY(fte_record(ctx, 4));
    const double scale = gather_scale(a);
    if (a.ntar > 0 && ts_g > 0) {
        if (ff) FTE_LAUNCH(ctx, k_ff_split, ew_grid(ctx, 2LL * (long long)G), 256, 0, H, 2LL * (long long)G);
        FTE_TRY(launch_gather_tiled(ctx, a, tb_g, wp, H, scale));
    } else if (a.ntar > 0) {
        FTE_CUDA_TRY(fte_smem_ceiling(k_gather, (int)sm_pt));
        FTE_LAUNCH(ctx, k_gather, pt_grid(ctx, a.ntar), kPtThreads, sm_pt, a.ptar, a.ntar, wp, (const double*)H,
                   (const double*)(H + G), scale, a.uk);
    }
    FTE_TRY(fte_record(ctx, 5));
    (void)info;
    return FTE_OK;
}

// ===========================================================================
// Work lists of many float-float k-space evaluations (the batches of plans).
//
// A batch evaluates many (plan, density vector) pairs.  Where a plan's
// k-space part is the float-float form on block transforms with tiled spread
// and gather (what the tuned choice picks for batches at tol >= 1e-11), its
// evaluations become items of one work list per stage instead of one launch
// per stage and evaluation: grid clearing, window records, spread (Stokeslet
// and stresslet), the y transforms, the x transforms, the multipliers, the
// inverse transforms and the gather each run as one launch over every item's
// blocks (a block reads its item's parameters from a device array; transforms
// are grouped by line length so that a short line's block does not carry a
// long line's shared memory, spread and gather items by the CTAs per SM their
// tile allows and the gather's by window support).  The arithmetic is the
// per-call kernels' own (the same device functions), so results match the
// per-plan path.
// ===========================================================================
namespace {

struct KItem {
    WinParams wp;
    FftDev py, px;
    FfFilt ffc;
    int kind, ngs, Mx, My, Kh, PM;
    int64_t nsrc, ntar;
    double* H;    // the spread's FP64 grids, later the float-float grids of the gather
    float4* Hf;   // float-float half spectra
    FfWin* recs;  // window records of the sources in tile order
    const double *psrc, *f, *nrm, *wts;
    const int *toff_s, *perm_s;
    int ts_s, ntx_s, nty_s;
    const double* ptar;
    const int *toff_g, *perm_g;
    int ts_g, ntx_g, nty_g;
    double scale;
    double2* uk;
};

constexpr int kZeroPerThread = 8;
constexpr int kFftClasses = 4;
int fft_class(int m) { return m <= 256 ? 0 : (m <= 1024 ? 1 : (m <= 4096 ? 2 : 3)); }
// Spread and gather items are grouped by the CTAs per SM their shared memory
// allows (1..kOccClasses): a launch reserves its largest item's shared memory
// for every block, so that plans with larger tiles (autotuned sizes differ per
// plan) would otherwise lower every other plan's occupancy.
constexpr int kOccClasses = 8;
int occ_class(size_t smem) {
    const size_t per_sm = 228 * 1024, reserved = 1024;  // per SM; per CTA
    const size_t c = per_sm / (smem + reserved);
    return (int)(c < 1 ? 0 : (c > kOccClasses ? kOccClasses - 1 : c - 1));
}

__global__ void k_zero_multi(const KItem* __restrict__ items, const int2* __restrict__ wl) {
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const size_t n = (size_t)it.ngs * it.Mx * it.My;
    const size_t base = (size_t)w.y * blockDim.x * kZeroPerThread;
    for (int j = 0; j < kZeroPerThread; j++) {
        const size_t i = base + (size_t)j * blockDim.x + threadIdx.x;
        if (i < n) it.H[i] = 0.0;
    }
}

__global__ void k_ff_win_multi(const KItem* __restrict__ items, const int2* __restrict__ wl) {
    __shared__ float2 etab[64];
    load_etab(etab);
    __syncthreads();
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const int64_t k = (int64_t)w.y * blockDim.x + threadIdx.x;
    if (k < it.nsrc) {
        const WinParams wp = it.wp;
        ff_win_rec(it.kind, it.psrc, it.f, it.nrm, it.wts, it.perm_s, k, wp, etab, it.recs);
    }
}

template <int NG>
__global__ void __launch_bounds__(kColThreads) k_spread_ff_multi(const KItem* __restrict__ items,
                                                                const int2* __restrict__ wl) {
    extern __shared__ __align__(16) unsigned char shraw[];
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const WinParams wp = it.wp;
    const size_t G = (size_t)it.Mx * it.My;
    spread_ff_run<NG>(it.recs, it.toff_s, it.ts_s, it.ntx_s, it.nty_s, wp, it.H, it.H + G,
                      NG == 3 ? it.H + 2 * G : nullptr, w.y, it.ntx_s * it.nty_s, shraw);
}

__global__ void __launch_bounds__(512, 2) k_fft_y_r2c_ff_multi(const KItem* __restrict__ items,
                                                               const int2* __restrict__ wl) {
    extern __shared__ __align__(16) unsigned char shff[];
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const FftDev plan = it.py;
    const int half = it.Mx / 2;
    fft_y_r2c_ff_line(it.H, it.Hf, it.Mx, it.My, plan, w.y % half, w.y / half, shff);
}

__global__ void __launch_bounds__(512, 2) k_fft_x_ff_multi(const KItem* __restrict__ items,
                                                           const int2* __restrict__ wl, int inv) {
    extern __shared__ __align__(16) unsigned char shff[];
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const FftDev plan = it.px;
    fft_x_ff_line(it.Hf, it.Mx, it.Kh, plan, inv, w.y % it.Kh, w.y / it.Kh, shff);
}

__global__ void __launch_bounds__(512, 2) k_fft_y_c2r_ff_multi(const KItem* __restrict__ items,
                                                               const int2* __restrict__ wl) {
    extern __shared__ __align__(16) unsigned char shff[];
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const FftDev plan = it.py;
    const int half = it.Mx / 2;
    fft_y_c2r_ff_line(it.Hf, reinterpret_cast<float2*>(it.H), it.Mx, it.My, plan, w.y % half, w.y / half, shff);
}

template <int KIND>
__global__ void k_filter_ff_multi(const KItem* __restrict__ items, const int2* __restrict__ wl) {
    __shared__ float2 etab[64];
    load_etab(etab);
    __syncthreads();
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const FfFilt f = it.ffc;
    const size_t GS = (size_t)it.Mx * it.Kh;
    filter_ff_run<KIND>(it.Hf, it.Mx, it.My, f, it.ngs, (size_t)w.y * blockDim.x + threadIdx.x, GS, etab);
}

template <int PM>
__global__ void __launch_bounds__(kTileThreads, 5) k_gather_ff_multi(const KItem* __restrict__ items,
                                                                     const int2* __restrict__ wl) {
    extern __shared__ __align__(16) unsigned char shraw[];
    __shared__ float2 etab[64];
    const int2 w = wl[blockIdx.x];
    const KItem& it = items[w.x];
    const WinParams wp = it.wp;
    const size_t G = (size_t)it.Mx * it.My;
    const float2* Hf = reinterpret_cast<const float2*>(it.H);
    gather_ff_run<PM>(it.ptar, it.toff_g, it.perm_g, it.ts_g, it.ntx_g, it.nty_g, wp, Hf, Hf + G, it.scale, it.uk, w.y,
                      it.ntx_g * it.nty_g, shraw, etab);
}

}  // namespace

struct KMulti {
    struct List {
        std::vector<int2> h;
        int2* d = nullptr;
        size_t smem = 0;
        int threads = 0;
        void add(int item, int n) {
            for (int j = 0; j < n; j++) h.push_back(make_int2(item, j));
        }
    };
    std::vector<KItem> items;
    KItem* ditems = nullptr;
    char* mem = nullptr;
    // spread[grids 2/3][occupancy class], gather[support class][occupancy class]
    List zero, win, spread[2][kOccClasses], yr2c[kFftClasses], xf[kFftClasses], filt[2], xi[kFftClasses],
        yc2r[kFftClasses], gather[kGatherPmClasses][kOccClasses];
    template <typename F>
    void each(F fn) {
        fn(zero);
        fn(win);
        for (auto& g : spread)
            for (auto& l : g) fn(l);
        for (auto& l : yr2c) fn(l);
        for (auto& l : xf) fn(l);
        for (auto& l : filt) fn(l);
        for (auto& l : xi) fn(l);
        for (auto& l : yc2r) fn(l);
        for (auto& g : gather)
            for (auto& l : g) fn(l);
    }
};

int fte_kmulti_create(KMulti** out) {
    *out = new (std::nothrow) KMulti();
    if (!*out) {
        fte_set_error("out of host memory");
        return FTE_ERR_ALLOC;
    }
    return FTE_OK;
}

void fte_kmulti_destroy(KMulti* km) {
    if (!km) return;
    if (km->mem) cudaFree(km->mem);
    delete km;
}

int fte_kmulti_add(KMulti* km, fte_context* ctx, WsCarver& wc, const KspaceArgs& a, bool* taken) {
    *taken = false;
    if (a.form != FTE_FORM_FF || !a.pre_src || !a.pre_tar) return FTE_OK;
    const int Mx = a.Mx, My = a.My, Kh = My / 2 + 1;
    if (!fte_fft_fits_block(My, sizeof(double2)) || !fte_fft_fits_block(Mx, sizeof(double2))) return FTE_OK;
    const int PM = gather_ff_pm(a.P + 1);
    if (!PM) return FTE_OK;
    int ts_s = 0, ts_g = 0;
    FTE_TRY(resolve_tiles(ctx, a, &ts_s, &ts_g));
    if ((a.nsrc > 0 && (ts_s == 0 || a.pre_src->ts != ts_s)) || (a.ntar > 0 && (ts_g == 0 || a.pre_tar->ts != ts_g)))
        return FTE_OK;
    const double kmax = FTE_PI * (Mx / a.Lx > My / a.Ly ? Mx / a.Lx : My / a.Ly);
    if (fabs(1.0 - a.eta) * 2.0 * kmax * kmax / (4.0 * a.xi * a.xi) >= 75.0) return FTE_OK;  // FP64 multiplier
    KItem it;
    std::memset(&it, 0, sizeof(it));
    it.wp = win_params(a);
    FTE_TRY(fte_get_plan(ctx, My, &it.py));
    FTE_TRY(fte_get_plan(ctx, Mx, &it.px));
    if (2 * (size_t)it.py.m * sizeof(float4) > (size_t)ctx->max_smem_optin ||
        2 * (size_t)it.px.m * sizeof(float4) > (size_t)ctx->max_smem_optin)
        return FTE_OK;
    // the scratch as fte_kspace_run carves it: grids, half spectra, records
    const int ng = a.kind == FTE_KIND_SLP ? 2 : 4;
    const size_t G = (size_t)Mx * My;
    it.H = wc.take<double>(ng * G);
    it.Hf = reinterpret_cast<float4*>(wc.take<double2>(ng * (size_t)Mx * Kh));
    it.recs = a.nsrc > 0 ? wc.take<FfWin>(a.nsrc) : nullptr;
    FTE_WS_CHECK(wc);
    it.ffc = ff_filter_consts(a.Lx, a.Ly, a.xi, a.eta);
    it.kind = a.kind;
    it.ngs = a.kind == FTE_KIND_SLP ? 2 : 3;
    it.Mx = Mx;
    it.My = My;
    it.Kh = Kh;
    it.PM = PM;
    it.nsrc = a.nsrc;
    it.ntar = a.ntar;
    it.psrc = a.psrc;
    it.f = a.f;
    it.nrm = a.nrm;
    it.wts = a.wts;
    it.toff_s = a.pre_src->off;
    it.perm_s = a.pre_src->perm;
    it.ts_s = a.pre_src->ts;
    it.ntx_s = a.nsrc > 0 ? a.pre_src->ntx : 0;
    it.nty_s = a.nsrc > 0 ? a.pre_src->nty : 0;
    it.ptar = a.ptar;
    it.toff_g = a.pre_tar->off;
    it.perm_g = a.pre_tar->perm;
    it.ts_g = a.pre_tar->ts;
    it.ntx_g = a.ntar > 0 ? a.pre_tar->ntx : 0;
    it.nty_g = a.ntar > 0 ? a.pre_tar->nty : 0;
    it.scale = gather_scale(a);
    it.uk = a.uk;
    const int i = (int)km->items.size();
    km->items.push_back(it);
    // work lists (blocks of every stage) and launch shapes
    const int an = it.wp.aniso;
    km->zero.add(i, (int)(((size_t)it.ngs * G + 256 * kZeroPerThread - 1) / (256 * kZeroPerThread)));
    if (a.nsrc > 0) {
        km->win.add(i, (int)((a.nsrc + 255) / 256));
        const size_t sm = spread_ff_smem(it.ts_s, a.P, it.ngs, an);
        KMulti::List& sp = km->spread[it.ngs == 2 ? 0 : 1][occ_class(sm)];
        sp.add(i, it.ntx_s * it.nty_s);
        sp.smem = std::max(sp.smem, sm);
    }
    const int cy = fft_class(it.py.m), cx = fft_class(it.px.m);
    const size_t smy = 2 * (size_t)it.py.m * sizeof(float4), smx = 2 * (size_t)it.px.m * sizeof(float4);
    auto shape = [](KMulti::List& l, size_t sm, int th) {
        l.smem = std::max(l.smem, sm);
        l.threads = std::max(l.threads, th);
    };
    km->yr2c[cy].add(i, (Mx / 2) * it.ngs);
    shape(km->yr2c[cy], smy, fft_threads(it.py.m));
    km->xf[cx].add(i, Kh * it.ngs);
    shape(km->xf[cx], smx, fft_threads(it.px.m));
    km->filt[a.kind == FTE_KIND_SLP ? 0 : 1].add(i, (int)(((size_t)Mx * Kh + 255) / 256));
    km->xi[cx].add(i, Kh * 2);
    shape(km->xi[cx], smx, fft_threads(it.px.m));
    km->yc2r[cy].add(i, (Mx / 2) * 2);
    shape(km->yc2r[cy], smy, fft_threads(it.py.m));
    if (a.ntar > 0) {
        const size_t sm = gather_ff_smem(it.ts_g, a.P, an);
        KMulti::List& ga = km->gather[gather_pm_class(PM)][occ_class(sm)];
        ga.add(i, it.ntx_g * it.nty_g);
        ga.smem = std::max(ga.smem, sm);
    }
    *taken = true;
    return FTE_OK;
}

int fte_kmulti_finalize(KMulti* km, fte_context* ctx) {
    if (km->items.empty()) return FTE_OK;
    size_t need = ws_bytes(km->items.size() * sizeof(KItem), 1) + 4096;
    km->each([&](KMulti::List& l) { need += ws_bytes(l.h.size() * sizeof(int2), 1); });
    if (fte_alloc_should_fail() || cudaMalloc(&km->mem, need) != cudaSuccess) {
        cudaGetLastError();
        km->mem = nullptr;
        fte_set_error("batch: %zu bytes of device memory for the k-space work lists not available", need);
        return FTE_ERR_ALLOC;
    }
    WsCarver c{km->mem, 0, need};
    km->ditems = c.take<KItem>(km->items.size());
    km->each([&](KMulti::List& l) { l.d = l.h.empty() ? nullptr : c.take<int2>(l.h.size()); });
    FTE_WS_CHECK(c);
    FTE_CUDA_TRY(cudaMemcpyAsync(km->ditems, km->items.data(), km->items.size() * sizeof(KItem),
                                 cudaMemcpyHostToDevice, ctx->stream));
    cudaError_t e = cudaSuccess;
    km->each([&](KMulti::List& l) {
        if (l.d && e == cudaSuccess)
            e = cudaMemcpyAsync(l.d, l.h.data(), l.h.size() * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream);
    });
    FTE_CUDA_TRY(e);
    FTE_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return FTE_OK;
}

int fte_kmulti_items(const KMulti* km) { return km ? (int)km->items.size() : 0; }

int fte_kmulti_run(KMulti* km, fte_context* ctx) {
    if (!km || km->items.empty()) return FTE_OK;
    const KItem* it = km->ditems;
    auto n = [](const KMulti::List& l) { return (int)l.h.size(); };
    if (n(km->zero)) FTE_LAUNCH(ctx, k_zero_multi, n(km->zero), 256, 0, it, (const int2*)km->zero.d);
    if (n(km->win)) FTE_LAUNCH(ctx, k_ff_win_multi, n(km->win), 256, 0, it, (const int2*)km->win.d);
    for (auto& l : km->spread[0])
        if (n(l)) {
            FTE_CUDA_TRY(fte_smem_ceiling(k_spread_ff_multi<2>, l.smem));
            FTE_LAUNCH(ctx, k_spread_ff_multi<2>, n(l), kColThreads, l.smem, it, (const int2*)l.d);
        }
    for (auto& l : km->spread[1])
        if (n(l)) {
            FTE_CUDA_TRY(fte_smem_ceiling(k_spread_ff_multi<3>, l.smem));
            FTE_LAUNCH(ctx, k_spread_ff_multi<3>, n(l), kColThreads, l.smem, it, (const int2*)l.d);
        }
    for (auto& l : km->yr2c)
        if (n(l)) {
            FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_r2c_ff_multi, l.smem));
            FTE_LAUNCH(ctx, k_fft_y_r2c_ff_multi, n(l), l.threads, l.smem, it, (const int2*)l.d);
        }
    for (auto& l : km->xf)
        if (n(l)) {
            FTE_CUDA_TRY(fte_smem_ceiling(k_fft_x_ff_multi, l.smem));
            FTE_LAUNCH(ctx, k_fft_x_ff_multi, n(l), l.threads, l.smem, it, (const int2*)l.d, 0);
        }
    if (n(km->filt[0])) FTE_LAUNCH(ctx, k_filter_ff_multi<FTE_KIND_SLP>, n(km->filt[0]), 256, 0, it,
                                   (const int2*)km->filt[0].d);
    if (n(km->filt[1])) FTE_LAUNCH(ctx, k_filter_ff_multi<FTE_KIND_DLP>, n(km->filt[1]), 256, 0, it,
                                   (const int2*)km->filt[1].d);
    for (auto& l : km->xi)
        if (n(l)) {
            FTE_CUDA_TRY(fte_smem_ceiling(k_fft_x_ff_multi, l.smem));
            FTE_LAUNCH(ctx, k_fft_x_ff_multi, n(l), l.threads, l.smem, it, (const int2*)l.d, 1);
        }
    for (auto& l : km->yc2r)
        if (n(l)) {
            FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_c2r_ff_multi, l.smem));
            FTE_LAUNCH(ctx, k_fft_y_c2r_ff_multi, n(l), l.threads, l.smem, it, (const int2*)l.d);
        }
    auto gather_class = [&](auto kern, int cls) -> int {
        for (auto& l : km->gather[cls])
            if (n(l)) {
                FTE_CUDA_TRY(fte_smem_ceiling(kern, l.smem));
                FTE_LAUNCH(ctx, kern, n(l), kTileThreads, l.smem, it, (const int2*)l.d);
            }
        return FTE_OK;
    };
    FTE_TRY(gather_class(k_gather_ff_multi<16>, 0));
    FTE_TRY(gather_class(k_gather_ff_multi<17>, 1));
    FTE_TRY(gather_class(k_gather_ff_multi<19>, 2));
    FTE_TRY(gather_class(k_gather_ff_multi<21>, 3));
    FTE_TRY(gather_class(k_gather_ff_multi<23>, 4));
    FTE_TRY(gather_class(k_gather_ff_multi<24>, 5));
    FTE_TRY(gather_class(k_gather_ff_multi<25>, 6));
    FTE_TRY(gather_class(k_gather_ff_multi<32>, 7));
    return FTE_OK;
}

// ===========================================================================
// k-space sums of the other quantities (FP64): the velocity pipeline's spread,
// transforms and gather around the quantity's filter.  The filter stores the
// Hermitian part of the reference's filtered spectrum, (G(k) + conj G(-k)) / 2
// with G(-k) evaluated at the wave numbers the reference assigns to the index
// of -k (Nyquist rows and columns keep +k), which is what real(ifft2) of the
// reference's full spectrum equals.
// ===========================================================================
namespace {
template <int KIND, int Q>
__global__ void k_filter_q(double2* __restrict__ Hh, int Mx, int My, double Lx, double Ly, double xi, double eta) {
    constexpr int NG = KIND == FTE_KIND_SLP ? 2 : 4;
    constexpr int NO = fte_q_nout(Q);
    const int Kh = My / 2 + 1;
    const size_t GS = (size_t)Mx * Kh;
    const double tpx = 2.0 * FTE_PI / Lx, tpy = 2.0 * FTE_PI / Ly;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < GS; idx += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx / Kh), k = (int)(idx % Kh);
        double2 in[NG], out[NO], out2[NO];
#pragma unroll
        for (int g = 0; g < NG; g++) in[g] = Hh[g * GS + idx];
        if (j == 0 && k == 0) {
#pragma unroll
            for (int o = 0; o < NO; o++) out[o] = make_double2(0.0, 0.0);
        } else {
            const double k1 = j <= Mx / 2 ? tpx * j : tpx * (j - Mx);
            const double k2 = tpy * k;
            fte_q_apply<KIND, Q>(k1, k2, xi, eta, in, out);
            const bool nyq_x = 2 * j == Mx, nyq_y = 2 * k == My;
            double2 cin[NG];
#pragma unroll
            for (int g = 0; g < NG; g++) cin[g] = make_double2(in[g].x, -in[g].y);
            fte_q_apply<KIND, Q>(nyq_x ? k1 : -k1, nyq_y ? k2 : -k2, xi, eta, cin, out2);
#pragma unroll
            for (int o = 0; o < NO; o++)
                out[o] = make_double2(0.5 * (out[o].x + out2[o].x), 0.5 * (out[o].y - out2[o].y));
        }
#pragma unroll
        for (int o = 0; o < NO; o++) Hh[o * GS + idx] = out[o];
    }
}

// out[t * no + c] from gathered component pairs
__global__ void k_q_pack(const double2* __restrict__ a, const double2* __restrict__ b, int64_t n, int no,
                         double* __restrict__ out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const double2 u = a[t];
        if (no == 1) {
            out[t] = u.x;
        } else {
            const double2 v = b[t];
            out[4 * t] = u.x;
            out[4 * t + 1] = u.y;
            out[4 * t + 2] = v.x;
            out[4 * t + 3] = v.y;
        }
    }
}

template <int KIND>
int q_filter_launch(fte_context* ctx, int q, double2* Hh, const KspaceArgs& a) {
    int fb = (int)(((size_t)a.Mx * (a.My / 2 + 1) + 255) / 256);
    if (fb > ctx->num_sms * 32) fb = ctx->num_sms * 32;
    switch (q) {
        case FTE_Q_PRESSURE:
            FTE_LAUNCH(ctx, (k_filter_q<KIND, FTE_Q_PRESSURE>), fb, 256, 0, Hh, a.Mx, a.My, a.Lx, a.Ly, a.xi, a.eta);
            return FTE_OK;
        case FTE_Q_PRESSURE_GRAD:
            FTE_LAUNCH(ctx, (k_filter_q<KIND, FTE_Q_PRESSURE_GRAD>), fb, 256, 0, Hh, a.Mx, a.My, a.Lx, a.Ly, a.xi,
                       a.eta);
            return FTE_OK;
        case FTE_Q_GRADIENT:
            FTE_LAUNCH(ctx, (k_filter_q<KIND, FTE_Q_GRADIENT>), fb, 256, 0, Hh, a.Mx, a.My, a.Lx, a.Ly, a.xi, a.eta);
            return FTE_OK;
        case FTE_Q_STRESS:
            FTE_LAUNCH(ctx, (k_filter_q<KIND, FTE_Q_STRESS>), fb, 256, 0, Hh, a.Mx, a.My, a.Lx, a.Ly, a.xi, a.eta);
            return FTE_OK;
        case FTE_Q_VORTICITY:
            FTE_LAUNCH(ctx, (k_filter_q<KIND, FTE_Q_VORTICITY>), fb, 256, 0, Hh, a.Mx, a.My, a.Lx, a.Ly, a.xi, a.eta);
            return FTE_OK;
        default: break;
    }
    fte_set_error("unknown quantity %d", q);
    return FTE_ERR_INVALID;
}
}  // namespace

size_t fte_q_kspace_ws(int Mx, int My, int64_t nsrc, int64_t ntar) {
    // four grids cover every kind's inputs and every quantity's outputs
    return fte_kspace_ws(FTE_KIND_DLP, FTE_FORM_PLAIN, Mx, My, nsrc, ntar) + 2 * ws_bytes((size_t)ntar + 1, 16) + 4096;
}

int fte_q_kspace_run(fte_context* ctx, WsCarver& wc, int q, const KspaceArgs& a, double* out) {
    const int ng = a.kind == FTE_KIND_SLP ? 2 : 4;
    const int no = fte_q_nout(q);
    const int nh = ng > no ? ng : no;  // grids held at once
    const int Mx = a.Mx, My = a.My;
    const size_t G = (size_t)Mx * My;
    const int Kh = My / 2 + 1;
    double* H = wc.take<double>(4 * G);
    double2* Hh = wc.take<double2>(4 * (size_t)Mx * Kh);
    double2* ga = wc.take<double2>((size_t)a.ntar + 1);
    double2* gb = wc.take<double2>((size_t)a.ntar + 1);
    FTE_WS_CHECK(wc);
    const WinParams wp = win_params(a);
    const bool long_y = !fte_fft_fits_block(My, sizeof(double2));
    const bool long_x = !fte_fft_fits_block(Mx, sizeof(double2));
    FftDev py{}, px{};
    LongFft ly, lx;
    if (long_y)
        FTE_TRY(fte_get_long_plan(ctx, My, &ly));
    else
        FTE_TRY(fte_get_plan(ctx, My, &py));
    if (long_x)
        FTE_TRY(fte_get_long_plan(ctx, Mx, &lx));
    else
        FTE_TRY(fte_get_plan(ctx, Mx, &px));
    const size_t sm_y = 2 * (size_t)py.m * sizeof(double2), sm_x = 2 * (size_t)px.m * sizeof(double2);
    if (sm_y > (size_t)ctx->max_smem_optin || sm_x > (size_t)ctx->max_smem_optin) {
        fte_set_error("grid %d x %d beyond this device's shared memory", Mx, My);
        return FTE_ERR_UNSUPPORTED;
    }
    double2* S = long_y ? wc.take<double2>((size_t)nh * (Mx / 2) * My) : nullptr;
    const size_t lsy = long_y ? fte_long_scratch(My, (long long)nh * (Mx / 2)) : 0;
    const size_t lsx = long_x ? fte_long_scratch(Mx, (long long)nh * Kh) : 0;
    double2* LS = (lsy || lsx) ? wc.take<double2>(lsy > lsx ? lsy : lsx) : nullptr;
    FTE_WS_CHECK(wc);
    const LineMap rows{(long long)My, 0, 1, 1};
    const LineMap cols{(long long)Mx * Kh, 1, (long long)Kh, Kh};

    int ts_s = 0, ts_g = 0;
    FTE_TRY(resolve_tiles(ctx, a, &ts_s, &ts_g));
    if (!ts_s || !ts_g) {
        fte_set_error("window support P=%d too wide for the spread/gather tiles", a.P);
        return FTE_ERR_UNSUPPORTED;
    }
    FTE_CUDA_TRY(cudaMemsetAsync(H, 0, sizeof(double) * ng * G, ctx->stream));
    if (a.nsrc > 0) {
        TileBins tb;
        WsCarver w2 = wc;
        FTE_TRY(fte_tiles_build(ctx, w2, a.psrc, a.nsrc, a.Lx, a.Ly, wp.h, wp.hy, ts_s, (Mx + ts_s - 1) / ts_s,
                                (My + ts_s - 1) / ts_s, &tb));
        FTE_WS_CHECK(w2);
        FTE_TRY(launch_spread_tiled(ctx, a, tb, wp, H, nullptr));
    }
    // forward: ng grids
    if (!long_y) {
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_r2c, (int)sm_y));
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_c2r, (int)sm_y));
        FTE_LAUNCH(ctx, k_fft_y_r2c, dim3(Mx / 2, ng), fft_threads(py.m), sm_y, (const double*)H, Hh, Mx, My, py);
    } else {
        FTE_LAUNCH(ctx, k_ly_pack_r2c, ew_grid(ctx, (long long)ng * (Mx / 2) * My), 256, 0, (const double*)H, S, Mx,
                   My, ng);
        FTE_TRY(fte_long_fft(ctx, ly, S, rows, (long long)ng * (Mx / 2), false, LS));
        FTE_LAUNCH(ctx, k_ly_unpack_r2c, ew_grid(ctx, (long long)ng * (Mx / 2) * Kh), 256, 0, (const double2*)S, Hh,
                   Mx, My, ng);
    }
    if (!long_x) {
        FTE_CUDA_TRY(fte_smem_ceiling(k_fft_x, (int)sm_x));
        FTE_LAUNCH(ctx, k_fft_x, dim3(Kh, ng), fft_threads(px.m), sm_x, Hh, Mx, Kh, px, 0);
    } else {
        FTE_TRY(fte_long_fft(ctx, lx, Hh, cols, (long long)ng * Kh, false, LS));
    }
    if (a.kind == FTE_KIND_SLP)
        FTE_TRY(q_filter_launch<FTE_KIND_SLP>(ctx, q, Hh, a));
    else
        FTE_TRY(q_filter_launch<FTE_KIND_DLP>(ctx, q, Hh, a));
    // inverse: no grids
    if (!long_x)
        FTE_LAUNCH(ctx, k_fft_x, dim3(Kh, no), fft_threads(px.m), sm_x, Hh, Mx, Kh, px, 1);
    else
        FTE_TRY(fte_long_fft(ctx, lx, Hh, cols, (long long)no * Kh, true, LS));
    if (!long_y) {
        FTE_LAUNCH(ctx, k_fft_y_c2r, dim3(Mx / 2, no), fft_threads(py.m), sm_y, (const double2*)Hh, H, Mx, My, py);
    } else {
        FTE_LAUNCH(ctx, k_ly_pack_c2r, ew_grid(ctx, (long long)no * (Mx / 2) * Kh), 256, 0, (const double2*)Hh, S, Mx,
                   My, no);
        FTE_TRY(fte_long_fft(ctx, ly, S, rows, (long long)no * (Mx / 2), true, LS));
        FTE_LAUNCH(ctx, k_ly_unpack_c2r, ew_grid(ctx, (long long)no * (Mx / 2) * My), 256, 0, (const double2*)S, H,
                   Mx, My, no);
    }
    if (a.ntar == 0) return FTE_OK;
    // gather pairs of grids
    TileBins tb;
    FTE_TRY(fte_tiles_build(ctx, wc, a.ptar, a.ntar, a.Lx, a.Ly, wp.h, wp.hy, ts_g, (Mx + ts_g - 1) / ts_g,
                            (My + ts_g - 1) / ts_g, &tb, tile_region(ts_g, a.P)));
    FTE_WS_CHECK(wc);
    const double scale = gather_scale(a);
    KspaceArgs ag = a;
    ag.form = FTE_FORM_PLAIN;
    if (no == 2) {
        ag.uk = reinterpret_cast<double2*>(out);
        FTE_TRY(launch_gather_tiled(ctx, ag, tb, wp, H, scale));
        return FTE_OK;
    }
    ag.uk = ga;
    FTE_TRY(launch_gather_tiled(ctx, ag, tb, wp, H, scale));  // grids 0 (and 1)
    if (no == 4) {
        ag.uk = gb;
        FTE_TRY(launch_gather_tiled(ctx, ag, tb, wp, H + 2 * G, scale));  // grids 2, 3
    }
    FTE_LAUNCH(ctx, k_q_pack, ew_grid(ctx, a.ntar), 256, 0, (const double2*)ga, (const double2*)gb, (int64_t)a.ntar,
               no, out);
    return FTE_OK;
}

// ===========================================================================
// Stokeslet k-space sum without device allocation.
//
// Some callers cannot call cudaMalloc: solvers embedded in a host application
// that owns every byte of device memory through its own pool, real-time loops
// where an allocation (and the device synchronisation cudaMalloc/cudaFree can
// imply) is not allowed after start-up, and plugins whose host forbids
// allocation outside its initialisation phase.  fte_slp_kspace_noalloc serves
// them: it computes exactly what fte_slp_kspace computes, but takes every
// byte of scratch (the two real grids, their half spectra and the FFT tables)
// from one file-scope device array of fixed size instead of a context
// workspace.  The caller passes device pointers to the inputs and the output
// and a stream; nothing is allocated on the device or the host.
//
// Limits: Mx, My <= FTE_NOALLOC_MAX_SIDE (512) and Mx*My <= FTE_NOALLOC_MAX_NODES
// (512*512); larger grids are rejected with FTE_ERR_UNSUPPORTED.  The array
// (about 8.5 MB) stays resident on every GPU that loads the library until the
// process exits.  All calls share it and it keeps the previous call's
// contents, so calls that overlap on the GPU (different streams, or different
// host threads on one device) race and must be serialised by the caller.
// ===========================================================================
namespace {

constexpr long kNaMaxSide = FTE_NOALLOC_MAX_SIDE;
constexpr long kNaMaxNodes = FTE_NOALLOC_MAX_NODES;
constexpr long kNaMaxFft = 1024;  // inner FFT length for any side <= 512 (7-smooth m >= 2n-1)
// doubles: 2 real grids, 2 half spectra (Mx (My/2+1) complex each), and per
// direction the twiddle, chirp and Bluestein tables (complex, <= kNaMaxFft each)
constexpr long kNaGrid = 2 * kNaMaxNodes;
constexpr long kNaSpec = 2 * 2 * (kNaMaxNodes / 2 + kNaMaxSide);
constexpr long kNaTables = 2 * 3 * 2 * kNaMaxFft;
constexpr long kNaDoubles = kNaGrid + kNaSpec + kNaTables;

static __device__ __align__(256) double g_fte_noalloc_scratch[kNaDoubles];

// Device address of the array per device ordinal, looked up once per device.
std::mutex g_na_mu;
double* g_na_ptr[256] = {nullptr};

int na_scratch(double** out) {
    int dev = 0;
    FTE_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        fte_set_error("fte_slp_kspace_noalloc: device ordinal %d out of range", dev);
        return FTE_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_fte_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            fte_set_error("fte_slp_kspace_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return FTE_ERR_CUDA;
        }
        g_na_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_na_ptr[dev];
    return FTE_OK;
}

// radices of a 7-smooth length (8s first), no heap
bool na_radices(int n, int* rad, int* nrad) {
    int c2 = 0, c3 = 0, c5 = 0, c7 = 0, v = n;
    while (v % 2 == 0) { v /= 2; c2++; }
    while (v % 3 == 0) { v /= 3; c3++; }
    while (v % 5 == 0) { v /= 5; c5++; }
    while (v % 7 == 0) { v /= 7; c7++; }
    if (v != 1) return false;
    int k = 0;
    for (; c2 >= 3; c2 -= 3) rad[k++] = 8;
    if (c2 == 2) rad[k++] = 4;
    if (c2 == 1) rad[k++] = 2;
    for (int i = 0; i < c3; i++) rad[k++] = 3;
    for (int i = 0; i < c5; i++) rad[k++] = 5;
    for (int i = 0; i < c7; i++) rad[k++] = 7;
    *nrad = k;
    return k <= 24;
}

// FFT plan of length n with its tables at `tab` (3 * kNaMaxFft complex).
bool na_plan(int n, double2* tab, FftDev* p) {
    int rad[32], nrad = 0;
    p->n = n;
    if (na_radices(n, rad, &nrad)) {
        p->bluestein = 0;
        p->m = n;
    } else {
        int m = 2 * n - 1;
        while (!na_radices(m, rad, &nrad)) m++;
        p->bluestein = 1;
        p->m = m;
    }
    if (p->m > kNaMaxFft) return false;
    p->nrad = nrad;
    for (int i = 0; i < 24; i++) p->rad[i] = i < nrad ? rad[i] : 0;
    p->tw = tab;
    p->chirp = tab + kNaMaxFft;
    p->bhat = tab + 2 * kNaMaxFft;
    p->tw32 = nullptr;
    p->chirp32 = nullptr;
    p->bhat32 = nullptr;
    return true;
}

// twiddles exp(-2 pi i t/m) and the chirp exp(-i pi k^2/n), from sincospi
__global__ void k_na_tables(double2* tw, double2* chirp, int n, int m, int bluestein) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m; t += gridDim.x * blockDim.x) {
        double s, c;
        if (2 * t <= m)
            sincospi(-2.0 * (double)t / (double)m, &s, &c);
        else
            sincospi(2.0 * (double)(m - t) / (double)m, &s, &c);
        tw[t] = make_double2(c, s);
        if (bluestein && t < n) {
            long long k2 = ((long long)t * t) % (2LL * n);
            sincospi(-(double)k2 / (double)n, &s, &c);
            chirp[t] = make_double2(c, s);
        }
    }
}

// Bluestein kernel: DFT_m of the wrapped conjugate chirp, divided by m
__global__ void k_na_bhat(FftDev p, double2* bhat) {
    extern __shared__ double2 shc[];
    double2* A = shc;
    double2* B = shc + p.m;
    for (int k = threadIdx.x; k < p.m; k += blockDim.x) {
        double2 v = make_double2(0.0, 0.0);
        int j = k < p.n ? k : (k > p.m - p.n ? p.m - k : -1);
        if (j >= 0) {
            double2 c = p.chirp[j];
            v = make_double2(c.x, -c.y);
        }
        A[k] = v;
    }
    double2* R = fft_inner<double>(A, B, p, false);
    double inv = 1.0 / p.m;
    for (int k = threadIdx.x; k < p.m; k += blockDim.x) bhat[k] = make_double2(R[k].x * inv, R[k].y * inv);
}

#define NA_LAUNCH(kernel, grid, block, smem, stream, ...)                                          \
    do {                                                                                           \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                                \
        cudaError_t e_ = cudaGetLastError();                                                       \
        if (e_ != cudaSuccess) {                                                                   \
            fte_set_error("fte_slp_kspace_noalloc: launch of %s failed: %s", #kernel,              \
                          cudaGetErrorString(e_));                                                 \
            return FTE_ERR_CUDA;                                                                   \
        }                                                                                          \
    } while (0)

}  // namespace

extern "C" int fte_slp_kspace_noalloc(const double* psrc, int64_t nsrc, const double* ptar, int64_t ntar, double xi,
                                      double eta, const double* f, int Mx, int My, double Lx, double Ly, double w,
                                      int P, double* uk, void* stream_handle) {
    cudaStream_t stream = (cudaStream_t)stream_handle;
    if (nsrc < 0 || ntar < 0 || nsrc > 2000000000LL || ntar > 2000000000LL) {
        fte_set_error("fte_slp_kspace_noalloc: point counts out of range");
        return FTE_ERR_INVALID;
    }
    if ((nsrc > 0 && (!psrc || !f)) || (ntar > 0 && (!ptar || !uk))) {
        fte_set_error("fte_slp_kspace_noalloc: null array argument");
        return FTE_ERR_INVALID;
    }
    if (!(Lx > 0) || !(Ly > 0) || !isfinite(Lx) || !isfinite(Ly) || !(xi > 0) || !isfinite(xi) || !(eta > 0) ||
        !isfinite(eta) || !isfinite(w)) {
        fte_set_error("fte_slp_kspace_noalloc: Lx, Ly, xi, eta must be positive and finite, w finite");
        return FTE_ERR_INVALID;
    }
    if (P < 2 || P % 2 != 0 || P > 64) {
        fte_set_error("fte_slp_kspace_noalloc: window support P must be even and in [2, 64] (P=%d)", P);
        return FTE_ERR_INVALID;
    }
    if (Mx < 2 || My < 2 || Mx % 2 || My % 2) {
        fte_set_error("fte_slp_kspace_noalloc: grid sizes must be even and >= 2 (Mx=%d, My=%d)", Mx, My);
        return FTE_ERR_INVALID;
    }
    double hx = Lx / Mx, hy = Ly / My;
    if (fabs(hx - hy) > 1e-12 * fmax(hx, hy)) {
        fte_set_error("fte_slp_kspace_noalloc: grid spacing must be equal in x and y");
        return FTE_ERR_INVALID;
    }
    if (Mx > kNaMaxSide || My > kNaMaxSide || (long)Mx * My > kNaMaxNodes) {
        fte_set_error("fte_slp_kspace_noalloc: grid %d x %d exceeds the fixed scratch (sides <= %ld, Mx*My <= %ld); "
                      "use fte_slp_kspace",
                      Mx, My, kNaMaxSide, kNaMaxNodes);
        return FTE_ERR_UNSUPPORTED;
    }
    double* base = nullptr;
    FTE_TRY(na_scratch(&base));
    const int Kh = My / 2 + 1;
    const size_t G = (size_t)Mx * My;
    double* H = base;                                           // 2 real grids
    double2* Hh = reinterpret_cast<double2*>(base + kNaGrid);   // 2 half spectra
    double2* tab = reinterpret_cast<double2*>(base + kNaGrid + kNaSpec);
    FftDev py{}, px{};
    if (!na_plan(My, tab, &py) || !na_plan(Mx, tab + 3 * kNaMaxFft, &px)) {
        fte_set_error("fte_slp_kspace_noalloc: FFT length beyond the fixed tables");
        return FTE_ERR_UNSUPPORTED;
    }
    // FFT tables of this call's sizes (the previous call may have used others)
    NA_LAUNCH(k_na_tables, 4, 256, 0, stream, const_cast<double2*>(py.tw), const_cast<double2*>(py.chirp), My, py.m,
              py.bluestein);
    NA_LAUNCH(k_na_tables, 4, 256, 0, stream, const_cast<double2*>(px.tw), const_cast<double2*>(px.chirp), Mx, px.m,
              px.bluestein);
    if (py.bluestein)
        NA_LAUNCH(k_na_bhat, 1, fft_threads(py.m), 2 * py.m * sizeof(double2), stream, py,
                  const_cast<double2*>(py.bhat));
    if (px.bluestein)
        NA_LAUNCH(k_na_bhat, 1, fft_threads(px.m), 2 * px.m * sizeof(double2), stream, px,
                  const_cast<double2*>(px.bhat));
    // the spread accumulates with atomics: the grids must start at zero
    FTE_CUDA_TRY(cudaMemsetAsync(H, 0, sizeof(double) * 2 * G, stream));
    WinParams wp;
    wp.Lx = Lx;
    wp.Ly = Ly;
    wp.h = Lx / Mx;
    wp.rh = 1.0 / wp.h;
    wp.xi = xi;
    wp.eta = eta;
    wp.w = w;
    wp.P = P;
    wp.Mx = Mx;
    wp.My = My;
    wp.hy = wp.h;  // equal steps (checked above)
    wp.rhy = wp.rh;
    wp.wy = wp.w;
    wp.aniso = 0;
    const int P1 = P + 1;
    const size_t sm_pt = (size_t)(((P1 + 1) & ~1) + kPtThreads * P1) * sizeof(double);
    const size_t sm_y = 2 * (size_t)py.m * sizeof(double2), sm_x = 2 * (size_t)px.m * sizeof(double2);
    auto blocks = [](int64_t n) {
        int64_t b = (n + kPtThreads - 1) / kPtThreads;
        return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
    };
    // dynamic shared-memory ceilings: raised once per kernel and device and
    // never lowered (shared with the other entries), checked against these sizes
    FTE_CUDA_TRY(fte_smem_ceiling(k_spread<2>, (int)sm_pt));
    FTE_CUDA_TRY(fte_smem_ceiling(k_gather, (int)sm_pt));
    FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_r2c, (int)sm_y));
    FTE_CUDA_TRY(fte_smem_ceiling(k_fft_y_c2r, (int)sm_y));
    FTE_CUDA_TRY(fte_smem_ceiling(k_fft_x, (int)sm_x));
    if (nsrc > 0)
        NA_LAUNCH(k_spread<2>, blocks(nsrc), kPtThreads, sm_pt, stream, psrc, f, (const double*)nullptr,
                  (const double*)nullptr, nsrc, wp, H);
    NA_LAUNCH(k_fft_y_r2c, dim3(Mx / 2, 2), fft_threads(py.m), sm_y, stream, (const double*)H, Hh, Mx, My, py);
    NA_LAUNCH(k_fft_x, dim3(Kh, 2), fft_threads(px.m), sm_x, stream, Hh, Mx, Kh, px, 0);
    int fb = (int)(((size_t)Mx * Kh + 255) / 256);
    NA_LAUNCH((k_filter<FTE_KIND_SLP, double2>), fb, 256, 0, stream, Hh, Mx, My, Lx, Ly, xi, eta, 2);
    NA_LAUNCH(k_fft_x, dim3(Kh, 2), fft_threads(px.m), sm_x, stream, Hh, Mx, Kh, px, 1);
    NA_LAUNCH(k_fft_y_c2r, dim3(Mx / 2, 2), fft_threads(py.m), sm_y, stream, (const double2*)Hh, H, Mx, My, py);
    double s = 4 * xi * xi / eta;
    s = s * s * wp.h * wp.h / FTE_PI;
    double scale = s / (4 * FTE_PI) / ((double)Mx * (double)My);
    if (ntar > 0)
        NA_LAUNCH(k_gather, blocks(ntar), kPtThreads, sm_pt, stream, ptar, ntar, wp, (const double*)H,
                  (const double*)(H + G), scale, reinterpret_cast<double2*>(uk));
    return FTE_OK;
}
