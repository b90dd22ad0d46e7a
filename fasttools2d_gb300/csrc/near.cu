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
// warp sweeps its targets one after another: its lanes test the staged
// sources 32 at a time with a conservative FP32 distance test, compact the
// survivors into per-warp ring queues (ballot + popc), and every full queue
// of 32 candidate pairs is evaluated with all lanes busy in FP64 (exact
// cutoff test, exp, E1).  Queue entries carry the slot of their target, so
// up to four targets are in flight and a target's last, partial batch is
// filled by the next targets' pairs.  GB300's FP64 pipe issues a warp
// instruction every ~16 cycles per SM whatever the number of active lanes,
// so full batches are what keeps the FP64 work proportional to the pairs
// inside the cutoff.
#include "fte_internal.cuh"
#include "ff.cuh"

#define FTE_E1_STORAGE_R static __constant__
#define FTE_E1_STORAGE_G static __device__ const
#include "fte_e1_coeffs.h"

namespace {

// CTA shape per layout.  The float-float kernel runs 4 warps per CTA and 4
// CTAs per SM: a box's targets are shared by fewer warps (longer runs of
// targets per warp, fewer queue drains per box) and boxes overlap across
// more CTAs.  The FP64 kernel keeps 8 warps and 2 CTAs (its larger staged
// sources want the bigger shared-memory share).
template <bool L>
struct NearCfg {
    static constexpr int threads = L ? 128 : 256;
    static constexpr int warps = threads / 32;
    static constexpr int ctas = L ? 5 : 2;          // per SM
    static constexpr int grid_per_sm = L ? 32 : 16;  // grid-stride launch size
    // dynamic shared memory per CTA; five float-float CTAs per SM fit with
    // 0.8 KB to spare (dynamic + 464 B static + the 1 KB the runtime
    // reserves per CTA, x 5, against 228 KB): more static shared memory in
    // the kernel drops it to four CTAs unless this shrinks
    static constexpr size_t budget = L ? 44 * 1024 : 110 * 1024;
};
constexpr int kQueue = 128;  // ring entries per warp and class (a sweep step adds up to 64)
constexpr int kGtab = FTE_E1_NPIECE_G * (FTE_E1_DEG_G + 1);
constexpr int kKtab = FTE_K_NPIECE * (FTE_K_DEG + 1);

struct NearParams {
    int nsx, nsy, nb;
    const int* __restrict__ src_off;
    const double2* __restrict__ spos;
    // densities of the sorted sources; vector v at q* + v * qstride
    const double* __restrict__ q0;  // SLP: f1 ; DLP: S11 = f1 n1
    const double* __restrict__ q1;  // SLP: f2 ; DLP: S12 + S21
    const double* __restrict__ q2;  // DLP: S22
    long long qstride;
    const int* __restrict__ tar_off;
    const double2* __restrict__ tpos;
    const int* __restrict__ tidx;
    double Lx, Ly, xi, xi2, inv_xi2, selfc, cutoffsq, pf;
    double bsx, bsy;  // box sides Lx / nsx, Ly / nsy
    float cut32;
    // pairs with xi^2 r^2 >= x32 are evaluated in FP32 (their terms are
    // below the tolerance's reach of FP32 rounding); +inf: all FP64
    float x32;
    // mixed form at tolerances the float-float class meets: the FP64 pairs
    // with x >= 1 are evaluated in float-float (ffnear = 1); constants as
    // float-float
    int ffnear;
    float2 xi2ff, pfff, cutff, selcff;
    // float-float class: per sorted source, its position relative to the
    // centre of its own box (x hi, x lo, y hi, y lo) and its staged density
    // values as float-float, value c of vector v at qff[(v * kDen + c) *
    // qffstride + i]; box sides as float-float (written by fte_near_ff_prep)
    const float4* __restrict__ sff;
    const float2* __restrict__ qff;
    long long qffstride;
    float2 bsxff, bsyff;
    int cap;
    double2* __restrict__ ur;  // vector v at ur + v * ustride
    long long ustride;
};

// centre of box (bx, by): the reference frame of the box-relative FP32 and
// float-float coordinates (the same expression wherever they are formed)
__device__ __forceinline__ double2 box_centre(const NearParams& prm, int bx, int by) {
    return make_double2(fma(bx + 0.5, prm.bsx, -0.5 * prm.Lx), fma(by + 0.5, prm.bsy, -0.5 * prm.Ly));
}

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

// exp(-x) for x >= 0 (0 beyond 700): 2^(-n/64) exp(-r) with n = round(64 x / ln 2),
// r = x - n ln2/64 (Cody-Waite), exp(-r) by its degree-6 Taylor polynomial
// (|r| <= ln2/128, truncation < 3e-20), 2^(-j/64) from a 64-entry table and
// the power of two applied to the exponent field.  11 FP64 operations.
__device__ __forceinline__ double fte_expm(double x, const double* __restrict__ tab) {
    const double magic = 6755399441055744.0;  // 1.5 * 2^52
    double t = fma(x, FTE_EXP_INV_LN2_64, magic);
    double nd = t - magic;
    int n = __double2loint(t);
    double r = fma(nd, -FTE_EXP_LN2_64_HI, x);
    r = fma(nd, -FTE_EXP_LN2_64_LO, r);
    double p = fte_exp_poly[6];
#pragma unroll
    for (int k = 5; k >= 0; k--) p = fma(p, r, fte_exp_poly[k]);
    double v = p * tab[n & 63];
    v = __hiloint2double(__double2hiint(v) - ((n >> 6) << 20), __double2loint(v));
    return x > 700.0 ? 0.0 : v;
}

// 1/a from the FP32 hardware reciprocal and two Newton steps in FP64.
__device__ __forceinline__ double fte_rcp(double a) {
    float af = __double2float_rn(a);
    float yf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(af));
    double y = (double)yf;
    double e = fma(-a, y, 1.0);
    y = fma(y, e, y);
    e = fma(-a, y, 1.0);
    return fma(y, e, y);
}

// K(x) = 0.5 e^x E1(x) - 1 for x >= 1 (eighth-octave pieces; a value marginally
// below 1, from the FP32 classification, extrapolates the first piece).
__device__ __forceinline__ double fte_kfun(double x, const double* __restrict__ ktab) {
    long long bits = __double_as_longlong(x);
    int e = (int)(bits >> 52) - 1023;
    int q = (int)((bits >> 49) & 7);
    double mant = __longlong_as_double((bits & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
    if (e < 0) {
        e = 0;
        q = 0;
        mant = x;
    } else if (e > 9) {  // exp(-x) underflows there; stay inside the table
        e = 9;
        q = 7;
        mant = 2.0;
    }
    double mid = __longlong_as_double(0x3FF0000000000000LL | ((long long)q << 49) | (1LL << 48));
    double t = (mant - mid) * 16.0;
    const double* c = ktab + (8 * e + q) * (FTE_K_DEG + 1);
    double k = c[FTE_K_DEG];
#pragma unroll
    for (int j = FTE_K_DEG - 1; j >= 0; j--) k = fma(k, t, c[j]);
    return k;
}

// The same K(x) in FP32 from an FP32 copy of the table (pairs of the FP32
// class only: x >= 1, relative error ~1e-7).
__device__ __forceinline__ float fte_kfun32(float x, const float* __restrict__ ktab) {
    int bits = __float_as_int(x);
    int e = (bits >> 23) - 127;
    int q = (bits >> 20) & 7;
    float mant = __int_as_float((bits & 0x007FFFFF) | 0x3F800000);
    if (e < 0) {
        e = 0;
        q = 0;
        mant = x;
    } else if (e > 9) {
        e = 9;
        q = 7;
        mant = 2.0f;
    }
    float mid = __int_as_float(0x3F800000 | (q << 20) | (1 << 19));
    float t = (mant - mid) * 16.0f;
    const float* c = ktab + (8 * e + q) * (FTE_K_DEG + 1);
    float k = c[FTE_K_DEG];
#pragma unroll
    for (int j = FTE_K_DEG - 1; j >= 0; j--) k = fmaf(k, t, c[j]);
    return k;
}

// K(x) in float-float from the float-float table (x >= 1 less a rounding
// margin): the piece and t from x.hi, t's low part from x.lo; Horner with
// the degree-10..5 terms in FP32 (relative size below 1e-7 of K) and the
// rest in float-float.  Relative error ~5e-15.
__device__ __forceinline__ float2 fte_kfun_ff(float2 x, const float2* __restrict__ ktab) {
    const int bits = __float_as_int(x.x);
    int e = (bits >> 23) - 127;
    int q = (bits >> 20) & 7;
    float mant = __int_as_float((bits & 0x007FFFFF) | 0x3F800000);
    float sc = __int_as_float((127 - e) << 23);  // 2^-e
    if (e < 0) {
        e = 0;
        q = 0;
        mant = x.x;
        sc = 1.0f;
    } else if (e > 9) {
        e = 9;
        q = 7;
        mant = 2.0f;
        sc = 0.0f;
    }
    const float mid = __int_as_float(0x3F800000 | (q << 20) | (1 << 19));
    const float2 t = ff_norm(__fmul_rn(__fsub_rn(mant, mid), 16.0f), __fmul_rn(__fmul_rn(x.y, sc), 16.0f));
    const float2* c = ktab + (8 * e + q) * (FTE_K_DEG + 1);
    float k = c[FTE_K_DEG].x;
#pragma unroll
    for (int j = FTE_K_DEG - 1; j >= 5; j--) k = __fmaf_rn(k, t.x, c[j].x);
    float2 kk = make_float2(k, 0.0f);
#pragma unroll
    for (int j = 4; j >= 0; j--) kk = ff_add(ff_mul(kk, t), c[j]);
    return kk;
}

// ln x in float-float for a normal x.hi > 0: x = m 2^e with m in [1, 2),
// y0 = logf(m) (about an ulp) and one Newton step y0 + m e^-y0 - 1, plus
// e ln 2.  Absolute error ~1e-13.
__device__ __forceinline__ float2 fte_log_ff(float2 x, const float2* __restrict__ etab) {
    const int e = (__float_as_int(x.x) >> 23) - 127;
    const float sc = __int_as_float((127 - e) << 23);  // 2^-e
    const float2 m = make_float2(__fmul_rn(x.x, sc), __fmul_rn(x.y, sc));
    const float y0 = logf(m.x);
    const float2 t = ff_add(ff_mul(m, fte_expm_ff(make_float2(y0, 0.0f), etab)), make_float2(-1.0f, 0.0f));
    const float2 y = ff_add(make_float2(y0, 0.0f), t);
    const float2 ln2 = make_float2(6.931471825e-01f, -1.904654212e-09f);
    return ff_add(y, ff_mulf(ln2, (float)e));
}

// 0.5 E1(x) - e^-x for 0 < x < 1 in float-float: E1 = -gamma - ln x +
// x R(2x - 1) with the degree-11..6 terms of R in FP32 (below 4e-7 of R) and
// the rest in float-float (R's coefficients as float-float in rtab).
// Absolute error ~1e-13.
__device__ __forceinline__ float2 fte_slp_small_ff(float2 x, float2 emx, const float2* __restrict__ rtab,
                                                   const float2* __restrict__ etab) {
    const float2 t = ff_add(make_float2(__fadd_rn(x.x, x.x), __fadd_rn(x.y, x.y)), make_float2(-1.0f, 0.0f));
    float k = rtab[FTE_E1_DEG_R].x;
#pragma unroll
    for (int j = FTE_E1_DEG_R - 1; j >= 6; j--) k = __fmaf_rn(k, t.x, rtab[j].x);
    float2 kk = make_float2(k, 0.0f);
#pragma unroll
    for (int j = 5; j >= 0; j--) kk = ff_add(ff_mul(kk, t), rtab[j]);
    const float2 g = make_float2(5.772156715e-01f, -6.637773886e-09f);  // Euler's gamma
    float2 E = ff_add(ff_mul(x, kk), ff_neg(g));
    E = ff_add(E, ff_neg(fte_log_ff(x, etab)));
    return ff_add(make_float2(__fmul_rn(E.x, 0.5f), __fmul_rn(E.y, 0.5f)), ff_neg(emx));
}

// Shared-memory layout of the near-field kernels (per CTA):
//   K(x) table, exp table, their float-float copies, FP32 K(x) table, then
//   per staged source: x, y (FP64), NV density sets (SLP: f1, f2; DLP: S11,
//   (S12+S21)/2, S22, S11+S22) in FP64 and in FP32, FP32 box-relative
//   position, and with the float-float class the low parts of the position
//   and the densities; then three 64-entry rings per warp.
template <int KIND, int NV>
struct NearSmem {
    static constexpr int kDen = KIND == FTE_KIND_SLP ? 2 : 4;
    // targets a warp keeps in flight (ring entries carry the slot): the
    // accumulators cost NSLOT * NV * 2 doubles per lane
    static constexpr int kSlots = NV == 1 ? 4 : (NV == 2 ? 2 : 1);
    // the float-float kernel: the Stokeslet with one vector keeps four
    // targets' sums in shared memory (a float4 per lane and slot: selecting
    // among four register copies cost more than the loads; 1e6 points:
    // near 3.31 -> 3.09 ms at tol 1e-10, 4.07 -> 2.87 ms at 1e-8); the
    // others keep two (one beyond two vectors) in registers, since the
    // stresslet's larger staged sources need that shared memory (its
    // neighbourhoods then split into more chunks: 2.48 -> 3.03 ms)
    static constexpr bool kAccSmem = KIND == FTE_KIND_SLP && NV == 1;
    static constexpr int kSlotsFF = kAccSmem ? 4 : (NV <= 2 ? 2 : 1);
    // doubles before the staged sources: the FP64 kernel's K(x) and exp
    // tables, or the float-float kernel's K(x), exp and small-x E1 tables,
    // then the FP32 K(x) table
    __host__ __device__ static constexpr int head(bool ff) {
        return (ff ? kKtab + 64 + 12 : kKtab + 64) + kKtab / 2 + 1;
    }
    // per staged source: FP64 layout (x, y, densities; FP32 copies) or, with
    // the float-float class, float-float only (position and densities as
    // FP32 + low part)
    __host__ __device__ static size_t per_source(bool ff) {
        return ff ? 2 * sizeof(float2) + 2 * kDen * NV * sizeof(float)
                  : (2 + kDen * NV) * sizeof(double) + sizeof(float2) + kDen * NV * sizeof(float);
    }
    __host__ __device__ static size_t acc_bytes(bool ff) {
        return ff && kAccSmem ? (size_t)NearCfg<true>::warps * kSlotsFF * NV * 32 * sizeof(float4) + 16 : 0;
    }
    __host__ __device__ static size_t bytes(int cap, bool ff) {
        return head(ff) * sizeof(double) + (size_t)cap * per_source(ff) +
               (ff ? NearCfg<true>::warps : NearCfg<false>::warps) * 3 * kQueue * sizeof(int) + acc_bytes(ff) + 64;
    }
};

// All targets of box b against the 3x3 neighbourhood of sources, for NV
// density vectors at once: the pair geometry and the special functions are
// evaluated once per pair and shared by the vectors.
template <int KIND, int NV, bool FF>
// (part `part` of `nparts` of the box's targets: a problem with fewer boxes
// than the GPU has CTA slots splits each box's targets over several CTAs)
__device__ __forceinline__ void near_box(const NearParams& prm, int b, int part, int nparts, unsigned char* smem_raw,
                                         int* nb_box, int* nb_start, double* nb_shx, double* nb_shy) {
    constexpr int kDen = NearSmem<KIND, NV>::kDen;
    // float-float class (FF)
    constexpr bool ffn = FF;
    constexpr int kNearThreads = NearCfg<ffn>::threads;
    constexpr int kNearWarps = NearCfg<ffn>::warps;
    // targets in flight (up to four for one density vector): a target's
    // sums stay open until the rings have evaluated its pairs, so that
    // batches fill up with later targets' pairs instead of being drained
    // half empty; the sums live in registers (selected per entry) except the
    // float-float Stokeslet's with one vector (shared memory, NearSmem)
    constexpr int NSLOT = ffn ? NearSmem<KIND, NV>::kSlotsFF : NearSmem<KIND, NV>::kSlots;
    const int cap = prm.cap;
    // tables: FP64 kernel: ktab, etab, ktab32; float-float kernel: ktabff,
    // etabff, rtabff, ktab32
    const double* ktab = reinterpret_cast<const double*>(smem_raw);
    const double* etab = ktab + kKtab;
    const float2* ktabff = reinterpret_cast<const float2*>(smem_raw);
    const float2* etabff = ktabff + kKtab;
    const float2* rtabff = etabff + 64;
    const float* ktab32 = ffn ? reinterpret_cast<const float*>(rtabff + 12) : reinterpret_cast<const float*>(etab + 64);
    // FP64 layout: x, y, densities (FP64), FP32 position, FP32 densities;
    // float-float layout: FP32 position, FP32 densities, their low parts
    double* const s0 = reinterpret_cast<double*>(smem_raw) + NearSmem<KIND, NV>::head(ffn);
    double* sx = ffn ? nullptr : s0;
    double* sy = ffn ? nullptr : s0 + cap;
    double* den = ffn ? nullptr : s0 + 2 * cap;  // den[(v * kDen + c) * cap + i]
    float2* s32 = ffn ? reinterpret_cast<float2*>(s0) : reinterpret_cast<float2*>(s0 + (size_t)(2 + kDen * NV) * cap);
    float* den32 = reinterpret_cast<float*>(s32 + cap);  // den32[(v * kDen + c) * cap + i]
    float2* slo = reinterpret_cast<float2*>(den32 + (size_t)kDen * NV * cap);
    float* dlo = reinterpret_cast<float*>(slo + (ffn ? cap : 0));
    int* qbuf = reinterpret_cast<int*>(dlo + (ffn ? (size_t)kDen * NV * cap : 0));
    // float-float class with sums in shared memory: [warp][slot][vector][lane]
    // (16-byte aligned)
    float4* const accs = reinterpret_cast<float4*>(
        (reinterpret_cast<uintptr_t>(qbuf + kNearWarps * 3 * kQueue) + 15) & ~static_cast<uintptr_t>(15));

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // per warp: ring 0 = pairs with x >= 1 (FP64, or float-float when ffn),
    // ring 1 = x < 1 (FP64; the stresslet's only with ffn, else its FP64
    // pairs all take ring 0), ring 2 = the FP32 class (x >= x32)
    int* qf = qbuf + warp * 3 * kQueue;
    int* qn = qf + kQueue;
    int* qs = qn + kQueue;
    // per warp and target slot: the target's position and its FP32-class sums
    // (ring entries carry the slot in two bits; the FP32-class sums of a
    // warp hold two components per slot and vector)
    static_assert(NSLOT >= 1 && NSLOT <= 4 && (NSLOT & (NSLOT - 1)) == 0, "target slots");
    constexpr int kFsum = 2 * NSLOT * NV > 8 ? 2 * NSLOT * NV : 8;
    __shared__ double2 tslot[kNearWarps * 4];
    __shared__ float4 tslot_ff[kNearWarps * 4];  // box-relative (x hi, x lo, y hi, y lo)
    __shared__ float fsum_all[kNearWarps * kFsum];
    double2* tsl = tslot + warp * 4;
    float4* tsf = tslot_ff + warp * 4;
    float* fsw = fsum_all + warp * kFsum;
    const float x32 = prm.x32;
    const float cutf = (float)prm.cutoffsq;
    const float pf32 = (float)prm.pf;
    const unsigned lt_mask = (1u << lane) - 1u;
    const double inv4pi = 1.0 / (4.0 * FTE_PI);
    const float xi2f = (float)prm.xi2;

    const int tb0 = prm.tar_off[b], ntb = prm.tar_off[b + 1] - tb0;
    int t0 = tb0, nt = ntb;
    if (nparts > 1) {
        t0 = tb0 + (int)((long long)ntb * part / nparts);
        nt = tb0 + (int)((long long)ntb * (part + 1) / nparts) - t0;
    }
    if (nt == 0) return;
    const int bx = b % prm.nsx, by = b / prm.nsx;
    __syncthreads();  // the previous box is done with the staging buffers
    if (tid < 9) {
        // own box first, then the reference's neighbour order (ilist_x/ilist_y)
        const int ox = tid == 0 ? 0 : (tid <= 3 ? -1 : (tid <= 5 ? 0 : 1));
        const int oy = tid == 0 ? 0 : ((tid == 1 || tid == 4 || tid == 6) ? -1 : ((tid == 2 || tid == 7) ? 0 : 1));
        int psx = bx + ox, psy = by + oy;
        int tx = (psx + prm.nsx) % prm.nsx, ty = (psy + prm.nsy) % prm.nsy;
        int sb = ty * prm.nsx + tx;
        nb_box[tid] = sb;
        if (!ffn) {  // image shifts (the float-float staging adds whole box sides instead)
            nb_shx[tid] = (prm.Lx * (psx - tx)) / prm.nsx;
            nb_shy[tid] = (prm.Ly * (psy - ty)) / prm.nsy;
        }
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
    const double2 bc = box_centre(prm, bx, by);
    const double cx = bc.x, cy = bc.y;

    if (S == 0) {
        for (int t = tid; t < nt; t += kNearThreads)
            for (int v = 0; v < NV; v++) prm.ur[v * prm.ustride + prm.tidx[t0 + t]] = make_double2(0.0, 0.0);
        return;
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
            if constexpr (ffn) {
                // own-box-relative position + the neighbour's offset (a whole
                // number of box sides), densities as prepared
                const int oxe = e == 0 ? 0 : (e <= 3 ? -1 : (e <= 5 ? 0 : 1));
                const int oye = e == 0 ? 0 : ((e == 1 || e == 4 || e == 6) ? -1 : ((e == 2 || e == 7) ? 0 : 1));
                const float4 r = prm.sff[si];
                const float2 px = ff_add(make_float2(r.x, r.y), make_float2(oxe * prm.bsxff.x, oxe * prm.bsxff.y));
                const float2 py = ff_add(make_float2(r.z, r.w), make_float2(oye * prm.bsyff.x, oye * prm.bsyff.y));
                s32[i] = make_float2(px.x, py.x);
                slo[i] = make_float2(px.y, py.y);
#pragma unroll
                for (int v = 0; v < NV; v++)
#pragma unroll
                    for (int c = 0; c < kDen; c++) {
                        const float2 q = prm.qff[(size_t)(v * kDen + c) * prm.qffstride + si];
                        den32[(size_t)(v * kDen + c) * cap + i] = q.x;
                        dlo[(size_t)(v * kDen + c) * cap + i] = q.y;
                    }
                continue;
            }
            double2 p = prm.spos[si];
            double xs = p.x + nb_shx[e], ys = p.y + nb_shy[e];
            sx[i] = xs;
            sy[i] = ys;
#pragma unroll
            for (int v = 0; v < NV; v++) {
                const long long o = v * prm.qstride + si;
                double* d = den + (size_t)v * kDen * cap + i;
                float* d32 = den32 + (size_t)v * kDen * cap + i;
                if (KIND == FTE_KIND_SLP) {
                    d[0] = prm.q0[o];
                    d[cap] = prm.q1[o];
                    d32[0] = (float)d[0];
                    d32[cap] = (float)d[cap];
                } else {
                    // S11, (S12 + S21)/2, S22, S11 + S22
                    double s11 = prm.q0[o], ssym = prm.q1[o], s22 = prm.q2[o];
                    d[0] = s11;
                    d[cap] = 0.5 * ssym;
                    d[2 * cap] = s22;
                    d[3 * cap] = s11 + s22;
                    d32[0] = (float)s11;
                    d32[cap] = (float)(0.5 * ssym);
                    d32[2 * cap] = (float)s22;
                    d32[3 * cap] = (float)(s11 + s22);
                }
            }
            s32[i] = make_float2((float)(xs - cx), (float)(ys - cy));
        }
        __syncthreads();
        const int own_lim = n_own - chunk;  // local index < own_lim: own box

        // A warp keeps up to NSLOT of its targets in flight.  FP64 ring
        // entries are (staged source << 2 | slot), the lanes accumulate per
        // slot, and a target is reduced once the rings have passed every
        // entry it pushed: the batch that would end one target's sweep half
        // empty fills up with the next targets' pairs instead.  The FP32 class
        // is cheap and is finished per target.
        const int ntw = warp < nt ? (nt - warp + kNearWarps - 1) / kNearWarps : 0;
        // x below which a Stokeslet pair takes ring qn
        const float xsplit = 1.0f;
        // Stokeslet with the FP32 class from x = 1 (tol >= ~7e-8): ring qf
        // (1 <= x < x32) stays empty, its ballots and stores are skipped
        const bool slp_no_f = KIND == FTE_KIND_SLP && x32 <= xsplit;
        int Pf = 0, Ef = 0, Pn = 0, En = 0;  // pushed / evaluated counts of rings qf, qn
        int tailF[NSLOT], tailN[NSLOT];      // Pf, Pn after each slot's sweep
        double acc[NSLOT][NV][2];
        // float-float class: (sum, low parts) per component per slot, in
        // registers or (kAccSmem) this lane's entries in shared memory
        constexpr bool acc_smem = NearSmem<KIND, NV>::kAccSmem;
        float4* const accw = accs + (size_t)warp * NSLOT * NV * 32 + lane;
        float accf[acc_smem ? 1 : NSLOT][NV][4];
        float acc32[NV][2];
#pragma unroll
        for (int j = 0; j < NSLOT; j++) {
            tailF[j] = tailN[j] = 0;
#pragma unroll
            for (int v = 0; v < NV; v++) {
                acc[j][v][0] = acc[j][v][1] = 0.0;
                if constexpr (acc_smem) {
                    if (ffn) accw[(j * NV + v) * 32] = make_float4(0.f, 0.f, 0.f, 0.f);
                } else {
                    accf[j][v][0] = accf[j][v][1] = accf[j][v][2] = accf[j][v][3] = 0.0f;
                }
            }
        }
#pragma unroll
        for (int v = 0; v < NV; v++) acc32[v][0] = acc32[v][1] = 0.0f;
        float tx32 = 0.0f, ty32 = 0.0f;  // box-relative position of the target being swept
        // FP64 accumulators in use (the float-float form has no FP64 pairs)
        constexpr bool any64 = !ffn;

        // slot `tag`'s accumulators of vector v, selected into (a0, a1) and
        // back: selects only (written as conditional expressions, which
        // compile to selects rather than branches), no FP64 work per slot
        auto acc_get = [&](int tag, int v, double& a0, double& a1) {
            a0 = acc[0][v][0];
            a1 = acc[0][v][1];
#pragma unroll
            for (int j = 1; j < NSLOT; j++)
                {
                    const bool m = tag == j;
                    a0 = m ? acc[j][v][0] : a0;
                    a1 = m ? acc[j][v][1] : a1;
                }
        };
        auto acc_put = [&](int tag, int v, double a0, double a1) {
#pragma unroll
            for (int j = 0; j < NSLOT; j++)
                {
                    const bool m = tag == j;
                    acc[j][v][0] = m ? a0 : acc[j][v][0];
                    acc[j][v][1] = m ? a1 : acc[j][v][1];
                }
        };
        // (each lane reads and writes only its own entries: no barrier)
        // (selects written as conditional expressions, no branches)
        auto accf_get = [&](int tag, int v, float* a) {
            if constexpr (acc_smem) {
                const float4 t = accw[(tag * NV + v) * 32];
                a[0] = t.x;
                a[1] = t.y;
                a[2] = t.z;
                a[3] = t.w;
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++) a[i] = accf[0][v][i];
#pragma unroll
                for (int j = 1; j < NSLOT; j++) {
                    const bool m = tag == j;
#pragma unroll
                    for (int i = 0; i < 4; i++) a[i] = m ? accf[j][v][i] : a[i];
                }
            }
        };
        auto accf_put = [&](int tag, int v, const float* a) {
            if constexpr (acc_smem) {
                accw[(tag * NV + v) * 32] = make_float4(a[0], a[1], a[2], a[3]);
            } else {
#pragma unroll
                for (int j = 0; j < NSLOT; j++) {
                    const bool m = tag == j;
#pragma unroll
                    for (int i = 0; i < 4; i++) accf[j][v][i] = m ? a[i] : accf[j][v][i];
                }
            }
        };

        // FP32 class: the same pair terms in FP32 from box-relative
        // positions, accumulated per lane in FP32 for the target being swept
        auto eval_slp32 = [&](int s) {
            const float2 q = s32[s];
            const float dx = tx32 - q.x, dy = ty32 - q.y;
            const float r2 = fmaf(dx, dx, dy * dy);
            if (!(s < own_lim) && !(r2 < cutf)) return;
            const float x = r2 * xi2f;
            const float e = expf(-x);
            const float A = e * fte_kfun32(x, ktab32);
            const float gr = __fdividef(e, r2);
#pragma unroll
            for (int v = 0; v < NV; v++) {
                const float* d = den32 + (size_t)v * 2 * cap + s;
                const float fx = d[0], fy = d[cap];
                const float c = gr * fmaf(dx, fx, dy * fy);
                acc32[v][0] = fmaf(A, fx, fmaf(c, dx, acc32[v][0]));
                acc32[v][1] = fmaf(A, fy, fmaf(c, dy, acc32[v][1]));
            }
        };
        auto eval_dlp32 = [&](int s) {
            const float2 q = s32[s];
            const float dx = tx32 - q.x, dy = ty32 - q.y;
            const float r2 = fmaf(dx, dx, dy * dy);
            if (!(s < own_lim) && !(r2 < cutf)) return;
            const float x = r2 * xi2f;
            const float e2 = expf(-x);
            const float ir2 = __frcp_rn(r2);
            const float facb = -4.0f * (1.0f + x) * ir2 * ir2;
#pragma unroll
            for (int v = 0; v < NV; v++) {
                const float* d = den32 + (size_t)v * 4 * cap + s;
                const float s11 = d[0], h = d[cap], s22 = d[2 * cap], tr = d[3 * cap];
                const float u = fmaf(dx, s11, dy * h);
                const float w = fmaf(dy, s22, dx * h);
                const float fQ = facb * fmaf(dx, u, dy * w);
                const float w1 = fmaf(dx, tr, u + u);
                const float w2 = fmaf(dy, tr, w + w);
                acc32[v][0] = fmaf(e2, fmaf(fQ, dx, pf32 * w1), acc32[v][0]);
                acc32[v][1] = fmaf(e2, fmaf(fQ, dy, pf32 * w2), acc32[v][1]);
            }
        };

        // Stokeslet pair (mex_stokes_slp_real.cpp:161-225 / 264-323):
        //   u += (0.5 E1(x) - e^-x) f + e^-x (r.f) r / r^2,   x = xi^2 r^2
        auto eval_slp = [&](int ent, bool small_x) {
            const int s = ent >> 2, tag = ent & 3;
            const double2 tp = tsl[tag];
            double dx = tp.x - sx[s], dy = tp.y - sy[s];
            double r2 = fma(dx, dx, dy * dy);
            bool own = s < own_lim;
            if (own && fabs(r2) < 1e-15) {
#pragma unroll
                for (int v = 0; v < NV; v++) {
                    const double* d = den + (size_t)v * 2 * cap + s;
                    double a0, a1;
                    acc_get(tag, v, a0, a1);
                    a0 = fma(prm.selfc, d[0], a0);
                    a1 = fma(prm.selfc, d[cap], a1);
                    acc_put(tag, v, a0, a1);
                }
                return;
            }
            if (!own && !(r2 < prm.cutoffsq)) return;
            double x = r2 * prm.xi2;
            double emx = fte_expm(x, etab);
            double A;
            if (small_x) {
                double tt = fma(2.0, x, -1.0);
                double R = fte_e1_coef_r[FTE_E1_DEG_R];
#pragma unroll
                for (int k = FTE_E1_DEG_R - 1; k >= 0; k--) R = fma(R, tt, fte_e1_coef_r[k]);
                double E = fma(x, R, -FTE_EULER - log(x));
                A = fma(0.5, E, -emx);
            } else {
                A = emx * fte_kfun(x, ktab);
            }
            double gr = emx * fte_rcp(r2);
#pragma unroll
            for (int v = 0; v < NV; v++) {
                const double* d = den + (size_t)v * 2 * cap + s;
                double fx = d[0], fy = d[cap];
                double c = gr * fma(dx, fx, dy * fy);
                double a0, a1;
                acc_get(tag, v, a0, a1);
                a0 = fma(A, fx, fma(c, dx, a0));
                a1 = fma(A, fy, fma(c, dy, a1));
                acc_put(tag, v, a0, a1);
            }
        };
        // stresslet pair (mex_stokes_dlp_real.cpp:117-138 / 162-181):
        //   u_i += e^-x [ -4 (1+x) r_i (r.S.r)/r^4 + 2 xi^2 (f_i (r.n) + n_i (r.f) + (f.n) r_i) ]
        auto eval_dlp = [&](int ent) {
            const int s = ent >> 2, tag = ent & 3;
            const double2 tp = tsl[tag];
            double dx = tp.x - sx[s], dy = tp.y - sy[s];
            double r2 = fma(dx, dx, dy * dy);
            bool own = s < own_lim;
            if (own ? (r2 == 0.0) : !(r2 < prm.cutoffsq)) return;
            double x = r2 * prm.xi2;
            double e2 = fte_expm(x, etab);
            double ir2 = fte_rcp(r2);
            double facb = -4.0 * (1.0 + x) * ir2 * ir2;
#pragma unroll
            for (int v = 0; v < NV; v++) {
                const double* d = den + (size_t)v * 4 * cap + s;
                double s11 = d[0], h = d[cap], s22 = d[2 * cap], tr = d[3 * cap];
                double u = fma(dx, s11, dy * h);  // (S r)_1 with S symmetrised
                double w = fma(dy, s22, dx * h);  // (S r)_2
                double Q = fma(dx, u, dy * w);    // r.S.r
                double fQ = facb * Q;
                double w1 = fma(dx, tr, u + u);   // f_1 (r.n) + n_1 (r.f) + (f.n) r_1
                double w2 = fma(dy, tr, w + w);
                double a0, a1;
                acc_get(tag, v, a0, a1);
                a0 = fma(e2, fma(fQ, dx, prm.pf * w1), a0);
                a1 = fma(e2, fma(fQ, dy, prm.pf * w2), a1);
                acc_put(tag, v, a0, a1);
            }
        };

        // The same pair terms in float-float (pairs with x >= 1 at mixed-form
        // tolerances from 1e-11): box-relative positions and densities as
        // (FP32, low part), relative error ~1e-13 per term.
        auto ff_geom = [&](int s, int tag, float2& dx, float2& dy, float2& r2) {
            const float4 tq = tsf[tag];
            const float2 sh = s32[s], sl = slo[s];
            dx = ff_add(make_float2(tq.x, tq.y), make_float2(-sh.x, -sl.x));
            dy = ff_add(make_float2(tq.z, tq.w), make_float2(-sh.y, -sl.y));
            r2 = ff_add(ff_sqr(dx), ff_sqr(dy));
        };
        // u += A f + gr (r.f) r for every vector (Stokeslet, float-float)
        auto slp_ff_add = [&](int s, int tag, float2 dx, float2 dy, float2 A, float2 gr) {
#pragma unroll
            for (int v = 0; v < NV; v++) {
                const float* d = den32 + (size_t)v * 2 * cap + s;
                const float* dl = dlo + (size_t)v * 2 * cap + s;
                const float2 fx = make_float2(d[0], dl[0]), fy = make_float2(d[cap], dl[cap]);
                const float2 c = ff_mul(gr, ff_add(ff_mul(dx, fx), ff_mul(dy, fy)));
                float a[4];
                accf_get(tag, v, a);
                ff_acc(ff_add(ff_mul(A, fx), ff_mul(c, dx)), a[0], a[1]);
                ff_acc(ff_add(ff_mul(A, fy), ff_mul(c, dy)), a[2], a[3]);
                accf_put(tag, v, a);
            }
        };
        // x >= 1: A = e^-x K(x)
        auto eval_slp_ff = [&](int ent) {
            {
                const int s = ent >> 2, tag = ent & 3;
                float2 dx, dy, r2;
                ff_geom(s, tag, dx, dy, r2);
                if (!(s < own_lim) && !ff_lt(r2, prm.cutff)) return;
                const float2 x = ff_mul(r2, prm.xi2ff);
                const float2 emx = fte_expm_ff(x, etabff);
                slp_ff_add(s, tag, dx, dy, ff_mul(emx, fte_kfun_ff(x, ktabff)), ff_mul(emx, ff_rcp(r2)));
            }
        };
        // x < 1: A = 0.5 E1(x) - e^-x by its series; the self term
        // (-1 - gamma/2 - log xi) f for a coincident source of the own box
        auto eval_slp_ff_small = [&](int ent) {
            {
                const int s = ent >> 2, tag = ent & 3;
                float2 dx, dy, r2;
                ff_geom(s, tag, dx, dy, r2);
                const bool own = s < own_lim;
                if (own && r2.x < 1e-15f) {
#pragma unroll
                    for (int v = 0; v < NV; v++) {
                        const float* d = den32 + (size_t)v * 2 * cap + s;
                        const float* dl = dlo + (size_t)v * 2 * cap + s;
                        float a[4];
                        accf_get(tag, v, a);
                        ff_acc(ff_mul(prm.selcff, make_float2(d[0], dl[0])), a[0], a[1]);
                        ff_acc(ff_mul(prm.selcff, make_float2(d[cap], dl[cap])), a[2], a[3]);
                        accf_put(tag, v, a);
                    }
                    return;
                }
                if (!own && !ff_lt(r2, prm.cutff)) return;
                const float2 x = ff_mul(r2, prm.xi2ff);
                const float2 emx = fte_expm_ff(x, etabff);
                slp_ff_add(s, tag, dx, dy, fte_slp_small_ff(x, emx, rtabff, etabff), ff_mul(emx, ff_rcp(r2)));
            }
        };
        auto eval_dlp_ff = [&](int ent) {
            {
                const int s = ent >> 2, tag = ent & 3;
                float2 dx, dy, r2;
                ff_geom(s, tag, dx, dy, r2);
                if (s < own_lim ? (r2.x == 0.0f && r2.y == 0.0f) : !ff_lt(r2, prm.cutff)) return;
                const float2 x = ff_mul(r2, prm.xi2ff);
                const float2 e2 = fte_expm_ff(x, etabff);
                const float2 ir2 = ff_rcp(r2);
                const float2 facb = ff_mulf(ff_mul(ff_add(make_float2(1.0f, 0.0f), x), ff_sqr(ir2)), -4.0f);
#pragma unroll
                for (int v = 0; v < NV; v++) {
                    const float* d = den32 + (size_t)v * 4 * cap + s;
                    const float* dl = dlo + (size_t)v * 4 * cap + s;
                    const float2 s11 = make_float2(d[0], dl[0]), h = make_float2(d[cap], dl[cap]);
                    const float2 s22 = make_float2(d[2 * cap], dl[2 * cap]), tr = make_float2(d[3 * cap], dl[3 * cap]);
                    const float2 u = ff_add(ff_mul(dx, s11), ff_mul(dy, h));
                    const float2 w = ff_add(ff_mul(dy, s22), ff_mul(dx, h));
                    const float2 fQ = ff_mul(facb, ff_add(ff_mul(dx, u), ff_mul(dy, w)));
                    const float2 w1 = ff_add(ff_mul(dx, tr), make_float2(2.0f * u.x, 2.0f * u.y));
                    const float2 w2 = ff_add(ff_mul(dy, tr), make_float2(2.0f * w.x, 2.0f * w.y));
                    const float2 t0 = ff_add(ff_mul(fQ, dx), ff_mul(prm.pfff, w1));
                    const float2 t1 = ff_add(ff_mul(fQ, dy), ff_mul(prm.pfff, w2));
                    float a[4];
                    accf_get(tag, v, a);
                    ff_acc(ff_mul(e2, t0), a[0], a[1]);
                    ff_acc(ff_mul(e2, t1), a[2], a[3]);
                    accf_put(tag, v, a);
                }
            }
        };
        // ring qf: the Stokeslet's x >= 1 and every stresslet pair; ring qn:
        // the Stokeslet's x < 1 (float-float when ffn, else FP64)
        auto evalF = [&](int ent) {
            if (KIND == FTE_KIND_SLP) {
                if (ffn)
                    eval_slp_ff(ent);
                else
                    eval_slp(ent, false);
            } else {
                if (ffn)
                    eval_dlp_ff(ent);
                else
                    eval_dlp(ent);
            }
        };
        auto evalN = [&](int ent) {
            if (KIND == FTE_KIND_SLP) {
                if (ffn)
                    eval_slp_ff_small(ent);
                else
                    eval_slp(ent, true);
            } else {
                eval_dlp(ent);
            }
        };

        // evaluate everything pending in ring qf (if df) and qn (if dn);
        // both hold fewer than 32 entries here
        // (one call site per ring: each inlined copy of a pair evaluation
        // is hundreds of instructions, and copies at several sites made
        // the kernel wait on instruction fetch)
        auto drain = [&](bool df, bool dn) {
            const int cf = df ? Pf - Ef : 0, cn = dn ? Pn - En : 0;
            // the two rings share one pass when they fit in a warp (the two
            // divergent halves run one after the other either way)
            const bool one = cf + cn <= 32;
            const int ln = one ? lane - cf : lane;
            if (lane < cf) evalF(qf[(Ef + lane) & (kQueue - 1)]);
            if (ln >= 0 && ln < cn) evalN(qn[(En + ln) & (kQueue - 1)]);
            Ef += cf;
            En += cn;
            __syncwarp();
        };

        // target kk of this warp: finish its pairs, reduce its slot, store
        auto finalize = [&](int kk) {
            const int sl = kk & (NSLOT - 1);
            int tf = tailF[0], tn = tailN[0];
#pragma unroll
            for (int j = 1; j < NSLOT; j++)
                if (sl == j) tf = tailF[j], tn = tailN[j];
            const bool df = Ef < tf, dn = En < tn;
            if (df || dn) drain(df, dn);
            const int oi = prm.tidx[t0 + warp + kk * kNearWarps];
            const bool hi = (lane & 16) != 0;
#pragma unroll
            for (int v = 0; v < NV; v++) {
                // lanes 0-15 reduce component 0, lanes 16-31 component 1
                double keep = 0.0;
                if constexpr (any64) {
                    double a0, a1;
                    acc_get(sl, v, a0, a1);
                    keep = hi ? a1 : a0;
                    keep += __shfl_xor_sync(0xffffffffu, hi ? a0 : a1, 16);
#pragma unroll
                    for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
                    acc_put(sl, v, 0.0, 0.0);
                }
                if (ffn) {
                    // the float-float and FP32 sums, reduced in float-float
                    float a[4];
                    accf_get(sl, v, a);
                    float2 kf = hi ? make_float2(a[2], a[3]) : make_float2(a[0], a[1]);
                    const float2 sf = hi ? make_float2(a[0], a[1]) : make_float2(a[2], a[3]);
                    kf = ff_add(kf, make_float2(__shfl_xor_sync(0xffffffffu, sf.x, 16),
                                                __shfl_xor_sync(0xffffffffu, sf.y, 16)));
#pragma unroll
                    for (int o = 8; o > 0; o >>= 1)
                        kf = ff_add(kf, make_float2(__shfl_xor_sync(0xffffffffu, kf.x, o),
                                                    __shfl_xor_sync(0xffffffffu, kf.y, o)));
                    a[0] = a[1] = a[2] = a[3] = 0.0f;
                    accf_put(sl, v, a);
                    if ((lane & 15) == 0) {
                        kf = ff_add(kf, make_float2(fsw[(sl * NV + v) * 2 + (hi ? 1 : 0)], 0.0f));
                        const float2 i4p = make_float2(7.957746834e-02f, 3.210319122e-09f);  // 1 / (4 pi)
                        double val = ff_join(ff_mul(kf, i4p));
                        if constexpr (any64) val = fma(keep, inv4pi, val);
                        double* o = reinterpret_cast<double*>(prm.ur + v * prm.ustride + oi) + (hi ? 1 : 0);
                        if (chunk == 0)
                            *o = val;
                        else
                            *o += val;
                    }
                    continue;
                }
                if ((lane & 15) == 0) {
                    const double val = (keep + (double)fsw[(sl * NV + v) * 2 + (hi ? 1 : 0)]) * inv4pi;
                    double* o = reinterpret_cast<double*>(prm.ur + v * prm.ustride + oi) + (hi ? 1 : 0);
                    if (chunk == 0)
                        *o = val;
                    else
                        *o += val;
                }
            }
        };

        // the warp's next 32 targets are read and converted by its lanes at
        // once (lane l: target k0 + l); the one being swept is taken from
        // its lane
        double2 tpl = make_double2(0.0, 0.0);
        float4 tfl = make_float4(0.f, 0.f, 0.f, 0.f);
        // NSLOT - 1 steps past the last target finalize the targets still
        // in flight (one finalize site; its drain evaluates what the rings
        // still hold)
        for (int k = 0; k < ntw + NSLOT - 1; k++) {
            if (k < ntw) {
                const int slot = k & (NSLOT - 1);
                if ((k & 31) == 0 && k + lane < ntw) {
                    tpl = prm.tpos[t0 + warp + (k + lane) * kNearWarps];
                    const double rx = tpl.x - cx, ry = tpl.y - cy;
                    if (ffn) {
                        const float2 fx = ff_split(rx), fy = ff_split(ry);
                        tfl = make_float4(fx.x, fx.y, fy.x, fy.y);
                    } else {
                        tfl = make_float4((float)rx, 0.f, (float)ry, 0.f);
                    }
                }
                if (lane == (k & 31)) {
                    tsl[slot] = tpl;
                    tsf[slot] = tfl;
                }
                tx32 = __shfl_sync(0xffffffffu, tfl.x, k & 31);
                ty32 = __shfl_sync(0xffffffffu, tfl.z, k & 31);
                __syncwarp();
                int hs = 0, cs = 0;  // FP32-class ring head and count

                // candidate test of staged source s against the target being swept
                auto test = [&](int s, bool& pass, bool& small_x, bool& single) {
                    pass = small_x = single = false;
                    if (s < clen) {
                        const float2 q = s32[s];
                        float dx = q.x - tx32, dy = q.y - ty32;
                        float r2f = dx * dx + dy * dy;
                        pass = (s < own_lim) || (r2f < prm.cut32);
                        const float xf = r2f * xi2f;
                        small_x = xf < xsplit;
                        single = xf >= x32;
                    }
                };
                // NB = 2 batches of 32 candidates per step: independent tests in
                // flight and one set of ring updates (measured at 1e6 points:
                // stresslet near 8-9 % faster at tol 1e-10 and 1e-6, Stokeslet
                // 9 % faster at 1e-6 and 2 % slower at 1e-10).  The rings hold up
                // to 31 + 64 entries, and every full batch of 32 is evaluated
                // before the next step from a single call site each.
                constexpr int NB = 2;
                for (int base = 0; base < clen; base += 32 * NB) {
                    const int s0 = base + lane, s1 = base + 32 + lane;
                    bool p0, x0, g0, p1 = false, x1 = false, g1 = false;
                    test(s0, p0, x0, g0);
                    if constexpr (NB == 2) test(s1, p1, x1, g1);
                    {
                        const bool a0 = p0 && g0, a1 = p1 && g1;
                        const unsigned m0 = __ballot_sync(0xffffffffu, a0), m1 = NB == 2 ? __ballot_sync(0xffffffffu, a1) : 0u;
                        const int c0 = __popc(m0);
                        if (a0) qs[(hs + cs + __popc(m0 & lt_mask)) & (kQueue - 1)] = s0;
                        if (a1) qs[(hs + cs + c0 + __popc(m1 & lt_mask)) & (kQueue - 1)] = s1;
                        cs += c0 + __popc(m1);
                        p0 = p0 && !g0;
                        p1 = p1 && !g1;
                        __syncwarp();
                        while (cs >= 32) {
                            if (KIND == FTE_KIND_SLP)
                                eval_slp32(qs[(hs + lane) & (kQueue - 1)]);
                            else
                                eval_dlp32(qs[(hs + lane) & (kQueue - 1)]);
                            hs = (hs + 32) & (kQueue - 1);
                            cs -= 32;
                            __syncwarp();
                        }
                    }
                    const int e0 = (s0 << 2) | slot, e1 = (s1 << 2) | slot;
                    // the Stokeslet's pairs with x < 1 take ring qn (the series of
                    // E1); the stresslet has one pair formula
                    if constexpr (KIND == FTE_KIND_SLP) {
                        const bool f0 = p0 && !x0, n0 = p0 && x0, f1 = p1 && !x1, n1 = p1 && x1;
                        if (!slp_no_f) {
                            const unsigned mf0 = __ballot_sync(0xffffffffu, f0);
                            const unsigned mf1 = NB == 2 ? __ballot_sync(0xffffffffu, f1) : 0u;
                            const int cf0 = __popc(mf0);
                            if (f0) qf[(Pf + __popc(mf0 & lt_mask)) & (kQueue - 1)] = e0;
                            if (f1) qf[(Pf + cf0 + __popc(mf1 & lt_mask)) & (kQueue - 1)] = e1;
                            Pf += cf0 + __popc(mf1);
                        }
                        const unsigned mn0 = __ballot_sync(0xffffffffu, n0), mn1 = NB == 2 ? __ballot_sync(0xffffffffu, n1) : 0u;
                        const int cn0 = __popc(mn0);
                        if (n0) qn[(Pn + __popc(mn0 & lt_mask)) & (kQueue - 1)] = e0;
                        if (n1) qn[(Pn + cn0 + __popc(mn1 & lt_mask)) & (kQueue - 1)] = e1;
                        Pn += cn0 + __popc(mn1);
                    } else {
                        const unsigned mf0 = __ballot_sync(0xffffffffu, p0), mf1 = NB == 2 ? __ballot_sync(0xffffffffu, p1) : 0u;
                        const int cf0 = __popc(mf0);
                        if (p0) qf[(Pf + __popc(mf0 & lt_mask)) & (kQueue - 1)] = e0;
                        if (p1) qf[(Pf + cf0 + __popc(mf1 & lt_mask)) & (kQueue - 1)] = e1;
                        Pf += cf0 + __popc(mf1);
                    }
                    __syncwarp();
                    while (Pf - Ef >= 32) {
                        evalF(qf[(Ef + lane) & (kQueue - 1)]);
                        Ef += 32;
                        __syncwarp();
                    }
                    if constexpr (KIND == FTE_KIND_SLP) {
                        while (Pn - En >= 32) {
                            evalN(qn[(En + lane) & (kQueue - 1)]);
                            En += 32;
                            __syncwarp();
                        }
                    }
                }
                // the target's FP32 class: last partial batch, then its sums
                // (lanes 0-15 reduce component 0, lanes 16-31 component 1)
                if (lane < cs) {
                    if (KIND == FTE_KIND_SLP)
                        eval_slp32(qs[(hs + lane) & (kQueue - 1)]);
                    else
                        eval_dlp32(qs[(hs + lane) & (kQueue - 1)]);
                }
                {
                    const bool hi = (lane & 16) != 0;
#pragma unroll
                    for (int v = 0; v < NV; v++) {
                        float keep = hi ? acc32[v][1] : acc32[v][0];
                        keep += __shfl_xor_sync(0xffffffffu, hi ? acc32[v][0] : acc32[v][1], 16);
#pragma unroll
                        for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
                        if ((lane & 15) == 0) fsw[(slot * NV + v) * 2 + (hi ? 1 : 0)] = keep;
                        acc32[v][0] = acc32[v][1] = 0.0f;
                    }
                }
#pragma unroll
                for (int j = 0; j < NSLOT; j++)
                    if (slot == j) tailF[j] = Pf, tailN[j] = Pn;
            }
            // the oldest target in flight gives up its slot to target k + 1
            if (k >= NSLOT - 1) finalize(k - (NSLOT - 1));
        }
        __syncwarp();
    }
}

template <int KIND, int NV, bool FF>
__device__ __forceinline__ void near_load_tables(unsigned char* smem_raw) {
    constexpr bool ffn = FF;
    constexpr int kNearThreads = NearCfg<FF>::threads;
    if constexpr (ffn) {
        float2* ktabff = reinterpret_cast<float2*>(smem_raw);
        float2* etabff = ktabff + kKtab;
        float2* rtabff = etabff + 64;
        float* ktab32 = reinterpret_cast<float*>(rtabff + 12);
        for (int i = threadIdx.x; i < kKtab; i += kNearThreads) {
            const double c = (&fte_k_coef[0][0])[i];
            ktabff[i] = ff_split(c);
            ktab32[i] = (float)c;
        }
        for (int i = threadIdx.x; i < 64; i += kNearThreads) etabff[i] = ff_split(fte_exp_tab[i]);
        static_assert(FTE_E1_DEG_R + 1 <= 12, "small-x E1 table");
        for (int i = threadIdx.x; i <= FTE_E1_DEG_R; i += kNearThreads) rtabff[i] = ff_split(fte_e1_coef_r[i]);
    } else {
        double* ktab = reinterpret_cast<double*>(smem_raw);
        double* etab = ktab + kKtab;
        float* ktab32 = reinterpret_cast<float*>(etab + 64);
        for (int i = threadIdx.x; i < kKtab; i += kNearThreads) {
            const double c = (&fte_k_coef[0][0])[i];
            ktab[i] = c;
            ktab32[i] = (float)c;
        }
        for (int i = threadIdx.x; i < 64; i += kNearThreads) etab[i] = fte_exp_tab[i];
    }
}

// one problem: grid-stride over its boxes
template <int KIND, int NV, bool FF>
__global__ void __launch_bounds__(NearCfg<FF>::threads, NearCfg<FF>::ctas) k_near(const NearParams prm,
                                                                                   int nparts) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int nb_box[9], nb_start[10];
    __shared__ double nb_shx[9], nb_shy[9];
    near_load_tables<KIND, NV, FF>(smem_raw);
    for (int u = blockIdx.x; u < prm.nb * nparts; u += gridDim.x) {
        const int b = nparts > 1 ? u / nparts : u, part = nparts > 1 ? u % nparts : 0;
        near_box<KIND, NV, FF>(prm, b, part, nparts, smem_raw, nb_box, nb_start, nb_shx, nb_shy);
    }
}

// many problems: grid-stride over a (problem, box) work list; descriptions
// are stored in NearParamsHost slots (kParamStride bytes apart)
constexpr int kParamStride = sizeof(NearParamsHost);

template <int KIND, int NV, bool FF>
__global__ void __launch_bounds__(NearCfg<FF>::threads, NearCfg<FF>::ctas) k_near_batch(const unsigned char* __restrict__ plist,
                                                                const int2* __restrict__ items, int nitems) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int nb_box[9], nb_start[10];
    __shared__ double nb_shx[9], nb_shy[9];
    near_load_tables<KIND, NV, FF>(smem_raw);
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 w = items[it];
        // read in place (a register copy of the description would spill)
        const NearParams& prm = *reinterpret_cast<const NearParams*>(plist + (size_t)w.x * kParamStride);
        near_box<KIND, NV, FF>(prm, w.y, 0, 1, smem_raw, nb_box, nb_start, nb_shx, nb_shy);
    }
}

// Float-float data of the sorted sources for nv density vectors: position
// relative to the centre of the source's own box, and the staged density
// values (SLP: f1, f2; DLP: S11, (S12 + S21)/2, S22, S11 + S22) as
// float-float.  A warp per box.
// box b of one description, by one warp
template <int KIND>
__device__ __forceinline__ void near_ff_prep_box(const NearParams& prm, int nv, int b, float4* __restrict__ sff,
                                                 float2* __restrict__ qff) {
    constexpr int kDen = KIND == FTE_KIND_SLP ? 2 : 4;
    const int lane = threadIdx.x & 31;
    {
        const int bx = b % prm.nsx, by = b / prm.nsx;
        const double2 bc = box_centre(prm, bx, by);
        const double cx = bc.x, cy = bc.y;
        const int i1 = prm.src_off[b + 1];
        for (int i = prm.src_off[b] + lane; i < i1; i += 32) {
            const double2 p = prm.spos[i];
            const float2 fx = ff_split(p.x - cx), fy = ff_split(p.y - cy);
            sff[i] = make_float4(fx.x, fx.y, fy.x, fy.y);
            for (int v = 0; v < nv; v++) {
                const long long o = v * prm.qstride + i;
                float2* q = qff + (size_t)v * kDen * prm.qffstride + i;
                if (KIND == FTE_KIND_SLP) {
                    q[0] = ff_split(prm.q0[o]);
                    q[prm.qffstride] = ff_split(prm.q1[o]);
                } else {
                    const double s11 = prm.q0[o], s22 = prm.q2[o];
                    q[0] = ff_split(s11);
                    q[prm.qffstride] = ff_split(0.5 * prm.q1[o]);
                    q[2 * prm.qffstride] = ff_split(s22);
                    q[3 * prm.qffstride] = ff_split(s11 + s22);
                }
            }
        }
    }
}

template <int KIND>
__global__ void k_near_ff_prep(const NearParams prm, int nv, float4* __restrict__ sff, float2* __restrict__ qff) {
    const int wpb = blockDim.x >> 5;
    for (int b = blockIdx.x * wpb + (threadIdx.x >> 5); b < prm.nb; b += gridDim.x * wpb)
        near_ff_prep_box<KIND>(prm, nv, b, sff, qff);
}

// many descriptions at once: one warp per (description, box) work item
template <int KIND>
__global__ void k_near_ff_prep_batch(const unsigned char* __restrict__ plist, const int2* __restrict__ items,
                                     int nitems, int nv) {
    const int wpb = blockDim.x >> 5;
    const int it = blockIdx.x * wpb + (threadIdx.x >> 5);
    if (it >= nitems) return;
    const int2 w = items[it];
    const NearParams& prm = *reinterpret_cast<const NearParams*>(plist + (size_t)w.x * kParamStride);
    near_ff_prep_box<KIND>(prm, nv, w.y, const_cast<float4*>(prm.sff), const_cast<float2*>(prm.qff));
}

template <int KIND, int NV>
int near_cap(const fte_context* ctx, bool ff) {
    int cap = 2048;
    // shared memory of one of the CTAs an SM holds (227 KB per SM)
    const size_t b0 = ff ? NearCfg<true>::budget : NearCfg<false>::budget;
    const size_t budget = b0 < (size_t)ctx->max_smem_optin ? b0 : (size_t)ctx->max_smem_optin;
    while (cap > 64 && NearSmem<KIND, NV>::bytes(cap, ff) > budget) cap -= 32;
    return cap;
}
}  // namespace

int fte_near_classes(const fte_options* opt, double tol, double* x32, bool* ff) {
    *x32 = HUGE_VAL;
    *ff = false;
    if (!opt || opt->form != FTE_FORM_MIXED) return FTE_OK;
    switch (opt->near) {
        case FTE_NEAR_AUTO:
            *x32 = fte_near_fp32_threshold(tol);
            *ff = fte_near_ff_ok(tol);
            return FTE_OK;
        case FTE_NEAR_FP64: return FTE_OK;
        case FTE_NEAR_FF: *ff = true; return FTE_OK;
        default: fte_set_error("unknown near-pair arithmetic %d", opt->near); return FTE_ERR_INVALID;
    }
}

bool fte_near_ff_ok(double tol) {
    // float-float terms carry ~1e-13 relative error (exp, K(x) and the
    // reciprocal ~4e-14 each); from tol 1e-11 up that stays two orders below
    return tol >= 1e-11;
}

double fte_near_fp32_threshold(double tol) {
    // FP32 terms carry relative rounding ~1e-7 and a pair's terms scale with
    // e^-x (1 + x); pairs with e^-x (1 + x) <= 1e7 tol keep that rounding
    // at about tol of a single near term (the sum's scale is set by the FP64
    // pairs with x < 1, tens of them per target), and the per-pair rounding
    // errors add incoherently.  Never below x = 1 (the Stokeslet's log
    // branch stays FP64).
    const double target = 1e7 * tol;
    if (!(target > 0) || target >= 2.0 / std::exp(1.0)) return 1.0;
    double lo = 1.0, hi = 800.0;
    for (int it = 0; it < 100; it++) {
        double mid = 0.5 * (lo + hi);
        if (std::exp(-mid) * (1 + mid) > target)
            lo = mid;
        else
            hi = mid;
    }
    return hi;
}

void fte_near_fill_params(int kind, const CellList& cl, double xi, double Lx, double Ly, NearParamsHost* hp,
                          double x32, bool ff) {
    NearParams& p = *reinterpret_cast<NearParams*>(hp->raw);
    p.nsx = cl.nsx;
    p.nsy = cl.nsy;
    p.nb = cl.nb;
    p.src_off = cl.src_off;
    p.spos = cl.spos;
    p.q0 = cl.q0;
    p.q1 = cl.q1;
    p.q2 = cl.q2;
    p.qstride = cl.qstride;
    p.tar_off = cl.tar_off;
    p.tpos = cl.tpos;
    p.tidx = cl.tidx;
    p.Lx = Lx;
    p.Ly = Ly;
    p.xi = xi;
    p.xi2 = xi * xi;
    p.inv_xi2 = 1.0 / (xi * xi);
    p.selfc = -(1.0 + 0.5 * FTE_EULER) - log(xi);
    p.cutoffsq = cl.cutoffsq > 0.0 ? cl.cutoffsq : Lx * Ly / cl.nsx / cl.nsy;
    p.pf = 2.0 * xi * xi;
    p.bsx = Lx / cl.nsx;
    p.bsy = Ly / cl.nsy;
    double bsx = Lx / cl.nsx, bsy = Ly / cl.nsy;
    double bmax = bsx > bsy ? bsx : bsy;
    p.cut32 = (float)(p.cutoffsq + 1e-4 * bmax * bmax);
    p.x32 = x32 >= 1e30 ? INFINITY : (float)(x32 > 1.0 ? x32 : 1.0);
    p.ffnear = ff ? 1 : 0;
    {
        const float h = (float)p.xi2;
        p.xi2ff = make_float2(h, (float)(p.xi2 - (double)h));
        const float g = (float)p.pf;
        p.pfff = make_float2(g, (float)(p.pf - (double)g));
        const float c = (float)p.cutoffsq;
        p.cutff = make_float2(c, (float)(p.cutoffsq - (double)c));
        const float q = (float)p.selfc;
        p.selcff = make_float2(q, (float)(p.selfc - (double)q));
    }
    p.sff = nullptr;
    p.qff = nullptr;
    p.qffstride = 0;
    p.cap = 0;
    p.ur = nullptr;
    p.ustride = 0;
    (void)kind;
}

size_t fte_near_params_size() { return sizeof(NearParams); }

namespace {
template <int KIND, int NV>
int near_launch_one(fte_context* ctx, NearParams p) {
    const bool ff = p.ffnear != 0;
    p.cap = near_cap<KIND, NV>(ctx, ff);
    size_t smem = NearSmem<KIND, NV>::bytes(p.cap, ff);
    // boxes fewer than the CTAs the GPU holds at once: their targets split
    // over up to 8 CTAs each (each stages the neighbourhood again)
    auto parts = [&](int ctas) {
        const long long slots = (long long)ctx->num_sms * ctas;
        const long long q = p.nb > 0 ? (slots + p.nb - 1) / p.nb : 1;
        return (int)(q < 1 ? 1 : (q > 8 ? 8 : q));
    };
    if (ff) {
        using C = NearCfg<true>;
        const int np = parts(C::ctas);
        const long long units = (long long)p.nb * np;
        const int grid = units < ctx->num_sms * C::grid_per_sm ? (units > 0 ? (int)units : 1)
                                                                : ctx->num_sms * C::grid_per_sm;
        FTE_CUDA_TRY(
            fte_smem_ceiling(k_near<KIND, NV, true>, (int)smem));
        FTE_LAUNCH(ctx, (k_near<KIND, NV, true>), grid, C::threads, smem, p, np);
    } else {
        using C = NearCfg<false>;
        const int np = parts(C::ctas);
        const long long units = (long long)p.nb * np;
        const int grid = units < ctx->num_sms * C::grid_per_sm ? (units > 0 ? (int)units : 1)
                                                                : ctx->num_sms * C::grid_per_sm;
        FTE_CUDA_TRY(
            fte_smem_ceiling(k_near<KIND, NV, false>, (int)smem));
        FTE_LAUNCH(ctx, (k_near<KIND, NV, false>), grid, C::threads, smem, p, np);
    }
    return FTE_OK;
}

template <int KIND, int NV>
int near_launch_batch(fte_context* ctx, bool ff, const unsigned char* plist_dev, const int2* items, int nitems) {
    const size_t smem = NearSmem<KIND, NV>::bytes(near_cap<KIND, NV>(ctx, ff), ff);
    if (nitems < 1) return FTE_OK;
    if (ff) {
        using C = NearCfg<true>;
        const int grid = nitems < ctx->num_sms * C::grid_per_sm ? nitems : ctx->num_sms * C::grid_per_sm;
        FTE_CUDA_TRY(fte_smem_ceiling(k_near_batch<KIND, NV, true>, (int)smem));
        FTE_LAUNCH(ctx, (k_near_batch<KIND, NV, true>), grid, C::threads, smem, plist_dev, items, nitems);
    } else {
        using C = NearCfg<false>;
        const int grid = nitems < ctx->num_sms * C::grid_per_sm ? nitems : ctx->num_sms * C::grid_per_sm;
        FTE_CUDA_TRY(fte_smem_ceiling(k_near_batch<KIND, NV, false>, (int)smem));
        FTE_LAUNCH(ctx, (k_near_batch<KIND, NV, false>), grid, C::threads, smem, plist_dev, items, nitems);
    }
    return FTE_OK;
}
}  // namespace

bool fte_near_uses_ff(const NearParamsHost& hp) { return reinterpret_cast<const NearParams*>(hp.raw)->ffnear != 0; }

int fte_near_cap(const fte_context* ctx, int kind, int nv, bool ff) {
    if (kind == FTE_KIND_SLP) {
        switch (nv) {
            case 1: return near_cap<FTE_KIND_SLP, 1>(ctx, ff);
            case 2: return near_cap<FTE_KIND_SLP, 2>(ctx, ff);
            case 3: return near_cap<FTE_KIND_SLP, 3>(ctx, ff);
            default: return near_cap<FTE_KIND_SLP, 4>(ctx, ff);
        }
    }
    switch (nv) {
        case 1: return near_cap<FTE_KIND_DLP, 1>(ctx, ff);
        case 2: return near_cap<FTE_KIND_DLP, 2>(ctx, ff);
        case 3: return near_cap<FTE_KIND_DLP, 3>(ctx, ff);
        default: return near_cap<FTE_KIND_DLP, 4>(ctx, ff);
    }
}

int fte_near_launch_nv(fte_context* ctx, int kind, int nv, const NearParamsHost& hp, double2* ur, long long ustride) {
    NearParams p = *reinterpret_cast<const NearParams*>(hp.raw);
    p.ur = ur;
    p.ustride = ustride;
    if (nv < 1 || nv > 4) {
        fte_set_error("1 to 4 density vectors per near-field launch (got %d)", nv);
        return FTE_ERR_INVALID;
    }
    if (kind == FTE_KIND_SLP) {
        switch (nv) {
            case 1: return near_launch_one<FTE_KIND_SLP, 1>(ctx, p);
            case 2: return near_launch_one<FTE_KIND_SLP, 2>(ctx, p);
            case 3: return near_launch_one<FTE_KIND_SLP, 3>(ctx, p);
            default: return near_launch_one<FTE_KIND_SLP, 4>(ctx, p);
        }
    }
    switch (nv) {
        case 1: return near_launch_one<FTE_KIND_DLP, 1>(ctx, p);
        case 2: return near_launch_one<FTE_KIND_DLP, 2>(ctx, p);
        case 3: return near_launch_one<FTE_KIND_DLP, 3>(ctx, p);
        default: return near_launch_one<FTE_KIND_DLP, 4>(ctx, p);
    }
}

int fte_near_launch_batch(fte_context* ctx, int kind, int nv, bool ff, const void* plist_dev, const int2* items,
                          int nitems) {
    const unsigned char* pl = static_cast<const unsigned char*>(plist_dev);
    if (kind == FTE_KIND_SLP) {
        switch (nv) {
            case 1: return near_launch_batch<FTE_KIND_SLP, 1>(ctx, ff, pl, items, nitems);
            case 2: return near_launch_batch<FTE_KIND_SLP, 2>(ctx, ff, pl, items, nitems);
            case 3: return near_launch_batch<FTE_KIND_SLP, 3>(ctx, ff, pl, items, nitems);
            default: return near_launch_batch<FTE_KIND_SLP, 4>(ctx, ff, pl, items, nitems);
        }
    }
    switch (nv) {
        case 1: return near_launch_batch<FTE_KIND_DLP, 1>(ctx, ff, pl, items, nitems);
        case 2: return near_launch_batch<FTE_KIND_DLP, 2>(ctx, ff, pl, items, nitems);
        case 3: return near_launch_batch<FTE_KIND_DLP, 3>(ctx, ff, pl, items, nitems);
        default: return near_launch_batch<FTE_KIND_DLP, 4>(ctx, ff, pl, items, nitems);
    }
}

int fte_near_launch(fte_context* ctx, int kind, const CellList& cl, double xi, double Lx, double Ly, double2* ur,
                    double x32, bool ff, void* ffmem) {
    NearParamsHost hp;
    fte_near_fill_params(kind, cl, xi, Lx, Ly, &hp, x32, ff);
    if (ff) {
        if (!ffmem) {
            fte_set_error("internal: float-float near pairs without scratch");
            return FTE_ERR_INVALID;
        }
        fte_near_ff_attach(&hp, kind, 1, cl.nsrc, ffmem);
        FTE_TRY(fte_near_ff_prep(ctx, kind, 1, hp));
    }
    return fte_near_launch_nv(ctx, kind, 1, hp, ur, 0);
}

// ---- diagnostics: the special functions on the device (test hook) ------------
namespace {
__global__ void k_special_probe(int which, const double* __restrict__ x, double* __restrict__ out, int n) {
    __shared__ double gtab[kGtab];
    __shared__ double ktab[kKtab];
    __shared__ double etab[64];
    for (int i = threadIdx.x; i < kGtab; i += blockDim.x) gtab[i] = (&fte_e1_coef_g[0][0])[i];
    for (int i = threadIdx.x; i < kKtab; i += blockDim.x) ktab[i] = (&fte_k_coef[0][0])[i];
    for (int i = threadIdx.x; i < 64; i += blockDim.x) etab[i] = fte_exp_tab[i];
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = x[i];
    double r;
    switch (which) {
        case 0:  // E1(x)
            r = fte_e1(v, exp(-v), 1.0 / v, gtab);
            break;
        case 1:  // exp(-x), this project's evaluation
            r = fte_expm(v, etab);
            break;
        case 2: {  // 0.5 E1(x) - exp(-x) as the Stokeslet kernel evaluates it
            double emx = fte_expm(v, etab);
            if (v < 1.0) {
                double tt = fma(2.0, v, -1.0);
                double R = fte_e1_coef_r[FTE_E1_DEG_R];
                for (int k = FTE_E1_DEG_R - 1; k >= 0; k--) R = fma(R, tt, fte_e1_coef_r[k]);
                r = fma(0.5, fma(v, R, -FTE_EULER - log(v)), -emx);
            } else {
                r = emx * fte_kfun(v, ktab);
            }
            break;
        }
        case 3:  // 1/x
            r = fte_rcp(v);
            break;
        case 4:  // the drivers' coordinate wrap, box side 1
            r = fte_wrap_coord(v, 1.0, 1.0);
            break;
        default:  // the same, box side 2.75
            r = fte_wrap_coord(v, 2.75, 1.0 / 2.75);
            break;
    }
    out[i] = r;
}
}  // namespace

extern "C" int fte_debug_special(int which, const double* x_dev, double* out_dev, int n) {
    if (n <= 0) return FTE_OK;
    if (which < 0 || which > 5 || !x_dev || !out_dev) {
        fte_set_error("fte_debug_special: bad arguments");
        return FTE_ERR_INVALID;
    }
    k_special_probe<<<(n + 255) / 256, 256>>>(which, x_dev, out_dev, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        fte_set_error("fte_debug_special: %s", cudaGetErrorString(e));
        return FTE_ERR_CUDA;
    }
    return FTE_OK;
}

void fte_near_set_output(NearParamsHost* hp, double2* ur, long long ustride, int cap) {
    static_assert(sizeof(NearParams) <= sizeof(NearParamsHost::raw), "NearParamsHost too small");
    NearParams& p = *reinterpret_cast<NearParams*>(hp->raw);
    p.ur = ur;
    p.ustride = ustride;
    p.cap = cap;
}

size_t fte_near_ff_ws(int kind, int nv, int64_t nsrc) {
    const int kden = kind == FTE_KIND_SLP ? 2 : 4;
    return ws_bytes((size_t)nsrc + 1, sizeof(float4)) + ws_bytes((size_t)kden * nv * (nsrc + 1), sizeof(float2));
}

void fte_near_ff_attach(NearParamsHost* hp, int kind, int nv, int64_t nsrc, void* mem) {
    NearParams& p = *reinterpret_cast<NearParams*>(hp->raw);
    const int kden = kind == FTE_KIND_SLP ? 2 : 4;
    WsCarver w{static_cast<char*>(mem), 0, fte_near_ff_ws(kind, nv, nsrc)};
    p.sff = w.take<float4>((size_t)nsrc + 1);
    p.qff = w.take<float2>((size_t)kden * nv * (nsrc + 1));
    p.qffstride = nsrc;
    const double bx = p.Lx / p.nsx, by = p.Ly / p.nsy;
    const float hx = (float)bx, hy = (float)by;
    p.bsxff = make_float2(hx, (float)(bx - (double)hx));
    p.bsyff = make_float2(hy, (float)(by - (double)hy));
}

int fte_near_ff_prep_batch(fte_context* ctx, int kind, int nv, const void* plist_dev, const int2* items,
                           int nitems) {
    if (nitems < 1) return FTE_OK;
    const int grid = (nitems + 7) / 8;
    if (kind == FTE_KIND_SLP)
        FTE_LAUNCH(ctx, k_near_ff_prep_batch<FTE_KIND_SLP>, grid, 256, 0, (const unsigned char*)plist_dev, items,
                   nitems, nv);
    else
        FTE_LAUNCH(ctx, k_near_ff_prep_batch<FTE_KIND_DLP>, grid, 256, 0, (const unsigned char*)plist_dev, items,
                   nitems, nv);
    return FTE_OK;
}

int fte_near_ff_prep(fte_context* ctx, int kind, int nv, const NearParamsHost& hp) {
    const NearParams& p = *reinterpret_cast<const NearParams*>(hp.raw);
    if (!p.ffnear || p.nb == 0) return FTE_OK;
    if (!p.sff || !p.qff) {
        fte_set_error("internal: float-float near data not attached");
        return FTE_ERR_INVALID;
    }
    int grid = (p.nb + 7) / 8;
    if (grid > ctx->num_sms * 16) grid = ctx->num_sms * 16;
    float4* sff = const_cast<float4*>(p.sff);
    float2* qff = const_cast<float2*>(p.qff);
    if (kind == FTE_KIND_SLP)
        FTE_LAUNCH(ctx, k_near_ff_prep<FTE_KIND_SLP>, grid, 256, 0, p, nv, sff, qff);
    else
        FTE_LAUNCH(ctx, k_near_ff_prep<FTE_KIND_DLP>, grid, 256, 0, p, nv, sff, qff);
    return FTE_OK;
}
