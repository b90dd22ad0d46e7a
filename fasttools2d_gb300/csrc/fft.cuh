// fft.cuh -- block-cooperative 1-D complex FFT in shared memory.
//
// The reference obtains its transforms from MATLAB's fft2/ifft2
// (PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_kspace.cpp:80-81,176-177).
// Here one thread block transforms one sequence held in shared memory:
//   * Stockham autosort passes with radices 8, 4, 2, 3, 5, 7 (the mixed-radix
//     formulation of Govindaraju et al., "High performance discrete Fourier
//     transforms on graphics processors", SC 2008): pass with radix R and
//     Ns = product of the earlier radices reads v_r = x[j + r n/R], twiddles
//     by W_{Ns R}^{r (j mod Ns)}, does an R-point DFT and writes
//     y[(j/Ns) Ns R + (j mod Ns) + s Ns];
//   * lengths with a prime factor above 7 use Bluestein's chirp-z algorithm
//     (Bluestein 1970) over a 7-smooth length m >= 2n - 1.
// Twiddles come from FP64 tables computed on the host.  The transform is
// unnormalised; `inv` selects exp(+i...).
//
// Element types: double (FP64), float (FP32) and FfCx, complex float-float
// held in a float4 (re hi, re lo, im hi, im lo; ff.cuh) with float-float
// copies of the twiddle, chirp and root tables.
#pragma once

#include <type_traits>

#include "ff.cuh"
#include "fte_internal.cuh"

struct FfCx {};  // tag: complex float-float elements

// complex float-float arithmetic on float4 (declared ahead of the generic
// templates so that the FfCx instantiations pick them)
__device__ __forceinline__ float2 ffc_re(float4 a) { return make_float2(a.x, a.y); }
__device__ __forceinline__ float2 ffc_im(float4 a) { return make_float2(a.z, a.w); }
__device__ __forceinline__ float4 ffc_mk(float2 r, float2 i) { return make_float4(r.x, r.y, i.x, i.y); }
__device__ __forceinline__ float4 cadd(float4 a, float4 b) {
    return ffc_mk(ff_add(ffc_re(a), ffc_re(b)), ff_add(ffc_im(a), ffc_im(b)));
}
__device__ __forceinline__ float4 csub(float4 a, float4 b) {
    return ffc_mk(ff_add(ffc_re(a), ff_neg(ffc_re(b))), ff_add(ffc_im(a), ff_neg(ffc_im(b))));
}
__device__ __forceinline__ float4 cmul(float4 a, float4 b) {
    const float2 ar = ffc_re(a), ai = ffc_im(a), br = ffc_re(b), bi = ffc_im(b);
    return ffc_mk(ff_add(ff_mul(ar, br), ff_neg(ff_mul(ai, bi))), ff_add(ff_mul(ar, bi), ff_mul(ai, br)));
}
__device__ __forceinline__ float4 cconj(float4 a) { return make_float4(a.x, a.y, -a.z, -a.w); }
__device__ __forceinline__ float4 cmul_mi(float4 a, bool inv) {
    return inv ? make_float4(-a.z, -a.w, a.x, a.y) : make_float4(a.z, a.w, -a.x, -a.y);
}
// a times a real float-float number
__device__ __forceinline__ float4 cscale(float4 a, float2 c) { return ffc_mk(ff_mul(ffc_re(a), c), ff_mul(ffc_im(a), c)); }

template <typename T>
struct Cx;
template <>
struct Cx<double> {
    using V = double2;
    __device__ static V mk(double a, double b) { return make_double2(a, b); }
};
template <>
struct Cx<float> {
    using V = float2;
    __device__ static V mk(float a, float b) { return make_float2(a, b); }
};
template <>
struct Cx<FfCx> {
    using V = float4;
    __device__ static V mk(float a, float b) { return make_float4(a, 0.f, b, 0.f); }
};

template <typename V>
__device__ __forceinline__ V cadd(V a, V b) {
    V r;
    r.x = a.x + b.x;
    r.y = a.y + b.y;
    return r;
}
template <typename V>
__device__ __forceinline__ V csub(V a, V b) {
    V r;
    r.x = a.x - b.x;
    r.y = a.y - b.y;
    return r;
}
template <typename V>
__device__ __forceinline__ V cmul(V a, V b) {
    V r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename V>
__device__ __forceinline__ V cconj(V a) {
    a.y = -a.y;
    return a;
}
// multiply by -i (forward) or +i (inverse)
template <typename V>
__device__ __forceinline__ V cmul_mi(V a, bool inv) {
    V r;
    if (inv) {
        r.x = -a.y;
        r.y = a.x;
    } else {
        r.x = a.y;
        r.y = -a.x;
    }
    return r;
}

// cos/sin(2 pi m / R) for the generic small radices 3, 5, 7
__constant__ double fte_root3[2][3] = {{1.0, -0.5, -0.5},
                                       {0.0, 0.86602540378443864676, -0.86602540378443864676}};
__constant__ double fte_root5[2][5] = {
    {1.0, 0.30901699437494742410, -0.80901699437494742410, -0.80901699437494742410, 0.30901699437494742410},
    {0.0, 0.95105651629515357212, 0.58778525229247312917, -0.58778525229247312917, -0.95105651629515357212}};
__constant__ double fte_root7[2][7] = {
    {1.0, 0.62348980185873353053, -0.22252093395631440429, -0.90096886790241912624, -0.90096886790241912624,
     -0.22252093395631440429, 0.62348980185873353053},
    {0.0, 0.78183148246802980871, 0.97492791218182360702, 0.43388373911755812048, -0.43388373911755812048,
     -0.97492791218182360702, -0.78183148246802980871}};

// cos / sin (2 pi m / R) as float-float for R = 3, 5, 7
__constant__ float2 fte_root3ff[2][3] = {{{1.0f, 0.0f}, {-0.5f, 0.0f}, {-0.5f, 0.0f}},
                                         {{0.0f, 0.0f}, {8.660253882e-01f, 1.554362505e-08f},
                                          {-8.660253882e-01f, -1.554362505e-08f}}};
__constant__ float2 fte_root5ff[2][5] = {
    {{1.0f, 0.0f}, {3.090170026e-01f, -8.207602598e-09f}, {-8.090170026e-01f, 8.207602598e-09f},
     {-8.090170026e-01f, 8.207602598e-09f}, {3.090170026e-01f, -8.207602598e-09f}},
    {{0.0f, 0.0f}, {9.510565400e-01f, -2.371720598e-08f}, {5.877852440e-01f, 8.304436250e-09f},
     {-5.877852440e-01f, -8.304436250e-09f}, {-9.510565400e-01f, 2.371720598e-08f}}};
__constant__ float2 fte_root7ff[2][7] = {
    {{1.0f, 0.0f}, {6.234897971e-01f, 4.743407445e-09f}, {-2.225209326e-01f, -1.401115779e-09f},
     {-9.009688497e-01f, -1.824345297e-08f}, {-9.009688497e-01f, -1.824345297e-08f},
     {-2.225209326e-01f, -1.401115779e-09f}, {6.234897971e-01f, 4.743407445e-09f}},
    {{0.0f, 0.0f}, {7.818315029e-01f, -2.044639835e-08f}, {9.749279022e-01f, 9.960143821e-09f},
     {4.338837266e-01f, 1.252072579e-08f}, {-4.338837266e-01f, -1.252072579e-08f},
     {-9.749279022e-01f, -9.960143821e-09f}, {-7.818315029e-01f, 2.044639835e-08f}}};

// R-point DFT in float-float (the same butterflies as dft_small)
template <int R>
__device__ __forceinline__ void dft_small_ff(float4* v, bool inv) {
    if constexpr (R == 2) {
        const float4 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        const float4 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        const float4 t2 = cadd(v[1], v[3]), t3 = cmul_mi(csub(v[1], v[3]), inv);
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    } else if constexpr (R == 8) {
        float4 e[4] = {v[0], v[2], v[4], v[6]};
        float4 o[4] = {v[1], v[3], v[5], v[7]};
        dft_small_ff<4>(e, inv);
        dft_small_ff<4>(o, inv);
        // W8 = (1 - i)/sqrt 2 (forward), (1 + i)/sqrt 2 (inverse); W8^3 = -i W8
        const float2 r2 = make_float2(7.071067691e-01f, 1.210161749e-08f);
        const float4 s1 = cscale(o[1], r2), s3 = cscale(o[3], r2);
        const float4 o1 = inv ? ffc_mk(ff_add(ffc_re(s1), ff_neg(ffc_im(s1))), ff_add(ffc_im(s1), ffc_re(s1)))
                              : ffc_mk(ff_add(ffc_re(s1), ffc_im(s1)), ff_add(ffc_im(s1), ff_neg(ffc_re(s1))));
        // W8^3 o3 = (-1 - i)/sqrt 2 o3 (forward), (-1 + i)/sqrt 2 o3 (inverse)
        const float4 o3 = inv ? ffc_mk(ff_neg(ff_add(ffc_re(s3), ffc_im(s3))), ff_add(ffc_re(s3), ff_neg(ffc_im(s3))))
                              : ffc_mk(ff_add(ffc_im(s3), ff_neg(ffc_re(s3))), ff_neg(ff_add(ffc_re(s3), ffc_im(s3))));
        const float4 o2 = cmul_mi(o[2], inv);
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    } else {
        constexpr int H = (R - 1) / 2;
        const float2* rc = R == 3 ? fte_root3ff[0] : (R == 5 ? fte_root5ff[0] : fte_root7ff[0]);
        const float2* rs = R == 3 ? fte_root3ff[1] : (R == 5 ? fte_root5ff[1] : fte_root7ff[1]);
        float4 t[H], u[H];
        float4 out0 = v[0];
#pragma unroll
        for (int r = 1; r <= H; r++) {
            t[r - 1] = cadd(v[r], v[R - r]);
            u[r - 1] = csub(v[r], v[R - r]);
            out0 = cadd(out0, t[r - 1]);
        }
#pragma unroll
        for (int s = 1; s <= H; s++) {
            float4 A = v[0], B = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int r = 1; r <= H; r++) {
                const int m = (r * s) % R;
                A = cadd(A, cscale(t[r - 1], rc[m]));
                B = cadd(B, cscale(u[r - 1], rs[m]));
            }
            // -i B = (B.im, -B.re); forward: out_s = A - iB, out_{R-s} = A + iB
            const float4 mib = make_float4(B.z, B.w, -B.x, -B.y);
            const float4 am = cadd(A, mib), ap = csub(A, mib);
            v[s] = inv ? ap : am;
            v[R - s] = inv ? am : ap;
        }
        v[0] = out0;
    }
}

template <typename T, int R>
__device__ __forceinline__ void dft_small(typename Cx<T>::V* v, bool inv) {
    using V = typename Cx<T>::V;
    if constexpr (std::is_same<T, FfCx>::value) {
        dft_small_ff<R>(v, inv);
    } else if constexpr (R == 2) {
        V a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        V t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        V t2 = cadd(v[1], v[3]), t3 = cmul_mi(csub(v[1], v[3]), inv);
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    } else if constexpr (R == 8) {
        V e[4] = {v[0], v[2], v[4], v[6]};
        V o[4] = {v[1], v[3], v[5], v[7]};
        dft_small<T, 4>(e, inv);
        dft_small<T, 4>(o, inv);
        const T r2 = (T)0.70710678118654752440;
        // W8^s for s = 0..3 (forward exp(-i pi s/4), inverse conj)
        V w1 = Cx<T>::mk(r2, inv ? r2 : -r2);
        V w3 = Cx<T>::mk(-r2, inv ? r2 : -r2);
        V o1 = cmul(o[1], w1), o2 = cmul_mi(o[2], inv), o3 = cmul(o[3], w3);
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    } else {
        // odd R: pair the inputs r and R - r.  With t_r = v_r + v_{R-r},
        // u_r = v_r - v_{R-r} (r = 1..H, H = (R-1)/2):
        //   out_0     = v_0 + sum_r t_r
        //   out_s     = A_s - i B_s,  out_{R-s} = A_s + i B_s   (forward; inverse swaps)
        //   A_s = v_0 + sum_r cos(2 pi r s / R) t_r,  B_s = sum_r sin(2 pi r s / R) u_r
        // about a third of the arithmetic of the direct sum over all r, s.
        constexpr int H = (R - 1) / 2;
        const double* rc = R == 3 ? fte_root3[0] : (R == 5 ? fte_root5[0] : fte_root7[0]);
        const double* rs = R == 3 ? fte_root3[1] : (R == 5 ? fte_root5[1] : fte_root7[1]);
        V t[H], u[H];
        V out0 = v[0];
#pragma unroll
        for (int r = 1; r <= H; r++) {
            t[r - 1] = cadd(v[r], v[R - r]);
            u[r - 1] = csub(v[r], v[R - r]);
            out0 = cadd(out0, t[r - 1]);
        }
#pragma unroll
        for (int s = 1; s <= H; s++) {
            T ax = v[0].x, ay = v[0].y, bx = 0, by = 0;
#pragma unroll
            for (int r = 1; r <= H; r++) {
                const int m = (r * s) % R;
                const T c = (T)rc[m], sn = (T)rs[m];
                ax += c * t[r - 1].x;
                ay += c * t[r - 1].y;
                bx += sn * u[r - 1].x;
                by += sn * u[r - 1].y;
            }
            // -i B = (by, -bx); forward: out_s = A - iB, out_{R-s} = A + iB
            const V am = Cx<T>::mk(ax + by, ay - bx), ap = Cx<T>::mk(ax - by, ay + bx);
            v[s] = inv ? ap : am;
            v[R - s] = inv ? am : ap;
        }
        v[0] = out0;
    }
}

template <typename T>
__device__ __forceinline__ typename Cx<T>::V tw_load(const FftDev& p, int idx);
template <>
__device__ __forceinline__ double2 tw_load<double>(const FftDev& p, int idx) {
    return __ldg(p.tw + idx);
}
template <>
__device__ __forceinline__ float2 tw_load<float>(const FftDev& p, int idx) {
    return __ldg(p.tw32 + idx);
}
template <>
__device__ __forceinline__ float4 tw_load<FfCx>(const FftDev& p, int idx) {
    return __ldg(p.twff + idx);
}

template <typename T, int R>
__device__ __forceinline__ void stockham_pass(const typename Cx<T>::V* __restrict__ in, typename Cx<T>::V* __restrict__ out,
                                              int n, int Ns, const FftDev& p, bool inv) {
    using V = typename Cx<T>::V;
    const int nb = n / R;
    const int twstep = n / (Ns * R);
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        int k = j % Ns;
        V v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = in[j + r * nb];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; r++) {
                V w = tw_load<T>(p, r * k * twstep);
                if (inv) w = cconj(w);
                v[r] = cmul(v[r], w);
            }
        }
        dft_small<T, R>(v, inv);
        int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int s = 0; s < R; s++) out[idxD + s * Ns] = v[s];
    }
}

// Transform of length p.m (the inner, 7-smooth length) held in a; b is
// scratch of the same length.  Returns the buffer holding the result.
template <typename T>
__device__ typename Cx<T>::V* fft_inner(typename Cx<T>::V* a, typename Cx<T>::V* b, const FftDev& p, bool inv) {
    using V = typename Cx<T>::V;
    V* src = a;
    V* dst = b;
    int Ns = 1;
    const int n = p.m;
    for (int s = 0; s < p.nrad; s++) {
        __syncthreads();
        switch (p.rad[s]) {
            case 2: stockham_pass<T, 2>(src, dst, n, Ns, p, inv); break;
            case 3: stockham_pass<T, 3>(src, dst, n, Ns, p, inv); break;
            case 4: stockham_pass<T, 4>(src, dst, n, Ns, p, inv); break;
            case 5: stockham_pass<T, 5>(src, dst, n, Ns, p, inv); break;
            case 7: stockham_pass<T, 7>(src, dst, n, Ns, p, inv); break;
            default: stockham_pass<T, 8>(src, dst, n, Ns, p, inv); break;
        }
        Ns *= p.rad[s];
        V* t = src;
        src = dst;
        dst = t;
    }
    __syncthreads();
    return src;
}

template <typename T>
__device__ __forceinline__ typename Cx<T>::V chirp_load(const FftDev& p, int k) {
    if constexpr (std::is_same<T, FfCx>::value) {
        return __ldg(p.chirpff + k);
    } else if constexpr (sizeof(T) == 8) {
        return __ldg(p.chirp + k);
    } else {
        return __ldg(p.chirp32 + k);
    }
}
template <typename T>
__device__ __forceinline__ typename Cx<T>::V bhat_load(const FftDev& p, int k) {
    if constexpr (std::is_same<T, FfCx>::value) {
        return __ldg(p.bhatff + k);
    } else if constexpr (sizeof(T) == 8) {
        return __ldg(p.bhat + k);
    } else {
        return __ldg(p.bhat32 + k);
    }
}

// Full length-n transform of the data in a[0..n) (a and b each hold p.m
// elements).  Returns the buffer holding the n results.
template <typename T>
__device__ typename Cx<T>::V* fft_block(typename Cx<T>::V* a, typename Cx<T>::V* b, const FftDev& p, bool inv) {
    using V = typename Cx<T>::V;
    if (!p.bluestein) return fft_inner<T>(a, b, p, inv);
    // Bluestein: y_k = c_k sum_j (x_j c_j) conj(c_{k-j}),  c_k = exp(-i pi k^2/n).
    // The inverse transform is conj(forward(conj(x))).
    __syncthreads();
    for (int k = threadIdx.x; k < p.m; k += blockDim.x) {
        V v;
        if (k < p.n) {
            V x = a[k];
            if (inv) x = cconj(x);
            v = cmul(x, chirp_load<T>(p, k));
        } else {
            v = Cx<T>::mk(0, 0);
        }
        a[k] = v;
    }
    V* r = fft_inner<T>(a, b, p, false);
    for (int k = threadIdx.x; k < p.m; k += blockDim.x) r[k] = cmul(r[k], bhat_load<T>(p, k));
    V* o = (r == a) ? b : a;
    V* r2 = fft_inner<T>(r, o, p, true);
    for (int k = threadIdx.x; k < p.n; k += blockDim.x) {
        V y = cmul(r2[k], chirp_load<T>(p, k));
        if (inv) y = cconj(y);
        r2[k] = y;
    }
    __syncthreads();
    return r2;
}
