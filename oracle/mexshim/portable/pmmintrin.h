/*
 * pmmintrin.h -- portable stand-in for the x86 SSE2/SSE3 double-precision
 * intrinsics header, for hosts without SSE (the aarch64 GPU hosts).
 * TEST INFRASTRUCTURE ONLY: it lets the reference's unmodified spectral
 * Ewald gateways (PeriodicEwald/src/mex/StokesSLP/mex_stokes_slp_real.cpp:4,
 * PeriodicEwald/src/mex/StokesDLP/mex_stokes_dlp_real.cpp:4 include
 * <pmmintrin.h>) compile where the real header does not exist.  The
 * Makefile puts this directory on the include path only on non-x86 hosts;
 * on x86-64 the compiler's own header is used (the CPU tests build one
 * x86 flavour with this header, FTE_PORTABLE_SSE_ON_X86, and compare it
 * bitwise with the flavour built on the compiler's header).
 *
 * Only the operations those gateways call are provided, each written from
 * the instruction's documented lane semantics on a two-lane vector of
 * doubles (GCC vector extension, which the compiler maps to NEON on
 * aarch64): lane 0 is the lower address.  Every lane operation is one IEEE
 * double operation, as on SSE2, so results match the x86 build when
 * floating-point contraction is off (-ffp-contract=off).
 */
#ifndef FTE_PORTABLE_PMMINTRIN_H
#define FTE_PORTABLE_PMMINTRIN_H

#if (defined(__x86_64__) || defined(__i386__)) && !defined(FTE_PORTABLE_SSE_ON_X86)
#error "oracle/mexshim/portable is for non-x86 hosts; use the compiler's pmmintrin.h on x86"
#endif

typedef double __m128d __attribute__((vector_size(16), aligned(16), may_alias));
typedef double fte_m128d_u __attribute__((vector_size(16), aligned(1), may_alias));

#define FTE_SSE_INLINE static inline __attribute__((always_inline))

/* {a0 + b0, a1 + b1} */
FTE_SSE_INLINE __m128d _mm_add_pd(__m128d a, __m128d b) { return a + b; }
/* {a0 - b0, a1 - b1} */
FTE_SSE_INLINE __m128d _mm_sub_pd(__m128d a, __m128d b) { return a - b; }
/* {a0 * b0, a1 * b1} */
FTE_SSE_INLINE __m128d _mm_mul_pd(__m128d a, __m128d b) { return a * b; }
/* SSE3 ADDSUBPD: {a0 - b0, a1 + b1} */
FTE_SSE_INLINE __m128d _mm_addsub_pd(__m128d a, __m128d b) {
    __m128d r = {a[0] - b[0], a[1] + b[1]};
    return r;
}
/* SSE3 HADDPD: {a0 + a1, b0 + b1} */
FTE_SSE_INLINE __m128d _mm_hadd_pd(__m128d a, __m128d b) {
    __m128d r = {a[0] + a[1], b[0] + b[1]};
    return r;
}
/* SSE3 HSUBPD: {a0 - a1, b0 - b1} */
FTE_SSE_INLINE __m128d _mm_hsub_pd(__m128d a, __m128d b) {
    __m128d r = {a[0] - a[1], b[0] - b[1]};
    return r;
}
/* MOVAPD load: p must be 16-byte aligned */
FTE_SSE_INLINE __m128d _mm_load_pd(const double* p) { return *(const __m128d*)p; }
/* MOVAPD store: p must be 16-byte aligned */
FTE_SSE_INLINE void _mm_store_pd(double* p, __m128d a) { *(__m128d*)p = a; }
/* MOVHPD store: the upper lane to *p */
FTE_SSE_INLINE void _mm_storeh_pd(double* p, __m128d a) { *p = a[1]; }
/* {x, x} */
FTE_SSE_INLINE __m128d _mm_set1_pd(double x) {
    __m128d r = {x, x};
    return r;
}
/* {a, b}: a in the lower lane */
FTE_SSE_INLINE __m128d _mm_setr_pd(double a, double b) {
    __m128d r = {a, b};
    return r;
}
/* {b, a}: the argument order of _mm_set_pd is high lane first */
FTE_SSE_INLINE __m128d _mm_set_pd(double a, double b) {
    __m128d r = {b, a};
    return r;
}
FTE_SSE_INLINE __m128d _mm_setzero_pd(void) {
    __m128d r = {0.0, 0.0};
    return r;
}
/* unaligned load / store */
FTE_SSE_INLINE __m128d _mm_loadu_pd(const double* p) { return *(const fte_m128d_u*)p; }
FTE_SSE_INLINE void _mm_storeu_pd(double* p, __m128d a) { *(fte_m128d_u*)p = a; }

#undef FTE_SSE_INLINE
#endif
