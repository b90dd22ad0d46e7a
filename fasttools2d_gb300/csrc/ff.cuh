// ff.cuh -- float-float arithmetic: a value is the unevaluated sum hi + lo of
// two FP32 numbers (float2 .x = hi, .y = lo), about 48 significant bits.
// GB300 issues FP32 at 64 times its FP64 rate, so float-float work on the
// FP32 pipe is several times faster than FP64 wherever ~1e-14 relative
// accuracy is enough.  Products use the exact FMA product (Dekker 1971, "A
// floating-point technique for extending the available precision"), sums
// Knuth's two-sum; the _rn intrinsics keep the compiler from contracting or
// reassociating the error-free steps.
#pragma once

__device__ __forceinline__ float2 ff_split(double v) {
    const float hi = __double2float_rn(v);
    return make_float2(hi, __double2float_rn(v - (double)hi));
}
__device__ __forceinline__ double ff_join(float s, float c) { return (double)s + (double)c; }
__device__ __forceinline__ double ff_join(float2 a) { return (double)a.x + (double)a.y; }
// (s + c) renormalised, |s| >= |c| or s == 0
__device__ __forceinline__ float2 ff_norm(float s, float c) {
    const float h = __fadd_rn(s, c);
    return make_float2(h, __fsub_rn(c, __fsub_rn(h, s)));
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
// a + b
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    return ff_norm(s, __fadd_rn(e, __fadd_rn(a.y, b.y)));
}
// a b (error below ~2^-46 |a b|)
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    return ff_norm(p, e);
}
// a b for an FP32 b
__device__ __forceinline__ float2 ff_mulf(float2 a, float b) {
    const float p = __fmul_rn(a.x, b);
    float e = __fmaf_rn(a.x, b, -p);
    e = __fmaf_rn(a.y, b, e);
    return ff_norm(p, e);
}
// a^2
__device__ __forceinline__ float2 ff_sqr(float2 a) {
    const float p = __fmul_rn(a.x, a.x);
    float e = __fmaf_rn(a.x, a.x, -p);
    e = __fmaf_rn(__fadd_rn(a.x, a.x), a.y, e);
    return ff_norm(p, e);
}
// (s, c) += a b, s the running sum and c the collected low-order parts
__device__ __forceinline__ void ff_mac(float2 a, float2 b, float& s, float& c) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, e));
}
// (s, c) += a b for FP32 a, b with Kahan's compensated summation (Kahan
// 1965, "Further remarks on reducing truncation errors"): the product rounded
// once together with the carried compensation, s + c the running sum; the
// sum's error stays near one rounding of the total while each product keeps
// its own FP32 rounding
__device__ __forceinline__ void fs_mac(float a, float b, float& s, float& c) {
    const float y = __fmaf_rn(a, b, c);
    const float t = __fadd_rn(s, y);
    c = __fadd_rn(__fsub_rn(s, t), y);
    s = t;
}
// (s, c) += a
__device__ __forceinline__ void ff_acc(float2 a, float& s, float& c) {
    const float t = __fadd_rn(s, a.x);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(a.x, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, a.y));
}
// 1/a: hardware reciprocal and one Newton step with the residual formed by
// FMA (relative error ~2e-14)
__device__ __forceinline__ float2 ff_rcp(float2 a) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(a.x));
    float e = __fmaf_rn(-a.x, y, 1.0f);
    e = __fmaf_rn(-a.y, y, e);
    return ff_norm(y, __fmul_rn(y, e));
}
// x^n, n >= 0, by binary powering
__device__ __forceinline__ float2 ff_powi(float2 x, int n) {
    float2 r = make_float2(1.f, 0.f);
    while (n) {
        if (n & 1) r = ff_mul(r, x);
        n >>= 1;
        if (n) x = ff_mul(x, x);
    }
    return r;
}
// a < b
__device__ __forceinline__ bool ff_lt(float2 a, float2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }

// exp(-x) in float-float for -80 < x < 80 (0 beyond 80): n = round(64 x /
// ln 2), r = x - n ln2/64 with ln2/64 split in three FP32 parts
// (the first with 13 trailing zero bits, so n C1 is exact for n < 8192);
// exp(-r), |r| <= ln2/128, as 1 - r + r^2/2 in float-float plus the cubic and
// higher Taylor terms in FP32 (they are below 3e-8); 2^(-j/64) from a
// float-float table.  Relative error ~4e-14.
__device__ __forceinline__ float2 fte_expm_ff(float2 x, const float2* __restrict__ tab) {
    const float C1 = 1.082611084e-02f, C2 = 4.313856607e-06f, C3 = -2.016456257e-13f;
    const int n = __float2int_rn(x.x * 9.233248138e+01f);
    const float nf = (float)n;
    const float rh = __fsub_rn(x.x, __fmul_rn(nf, C1));
    const float p2 = __fmul_rn(nf, C2);
    const float e2 = __fmaf_rn(nf, C2, -p2);
    // r = rh - p2 + (x.lo - e2 - n C3)
    const float s = __fsub_rn(rh, p2);
    const float bb = __fsub_rn(s, rh);
    float e = __fadd_rn(__fsub_rn(rh, __fsub_rn(s, bb)), __fsub_rn(-p2, bb));
    e = __fsub_rn(__fsub_rn(__fadd_rn(e, x.y), e2), __fmul_rn(nf, C3));
    const float2 r = ff_norm(s, e);
    const float r1 = r.x;
    float q = __fmaf_rn(r1, -1.0f / 120.0f, 1.0f / 24.0f);
    q = __fmaf_rn(r1, q, -1.0f / 6.0f);
    q = __fmul_rn(q, __fmul_rn(r1, __fmul_rn(r1, r1)));
    // r^2 / 2 in float-float
    const float p = __fmul_rn(r1, r1);
    float pe = __fmaf_rn(r1, r1, -p);
    pe = __fmaf_rn(__fadd_rn(r1, r1), r.y, pe);
    float2 h = ff_norm(__fmul_rn(p, 0.5f), __fmul_rn(pe, 0.5f));
    h = ff_add(h, make_float2(q, 0.0f));
    h = ff_add(h, ff_neg(r));
    h = ff_add(make_float2(1.0f, 0.0f), h);
    const float2 m = ff_mul(h, tab[n & 63]);
    const float sc = __int_as_float((127 - (n >> 6)) << 23);  // 2^-(n >> 6) (n >> 6 floors)
    return x.x < 80.0f ? make_float2(__fmul_rn(m.x, sc), __fmul_rn(m.y, sc)) : make_float2(0.0f, 0.0f);
}
