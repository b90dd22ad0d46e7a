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
// a < b
__device__ __forceinline__ bool ff_lt(float2 a, float2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }
