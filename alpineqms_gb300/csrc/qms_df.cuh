// qms_df.cuh -- double-float ("qdf") arithmetic: a value is the unevaluated sum h + l of two
// FP32 numbers with |l| <= ulp(h) / 2, about 48 significant bits.  GB300 executes FP64 at a
// small fraction of its FP32 rate, so the refinement residual of the mixed solver is
// evaluated in this format on the FP32 pipe.
//
// Building blocks (error-free transformations):
//   two_sum (Knuth, TAOCP vol. 2, 4.2.2):  s + e = a + b exactly, s = fl(a + b)
//   fast_two_sum (Dekker 1971):             the same when |a| >= |b|
//   two_prod with FMA:                      p + e = a b exactly, e = fma(a, b, -p)
// Addition is the "sloppy" double-word sum: its absolute error is a few units of 2^-48 of
// the larger operand, which is what a residual of difference-form rows needs.  Products follow
// the double-word times double-word scheme of Joldes, Muller and Popescu (ACM TOMS 44, 2017).
// Products return the pair without the final renormalisation (fast_two_sum): the high word is
// the float product and the low word gathers the rounding error and the cross terms, so |l|
// may reach a few units of ulp(h) instead of ulp(h) / 2 -- a product never cancels, so h still
// carries the value, and the next sum or product takes such a pair as it is.  Sums stay
// renormalised: a difference can cancel its high words, and a product of an unnormalised
// difference would lose the low word's cross term.
#pragma once
#include <cuda_runtime.h>

struct qdf {
    float h, l;
    __host__ __device__ qdf() : h(0.f), l(0.f) {}
    __host__ __device__ qdf(int v) : h((float)v), l(0.f) {}
    __host__ __device__ qdf(float v) : h(v), l(0.f) {}
    __host__ __device__ qdf(float a, float b) : h(a), l(b) {}
    // host only: the exact split of a double into its nearest float and the float of the rest
    __host__ explicit qdf(double d) {
        h = (float)d;
        l = (float)(d - (double)h);
    }
};

// Every operation below is an explicitly rounded intrinsic: the transformations are exact
// only if no product is contracted with a later sum into an FMA.
__device__ __forceinline__ void qdf_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void qdf_fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ qdf operator+(qdf x, qdf y) {
    float s, e;
    qdf_two_sum(x.h, y.h, s, e);
    e = __fadd_rn(e, __fadd_rn(x.l, y.l));
    qdf r;
    qdf_fast_two_sum(s, e, r.h, r.l);
    return r;
}
__device__ __forceinline__ qdf operator-(qdf x) { return qdf(-x.h, -x.l); }
__device__ __forceinline__ qdf operator-(qdf x, qdf y) { return x + (-y); }
__device__ __forceinline__ qdf operator*(qdf x, qdf y) {
    const float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return qdf(p, e);
}
// x / y: a float quotient, corrected once with the double-float remainder x - q y
__device__ __forceinline__ qdf operator/(qdf x, qdf y) {
    const float q1 = __fdiv_rn(x.h, y.h);
    const qdf r = x - y * qdf(q1);
    const float q2 = __fdiv_rn(r.h, y.h);
    qdf out;
    qdf_fast_two_sum(q1, q2, out.h, out.l);
    return out;
}
__device__ __forceinline__ qdf& operator+=(qdf& x, qdf y) { return x = x + y; }
__device__ __forceinline__ qdf fmax(qdf a, qdf b) { return (a.h > b.h || (a.h == b.h && a.l >= b.l)) ? a : b; }

// Split of a double into a qdf with integer operations only (no FP64 instruction): the high
// word keeps the leading 24 significant bits (truncated), the low word the float nearest to
// the remaining 29 bits.  Magnitudes below 2^-126 give 0, and the low word below 2^-74 is
// dropped (absolute errors under 1e-29); values this small do not occur in the solver.
__device__ __forceinline__ qdf qdf_split(double d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned e = (unsigned)(u >> 52) & 0x7FFu;
    if (e < 897u || e > 1150u) return qdf(0.f, 0.f);
    const unsigned sign = (unsigned)(u >> 63) << 31;
    const float h = __uint_as_float(sign | ((e - 896u) << 23) | ((unsigned)(u >> 29) & 0x7FFFFFu));
    const unsigned mlo = (unsigned)(u & 0x1FFFFFFFull);
    float l = 0.f;
    const int ee = (int)e - 1075;                 // exponent of the last bit of the double
    if (mlo != 0u && ee >= -126) {
        l = __uint2float_rn(mlo) * __uint_as_float((unsigned)(ee + 127) << 23);
        if (sign) l = -l;
    }
    return qdf(h, l);
}
