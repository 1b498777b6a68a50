// dfloat.cuh -- double-float ("float-float") arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum h + l of two floats, about 48 significant
// bits.  The algorithms are the classic error-free transformations: Knuth's
// TwoSum, Dekker's FastTwoSum and the FMA form of Dekker's TwoProduct
// (T. J. Dekker, "A floating-point technique for extending the available
// precision", Numer. Math. 18, 1971; the double-double library of Hida, Li
// and Bailey, 2001, uses the same building blocks).  On GB300 the FP64 pipe
// issues about one hundredth of the FP32 rate, so an FP64 kernel that is
// arithmetic-bound runs several times faster when its products and sums are
// taken in double-float; conversions from FP64 are done on the bits with
// integer operations, never on the FP64 pipe.
//
// Every operation uses the round-to-nearest intrinsics, so the compiler can
// neither contract nor reorder the error terms.
#pragma once
#include <cuda_runtime.h>

namespace ples {

struct dfl {
    float h, l;
};

__device__ __forceinline__ dfl two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a + b: TwoSum of the heads, the tails added to its error, renormalised.
// The error is a few units of 2^-47 of max(|a|, |b|) (an absolute bound,
// which is what a residual r = b - L(x) needs: its terms are summed, not
// divided).
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    dfl s = two_sum(a.h, b.h);
    s.l = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
    return fast_two_sum(s.h, s.l);
}

__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, dfl{-b.h, -b.l}); }

// a * b: the exact product of the heads (TwoProduct by FMA) plus the cross
// terms; relative error a few units of 2^-47
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}

// a*d + b1*s1 + b2*s2
__device__ __forceinline__ dfl df_dot3(dfl a, dfl d, dfl b1, dfl s1, dfl b2, dfl s2) {
    return df_add(df_add(df_mul(a, d), df_mul(b1, s1)), df_mul(b2, s2));
}

// 2^e as a float for -126 <= e <= 127
__device__ __forceinline__ float pow2f(int e) { return __uint_as_float((unsigned)(e + 127) << 23); }

// v * 2^o as a double-float, from the bits of v by integer operations.  The
// head is the top 24 significand bits of v (truncated), the tail the other
// 29 rounded to 24, so the split loses at most 2^-48 |v|.  With the scale
// applied: results below 2^-100 become zero (zeros and FP64 subnormals
// included) and keep no tail below 2^-74; results above 2^127, infinities
// and NaNs become infinite (a residual formed from them is not finite, which
// the solver reports as divergence).  The callers choose o so that the
// values they split lie near 1.
__device__ __forceinline__ dfl df_from_double(double v, int o) {
    const int hw = __double2hiint(v);
    const unsigned lw = (unsigned)__double2loint(v);
    const int e = ((hw >> 20) & 0x7FF) - 1023 + o;  // unbiased exponent of v * 2^o
    const unsigned sgn = (unsigned)hw & 0x80000000u;
    const unsigned m23 = (((unsigned)hw & 0xFFFFFu) << 3) | (lw >> 29);
    const unsigned hb = e > 127 ? 0x7F800000u : (e < -100 ? 0u : ((unsigned)(e + 127) << 23) | m23);
    // tail: (lw mod 2^29) units of 2^(e - 52).  Its top 23 and low 6 bits
    // become floats exactly by the 2^23 magic number (FP32 adds, no
    // conversion instruction) and are joined with one rounding; the scale
    // 2^(e - 52) is a normal float for e >= -74
    const unsigned t29 = lw & 0x1FFFFFFFu;
    const float th = __fsub_rn(__uint_as_float(0x4B000000u | (t29 >> 6)), 8388608.f);
    const float tl = __fsub_rn(__uint_as_float(0x4B000000u | (t29 & 63u)), 8388608.f);
    const float t = __fmul_rn(__fmaf_rn(th, 64.f, tl), pow2f(max(e, -74) - 52));
    return {__uint_as_float(sgn | hb), (e < -74 || e > 127) ? 0.f : (sgn ? -t : t)};
}

// the float nearest to a double-float times 2^-o (-126 <= -o <= 127)
__device__ __forceinline__ float df_to_float(dfl a, int o) { return __fmul_rn(__fadd_rn(a.h, a.l), pow2f(-o)); }

}  // namespace ples
