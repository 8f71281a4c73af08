// Float-float arithmetic ("double-single"): a value is the unevaluated sum
// hi + lo of two floats with |lo| <= ulp(hi) / 2, about 48 significant bits.
// Every operation runs on the FP32 pipe, which GB300 issues 64 times faster
// than the FP64 pipe.  The operations are built from the error-free
// transformations of floating-point arithmetic (Knuth's TwoSum, Dekker's
// FastTwoSum, and the exact product error of a fused multiply-add) and one
// Newton correction for division and square root; each is within a few units
// of 2^-48 of its operands' magnitude.  The explicit _rn intrinsics keep the
// compiler from contracting or reassociating the error terms.
#pragma once

#include <cuda_runtime.h>

namespace ibisgb {

#define IBISGB_FF_HD __host__ __device__ __forceinline__

struct FF {
    float hi, lo;

    FF() = default;
    IBISGB_FF_HD constexpr FF(float h, float l) : hi(h), lo(l) {}
    IBISGB_FF_HD constexpr FF(float h) : hi(h), lo(0.f) {}
    IBISGB_FF_HD constexpr FF(int h) : hi((float)h), lo(0.f) {}
    // from a double: hi is its rounding to float, lo the rounding of the rest.
    // Constant-folded for literals; at run time it costs a double subtraction,
    // so device code splits run-time doubles with d2ff instead.
    IBISGB_FF_HD constexpr FF(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

#if defined(__CUDA_ARCH__)
#define FF_ADD(a, b) __fadd_rn(a, b)
#define FF_SUB(a, b) __fsub_rn(a, b)
#define FF_MUL(a, b) __fmul_rn(a, b)
#define FF_FMA(a, b, c) __fmaf_rn(a, b, c)
#else
#define FF_ADD(a, b) ((a) + (b))
#define FF_SUB(a, b) ((a) - (b))
#define FF_MUL(a, b) ((a) * (b))
#define FF_FMA(a, b, c) fmaf(a, b, c)
#endif

// s + e = a + b exactly (TwoSum, any magnitudes)
IBISGB_FF_HD FF ff_two_sum(float a, float b) {
    const float s = FF_ADD(a, b);
    const float bb = FF_SUB(s, a);
    const float e = FF_ADD(FF_SUB(a, FF_SUB(s, bb)), FF_SUB(b, bb));
    return FF(s, e);
}
// s + e = a + b exactly when |a| >= |b| or a == 0 (FastTwoSum): renormalisation
IBISGB_FF_HD FF ff_fast_two_sum(float a, float b) {
    const float s = FF_ADD(a, b);
    return FF(s, FF_SUB(b, FF_SUB(s, a)));
}

IBISGB_FF_HD FF operator-(const FF& a) { return FF(-a.hi, -a.lo); }

IBISGB_FF_HD FF operator+(const FF& a, const FF& b) {
    FF s = ff_two_sum(a.hi, b.hi);
    const float e = FF_ADD(s.lo, FF_ADD(a.lo, b.lo));
    return ff_fast_two_sum(s.hi, e);
}
IBISGB_FF_HD FF operator+(const FF& a, float b) {
    FF s = ff_two_sum(a.hi, b);
    return ff_fast_two_sum(s.hi, FF_ADD(s.lo, a.lo));
}
IBISGB_FF_HD FF operator+(float a, const FF& b) { return b + a; }
IBISGB_FF_HD FF operator-(const FF& a, const FF& b) { return a + (-b); }
IBISGB_FF_HD FF operator-(const FF& a, float b) { return a + (-b); }
IBISGB_FF_HD FF operator-(float a, const FF& b) { return (-b) + a; }

IBISGB_FF_HD FF operator*(const FF& a, const FF& b) {
    const float p = FF_MUL(a.hi, b.hi);
    float e = FF_FMA(a.hi, b.hi, -p);
    e = FF_FMA(a.hi, b.lo, e);
    e = FF_FMA(a.lo, b.hi, e);
    return ff_fast_two_sum(p, e);
}
IBISGB_FF_HD FF operator*(const FF& a, float b) {
    const float p = FF_MUL(a.hi, b);
    float e = FF_FMA(a.hi, b, -p);
    e = FF_FMA(a.lo, b, e);
    return ff_fast_two_sum(p, e);
}
IBISGB_FF_HD FF operator*(float a, const FF& b) { return b * a; }

// a / b: a float quotient from the reciprocal, corrected once by the float-float
// remainder a - q b (the correction's own error is below 2^-46 |a / b|)
IBISGB_FF_HD FF operator/(const FF& a, const FF& b) {
    const float inv = 1.0f / b.hi;
    const float q1 = FF_MUL(a.hi, inv);
    const FF r = a - b * q1;
    const float q2 = FF_MUL(FF_ADD(r.hi, r.lo), inv);
    return ff_fast_two_sum(q1, q2);
}
IBISGB_FF_HD FF operator/(const FF& a, float b) { return a / FF(b); }
IBISGB_FF_HD FF operator/(float a, const FF& b) { return FF(a) / b; }

IBISGB_FF_HD FF& operator+=(FF& a, const FF& b) { return a = a + b; }
IBISGB_FF_HD FF& operator-=(FF& a, const FF& b) { return a = a - b; }
IBISGB_FF_HD FF& operator*=(FF& a, const FF& b) { return a = a * b; }
IBISGB_FF_HD FF& operator/=(FF& a, const FF& b) { return a = a / b; }

// comparisons of the represented values (hi first, then lo)
IBISGB_FF_HD bool operator<(const FF& a, const FF& b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
IBISGB_FF_HD bool operator>(const FF& a, const FF& b) { return b < a; }
IBISGB_FF_HD bool operator<=(const FF& a, const FF& b) { return !(b < a); }
IBISGB_FF_HD bool operator>=(const FF& a, const FF& b) { return !(a < b); }
IBISGB_FF_HD bool operator==(const FF& a, const FF& b) { return a.hi == b.hi && a.lo == b.lo; }
IBISGB_FF_HD bool operator!=(const FF& a, const FF& b) { return !(a == b); }

// square root: a float root corrected once by the exact remainder a - s^2
IBISGB_FF_HD FF ff_sqrt(const FF& a) {
    if (!(a.hi > 0.f)) return FF(a.hi == 0.f ? 0.f : sqrtf(a.hi), 0.f);  // 0, or NaN for a < 0
    const float s = sqrtf(a.hi);
    const float p = FF_MUL(s, s);
    const float pe = FF_FMA(s, s, -p);
    const float rem = FF_ADD(FF_SUB(FF_SUB(a.hi, p), pe), a.lo);
    return ff_fast_two_sum(s, FF_MUL(rem, 0.5f / s));
}
IBISGB_FF_HD FF ff_abs(const FF& a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f) ? -a : a; }
IBISGB_FF_HD FF ff_floor(const FF& a) {
    const float f = floorf(a.hi);
    if (f != a.hi) return FF(f, 0.f);
    return ff_fast_two_sum(f, floorf(a.lo));
}
IBISGB_FF_HD FF ff_copysign(const FF& m, const FF& s) {
    const bool neg_m = signbit(m.hi), neg_s = signbit(s.hi);
    return neg_m == neg_s ? m : -m;
}

// the double nearest hi + lo (one FP64 addition)
IBISGB_FF_HD double ff_to_double(const FF& a) { return (double)a.hi + (double)a.lo; }

#undef FF_ADD
#undef FF_SUB
#undef FF_MUL
#undef FF_FMA

}  // namespace ibisgb
