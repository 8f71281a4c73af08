// Forward-mode dual numbers for the tangent (Jacobian-vector product) kernels,
// with the semantics of ibis's Dual<T> (src/util/util/dual.h:11-346), so that
// the tangent of the residual reproduces the reference's dual-number Jv,
// branch choices included:
//   * comparisons look at the real part only;
//   * min/max return one operand chosen by real part, ties return the second;
//   * abs flips both parts when the real part is negative;
//   * floor is applied to both parts; copysign keeps or flips the dual part;
//   * pow(b, p) = (b^p, b' p b^(p-1) + p' b^p log b).
// DualT<true> (Dual) is that type.  DualT<false> (DualA) differs only in floor,
// whose dual part it sets to zero, the derivative of a step function: the
// reference's rule makes the tangent of LDFSS2 (whose switches go through floor)
// nonlinear in the direction, which no adjoint can transpose, so the adjoint
// kernels evaluate local derivatives with DualA.
#pragma once

#include <cuda_runtime.h>

namespace ibisgb {

template <bool RefFloor>
struct DualT {
    double re, du;
    __host__ __device__ __forceinline__ DualT() : re(0.0), du(0.0) {}
    __host__ __device__ __forceinline__ DualT(double r) : re(r), du(0.0) {}
    __host__ __device__ __forceinline__ DualT(double r, double d) : re(r), du(d) {}
    __host__ __device__ __forceinline__ explicit DualT(float r) : re((double)r), du(0.0) {}
    __host__ __device__ __forceinline__ explicit DualT(int r) : re((double)r), du(0.0) {}
    __device__ __forceinline__ DualT operator-() const { return DualT(-re, -du); }
    __device__ __forceinline__ DualT& operator+=(const DualT& o) { re += o.re; du += o.du; return *this; }
    __device__ __forceinline__ DualT& operator-=(const DualT& o) { re -= o.re; du -= o.du; return *this; }
};

template <bool B>
__device__ __forceinline__ DualT<B> operator+(const DualT<B>& a, const DualT<B>& b) {
    return DualT<B>(a.re + b.re, a.du + b.du);
}
template <bool B>
__device__ __forceinline__ DualT<B> operator-(const DualT<B>& a, const DualT<B>& b) {
    return DualT<B>(a.re - b.re, a.du - b.du);
}
template <bool B>
__device__ __forceinline__ DualT<B> operator*(const DualT<B>& a, const DualT<B>& b) {
    return DualT<B>(a.re * b.re, a.re * b.du + a.du * b.re);
}
template <bool B>
__device__ __forceinline__ DualT<B> operator/(const DualT<B>& a, const DualT<B>& b) {
    return DualT<B>(a.re / b.re, (a.du * b.re - a.re * b.du) / (b.re * b.re));
}
template <bool B> __device__ __forceinline__ bool operator<(const DualT<B>& a, const DualT<B>& b) { return a.re < b.re; }
template <bool B> __device__ __forceinline__ bool operator>(const DualT<B>& a, const DualT<B>& b) { return a.re > b.re; }
template <bool B> __device__ __forceinline__ bool operator<=(const DualT<B>& a, const DualT<B>& b) { return a.re <= b.re; }
template <bool B> __device__ __forceinline__ bool operator>=(const DualT<B>& a, const DualT<B>& b) { return a.re >= b.re; }
template <bool B> __device__ __forceinline__ bool operator==(const DualT<B>& a, const DualT<B>& b) { return a.re == b.re; }
template <bool B> __device__ __forceinline__ bool operator!=(const DualT<B>& a, const DualT<B>& b) { return a.re != b.re; }

template <bool B>
__device__ __forceinline__ DualT<B> dual_sqrt(DualT<B> d) {
    double r = sqrt(d.re);
    return DualT<B>(r, d.du / (2.0 * r));
}
template <bool B>
__device__ __forceinline__ DualT<B> dual_pow(DualT<B> b, DualT<B> p) {
    double r = pow(b.re, p.re);
    return DualT<B>(r, b.du * p.re * pow(b.re, p.re - 1.0) + p.du * r * log(b.re));
}
template <bool B>
__device__ __forceinline__ DualT<B> dual_copysign(DualT<B> m, DualT<B> s) {
    double r = copysign(m.re, s.re);
    return DualT<B>(r, (r - m.re) < 1e-15 ? m.du : -m.du);
}

template <> __device__ __forceinline__ Dual d_sqrt<Dual>(Dual d) { return dual_sqrt(d); }
template <> __device__ __forceinline__ DualA d_sqrt<DualA>(DualA d) { return dual_sqrt(d); }
template <> __device__ __forceinline__ Dual d_abs<Dual>(Dual d) { return d.re < 0.0 ? -d : d; }
template <> __device__ __forceinline__ DualA d_abs<DualA>(DualA d) { return d.re < 0.0 ? -d : d; }
template <> __device__ __forceinline__ Dual d_pow<Dual>(Dual b, Dual p) { return dual_pow(b, p); }
template <> __device__ __forceinline__ DualA d_pow<DualA>(DualA b, DualA p) { return dual_pow(b, p); }
template <> __device__ __forceinline__ Dual d_floor<Dual>(Dual d) { return Dual(floor(d.re), floor(d.du)); }
template <> __device__ __forceinline__ DualA d_floor<DualA>(DualA d) { return DualA(floor(d.re), 0.0); }
template <> __device__ __forceinline__ Dual d_copysign<Dual>(Dual m, Dual s) { return dual_copysign(m, s); }
template <> __device__ __forceinline__ DualA d_copysign<DualA>(DualA m, DualA s) { return dual_copysign(m, s); }
template <> __device__ __forceinline__ Dual d_min<Dual>(Dual a, Dual b) { return a.re < b.re ? a : b; }
template <> __device__ __forceinline__ DualA d_min<DualA>(DualA a, DualA b) { return a.re < b.re ? a : b; }
template <> __device__ __forceinline__ Dual d_max<Dual>(Dual a, Dual b) { return a.re > b.re ? a : b; }
template <> __device__ __forceinline__ DualA d_max<DualA>(DualA a, DualA b) { return a.re > b.re ? a : b; }

template <bool B>
__device__ __forceinline__ double real_of(const DualT<B>& x) { return x.re; }

}  // namespace ibisgb
