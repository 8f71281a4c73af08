// Forward-mode dual numbers for the tangent (Jacobian-vector product) kernels,
// with the semantics of ibis's Dual<T> (src/util/util/dual.h:11-346), so that
// the tangent of the residual reproduces the reference's dual-number Jv,
// branch choices included:
//   * comparisons look at the real part only;
//   * min/max return one operand chosen by real part, ties return the second;
//   * abs flips both parts when the real part is negative;
//   * floor is applied to both parts; copysign keeps or flips the dual part;
//   * pow(b, p) = (b^p, b' p b^(p-1) + p' b^p log b).
#pragma once

#include <cuda_runtime.h>

namespace ibisgb {

struct Dual {
    double re, du;
    __host__ __device__ __forceinline__ Dual() : re(0.0), du(0.0) {}
    __host__ __device__ __forceinline__ Dual(double r) : re(r), du(0.0) {}
    __host__ __device__ __forceinline__ Dual(double r, double d) : re(r), du(d) {}
    __host__ __device__ __forceinline__ explicit Dual(float r) : re((double)r), du(0.0) {}
    __host__ __device__ __forceinline__ explicit Dual(int r) : re((double)r), du(0.0) {}
    __device__ __forceinline__ Dual operator-() const { return Dual(-re, -du); }
    __device__ __forceinline__ Dual& operator+=(const Dual& o) { re += o.re; du += o.du; return *this; }
    __device__ __forceinline__ Dual& operator-=(const Dual& o) { re -= o.re; du -= o.du; return *this; }
};

__device__ __forceinline__ Dual operator+(const Dual& a, const Dual& b) { return Dual(a.re + b.re, a.du + b.du); }
__device__ __forceinline__ Dual operator-(const Dual& a, const Dual& b) { return Dual(a.re - b.re, a.du - b.du); }
__device__ __forceinline__ Dual operator*(const Dual& a, const Dual& b) {
    return Dual(a.re * b.re, a.re * b.du + a.du * b.re);
}
__device__ __forceinline__ Dual operator/(const Dual& a, const Dual& b) {
    return Dual(a.re / b.re, (a.du * b.re - a.re * b.du) / (b.re * b.re));
}
__device__ __forceinline__ bool operator<(const Dual& a, const Dual& b) { return a.re < b.re; }
__device__ __forceinline__ bool operator>(const Dual& a, const Dual& b) { return a.re > b.re; }
__device__ __forceinline__ bool operator<=(const Dual& a, const Dual& b) { return a.re <= b.re; }
__device__ __forceinline__ bool operator>=(const Dual& a, const Dual& b) { return a.re >= b.re; }
__device__ __forceinline__ bool operator==(const Dual& a, const Dual& b) { return a.re == b.re; }
__device__ __forceinline__ bool operator!=(const Dual& a, const Dual& b) { return a.re != b.re; }

template <> __device__ __forceinline__ Dual d_sqrt<Dual>(Dual d) {
    double r = sqrt(d.re);
    return Dual(r, d.du / (2.0 * r));
}
template <> __device__ __forceinline__ Dual d_abs<Dual>(Dual d) { return d.re < 0.0 ? -d : d; }
template <> __device__ __forceinline__ Dual d_pow<Dual>(Dual b, Dual p) {
    double r = pow(b.re, p.re);
    return Dual(r, b.du * p.re * pow(b.re, p.re - 1.0) + p.du * r * log(b.re));
}
template <> __device__ __forceinline__ Dual d_floor<Dual>(Dual d) { return Dual(floor(d.re), floor(d.du)); }
template <> __device__ __forceinline__ Dual d_copysign<Dual>(Dual m, Dual s) {
    double r = copysign(m.re, s.re);
    return Dual(r, (r - m.re) < 1e-15 ? m.du : -m.du);
}
__device__ __forceinline__ double real_of(const Dual& x) { return x.re; }

template <> __device__ __forceinline__ Dual d_min<Dual>(Dual a, Dual b) { return a.re < b.re ? a : b; }
template <> __device__ __forceinline__ Dual d_max<Dual>(Dual a, Dual b) { return a.re > b.re ? a : b; }

}  // namespace ibisgb
