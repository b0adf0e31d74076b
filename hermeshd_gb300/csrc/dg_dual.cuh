// dg_dual.cuh -- forward-mode dual numbers for the adjoint kernels.
//
// Dual{v, d} carries a value and one directional derivative.  The point-wise
// physics of dg_physics.cuh (primitives, point flux, HLLC, Roe) is templated
// on its arithmetic type; instantiated with Dual it returns, besides the
// primal result, the derivative along the seeded input direction -- one
// column of the point Jacobian per pass.  Branches (floors, HLLC wave
// selection, min/max) follow the primal values, i.e. the derivative of the
// branch that is active, which is the derivative of the reference's
// piecewise-smooth scheme away from its switching surfaces.
//
// The type and its functions live in a nested namespace: found by
// argument-dependent lookup for Dual arguments, they do not hide the
// double-precision math functions from unqualified calls in namespace hermes.
#pragma once

#include <cmath>

namespace hermes {
namespace ad {

struct Dual {
    double v, d;
    __host__ __device__ Dual() : v(0.0), d(0.0) {}
    __host__ __device__ Dual(double x) : v(x), d(0.0) {}
    __host__ __device__ Dual(double x, double dx) : v(x), d(dx) {}
};

__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { a = a + b; return a; }
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { a = a - b; return a; }
__device__ __forceinline__ Dual& operator*=(Dual& a, Dual b) { a = a * b; return a; }
__device__ __forceinline__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(Dual a, Dual b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
__device__ __forceinline__ bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
__device__ __forceinline__ bool operator==(Dual a, Dual b) { return a.v == b.v; }
__device__ __forceinline__ bool operator!=(Dual a, Dual b) { return a.v != b.v; }

__device__ __forceinline__ Dual fma(Dual a, Dual b, Dual c) {
    return Dual(::fma(a.v, b.v, c.v), a.d * b.v + a.v * b.d + c.d);
}
__device__ __forceinline__ Dual sqrt(Dual a) {
    const double s = ::sqrt(a.v);
    return Dual(s, a.d / (2.0 * s));
}
__device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0.0 ? -a : a; }
__device__ __forceinline__ Dual fmin(Dual a, Dual b) { return (b.v < a.v) ? b : a; }
__device__ __forceinline__ Dual fmax(Dual a, Dual b) { return (b.v > a.v) ? b : a; }
__device__ __forceinline__ Dual pow(Dual a, Dual b) {
    // only constant exponents occur (Tait EOS)
    const double p = ::pow(a.v, b.v);
    return Dual(p, b.v * ::pow(a.v, b.v - 1.0) * a.d);
}

}  // namespace ad

using ad::Dual;

}  // namespace hermes
