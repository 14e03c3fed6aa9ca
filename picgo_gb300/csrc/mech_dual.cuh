// Forward-mode dual numbers for the Hessian-vector products: a value and its
// derivative along one direction.  Evaluating a force routine on positions
// x + eps v with eps infinitesimal gives F(x) in .v and dF/dx . v in .d, i.e.
// minus the Hessian of the energy applied to v.  Only the operations the force
// routines use are defined; comparisons look at the value.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace mech {

// the dual overloads below would hide the C library's functions from
// unqualified calls inside this namespace; keep both visible
using ::atan2;
using ::cos;
using ::exp;
using ::fabs;
using ::fmax;
using ::sin;
using ::sqrt;

struct Dual {
    double v, d;
    __host__ __device__ Dual() : v(0.0), d(0.0) {}
    __host__ __device__ Dual(double a) : v(a), d(0.0) {}
    __host__ __device__ Dual(double a, double b) : v(a), d(b) {}
    __host__ __device__ Dual& operator+=(const Dual& o) { v += o.v; d += o.d; return *this; }
    __host__ __device__ Dual& operator-=(const Dual& o) { v -= o.v; d -= o.d; return *this; }
    __host__ __device__ Dual& operator*=(const Dual& o) { d = d * o.v + v * o.d; v *= o.v; return *this; }
};

__host__ __device__ inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__host__ __device__ inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__host__ __device__ inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__host__ __device__ inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__host__ __device__ inline Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return Dual(q, (a.d - q * b.d) / b.v);
}
__host__ __device__ inline Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
__host__ __device__ inline Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
__host__ __device__ inline Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
__host__ __device__ inline Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
__host__ __device__ inline Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
__host__ __device__ inline Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
__host__ __device__ inline Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
__host__ __device__ inline Dual operator/(double a, Dual b) {
    const double q = a / b.v;
    return Dual(q, -q * b.d / b.v);
}

__host__ __device__ inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
__host__ __device__ inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
__host__ __device__ inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
__host__ __device__ inline bool operator>=(Dual a, Dual b) { return a.v >= b.v; }

__device__ inline Dual sqrt(Dual a) {
    const double s = ::sqrt(a.v);
    return Dual(s, a.d / (2.0 * s));
}
__device__ inline Dual fabs(Dual a) { return a.v < 0 ? -a : a; }
__device__ inline Dual fmax(Dual a, Dual b) { return a.v >= b.v ? a : b; }
__device__ inline Dual exp(Dual a) {
    const double e = ::exp(a.v);
    return Dual(e, e * a.d);
}
__device__ inline Dual cos(Dual a) { return Dual(::cos(a.v), -::sin(a.v) * a.d); }
__device__ inline Dual sin(Dual a) { return Dual(::sin(a.v), ::cos(a.v) * a.d); }
// d atan2(y, x) = (x dy - y dx) / (x^2 + y^2)
__device__ inline Dual atan2(Dual y, Dual x) {
    return Dual(::atan2(y.v, x.v), (x.v * y.d - y.v * x.d) / (x.v * x.v + y.v * y.v));
}
__device__ inline Dual atan_of(Dual a) { return Dual(::atan(a.v), a.d / (1.0 + a.v * a.v)); }
__device__ inline bool near_zero_theta(Dual t) { return ::fabs(t.v - 0.0) < 1e-6; }

}  // namespace mech
