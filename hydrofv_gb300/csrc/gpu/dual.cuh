/*
 * dual.cuh -- forward-mode dual numbers for the tangent-linear step.
 *
 * Dual{v, d} carries a value and its directional derivative.  Every
 * operator computes the value with exactly the operation the plain double
 * code performs (so a kernel instantiated with Dual reproduces the FP64
 * primal bit for bit when compiled with --fmad=false) and the derivative by
 * the chain rule.  Comparisons look at the value only: a template run on
 * Dual takes the branches the primal takes, which is what "branches
 * replayed from the forward pass" means for the tangent-linear model.
 *
 * Conventions at non-differentiable points, shared with the hand-written
 * reverse-mode code (adjoint_numerics.cuh) so that the two are exact
 * transposes of each other:
 *   fabs(x)     derivative sign(x), +1 at x == 0;
 *   fmin(x, y)  the derivative of x unless y < x (ties take x);
 *   pow(x, y)   y is a constant (its derivative is ignored).
 */
#ifndef HYDRO_GPU_DUAL_CUH
#define HYDRO_GPU_DUAL_CUH

#include <math.h>

#include "pow_int.cuh"

#ifdef __CUDACC__
#define DHD __host__ __device__ __forceinline__
#else
#define DHD static inline
#endif

namespace hydro {

struct Dual {
    double v, d;
    DHD Dual() : v(0.0), d(0.0) {}
    DHD Dual(double x) : v(x), d(0.0) {}
    DHD Dual(double x, double dx) : v(x), d(dx) {}
    DHD explicit operator double() const { return v; }
};

DHD Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
DHD Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
DHD Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
DHD Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
DHD Dual operator/(Dual a, Dual b)
{
    const double q = dv(a.v, b.v);
    return Dual(q, dv(a.d - q * b.d, b.v));
}
DHD Dual &operator+=(Dual &a, Dual b) { a = a + b; return a; }
DHD Dual &operator-=(Dual &a, Dual b) { a = a - b; return a; }

DHD bool operator<(Dual a, Dual b) { return a.v < b.v; }
DHD bool operator>(Dual a, Dual b) { return a.v > b.v; }
DHD bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
DHD bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
DHD bool operator==(Dual a, Dual b) { return a.v == b.v; }
DHD bool operator!=(Dual a, Dual b) { return a.v != b.v; }

DHD Dual sqrt(Dual a)
{
    const double s = sq(a.v);
    return Dual(s, dv(a.d, 2.0 * s));
}

DHD Dual fabs(Dual a) { return (a.v < 0.0) ? -a : a; }

DHD Dual fmin(Dual a, Dual b) { return (b.v < a.v) ? b : a; }

/* x^y with a constant exponent: d = y * x^y / x * dx. */
DHD Dual pow(Dual x, Dual y)
{
    const double p = pw(x.v, y.v);
    return Dual(p, y.v * dv(p, x.v) * x.d);
}

}  // namespace hydro

#endif
