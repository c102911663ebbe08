// Forward-mode dual number with one tangent direction, used to differentiate
// the Gauss-point physics (vefem_physics.cuh) for the exact Jacobian.
// sqrt and fabs take the derivative 0 at 0 (a subgradient), where the
// classical derivative does not exist; sqrt of a negative (round-off)
// argument is 0 with derivative 0.
#pragma once

#include <math.h>

#include <type_traits>

#include "vefem_scalar.cuh"

#ifdef __CUDACC__
#define VD_HD __host__ __device__ __forceinline__
#else
#define VD_HD inline
#endif

namespace vefem {

// plain overloads: the Dual templates below would otherwise hide the global
// math functions from unqualified calls inside this namespace
VD_HD double sqrt(double x) { return ::sqrt(x); }
VD_HD float sqrt(float x) { return ::sqrtf(x); }
VD_HD double exp(double x) { return ::exp(x); }
VD_HD float exp(float x) { return ::expf(x); }
VD_HD double fabs(double x) { return ::fabs(x); }
VD_HD float fabs(float x) { return ::fabsf(x); }

template <class T>
struct Dual {
    T v, d;
    VD_HD Dual() : v(0), d(0) {}
    VD_HD Dual(double x) : v((T)x), d(0) {}
    VD_HD Dual(T x, T dx) : v(x), d(dx) {}
};

template <class T>
struct ScalarOf<Dual<T>> {
    typedef T type;
};

template <class T> VD_HD Dual<T> operator+(Dual<T> a, Dual<T> b) { return Dual<T>(a.v + b.v, a.d + b.d); }
template <class T> VD_HD Dual<T> operator-(Dual<T> a, Dual<T> b) { return Dual<T>(a.v - b.v, a.d - b.d); }
template <class T> VD_HD Dual<T> operator*(Dual<T> a, Dual<T> b)
{
    return Dual<T>(a.v * b.v, a.d * b.v + a.v * b.d);
}
template <class T> VD_HD Dual<T> operator/(Dual<T> a, Dual<T> b)
{
    const T q = a.v / b.v;
    return Dual<T>(q, (a.d - q * b.d) / b.v);
}
template <class T> VD_HD Dual<T> operator-(Dual<T> a) { return Dual<T>(-a.v, -a.d); }

// Dual (op) scalar: the scalar is converted to T once (a float path never
// widens to FP64, whose pipe is narrow on this GPU; literals fold)
#define VD_SCALAR template <class T, class U, typename std::enable_if<std::is_arithmetic<U>::value, int>::type = 0>
VD_SCALAR VD_HD Dual<T> operator+(Dual<T> a, U b) { return Dual<T>(a.v + (T)b, a.d); }
VD_SCALAR VD_HD Dual<T> operator-(Dual<T> a, U b) { return Dual<T>(a.v - (T)b, a.d); }
VD_SCALAR VD_HD Dual<T> operator*(Dual<T> a, U b) { return Dual<T>(a.v * (T)b, a.d * (T)b); }
VD_SCALAR VD_HD Dual<T> operator/(Dual<T> a, U b) { return Dual<T>(a.v / (T)b, a.d / (T)b); }
VD_SCALAR VD_HD Dual<T> operator+(U a, Dual<T> b) { return Dual<T>((T)a + b.v, b.d); }
VD_SCALAR VD_HD Dual<T> operator-(U a, Dual<T> b) { return Dual<T>((T)a - b.v, -b.d); }
VD_SCALAR VD_HD Dual<T> operator*(U a, Dual<T> b) { return Dual<T>((T)a * b.v, (T)a * b.d); }
VD_SCALAR VD_HD Dual<T> operator/(U a, Dual<T> b)
{
    const T q = (T)a / b.v;
    return Dual<T>(q, -q * b.d / b.v);
}
#undef VD_SCALAR

template <class T> VD_HD Dual<T> sqrt(Dual<T> a)
{
    // A negative argument is round-off of a quantity that is non-negative in
    // the FP64 residual: the magnitude sqrt(0.5 C:C^T) of the constitutive
    // residual C, which vanishes for an exact parallel-flow state, rounds
    // below zero in FP32 when C12 and C21 are noise of opposite signs.  The
    // Jacobian then takes value and derivative 0 (the subgradient at 0)
    // instead of NaN; a NaN argument stays NaN.
    if (a.v < (T)0) return Dual<T>((T)0, (T)0);
    const T r = sqrt(a.v);
    return Dual<T>(r, r > (T)0 ? a.d / (r + r) : (T)0);
}
template <class T> VD_HD Dual<T> exp(Dual<T> a)
{
    const T e = exp(a.v);
    return Dual<T>(e, e * a.d);
}
template <class T> VD_HD Dual<T> fabs(Dual<T> a)
{
    return Dual<T>(fabs(a.v), a.v > (T)0 ? a.d : (a.v < (T)0 ? -a.d : (T)0));
}

}  // namespace vefem
