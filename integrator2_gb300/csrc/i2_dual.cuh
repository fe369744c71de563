// i2_dual.cuh -- forward-mode dual numbers for the adjoint kernels.
//
// Dual<T, N> carries a value and its derivatives with respect to N seeded inputs (here the three
// coordinates of one mesh vertex).  The templated geometry and integrands of i2_device.cuh run on
// it unchanged; every elementary operation applies its derivative rule, so the derivative of a
// pair integral is exact to rounding for the arithmetic the forward pass performs.  Branches
// (the reference's EPS tests, tier and refinement decisions) compare values only.  The math
// functions live in this namespace and are found by argument-dependent lookup; plain double code
// never sees them.
#pragma once

#include <cuda_runtime.h>

namespace i2 {
namespace ad {

template <class T, int N>
struct Dual {
    T v;
    T d[N];
    __device__ __forceinline__ Dual() {}
    __device__ __forceinline__ Dual(double x) : v((T)x)
    {
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = T(0);
    }
};

template <class T, int N>
__device__ __forceinline__ T value_of(const Dual<T, N> &a)
{
    return a.v;
}

// value and one derivative rule: f(a) with f'(a) = g
template <class T, int N>
__device__ __forceinline__ Dual<T, N> chain(const Dual<T, N> &a, T f, T g)
{
    Dual<T, N> r;
    r.v = f;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = g * a.d[k];
    return r;
}

template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator+(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N> &a)
{
    Dual<T, N> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator*(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator/(const Dual<T, N> &a, const Dual<T, N> &b)
{
    Dual<T, N> r;
    const T inv = T(1) / b.v;
    r.v = a.v * inv;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
    return r;
}
// with plain scalars
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator+(const Dual<T, N> &a, double s)
{
    Dual<T, N> r = a;
    r.v = a.v + (T)s;
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator+(double s, const Dual<T, N> &a)
{
    return a + s;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator-(const Dual<T, N> &a, double s)
{
    Dual<T, N> r = a;
    r.v = a.v - (T)s;
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator-(double s, const Dual<T, N> &a)
{
    Dual<T, N> r;
    r.v = (T)s - a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator*(const Dual<T, N> &a, double s)
{
    Dual<T, N> r;
    r.v = a.v * (T)s;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * (T)s;
    return r;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator*(double s, const Dual<T, N> &a)
{
    return a * s;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator/(const Dual<T, N> &a, double s)
{
    return a * (1.0 / s);
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> operator/(double s, const Dual<T, N> &a)
{
    const T inv = T(1) / a.v;
    const T f = (T)s * inv;
    return chain(a, f, -f * inv);
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> &operator+=(Dual<T, N> &a, const Dual<T, N> &b)
{
    a = a + b;
    return a;
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> &operator-=(Dual<T, N> &a, const Dual<T, N> &b)
{
    a = a - b;
    return a;
}

// comparisons look at values only
#define I2_DUAL_CMP(op)                                                                                                \
    template <class T, int N>                                                                                          \
    __device__ __forceinline__ bool operator op(const Dual<T, N> &a, const Dual<T, N> &b)                              \
    {                                                                                                                  \
        return a.v op b.v;                                                                                             \
    }                                                                                                                  \
    template <class T, int N>                                                                                          \
    __device__ __forceinline__ bool operator op(const Dual<T, N> &a, double b)                                         \
    {                                                                                                                  \
        return a.v op(T) b;                                                                                            \
    }                                                                                                                  \
    template <class T, int N>                                                                                          \
    __device__ __forceinline__ bool operator op(double a, const Dual<T, N> &b)                                         \
    {                                                                                                                  \
        return (T)a op b.v;                                                                                            \
    }
I2_DUAL_CMP(<)
I2_DUAL_CMP(>)
I2_DUAL_CMP(<=)
I2_DUAL_CMP(>=)
I2_DUAL_CMP(==)
I2_DUAL_CMP(!=)
#undef I2_DUAL_CMP

// elementary functions (derivative rules of calculus; the values come from CUDA's functions)
template <int N>
__device__ __forceinline__ Dual<double, N> sqrt(const Dual<double, N> &a)
{
    const double f = ::sqrt(a.v);
    return chain(a, f, 0.5 / f);
}
template <int N>
__device__ __forceinline__ Dual<float, N> sqrt(const Dual<float, N> &a)
{
    const float f = ::sqrtf(a.v);
    return chain(a, f, 0.5f / f);
}
template <int N>
__device__ __forceinline__ Dual<double, N> log(const Dual<double, N> &a)
{
    return chain(a, ::log(a.v), 1.0 / a.v);
}
template <int N>
__device__ __forceinline__ Dual<float, N> log(const Dual<float, N> &a)
{
    return chain(a, ::logf(a.v), 1.0f / a.v);
}
template <int N>
__device__ __forceinline__ Dual<double, N> log1p(const Dual<double, N> &a)
{
    return chain(a, ::log1p(a.v), 1.0 / (1.0 + a.v));
}
template <int N>
__device__ __forceinline__ Dual<float, N> log1p(const Dual<float, N> &a)
{
    return chain(a, ::log1pf(a.v), 1.0f / (1.0f + a.v));
}
template <int N>
__device__ __forceinline__ Dual<double, N> sin(const Dual<double, N> &a)
{
    double s, c;
    ::sincos(a.v, &s, &c);
    return chain(a, s, c);
}
template <int N>
__device__ __forceinline__ Dual<float, N> sin(const Dual<float, N> &a)
{
    float s, c;
    ::sincosf(a.v, &s, &c);
    return chain(a, s, c);
}
template <int N>
__device__ __forceinline__ Dual<double, N> cos(const Dual<double, N> &a)
{
    double s, c;
    ::sincos(a.v, &s, &c);
    return chain(a, c, -s);
}
template <int N>
__device__ __forceinline__ Dual<float, N> cos(const Dual<float, N> &a)
{
    float s, c;
    ::sincosf(a.v, &s, &c);
    return chain(a, c, -s);
}
template <int N>
__device__ __forceinline__ void sincos(const Dual<double, N> &a, Dual<double, N> *s, Dual<double, N> *c)
{
    double sv, cv;
    ::sincos(a.v, &sv, &cv);
    *s = chain(a, sv, cv);
    *c = chain(a, cv, -sv);
}
template <int N>
__device__ __forceinline__ void sincos(const Dual<float, N> &a, Dual<float, N> *s, Dual<float, N> *c)
{
    float sv, cv;
    ::sincosf(a.v, &sv, &cv);
    *s = chain(a, sv, cv);
    *c = chain(a, cv, -sv);
}
template <int N>
__device__ __forceinline__ Dual<double, N> tan(const Dual<double, N> &a)
{
    const double t = ::tan(a.v);
    return chain(a, t, 1.0 + t * t);
}
template <int N>
__device__ __forceinline__ Dual<float, N> tan(const Dual<float, N> &a)
{
    const float t = ::tanf(a.v);
    return chain(a, t, 1.0f + t * t);
}
template <int N>
__device__ __forceinline__ Dual<double, N> acos(const Dual<double, N> &a)
{
    return chain(a, ::acos(a.v), -1.0 / ::sqrt(1.0 - a.v * a.v));
}
template <int N>
__device__ __forceinline__ Dual<float, N> acos(const Dual<float, N> &a)
{
    return chain(a, ::acosf(a.v), -1.0f / ::sqrtf(1.0f - a.v * a.v));
}
// d atan2(y, x) = (x dy - y dx) / (x^2 + y^2)
template <class T, int N>
__device__ __forceinline__ Dual<T, N> atan2_rule(const Dual<T, N> &y, const Dual<T, N> &x, T f)
{
    Dual<T, N> r;
    r.v = f;
    const T inv = T(1) / (x.v * x.v + y.v * y.v);
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (x.v * y.d[k] - y.v * x.d[k]) * inv;
    return r;
}
template <int N>
__device__ __forceinline__ Dual<double, N> atan2(const Dual<double, N> &y, const Dual<double, N> &x)
{
    return atan2_rule(y, x, ::atan2(y.v, x.v));
}
template <int N>
__device__ __forceinline__ Dual<float, N> atan2(const Dual<float, N> &y, const Dual<float, N> &x)
{
    return atan2_rule(y, x, ::atan2f(y.v, x.v));
}
template <class T, int N>
__device__ __forceinline__ Dual<T, N> fabs(const Dual<T, N> &a)
{
    return a.v < T(0) ? -a : a;
}

} // namespace ad
} // namespace i2
