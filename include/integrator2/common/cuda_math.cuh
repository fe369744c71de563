// cuda_math.cuh -- Point3 (= double3) and double4 algebra with the reference's names and
// semantics (src/common/cuda_math.cuh, cuda_math.cu), usable in host and device code: + - and
// scalar products, dot, cross, lengths, normalize, the Runge rule's guarded component division
// (divide) and 1-norms, and the angle between two vectors with the reference's guards.
#ifndef I2_DROPIN_CUDA_MATH_CUH
#define I2_DROPIN_CUDA_MATH_CUH

#include "constants.h"

#include <cuda_runtime.h>

#include <cmath>

typedef double3 Point3;

__host__ __device__ inline double sqr(double x) { return x * x; }
// 0 within DOUBLE_MIN of zero, +1 above DOUBLE_MIN, -1 otherwise (x = DOUBLE_MIN itself gives -1, as in the reference)
__host__ __device__ inline double sign(double x)
{
    return fabs(x) < CONSTANTS::DOUBLE_MIN ? 0.0 : (x > CONSTANTS::DOUBLE_MIN ? 1.0 : -1.0);
}
// argument of a real number: 0 when clearly positive, pi otherwise
__host__ __device__ inline double arg(double x) { return x > CONSTANTS::DOUBLE_MIN ? 0.0 : CONSTANTS::PI; }

__host__ __device__ inline double4 assign_vector_part(const Point3 &v) { return make_double4(v.x, v.y, v.z, 0.0); }
__host__ __device__ inline Point3 extract_vector_part(const double4 &v) { return make_double3(v.x, v.y, v.z); }

__host__ __device__ inline double4 operator+(const double4 &a, const double4 &b) { return make_double4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__host__ __device__ inline double4 operator-(const double4 &a, const double4 &b) { return make_double4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__host__ __device__ inline double4 operator*(double s, const double4 &a) { return make_double4(s * a.x, s * a.y, s * a.z, s * a.w); }
__host__ __device__ inline void operator+=(double4 &a, const double4 &b) { a = a + b; }

__host__ __device__ inline Point3 operator+(const Point3 &a, const Point3 &b) { return make_double3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline Point3 operator-(const Point3 &a, const Point3 &b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline Point3 operator-(const Point3 &a) { return make_double3(-a.x, -a.y, -a.z); }
__host__ __device__ inline Point3 operator*(double s, const Point3 &a) { return make_double3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ inline void operator+=(Point3 &a, const Point3 &b) { a = a + b; }
__host__ __device__ inline void operator*=(Point3 &a, const double &s) { a = s * a; }
__host__ __device__ inline void operator/=(Point3 &a, const double &s) { a = make_double3(a.x / s, a.y / s, a.z / s); }

__host__ __device__ inline double dot(const Point3 &a, const Point3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline Point3 cross(const Point3 &a, const Point3 &b)
{
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ inline double vector_length2(const Point3 &v) { return dot(v, v); }
__host__ __device__ inline double vector_length(const Point3 &v) { return sqrt(vector_length2(v)); }
__host__ __device__ inline Point3 normalize(const Point3 &v) { return (1.0 / vector_length(v)) * v; }

// component-wise quotient; a component whose numerator and denominator are both negligible
// (below DOUBLE_MIN for the vector part, EPS_ZERO2 for the scalar part) is 0
__host__ __device__ inline double4 divide(const double4 &a, const double4 &b)
{
    const double e = CONSTANTS::DOUBLE_MIN, e2 = CONSTANTS::EPS_ZERO2;
    return make_double4(fabs(a.x) < e && fabs(b.x) < e ? 0.0 : a.x / b.x, fabs(a.y) < e && fabs(b.y) < e ? 0.0 : a.y / b.y,
                        fabs(a.z) < e && fabs(b.z) < e ? 0.0 : a.z / b.z, fabs(a.w) < e2 && fabs(b.w) < e2 ? 0.0 : a.w / b.w);
}
__host__ __device__ inline double norm1(const Point3 &v) { return fabs(v.x) + fabs(v.y) + fabs(v.z); }
__host__ __device__ inline double norm1(const double4 &v) { return fabs(v.x) + fabs(v.y) + fabs(v.z) + fabs(v.w); }

// angle between two vectors; 0 when either is shorter than EPS_ZERO (in the product of lengths),
// the cosine clamped to [-1, 1]
__host__ __device__ inline double angle(const Point3 &a, const Point3 &b)
{
    const double den = sqrt(vector_length2(a) * vector_length2(b));
    if (den < CONSTANTS::EPS_ZERO) return 0.0;
    const double c = dot(a, b) / den;
    return c >= 1.0 ? 0.0 : (c <= -1.0 ? CONSTANTS::PI : acos(c));
}

#endif
