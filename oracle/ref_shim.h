/*
 * ref_shim.h -- force-included when oracle/ref_build.sh compiles the reference's own sources
 * (andreyypopov/integrator2, src/) for the HOST.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference marks its math routines __device__ only.  Re-spelling __device__ as
 * __host__ __device__ lets the unmodified source also emit host copies of those routines,
 * so the oracle can be checked against the reference's own arithmetic (with the C library's
 * log/atan2/sincos/acos in place of the device math library).  rsqrt has no host
 * counterpart and becomes 1/sqrt.
 */
#pragma once
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>

#undef __device__
#define __device__ __host__ __attribute__((device))

__host__ __attribute__((device)) inline double i2ref_rsqrt(double x) { return 1.0 / sqrt(x); }
#define rsqrt i2ref_rsqrt
