// i2_dfloat.cuh -- double-float arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two binary32 numbers with |lo| <= ulp(hi)/2: about
// 48 significant bits (u^2, u = 2^-24) with binary32's exponent range.  GB300 runs FP64 at 1/64
// of the FP32 rate (1.25 against 78 TFLOP/s measured), so the stages of the mixed form that need
// more than FP32 (the adaptive potential of hard adjacent pairs and tier 2b) compute in this
// type rather than in double: an accurate addition costs 20 FP32 operations, a product 8, a
// logarithm about 90, against 64 FP32 issue slots for every FP64 operation.  Callers keep the
// magnitudes near 1 (geometry translated to a vertex and scaled by a power of two), so neither
// the smaller exponent range nor subnormal low parts come into play.
//
// Algorithms (published; written here from their descriptions):
//   - error-free transforms: Knuth's TwoSum, Dekker's Fast2Sum, the FMA form of TwoProduct;
//   - addition, product, quotient: the double-word algorithms AccurateDWPlusDW, DWPlusFP,
//     DWTimesDW, DWTimesFP and DWDivDW of Joldes, Muller and Popescu, "Tight and rigorous error
//     bounds for basic building blocks of double-word arithmetic", ACM TOMS 44(2), 2017
//     (relative errors of a few u^2); the quotient takes its first approximations from an
//     approximate reciprocal, which its correction step absorbs;
//   - square root: the FP32 root from an approximate reciprocal square root and one Newton
//     correction carried in double-float (Karp and Markstein's form);
//   - logarithm: Tang's table-driven method (ACM TOMS 16(4), 1990): x = 2^k m, m in [0.75, 1.5),
//     F_j the breakpoint nearest m (spacing 1/512), u = (m - F_j)/F_j, log x = k ln2 + log F_j +
//     log1p(u) with |u| < 2^-9.5 and log1p(u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5);
//   - arctangent: reduction to t = min/max in [0, 1], breakpoints c_j = j/512 and
//     atan t = atan c_j + atan((t - c_j)/(1 + t c_j)), |argument| <= 2^-10, by its Taylor series
//     to the fifth power; the quadrant from the signs as for atan2.
// Relative accuracy, measured against float64 on the ranges used here: about 2^-44 for log and
// atan2, 2^-45 for the square root, a few u^2 for the arithmetic.
//
// The header compiles as plain C++ too (host arithmetic, for the CPU checks of the math).
#pragma once

#include <math.h>
#include <string.h>

#include "i2_dftables.h"

#if defined(__CUDACC__)
#define I2_DF_HD __host__ __device__ __forceinline__
// the transcendental functions are called, not inlined: a kernel evaluating several of them per
// point would otherwise outgrow the instruction cache (measured: instruction-fetch stalls were
// the largest stall reason of the inlined version)
#define I2_DF_CALL static __host__ __device__ __noinline__
#else
#define I2_DF_HD inline
#define I2_DF_CALL static inline
#endif

namespace i2 {

// the C library's overloads stay visible beside the double-float ones declared below
using ::acos;
using ::atan2;
using ::cos;
using ::fabs;
using ::log;
using ::sin;
using ::sincos;
using ::sqrt;
using ::tan;

struct dfl {
    float hi, lo;
    dfl() = default;
    I2_DF_HD constexpr dfl(float h, float l) : hi(h), lo(l) {}
    I2_DF_HD constexpr dfl(float f) : hi(f), lo(0.0f) {}
    // from a double: the nearest float and the float nearest the remainder (exact for the
    // literals the templated integrands use; an FP64 subtraction for run-time values)
    I2_DF_HD dfl(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
    I2_DF_HD explicit operator double() const { return (double)hi + (double)lo; }
};

struct alignas(16) dfl_log_entry {
    float log_hi, log_lo, inv_hi, inv_lo;
};
struct alignas(8) dfl_pair {
    float hi, lo;
};
struct alignas(16) dfl_sincos_entry {
    float s_hi, s_lo, c_hi, c_lo;
};

#if defined(__CUDACC__)
static __device__ const dfl_log_entry kDfLogTableDev[385] = I2_DF_LOG_TABLE;
static __device__ const dfl_pair kDfAtanTableDev[513] = I2_DF_ATAN_TABLE;
#endif
static const dfl_log_entry kDfLogTableHost[385] = I2_DF_LOG_TABLE;
static const dfl_pair kDfAtanTableHost[513] = I2_DF_ATAN_TABLE;
#if defined(__CUDACC__)
static __device__ const dfl_sincos_entry kDfSinCosTableDev[404] = I2_DF_SINCOS_TABLE;
#endif
static const dfl_sincos_entry kDfSinCosTableHost[404] = I2_DF_SINCOS_TABLE;

I2_DF_HD dfl_sincos_entry df_sincos_entry(int j)
{
#if defined(__CUDA_ARCH__)
    const float4 e = __ldg(reinterpret_cast<const float4 *>(kDfSinCosTableDev) + j);
    return dfl_sincos_entry{e.x, e.y, e.z, e.w};
#else
    return kDfSinCosTableHost[j];
#endif
}

I2_DF_HD dfl_log_entry df_log_entry(int j)
{
#if defined(__CUDA_ARCH__)
    const float4 e = __ldg(reinterpret_cast<const float4 *>(kDfLogTableDev) + j);
    return dfl_log_entry{e.x, e.y, e.z, e.w};
#else
    return kDfLogTableHost[j];
#endif
}

I2_DF_HD dfl_pair df_atan_entry(int j)
{
#if defined(__CUDA_ARCH__)
    const float2 e = __ldg(reinterpret_cast<const float2 *>(kDfAtanTableDev) + j);
    return dfl_pair{e.x, e.y};
#else
    return kDfAtanTableHost[j];
#endif
}

// ------------------------------------------------------------------ hardware approximations
I2_DF_HD float df_rcp_approx(float x)
{
#if defined(__CUDA_ARCH__)
    return __fdividef(1.0f, x);
#else
    return 1.0f / x;
#endif
}

I2_DF_HD float df_rsqrt_approx(float x)
{
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}

I2_DF_HD int df_float_bits(float x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_int(x);
#else
    int i;
    memcpy(&i, &x, sizeof i);
    return i;
#endif
}

I2_DF_HD float df_bits_float(int i)
{
#if defined(__CUDA_ARCH__)
    return __int_as_float(i);
#else
    float x;
    memcpy(&x, &i, sizeof x);
    return x;
#endif
}

I2_DF_HD int df_clamp(int j, int hi) { return j < 0 ? 0 : (j > hi ? hi : j); }

// ------------------------------------------------------------------ error-free transforms
I2_DF_HD dfl df_two_sum(float a, float b)
{
    const float s = a + b, bb = s - a;
    return dfl(s, (a - (s - bb)) + (b - bb));
}

// |a| >= |b| (or a == 0)
I2_DF_HD dfl df_fast_two_sum(float a, float b)
{
    const float s = a + b;
    return dfl(s, b - (s - a));
}

I2_DF_HD dfl df_two_prod(float a, float b)
{
    const float p = a * b;
    return dfl(p, fmaf(a, b, -p));
}

// ------------------------------------------------------------------ arithmetic
I2_DF_HD dfl operator-(dfl x) { return dfl(-x.hi, -x.lo); }

// AccurateDWPlusDW: exact cancellation handled (the low parts are summed error-free too)
I2_DF_HD dfl operator+(dfl x, dfl y)
{
    const dfl s = df_two_sum(x.hi, y.hi), t = df_two_sum(x.lo, y.lo);
    const dfl v = df_fast_two_sum(s.hi, s.lo + t.hi);
    return df_fast_two_sum(v.hi, t.lo + v.lo);
}
I2_DF_HD dfl operator-(dfl x, dfl y) { return x + (-y); }

// DWPlusFP
I2_DF_HD dfl operator+(dfl x, float y)
{
    const dfl s = df_two_sum(x.hi, y);
    return df_fast_two_sum(s.hi, x.lo + s.lo);
}
I2_DF_HD dfl operator+(float y, dfl x) { return x + y; }
I2_DF_HD dfl operator-(dfl x, float y) { return x + (-y); }
I2_DF_HD dfl operator-(float y, dfl x) { return (-x) + y; }

// DWTimesDW
I2_DF_HD dfl operator*(dfl x, dfl y)
{
    const dfl c = df_two_prod(x.hi, y.hi);
    const float cl2 = fmaf(x.lo, y.hi, x.hi * y.lo);
    return df_fast_two_sum(c.hi, c.lo + cl2);
}

// DWTimesFP
I2_DF_HD dfl operator*(dfl x, float y)
{
    const dfl c = df_two_prod(x.hi, y);
    return df_fast_two_sum(c.hi, fmaf(x.lo, y, c.lo));
}
I2_DF_HD dfl operator*(float y, dfl x) { return x * y; }

// DWDivDW: q1 from an approximate reciprocal, the exact residual x - y q1, one correction
I2_DF_HD dfl operator/(dfl x, dfl y)
{
    const float r = df_rcp_approx(y.hi);
    const float q1 = x.hi * r;
    const dfl p = y * q1;
    const float d = ((x.hi - p.hi) - p.lo) + x.lo;
    return df_fast_two_sum(q1, d * r);
}
I2_DF_HD dfl operator/(dfl x, float y) { return x / dfl(y); }

// mixed with double constants (the templated integrands' literals)
I2_DF_HD dfl operator+(dfl x, double y) { return x + dfl(y); }
I2_DF_HD dfl operator+(double y, dfl x) { return x + dfl(y); }
I2_DF_HD dfl operator-(dfl x, double y) { return x - dfl(y); }
I2_DF_HD dfl operator-(double y, dfl x) { return dfl(y) - x; }
I2_DF_HD dfl operator*(dfl x, double y) { return x * dfl(y); }
I2_DF_HD dfl operator*(double y, dfl x) { return x * dfl(y); }
I2_DF_HD dfl operator/(dfl x, double y) { return x / dfl(y); }
I2_DF_HD dfl operator/(double y, dfl x) { return dfl(y) / x; }

I2_DF_HD dfl &operator+=(dfl &x, dfl y) { return x = x + y; }
I2_DF_HD dfl &operator-=(dfl &x, dfl y) { return x = x - y; }
I2_DF_HD dfl &operator*=(dfl &x, dfl y) { return x = x * y; }

// exact scaling by 2^k (no overflow or underflow on the ranges used)
I2_DF_HD dfl df_ldexp(dfl x, int k) { return dfl(ldexpf(x.hi, k), ldexpf(x.lo, k)); }

// ------------------------------------------------------------------ comparisons
I2_DF_HD bool operator<(dfl a, dfl b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
I2_DF_HD bool operator>(dfl a, dfl b) { return b < a; }
I2_DF_HD bool operator<=(dfl a, dfl b) { return !(b < a); }
I2_DF_HD bool operator>=(dfl a, dfl b) { return !(a < b); }
I2_DF_HD bool operator==(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }
I2_DF_HD bool operator!=(dfl a, dfl b) { return !(a == b); }
I2_DF_HD bool operator<(dfl a, double b) { return a < dfl(b); }
I2_DF_HD bool operator>(dfl a, double b) { return dfl(b) < a; }
I2_DF_HD bool operator<=(dfl a, double b) { return !(dfl(b) < a); }
I2_DF_HD bool operator>=(dfl a, double b) { return !(a < dfl(b)); }
I2_DF_HD bool operator==(dfl a, double b) { return a == dfl(b); }
I2_DF_HD bool operator!=(dfl a, double b) { return !(a == dfl(b)); }

// ------------------------------------------------------------------ functions
I2_DF_HD dfl fabs(dfl x) { return x.hi < 0.0f ? -x : x; }

I2_DF_HD double value_of(dfl x) { return (double)x; }

// square root; 0 for x <= 0 (the callers take norms)
I2_DF_HD dfl sqrt(dfl x)
{
    if (!(x.hi > 0.0f)) return dfl(0.0f, 0.0f);
    const float r = df_rsqrt_approx(x.hi);
    const float s = x.hi * r;
    const dfl p = df_two_prod(s, s);
    const float d = ((x.hi - p.hi) - p.lo) + x.lo;
    return df_fast_two_sum(s, d * (0.5f * r));
}

// natural logarithm (Tang's table-driven method); -inf for 0, NaN below, +inf for +inf
I2_DF_CALL dfl log(dfl x)
{
    const float h = x.hi;
    if (!(h > 0.0f) || !(h < INFINITY)) return dfl(logf(h), 0.0f);
    const int bits = df_float_bits(h);
    int k = ((bits >> 23) & 0xff) - 127;
    float m = df_bits_float((bits & 0x7fffff) | 0x3f800000);  // [1, 2)
    if (k == -127) {  // subnormal high part: renormalise through an exact scaling
        const float hn = h * 16777216.0f;
        const int bn = df_float_bits(hn);
        k = ((bn >> 23) & 0xff) - 127 - 24;
        m = df_bits_float((bn & 0x7fffff) | 0x3f800000);
    }
    if (m >= 1.5f) {
        m *= 0.5f;
        k += 1;
    }
    const int j = df_clamp((int)((m - 0.75f) * 512.0f + 0.5f), 384);  // m - 0.75 is exact (Sterbenz)
    const float F = 0.75f + (float)j * (1.0f / 512.0f);
    const dfl_log_entry e = df_log_entry(j);
    const float sc = (k > -127 && k < 127) ? df_bits_float((127 - k) << 23) : ldexpf(1.0f, -k);  // 2^-k
    const dfl f = df_two_sum(m - F, x.lo * sc);  // m - F exact: |m - F| <= 2^-10
    const dfl u = f * dfl(e.inv_hi, e.inv_lo);
    const float uh = u.hi;
    const dfl sq = df_two_prod(uh, uh);
    const dfl half_sq = df_fast_two_sum(0.5f * sq.hi, 0.5f * fmaf(2.0f * uh, u.lo, sq.lo));
    const float u2 = uh * uh;  // the cubic term with u.lo's first-order part
    const float tail = fmaf(u2, u.lo, u2 * uh * fmaf(uh, fmaf(uh, 0.2f, -0.25f), 0.333333343f));
    dfl r = (u - half_sq) + tail;
    r = r + dfl(e.log_hi, e.log_lo);
    if (k != 0) {
        const float kf = (float)k;
        const dfl kl = df_two_prod(kf, I2_LN2_HI);
        r = r + df_fast_two_sum(kl.hi, fmaf(kf, I2_LN2_LO, kl.lo));
    }
    return r;
}

// atan2 with the quadrant and signed-zero conventions of the C library's atan2
I2_DF_CALL dfl atan2(dfl y, dfl x)
{
    const bool ny = signbit(y.hi), nx = signbit(x.hi);
    const dfl ay = ny ? -y : y, ax = nx ? -x : x;
    dfl r;
    if (ay.hi == 0.0f && ax.hi == 0.0f) {
        r = dfl(0.0f, 0.0f);
    } else {
        const bool swap = ax < ay;
        const dfl t = swap ? ax / ay : ay / ax;  // [0, 1]
        const int j = df_clamp((int)(t.hi * 512.0f + 0.5f), 512);
        const float c = (float)j * (1.0f / 512.0f);
        const dfl num = df_two_sum(t.hi - c, t.lo);  // t.hi - c exact
        const dfl den = (t * c) + 1.0f;
        const dfl d = num / den;
        const float dh = d.hi, d2 = dh * dh;
        const float tail = fmaf(-d2, d.lo, dh * d2 * fmaf(d2, 0.2f, -0.333333343f));  // with d.lo's first-order part
        const dfl_pair a = df_atan_entry(j);
        r = (d + tail) + dfl(a.hi, a.lo);
        if (swap) r = dfl(I2_HALFPI_HI, I2_HALFPI_LO) - r;
    }
    if (nx) r = dfl(I2_PI_HI, I2_PI_LO) - r;
    return ny ? -r : r;
}

// sine and cosine: x - n pi/2 with pi/2 in three parts (n the nearest integer to x 2/pi), the
// breakpoint c = j/512 nearest the remainder r (sin c, cos c tabulated), and the Taylor series
// of s = r - c, |s| <= 2^-10: sin s = s - s^3/6 + s^5/120, cos s = 1 - s^2/2 + s^4/24 - s^6/720;
// then the addition formulas and the quadrant of n.  For the moderate arguments of the closed
// forms (angles and their sums, |x| < 2^10).
I2_DF_CALL void sincos(dfl x, dfl *ps, dfl *pc)
{
    const float n = rintf(x.hi * 0.636619772f);
    dfl r = x;
    if (n != 0.0f) {
        r = r - df_two_prod(n, I2_PIO2_1);
        r = r - df_two_prod(n, I2_PIO2_2);
        r = r - n * I2_PIO2_3;
    }
    const float jf = rintf(r.hi * 512.0f);
    const float c0 = jf * (1.0f / 512.0f);
    const dfl sx = df_two_sum(r.hi - c0, r.lo);  // r.hi - c0 exact (Sterbenz)
    const float sh = sx.hi, s2 = sh * sh;
    const dfl sin_s = sx + fmaf(-0.5f * s2, sx.lo, sh * s2 * fmaf(s2, 0.00833333377f, -0.166666672f));
    const dfl sq = df_two_prod(sh, sh);
    const dfl half_sq = df_fast_two_sum(0.5f * sq.hi, 0.5f * fmaf(2.0f * sh, sx.lo, sq.lo));
    const dfl cos_s = (dfl(1.0f) - half_sq) + s2 * s2 * fmaf(s2, -0.00138888892f, 0.0416666679f);
    const dfl_sincos_entry e = df_sincos_entry(df_clamp((int)fabsf(jf), 403));
    const dfl S = jf < 0.0f ? dfl(-e.s_hi, -e.s_lo) : dfl(e.s_hi, e.s_lo), C(e.c_hi, e.c_lo);
    const dfl sr = S * cos_s + C * sin_s, cr = C * cos_s - S * sin_s;
    switch (((int)n) & 3) {
    case 0: *ps = sr; *pc = cr; break;
    case 1: *ps = cr; *pc = -sr; break;
    case 2: *ps = -sr; *pc = -cr; break;
    default: *ps = -cr; *pc = sr; break;
    }
}

I2_DF_HD dfl sin(dfl x)
{
    dfl s, c;
    sincos(x, &s, &c);
    return s;
}

I2_DF_HD dfl cos(dfl x)
{
    dfl s, c;
    sincos(x, &s, &c);
    return c;
}

I2_DF_HD dfl tan(dfl x)
{
    dfl s, c;
    sincos(x, &s, &c);
    return s / c;
}

// arccosine on [-1, 1] as atan2(sqrt((1 - c)(1 + c)), c)
I2_DF_HD dfl acos(dfl c)
{
    const dfl one(1.0f);
    return atan2(sqrt((one - c) * (one + c)), c);
}

} // namespace i2
