// Accuracy of the double-float arithmetic (integrator2_gb300/csrc/i2_dfloat.cuh) on the host:
// seeded random operands over the ranges the potential stages use, each result compared with the
// same operation in long double (64 or 113 significant bits).  Prints one line per operation:
// name, samples, largest relative error.
#include <cmath>
#include <cstdio>
#include <random>

#include "i2_dfloat.cuh"

using i2::dfl;

static dfl to_dfl(long double v)
{
    const float hi = (float)v;
    return dfl(hi, (float)(v - (long double)hi));
}
static long double val(dfl x) { return (long double)x.hi + (long double)x.lo; }
static long double rel(long double got, long double want) { return want == 0 ? fabsl(got) : fabsl(got - want) / fabsl(want); }

int main()
{
    std::mt19937_64 rng(2026);
    std::uniform_real_distribution<double> U(-1.0, 1.0), E(-20.0, 20.0);
    auto rnd = [&](double emin, double emax) {
        const double e = emin + (emax - emin) * (0.5 + 0.5 * U(rng));
        const long double m = (long double)U(rng) + (long double)U(rng) * 1e-9L;
        return to_dfl(m * powl(2.0L, e));
    };
    const int N = 200000;
    long double e_add = 0, e_sub = 0, e_mul = 0, e_div = 0, e_sqrt = 0, e_log = 0, e_log1 = 0, e_atan = 0, e_atan_small = 0;
    for (int i = 0; i < N; ++i) {
        const dfl a = rnd(-20, 20), b = rnd(-20, 20);
        const long double A = val(a), B = val(b);
        // addition: relative to the larger operand where the result cancels (the bound of the
        // accurate algorithm is relative to the exact result; measure that)
        e_add = fmaxl(e_add, rel(val(a + b), A + B));
        e_sub = fmaxl(e_sub, rel(val(a - b), A - B));
        e_mul = fmaxl(e_mul, rel(val(a * b), A * B));
        if (B != 0) e_div = fmaxl(e_div, rel(val(a / b), A / B));
        const dfl p = i2::fabs(a);
        e_sqrt = fmaxl(e_sqrt, rel(val(i2::sqrt(p)), sqrtl(val(p))));
        if (val(p) > 0) e_log = fmaxl(e_log, rel(val(i2::log(p)), logl(val(p))));
        // near 1, where log is small and its relative accuracy matters most
        // (the reference from the exact offset delta = (hi - 1) + lo: 1 + delta itself is not
        // representable in long double to the double-float's precision)
        const dfl q = dfl(1.0f) + rnd(-40, -2);
        const long double delta = ((long double)q.hi - 1.0L) + (long double)q.lo;
        if (delta != 0) e_log1 = fmaxl(e_log1, rel(val(i2::log(q)), log1pl(delta)));
        e_atan = fmaxl(e_atan, rel(val(i2::atan2(a, b)), atan2l(A, B)));
        const dfl s = rnd(-40, -1);
        e_atan_small = fmaxl(e_atan_small, rel(val(i2::atan2(s, i2::fabs(b))), atan2l(val(s), fabsl(B))));
    }
    // trigonometric functions on the closed forms' ranges
    long double e_sin = 0, e_cos = 0, e_tan = 0, e_acos = 0, e_sin_abs = 0;
    std::uniform_real_distribution<double> A(-7.0, 7.0), C1(-1.0, 1.0);
    for (int i = 0; i < N; ++i) {
        const dfl x = to_dfl((long double)A(rng) + (long double)U(rng) * 1e-9L);
        const long double X = val(x);
        // absolute error near the zeros, relative elsewhere
        const long double s = sinl(X), c = cosl(X);
        e_sin_abs = fmaxl(e_sin_abs, fabsl(val(i2::sin(x)) - s));
        if (fabsl(s) > 1e-3L) e_sin = fmaxl(e_sin, rel(val(i2::sin(x)), s));
        if (fabsl(c) > 1e-3L) e_cos = fmaxl(e_cos, rel(val(i2::cos(x)), c));
        if (fabsl(c) > 1e-2L) e_tan = fmaxl(e_tan, rel(val(i2::tan(x)), tanl(X)));
        const dfl y = to_dfl((long double)C1(rng) * (1.0L - 1e-7L));
        e_acos = fmaxl(e_acos, rel(val(i2::acos(y)), acosl(val(y))));
    }
    // small arguments of sin (relative), as the closed forms' half-angles near 0
    long double e_sin_small = 0;
    for (int i = 0; i < N; ++i) {
        const dfl x = rnd(-40, -3);
        e_sin_small = fmaxl(e_sin_small, rel(val(i2::sin(x)), sinl(val(x))));
    }
    printf("sin %d %.3Le\ncos %d %.3Le\ntan %d %.3Le\nacos %d %.3Le\nsin_abs %d %.3Le\nsin_small %d %.3Le\n", N, e_sin, N, e_cos, N, e_tan,
           N, e_acos, N, e_sin_abs, N, e_sin_small);
    // signed zeros and axes, as atan2
    const bool zeros = i2::atan2(dfl(0.0f), dfl(1.0f)).hi == 0.0f && !std::signbit(i2::atan2(dfl(0.0f), dfl(1.0f)).hi) &&
                       std::signbit(i2::atan2(dfl(-0.0f), dfl(1.0f)).hi) &&
                       fabsl(val(i2::atan2(dfl(0.0f), dfl(-1.0f))) - 3.14159265358979323846264L) < 1e-14L &&
                       fabsl(val(i2::atan2(dfl(-0.0f), dfl(-1.0f))) + 3.14159265358979323846264L) < 1e-14L &&
                       fabsl(val(i2::atan2(dfl(1.0f), dfl(0.0f))) - 1.57079632679489661923132L) < 1e-14L;
    printf("add %d %.3Le\nsub %d %.3Le\nmul %d %.3Le\ndiv %d %.3Le\nsqrt %d %.3Le\nlog %d %.3Le\nlog_near_1 %d %.3Le\n"
           "atan2 %d %.3Le\natan2_small %d %.3Le\nsigned_zeros %d %d\n",
           N, e_add, N, e_sub, N, e_mul, N, e_div, N, e_sqrt, N, e_log, N, e_log1, N, e_atan, N, e_atan_small, 1, zeros ? 1 : 0);
    return 0;
}
