// QuadratureFormula3d.cuh -- QuadratureFormula3D and the built-in triangle rules qf3D1 ... qf3D13
// (src/QuadratureFormula3d.cuh): barycentric coordinates (x, y; the third is 1 - x - y), weights
// and the rule's order (2^order enters the reference's Runge criterion).  The tables come from
// the library (i2_quadrature_builtin), so a program and the library use the same numbers.
#ifndef I2_DROPIN_QUADRATURE_FORMULA_3D_CUH
#define I2_DROPIN_QUADRATURE_FORMULA_3D_CUH

#include "../integrator2_gb300.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

struct QuadratureFormula3D {
    const std::vector<double2> coordinates;
    const std::vector<double> weights;
    const int order;
};

namespace i2dropin {
inline QuadratureFormula3D builtin_rule(int npoints)
{
    std::vector<double> c(2 * (size_t)npoints), w((size_t)npoints);
    int32_t order = 0;
    if (i2_quadrature_builtin(npoints, c.data(), w.data(), &order) != I2_OK) {
        std::fprintf(stderr, "no built-in %d-point rule: %s\n", npoints, i2_last_error());
        std::exit(EXIT_FAILURE);
    }
    std::vector<double2> xy((size_t)npoints);
    for (int k = 0; k < npoints; ++k) xy[k] = make_double2(c[2 * k], c[2 * k + 1]);
    return QuadratureFormula3D{xy, w, (int)order};
}
} // namespace i2dropin

inline const QuadratureFormula3D qf3D1 = i2dropin::builtin_rule(1);
inline const QuadratureFormula3D qf3D3 = i2dropin::builtin_rule(3);
inline const QuadratureFormula3D qf3D4 = i2dropin::builtin_rule(4);
inline const QuadratureFormula3D qf3D6 = i2dropin::builtin_rule(6);
inline const QuadratureFormula3D qf3D7 = i2dropin::builtin_rule(7);
inline const QuadratureFormula3D qf3D9 = i2dropin::builtin_rule(9);
inline const QuadratureFormula3D qf3D12 = i2dropin::builtin_rule(12);
inline const QuadratureFormula3D qf3D13 = i2dropin::builtin_rule(13);

#endif
