// constants.h -- named constants of the reference's interface (andreyypopov/integrator2,
// src/common/constants.h): the same names and values, so code written against the reference
// that reads them (CONSTANTS::PI, CONSTANTS::MAX_REFINE_LEVEL, ...) compiles unchanged.
#ifndef I2_DROPIN_CONSTANTS_H
#define I2_DROPIN_CONSTANTS_H

struct CONSTANTS {
    // tolerances of the reference's closed forms and its Runge criterion
    static constexpr double DOUBLE_MIN = 2e-6;
    static constexpr double EPS_ZERO = 1e-6;
    static constexpr double EPS_ZERO2 = 1e-10;
    static constexpr double EPS_PSI_THETA = EPS_ZERO;
    static constexpr double EPS_PSI_THETA2 = EPS_PSI_THETA * EPS_PSI_THETA;
    static constexpr double EPS_INTEGRATION = 1e-5;
    // mathematical constants
    static constexpr double ONE_THIRD = 1.0 / 3.0;
    static constexpr double PI = 3.14159265358979323846;
    static constexpr double TWO_PI = 2.0 * PI;
    static constexpr double RECIPROCAL_FOUR_PI = 1.0 / (4.0 * PI);
    // limits: deepest refinement level and largest Gauss rule (the library accepts the same)
    static constexpr int MAX_SIMPLE_NEIGHBORS_PER_CELL = 12;
    static constexpr int MAX_AUTO_REFINEMENT_TASK_COEFFICIENT = 4;
    static constexpr double MEMORY_REALLOCATION_COEFFICIENT = 1.25;
    static constexpr int MAX_REFINE_LEVEL = 5;
    static constexpr int MAX_GAUSS_POINTS = 13;
};

#endif
