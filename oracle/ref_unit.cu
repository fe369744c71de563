/*
 * ref_unit.cu -- one translation unit made of the reference's own sources (andreyypopov/
 * integrator2, src/), included unmodified.  TEST INFRASTRUCTURE ONLY.
 *
 * oracle/ref_cuda_build.sh compiles it for sm_103a into a cubin (device code only: the
 * reference's kernels, device functions and __constant__ quadrature tables) that
 * oracle/ref_cuda.py loads with the CUDA driver API on the GPU machine, where it launches the
 * reference's kernels in the order of its fixed-refinement host flow.  The product never loads it.
 */
#include "common/cuda_math.cu"
#include "common/cuda_helper.cu"
#include "Mesh3d.cu"
#include "NumericalIntegrator3d.cu"
#include "evaluators/evaluator3d.cu"
#include "evaluators/evaluatorJ3DK.cu"
