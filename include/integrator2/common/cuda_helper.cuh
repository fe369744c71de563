// cuda_helper.cuh -- CUDA error checking and launch-size helpers with the reference's names
// (src/common/cuda_helper.cuh): checkCudaErrors(call) prints the failing call with its file and
// line and ends the program, as the reference does; blocksForSize(n) rounds n up to blocks.
#ifndef I2_DROPIN_CUDA_HELPER_CUH
#define I2_DROPIN_CUDA_HELPER_CUH

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

const int gpuThreads = 256;
const int gpuThreadsMax = 1024;
const int gpuThreads2D = 16;

inline unsigned int blocksForSize(unsigned int n, unsigned int maxThreads = gpuThreads) { return (n + maxThreads - 1) / maxThreads; }

namespace i2dropin {
inline void check_cuda(cudaError_t e, const char *what, const char *file, int line)
{
    if (e == cudaSuccess) return;
    std::fprintf(stderr, "CUDA error at %s:%d code=%d (%s) \"%s\"\n", file, line, (int)e, cudaGetErrorString(e), what);
    std::exit(EXIT_FAILURE);
}
} // namespace i2dropin

#define checkCudaErrors(val) ::i2dropin::check_cuda((val), #val, __FILE__, __LINE__)

// free device memory in bytes, printed as the reference does after each pair class
inline size_t requestFreeDeviceMemoryAmount()
{
    size_t freeMemory = 0, totalMemory = 0;
    checkCudaErrors(cudaMemGetInfo(&freeMemory, &totalMemory));
    std::printf("GPU memory usage: %5.1f MBytes free out of total %5.1f MBytes\n", freeMemory / 1048576.0, totalMemory / 1048576.0);
    return freeMemory;
}

#endif
