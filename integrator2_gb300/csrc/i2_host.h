// i2_host.h -- host-side helpers shared by the library's translation units: the exception that
// carries an i2_status out of an entry point (caught at the C-ABI boundary), the checks that
// raise it, and the RAII device buffer every handle owns its memory through.
#pragma once

#include "integrator2_gb300.h"

#include <cuda_runtime.h>
#include <string>

namespace i2 {

struct Failure {
    i2_status code;
    std::string msg;
};

#define I2_CHECK_CUDA(call)                                                                                            \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) {                                                                                       \
            throw Failure{e_ == cudaErrorMemoryAllocation ? I2_ERR_OUT_OF_MEMORY : I2_ERR_CUDA,                        \
                          std::string(#call) + ": " + cudaGetErrorString(e_)};                                         \
        }                                                                                                              \
    } while (0)

#define I2_REQUIRE(cond, code, text)                                                                                   \
    do {                                                                                                               \
        if (!(cond)) throw Failure{code, text};                                                                        \
    } while (0)

// device buffer owned by one handle
template <class T>
struct DevBuf {
    T *ptr = nullptr;
    size_t count = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
    void reserve(size_t n)
    {
        if (n <= count && ptr) return;
        release();
        if (n == 0) return;
        I2_CHECK_CUDA(cudaMalloc(&ptr, n * sizeof(T)));
        count = n;
    }
};

} // namespace i2
