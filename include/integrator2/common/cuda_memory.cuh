// cuda_memory.cuh -- typed device / host allocation and copies with the reference's names and
// argument order (src/common/cuda_memory.cuh): sizes count elements, copies are asynchronous on
// the given stream (default: the legacy default stream), failures end the program.
#ifndef I2_DROPIN_CUDA_MEMORY_CUH
#define I2_DROPIN_CUDA_MEMORY_CUH

#include "cuda_helper.cuh"

template <class T> void allocate_device(T **ptr, size_t elements_num)
{
    if (elements_num) checkCudaErrors(cudaMalloc((void **)ptr, elements_num * sizeof(T)));
}
template <class T> void allocate_host(T **ptr, size_t elements_num)
{
    if (elements_num) checkCudaErrors(cudaMallocHost((void **)ptr, elements_num * sizeof(T)));
}
template <class T> void free_device(T *ptr)
{
    if (ptr) checkCudaErrors(cudaFree((void *)ptr));
}
template <class T> void free_host(T *ptr)
{
    if (ptr) checkCudaErrors(cudaFreeHost((void *)ptr));
}
template <class T> void zero_value_device(T *ptr, size_t elements_num, cudaStream_t stream = nullptr)
{
    if (elements_num) checkCudaErrors(cudaMemsetAsync((void *)ptr, 0, elements_num * sizeof(T), stream));
}
template <class T> void copy_h2d(const T *src, const T *dst, size_t elements_num, cudaStream_t stream = nullptr)
{
    if (elements_num) checkCudaErrors(cudaMemcpyAsync((void *)dst, (const void *)src, elements_num * sizeof(T), cudaMemcpyHostToDevice, stream));
}
template <class T> void copy_d2h(const T *src, const T *dst, size_t elements_num, cudaStream_t stream = nullptr)
{
    if (!elements_num) return;
    checkCudaErrors(cudaMemcpyAsync((void *)dst, (const void *)src, elements_num * sizeof(T), cudaMemcpyDeviceToHost, stream));
    checkCudaErrors(cudaStreamSynchronize(stream));  // the host reads the data right after the call
}
template <class T> void copy_d2d(const T *src, const T *dst, size_t elements_num, cudaStream_t stream = nullptr)
{
    if (elements_num) checkCudaErrors(cudaMemcpyAsync((void *)dst, (const void *)src, elements_num * sizeof(T), cudaMemcpyDeviceToDevice, stream));
}
template <class T> void copy_h2const(const T *src, const void *dst, size_t elements_num, cudaStream_t stream = nullptr)
{
    if (elements_num) checkCudaErrors(cudaMemcpyToSymbolAsync(dst, (const void *)src, elements_num * sizeof(T), 0, cudaMemcpyHostToDevice, stream));
}

#endif
