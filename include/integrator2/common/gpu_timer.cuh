// gpu_timer.cuh -- GpuTimer (src/common/gpu_timer.cuh): CUDA events around a region; stop()
// waits for the region, prints "Time for <message>: <ms> ms" when given a message and returns
// the time in ms.
#ifndef I2_DROPIN_GPU_TIMER_CUH
#define I2_DROPIN_GPU_TIMER_CUH

#include "cuda_helper.cuh"

class GpuTimer {
public:
    GpuTimer()
    {
        checkCudaErrors(cudaEventCreate(&startEvent));
        checkCudaErrors(cudaEventCreate(&stopEvent));
    }
    ~GpuTimer()
    {
        if (startEvent) cudaEventDestroy(startEvent);
        if (stopEvent) cudaEventDestroy(stopEvent);
    }
    GpuTimer(const GpuTimer &) = delete;
    GpuTimer &operator=(const GpuTimer &) = delete;
    void start(cudaStream_t stream = nullptr) { checkCudaErrors(cudaEventRecord(startEvent, stream)); }
    float stop(const char *message = nullptr, cudaStream_t stream = nullptr)
    {
        checkCudaErrors(cudaEventRecord(stopEvent, stream));
        checkCudaErrors(cudaEventSynchronize(stopEvent));
        float ms = 0.0f;
        checkCudaErrors(cudaEventElapsedTime(&ms, startEvent, stopEvent));
        if (message) std::printf("Time for %s: %6.3f ms\n", message, ms);
        return ms;
    }

    cudaEvent_t startEvent = nullptr;
    cudaEvent_t stopEvent = nullptr;
};

#endif
