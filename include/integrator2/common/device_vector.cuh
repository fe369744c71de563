// device_vector.cuh -- deviceVector<T>, the reference's owning device array
// (src/common/device_vector.cuh): public data / size / capacity, allocate, resize (growing by
// CONSTANTS::MEMORY_REALLOCATION_COEFFICIENT, contents not kept), swap, bytes; freed on
// destruction.  Copying is disabled (the reference's implicit shallow copy would free twice).
#ifndef I2_DROPIN_DEVICE_VECTOR_CUH
#define I2_DROPIN_DEVICE_VECTOR_CUH

#include "constants.h"
#include "cuda_memory.cuh"

template <class T> struct deviceVector {
    T *data = nullptr;
    int size = 0;
    int capacity = 0;

    deviceVector() = default;
    deviceVector(const deviceVector &) = delete;
    deviceVector &operator=(const deviceVector &) = delete;
    ~deviceVector() { free(); }

    void allocate(int new_size)
    {
        free();
        allocate_device(&data, (size_t)new_size);
        size = capacity = new_size;
    }
    size_t bytes() const { return (size_t)size * sizeof(T); }
    void swap(deviceVector<T> &other)
    {
        T *d = other.data;
        const int s = other.size, c = other.capacity;
        other.data = data;
        other.size = size;
        other.capacity = capacity;
        data = d;
        size = s;
        capacity = c;
    }
    void resize(int new_size)
    {
        if (new_size <= capacity) {
            size = new_size;
            return;
        }
        allocate((int)(CONSTANTS::MEMORY_REALLOCATION_COEFFICIENT * new_size));
        size = new_size;
    }

private:
    void free()
    {
        if (data) free_device(data);
        data = nullptr;
        size = capacity = 0;
    }
};

#endif
