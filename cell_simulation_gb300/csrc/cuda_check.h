// cuda_check.h — CUDA error checking that converts failures into cellsim::Error.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "internal.h"

#define CS_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t err__ = (call);                                                                \
        if (err__ != cudaSuccess)                                                                  \
            throw ::cellsim::Error(CS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err__)); \
    } while (0)

#define CS_LAUNCH_CHECK()                                                                          \
    do {                                                                                           \
        cudaError_t err__ = cudaGetLastError();                                                    \
        if (err__ != cudaSuccess)                                                                  \
            throw ::cellsim::Error(CS_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(err__)); \
    } while (0)

namespace cellsim {

// RAII device buffer.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { reset(); }
    void alloc(size_t count) {
        reset();
        n = count;
        if (count) CS_CUDA(cudaMalloc((void**)&p, sizeof(T) * count));
    }
    void reset() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return sizeof(T) * n; }
};

// Makes `device` current for the lifetime of the guard and restores the
// previous device afterwards.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        CS_CUDA(cudaSetDevice(dev));
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace cellsim
