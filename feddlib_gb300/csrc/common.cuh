// common.cuh -- shared types and device helpers of the GB300 assembly engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/feddgpu.h"

namespace fedd {

// ---------------------------------------------------------------- limits --
// Per-node limits of the incidence-gather assembly.  The structured 6-tet
// meshes need 24 incidences and 65 adjacent P2 nodes at most; general meshes
// beyond these limits are rejected with FEDD_ERR_CAPACITY.
constexpr int kMaxIncidence = 64;   // elements sharing one node
constexpr int kMaxAdjacency = 255;  // distinct neighbour nodes (uint8 slots)
constexpr int kSlotStride = 16;     // bytes of slot data per incidence

// Device error word (first error wins); read back by fedd_check.
enum DevErr : int { kDevOk = 0, kDevNonFinite = 1, kDevBadDet = 2, kDevCapacity = 3, kDevMesh = 4 };

__device__ __forceinline__ void set_dev_error(int *err, int code) {
    if (err) atomicCAS(err, 0, code);
}

// FP32 -> FP64 exactly, with integer ops only (the GB300 FP64 pipe runs at a
// small fraction of the FP32 rate, so the per-value conversion of the CSR
// output avoids it).  Denormal floats become signed zero; inf/nan map across.
__device__ __forceinline__ double f2d_exact(float f) {
    uint32_t b = __float_as_uint(f);
    uint32_t sign = b & 0x80000000u;
    uint32_t ex = (b >> 23) & 0xffu;
    uint32_t man = b & 0x7fffffu;
    uint32_t hi = sign | ((ex + 896u) << 20) | (man >> 3);
    hi = (ex == 0u) ? sign : hi;
    hi = (ex == 255u) ? (sign | 0x7ff00000u | (man >> 3)) : hi;
    uint32_t lo = (ex == 0u) ? 0u : (man << 29);
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ float ld_nc(const float *p) { return __ldg(p); }

// streaming (evict-first) store of the write-once CSR values
__device__ __forceinline__ void st_cs(double *p, double v) { __stcs(p, v); }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------ host side --
struct CudaError {
    cudaError_t code;
    const char *what;
};

#define FEDD_CUDA(call)                                                       \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) throw ::fedd::CudaError{e_, #call};            \
    } while (0)

struct Status {
    fedd_status code;
    std::string msg;
};

#define FEDD_FAIL(code, msg) throw ::fedd::Status{code, msg}

template <class T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() {}
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            FEDD_FAIL(FEDD_ERR_NOMEM, "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes failed");
        }
        n = count;
    }
    void upload(const T *h, size_t count, cudaStream_t s = 0) {
        alloc(count);
        if (count) FEDD_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void zero(cudaStream_t s = 0) {
        if (n) FEDD_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

inline unsigned ceil_div(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

}  // namespace fedd
