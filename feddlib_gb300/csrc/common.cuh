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
constexpr int kSlotLocal = 15;      // byte of the slot data holding the incidence's local node index

// Device error word (first error wins); read back by fedd_check.
// kDevTimeout: a bounded wait on the tensor cores gave up (the kernel freed
// its tensor memory and returned).
enum DevErr : int { kDevOk = 0, kDevNonFinite = 1, kDevBadDet = 2, kDevCapacity = 3, kDevMesh = 4, kDevTimeout = 5 };

#ifdef __CUDACC__  // device helpers: the host-only translation units skip them
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

// FP64 -> FP32 with round-to-nearest-even using integer ops only: the
// hardware conversion issues on the narrow FP64 pipe (about 1.6 results per
// clock per SM on GB300, against ~85 for the opposite direction).  Results
// below FP32's normal range flush to signed zero; overflow gives inf; NaN
// stays NaN.
__device__ __forceinline__ float d2f_rn(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t sign = hi & 0x80000000u;
    const int e11 = (int)((hi >> 20) & 0x7ffu);
    const int ex = e11 - 1023 + 127;
    const uint32_t man = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1fffffffu;
    const uint32_t up = (rem > 0x10000000u) || (rem == 0x10000000u && (man & 1u));
    uint32_t r = ((uint32_t)ex << 23) + man + up;
    r = (ex >= 255) ? 0x7f800000u : r;
    r = (ex <= 0) ? 0u : r;
    r = (e11 == 0x7ff && ((hi & 0xfffffu) | lo)) ? 0x7fc00000u : r;
    return __uint_as_float(sign | r);
}

// FP64 affine geometry of one tetrahedron, as the reference forms it
// (Helper::buildTransformation, feddlib/core/FE/Helper.cpp:196-222;
// SmallMatrix::computeDet / computeInverse, SmallMatrix.hpp:317-368):
// B = [x1 - x0, x2 - x0, x3 - x0] (columns), det B by cofactor expansion and
// B^-1 = adj(B) / det B, all in FP64; each entry of B^-1 is then rounded
// once to FP32 (Bi, row-major) for the FP32 element integrals.  Returns
// det B (signed, FP64).
__device__ __forceinline__ double geometry_fp64(const double *__restrict__ xyz, int32_t n0, int32_t n1, int32_t n2,
                                                int32_t n3, float *Bi) {
    const double x0 = xyz[3 * (int64_t)n0], y0 = xyz[3 * (int64_t)n0 + 1], z0 = xyz[3 * (int64_t)n0 + 2];
    const double B0 = xyz[3 * (int64_t)n1] - x0, B3 = xyz[3 * (int64_t)n1 + 1] - y0, B6 = xyz[3 * (int64_t)n1 + 2] - z0;
    const double B1 = xyz[3 * (int64_t)n2] - x0, B4 = xyz[3 * (int64_t)n2 + 1] - y0, B7 = xyz[3 * (int64_t)n2 + 2] - z0;
    const double B2 = xyz[3 * (int64_t)n3] - x0, B5 = xyz[3 * (int64_t)n3 + 1] - y0, B8 = xyz[3 * (int64_t)n3 + 2] - z0;
    const double C00 = B4 * B8 - B5 * B7, C01 = B5 * B6 - B3 * B8, C02 = B3 * B7 - B4 * B6;
    const double C10 = B2 * B7 - B1 * B8, C11 = B0 * B8 - B2 * B6, C12 = B1 * B6 - B0 * B7;
    const double C20 = B1 * B5 - B2 * B4, C21 = B2 * B3 - B0 * B5, C22 = B0 * B4 - B1 * B3;
    const double det = B0 * C00 + B1 * C01 + B2 * C02;
    const double id = 1.0 / det;
    Bi[0] = d2f_rn(C00 * id); Bi[1] = d2f_rn(C10 * id); Bi[2] = d2f_rn(C20 * id);
    Bi[3] = d2f_rn(C01 * id); Bi[4] = d2f_rn(C11 * id); Bi[5] = d2f_rn(C21 * id);
    Bi[6] = d2f_rn(C02 * id); Bi[7] = d2f_rn(C12 * id); Bi[8] = d2f_rn(C22 * id);
    return det;
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


// ---- asynchronous copies (cp.async) and per-node incidence lists ----------
__device__ __forceinline__ void cp_async4(void *smem_dst, const void *gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---- TF32 tensor-core products (mma.sync m16n8k8, FP32 accumulate) --------
// Fragments (g = lane / 4, tq = lane % 4): A row-major 16x8, a0 = A[g][tq],
// a1 = A[g+8][tq], a2 = A[g][tq+4], a3 = A[g+8][tq+4]; B 8x8, b0 = B[tq][g],
// b1 = B[tq+4][g]; C/D 16x8, c0 = C[g][2 tq], c1 = C[g][2 tq + 1],
// c2 = C[g+8][2 tq], c3 = C[g+8][2 tq + 1].  Callers split each operand into
// TF32 hi + lo parts and sum hi.hi + hi.lo + lo.hi (3xTF32: FP32-level products).
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// the node's incidence list, one coalesced load: lane k holds entries k and
// k + 32 (a node has at most kMaxIncidence = 64 incidences)
struct IncList {
    uint32_t lo, hi;
};
__device__ __forceinline__ IncList load_incidences(const uint32_t *__restrict__ inc, int64_t i0, int m, int lane) {
    IncList l;
    l.lo = lane < m ? __ldg(inc + i0 + lane) : 0u;
    l.hi = lane + 32 < m ? __ldg(inc + i0 + lane + 32) : 0u;
    return l;
}
__device__ __forceinline__ uint32_t incidence_at(const IncList &l, int t) {
    const uint32_t lo = __shfl_sync(0xffffffffu, l.lo, t & 31);
    const uint32_t hi = __shfl_sync(0xffffffffu, l.hi, t & 31);
    return t < 32 ? lo : hi;
}
#endif  // __CUDACC__

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
