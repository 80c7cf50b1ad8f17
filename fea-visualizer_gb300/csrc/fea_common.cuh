// fea_common.cuh -- shared device/host helpers of libfea_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <tuple>
#include <vector>

#include "fea_gpu.h"

namespace fea {

// ---- error plumbing (no exception crosses the C ABI) -----------------------
void set_error(const char* fmt, ...);

struct Error {
    int code;
};

#define FEA_CUDA_TRY(expr)                                                                     \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            ::fea::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(e_)); \
            throw ::fea::Error{e_ == cudaErrorMemoryAllocation ? FEA_ERR_OUT_OF_MEMORY          \
                                                               : FEA_ERR_CUDA};                \
        }                                                                                      \
    } while (0)

#define FEA_CHECK_LAUNCH() FEA_CUDA_TRY(cudaGetLastError())

inline int fail(int code, const char* msg) {
    set_error("%s", msg);
    return code;
}

// ---- sizes -----------------------------------------------------------------
constexpr int kBlock = 256;        // threads per block of the streaming kernels
constexpr int kMaxFields = 2;      // Gray-Scott solves u and v together

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

int num_sms();

// ---- field vectors: NF interleaved fields per unknown ------------------------
// Gray-Scott keeps (u, v) interleaved so one 8-byte (FP32) or 16-byte (FP64)
// load brings both operands of the paired SpMV.
template <typename R, int NF>
struct alignas(sizeof(R) * NF) FV {
    R v[NF];
};

// ---- device helpers ----------------------------------------------------------
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Deterministic block sum of NV doubles per thread; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&x)[NV], double* smem /* [32*NV] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        x[k] = warp_sum(x[k]);
        if (lane == 0) smem[wid * NV + k] = x[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double y = lane < nw ? smem[lane * NV + k] : 0.0;
            x[k] = warp_sum(y);
        }
    }
    __syncthreads();
}

// Last-block-done reduction.  Thread 0 of every block stores its block's NV
// totals to part[k * stride + blockIdx.x]; the block that finishes last sums
// all partials in a fixed order (so the result does not depend on which block
// finished last) and returns true in all its threads with the totals in out[]
// (valid in thread 0).  The ticket counter is reset for the next launch.
template <int NV>
__device__ bool last_block_commit(const double (&blk)[NV], double* part, int stride, unsigned int* ticket,
                                  double* smem, double (&out)[NV]) {
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) part[k * stride + blockIdx.x] = blk[k];
        __threadfence();
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    double y[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc += __ldcg(&part[k * stride + b]);
        y[k] = acc;
    }
    block_sum<NV>(y, smem);
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = y[k];
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// Fused multiply-add in the operands' own precision (the float overload runs
// on the FP32 pipe; nothing here may promote to double, whose pipe is narrow).
__device__ __forceinline__ float fmar(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmar(double a, double b, double c) { return __fma_rn(a, b, c); }

// Round-to-nearest arithmetic without contraction, so that FP32 operator
// values match the reference's per-entry evaluation bit for bit.
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

// ---- scans (pattern build) ------------------------------------------------------
// Exclusive prefix sum of n int32 values into out[0..n]; out[n] = total.
// Uses scratch from the caller's allocator; returns the total (synchronises).
int64_t exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st);

// ---- device memory owned by a handle ------------------------------------------
struct DeviceArena {
    DeviceArena() = default;
    DeviceArena(const DeviceArena&) = delete;
    DeviceArena& operator=(const DeviceArena&) = delete;
    std::vector<void*> ptrs;
    int64_t bytes = 0;
    template <typename T>
    T* alloc(int64_t count) {
        void* p = nullptr;
        size_t nb = (size_t)(count > 0 ? count : 1) * sizeof(T);
        FEA_CUDA_TRY(cudaMalloc(&p, nb));
        ptrs.push_back(p);
        bytes += (int64_t)nb;
        return static_cast<T*>(p);
    }
    void release() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
        bytes = 0;
    }
    ~DeviceArena() { release(); }
};

}  // namespace fea
