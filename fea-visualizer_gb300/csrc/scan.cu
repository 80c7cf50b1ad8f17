// scan.cu -- exclusive prefix sums used while building patterns (set-up only).
// Three phases: per-block sums, a recursive scan of the block sums, and the
// block-local scans offset by their block's prefix.
#include <vector>

#include "fea_common.cuh"

namespace fea {

namespace {

constexpr int kScanBlock = 1024;

__device__ __forceinline__ int64_t block_inclusive_scan(int64_t v, int64_t* sm) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) sm[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int64_t w = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sm[lane] = w;
    }
    __syncthreads();
    if (wid > 0) v += sm[wid - 1];
    __syncthreads();
    return v;
}

__global__ void k_block_sums(const int32_t* in, int64_t n, int64_t* sums) {
    __shared__ int64_t sm[32];
    int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
    int64_t v = i < n ? in[i] : 0;
    v = block_inclusive_scan(v, sm);
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = v;
}

__global__ void k_block_sums64(const int64_t* in, int64_t n, int64_t* sums) {
    __shared__ int64_t sm[32];
    int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
    int64_t v = i < n ? in[i] : 0;
    v = block_inclusive_scan(v, sm);
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = v;
}

__global__ void k_apply64(const int64_t* in, int64_t n, const int64_t* offs, int64_t* out) {
    __shared__ int64_t sm[32];
    int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
    int64_t x = i < n ? in[i] : 0;
    int64_t v = block_inclusive_scan(x, sm);
    int64_t base = offs ? offs[blockIdx.x] : 0;
    if (i < n) out[i] = base + v - x;
    if (i == n - 1) out[n] = base + v;
}

__global__ void k_apply32(const int32_t* in, int64_t n, const int64_t* offs, int32_t* out) {
    __shared__ int64_t sm[32];
    int64_t i = blockIdx.x * (int64_t)kScanBlock + threadIdx.x;
    int64_t x = i < n ? in[i] : 0;
    int64_t v = block_inclusive_scan(x, sm);
    int64_t base = offs ? offs[blockIdx.x] : 0;
    if (i < n) out[i] = (int32_t)(base + v - x);
    if (i == n - 1) out[n] = (int32_t)(base + v);
}

// Exclusive scan of int64 values: out[0..n], out[n] = total.
void scan64(DeviceArena& tmp, const int64_t* in, int64_t n, int64_t* out, cudaStream_t st) {
    int64_t nb = ceil_div(n, kScanBlock);
    if (nb <= 1) {
        k_apply64<<<1, kScanBlock, 0, st>>>(in, n, nullptr, out);
        FEA_CHECK_LAUNCH();
        return;
    }
    int64_t* sums = tmp.alloc<int64_t>(nb);
    int64_t* offs = tmp.alloc<int64_t>(nb + 1);
    k_block_sums64<<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, sums);
    FEA_CHECK_LAUNCH();
    scan64(tmp, sums, nb, offs, st);
    k_apply64<<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, offs, out);
    FEA_CHECK_LAUNCH();
}

}  // namespace

int64_t exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st) {
    if (n <= 0) {
        FEA_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int32_t), st));
        return 0;
    }
    DeviceArena tmp;
    int64_t nb = ceil_div(n, kScanBlock);
    int64_t* offs = nullptr;
    if (nb > 1) {
        int64_t* sums = tmp.alloc<int64_t>(nb);
        offs = tmp.alloc<int64_t>(nb + 1);
        k_block_sums<<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, sums);
        FEA_CHECK_LAUNCH();
        scan64(tmp, sums, nb, offs, st);
    }
    k_apply32<<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, offs, out);
    FEA_CHECK_LAUNCH();
    int64_t total = 0;
    // the total is checked against int32 range by recomputing it in 64 bits
    if (offs) {
        FEA_CUDA_TRY(cudaMemcpyAsync(&total, offs + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    } else {
        int32_t t32 = 0;
        FEA_CUDA_TRY(cudaMemcpyAsync(&t32, out + n, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        FEA_CUDA_TRY(cudaStreamSynchronize(st));
        total = t32;
    }
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    if (total > INT32_MAX) {
        set_error("prefix sum exceeds the int32 index range (%lld)", (long long)total);
        throw Error{FEA_ERR_TOO_LARGE};
    }
    return total;
}

}  // namespace fea
