// reduce.cuh -- deterministic FP64 sums of per-thread terms: warp shuffles,
// then one partial per block, then a fixed-order sum of the partials by one
// block (objective.cu and the projection's data-term epilogue, project.cuh).
#pragma once

#include <stdint.h>

namespace nr {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of v written to red[blk] by thread 0 (blockDim multiple of 32, <= 1024).
__device__ __forceinline__ void block_partial(double v, double* red, int64_t blk) {
    __shared__ double ws[32];
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    const int nt = blockDim.x * blockDim.y;
    v = warp_sum(v);
    if ((t & 31) == 0) ws[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        double s = (t < (nt >> 5)) ? ws[t] : 0.0;
        s = warp_sum(s);
        if (t == 0) red[blk] = s;
    }
}

// Fixed-order sum of n partials into out[0] by one block of 1024 threads.
__device__ __forceinline__ void sum_partials(const double* __restrict__ red, int64_t n,
                                             double* __restrict__ out) {
    __shared__ double ws[32];
    double s = 0.0;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) s += red[k];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = ws[threadIdx.x];
        t = warp_sum(t);
        if (threadIdx.x == 0) out[0] = t;
    }
    __syncthreads();
}

}  // namespace nr
