// Device helpers shared by the solver translation units: deterministic
// block reductions and the "last block to finish" pattern.
#pragma once

#include <cuda_runtime.h>

namespace isl {

template <typename T>
__device__ inline T ld(const T* p) { return __ldg(p); }

// fixed-order block reduction of a double (deterministic); result in thread 0
__device__ inline double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;
}

// true in every thread of the last block to finish
__device__ inline bool last_block(unsigned int* ticket) {
    __shared__ bool amLast;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(ticket, 1u);
        amLast = (t == gridDim.x - 1);
    }
    __syncthreads();
    return amLast;
}

// true in every thread of the last of `count` blocks sharing a ticket
__device__ inline bool last_of(unsigned int* ticket, unsigned int count) {
    __shared__ bool amLastOf;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(ticket, 1u);
        amLastOf = (t == count - 1);
    }
    __syncthreads();
    return amLastOf;
}

__device__ inline double reduce_parts(const double* part, int n, int stride, int off, double* sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(part + (size_t)i * stride + off);
    return block_sum(s, sh);
}


}  // namespace isl
