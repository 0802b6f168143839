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

// Ticket with release/acquire semantics at GPU scope: the release orders the
// partial sums thread 0 stored before it; the acquire of the block that draws
// the last ticket makes every block's partials visible to it (and, through the
// barrier that follows, to all of its threads).  Lighter than a sequentially
// consistent __threadfence() in every block.
__device__ inline unsigned ticket_acq_rel(unsigned* ticket) {
    unsigned t;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(t) : "l"(ticket) : "memory");
    return t;
}

// true in every thread of the last block to finish.  Only thread 0 wrote the
// block's partial sums, so only it takes the ticket.
__device__ inline bool last_block(unsigned int* ticket) {
    __shared__ bool amLast;
    __syncthreads();
    if (threadIdx.x == 0) amLast = (ticket_acq_rel(ticket) == gridDim.x - 1);
    __syncthreads();
    return amLast;
}

// true in every thread of the last of `count` blocks sharing a ticket
__device__ inline bool last_of(unsigned int* ticket, unsigned int count) {
    __shared__ bool amLastOf;
    __syncthreads();
    if (threadIdx.x == 0) amLastOf = (ticket_acq_rel(ticket) == count - 1);
    __syncthreads();
    return amLastOf;
}

// Sum of part[i*stride + off], i < n, by one block: the loads of a thread are
// issued together (unrolled) before they are added, in a fixed order.
__device__ inline double reduce_parts(const double* part, int n, int stride, int off, double* sh) {
    double s = 0.0;
    int i = threadIdx.x;
    for (; i + 3 * (int)blockDim.x < n; i += 4 * blockDim.x) {
        const double a = __ldcg(part + (size_t)i * stride + off);
        const double b = __ldcg(part + (size_t)(i + blockDim.x) * stride + off);
        const double c = __ldcg(part + (size_t)(i + 2 * blockDim.x) * stride + off);
        const double d = __ldcg(part + (size_t)(i + 3 * blockDim.x) * stride + off);
        s += (a + b) + (c + d);
    }
    for (; i < n; i += blockDim.x) s += __ldcg(part + (size_t)i * stride + off);
    return block_sum(s, sh);
}

// The two interleaved sums part[2i], part[2i+1] (i < n) in one pass.
__device__ inline void reduce_parts2(const double* part, int n, double* sh, double& out0, double& out1) {
    double s0 = 0.0, s1 = 0.0;
    const double2* p2 = reinterpret_cast<const double2*>(part);
    int i = threadIdx.x;
    for (; i + 3 * (int)blockDim.x < n; i += 4 * blockDim.x) {
        const double2 a = __ldcg(p2 + i), b = __ldcg(p2 + i + blockDim.x);
        const double2 c = __ldcg(p2 + i + 2 * blockDim.x), d = __ldcg(p2 + i + 3 * blockDim.x);
        s0 += (a.x + b.x) + (c.x + d.x);
        s1 += (a.y + b.y) + (c.y + d.y);
    }
    for (; i < n; i += blockDim.x) {
        const double2 a = __ldcg(p2 + i);
        s0 += a.x;
        s1 += a.y;
    }
    out0 = block_sum(s0, sh);
    out1 = block_sum(s1, sh);
}


}  // namespace isl
