// Device helpers shared by the solver translation units: deterministic
// block reductions and the "last block to finish" pattern.
#pragma once

#include <cuda_runtime.h>

#include "isl_df.cuh"

namespace isl {

template <typename T>
__device__ inline T ld(const T* p) { return __ldg(p); }

// Loads with a cache hint for data streamed once per kernel (not kept in L1)
__device__ __forceinline__ float ld_stream(const float* p) {
    float v;
    asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ int ld_stream(const int* p) {
    int v;
    asm volatile("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
// a 16-bit signed value, sign-extended
__device__ __forceinline__ int ld_stream(const short* p) {
    int v;
    asm volatile("ld.global.nc.L1::no_allocate.s16 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// Row dot product of a CSR matrix by a group of LPR lanes.  Every lane of the
// warp must call it the same number of times (the shuffles use the full-warp
// mask); lanes of a group without a row pass active = false and contribute 0.
template <typename TV, typename TX, int LPR>
__device__ inline TX row_dot(int row, bool active, const int* __restrict__ rowptr, const int* __restrict__ colind,
                             const TV* __restrict__ val, const TX* __restrict__ p, int lane) {
    TX acc = TX(0);
    if (active) {
        const int lo = rowptr[row], hi = rowptr[row + 1];
        for (int k = lo + lane; k < hi; k += LPR) acc += (TX)ld(val + k) * ld(p + ld(colind + k));
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, LPR);
    return acc;
}

// Software barrier across the blocks of a cooperative launch (every block is
// resident).  bar[0] counts arrivals, bar[1] is the generation.  Thread 0 of
// each block arrives with a release add (after the block barrier, so it
// publishes the writes of the whole block) and polls the generation with
// acquire loads, with an iteration limit: on expiry it sets *fault and the
// barrier reports false in every thread of the block.  A block that sees
// *fault set also reports false, so all blocks leave.  After the barrier,
// ordinary loads see every block's writes from before it (the acquire and
// the block barrier order them); only the non-coherent load path must not be
// used for data written inside the same launch.
constexpr unsigned GRID_SYNC_LIMIT = 1u << 22;
__device__ inline bool grid_sync(unsigned* bar, int* fault) {
    __shared__ int gs_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned gen, prev;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(gen) : "l"(bar + 1) : "memory");
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(prev) : "l"(bar) : "memory");
        if (prev + 1u == gridDim.x) {
            bar[0] = 0u;
            asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(bar + 1), "r"(gen + 1u) : "memory");
        } else {
            unsigned it = 0, g;
            for (;;) {
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(bar + 1) : "memory");
                if (g != gen) break;
                if (++it > GRID_SYNC_LIMIT || *(volatile int*)fault) { ok = 0; atomicExch(fault, 1); break; }
            }
        }
        if (*(volatile int*)fault) ok = 0;
        gs_ok = ok;
    }
    __syncthreads();
    return gs_ok != 0;
}

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

// a / b computed once by thread 0 and read by every thread of the block: an
// FP64 division is a sequence of FP64 operations, which run at 1/64 of the
// FP32 rate, so a block-wide division costs microseconds.  All threads of the
// block must call it (it holds two block barriers).
__device__ inline double block_div(double a, double b) {
    __shared__ double bd;
    if (threadIdx.x == 0) bd = a / b;
    __syncthreads();
    const double v = bd;
    __syncthreads();
    return v;
}

// Block sum of FP32 values: each warp adds its lanes in FP32 (the precision of
// the values), the warp sums are added in FP64 by warp 0.  FP64 arithmetic
// runs at 1/64 of the FP32 rate on this GPU, so the FP64 part is kept to one
// warp.  Fixed order; the result is valid in warp 0 (thread 0).
__device__ inline double block_sum_f(float v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = (double)v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;
}

// The same block sum with the warp sums added in double-float (about 48
// significant bits) on the FP32 pipe instead of FP64: a butterfly of df adds
// in warp 0 (TwoSum is exact, so both partners of a butterfly step compute
// the same bits).  sh: 32 floats.  Fixed order; valid in warp 0.
__device__ inline df block_sum_df(float v, float* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    df t = {0.f, 0.f};
    if (w == 0) {
        t.hi = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.f;
        for (int o = 16; o > 0; o >>= 1) {
            const df u = {__shfl_xor_sync(0xffffffffu, t.hi, o), __shfl_xor_sync(0xffffffffu, t.lo, o)};
            t = df_add_acc(t, u);
        }
    }
    return t;
}

// Two block sums at once (one pair of barriers): the bits of two
// block_sum_df calls.  sh: 64 floats.  Valid in warp 0.
__device__ inline void block_sum_df2(float a, float b, float* sh, df& oa, df& ob) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { sh[w] = a; sh[32 + w] = b; }
    __syncthreads();
    oa = ob = df{0.f, 0.f};
    if (w == 0) {
        const bool in = l < (int)(blockDim.x >> 5);
        oa.hi = in ? sh[l] : 0.f;
        ob.hi = in ? sh[32 + l] : 0.f;
        for (int o = 16; o > 0; o >>= 1) {
            const df ua = {__shfl_xor_sync(0xffffffffu, oa.hi, o), __shfl_xor_sync(0xffffffffu, oa.lo, o)};
            const df ub = {__shfl_xor_sync(0xffffffffu, ob.hi, o), __shfl_xor_sync(0xffffffffu, ob.lo, o)};
            oa = df_add_acc(oa, ua);
            ob = df_add_acc(ob, ub);
        }
    }
}

// the block sum matching the precision of the summed values
__device__ inline double block_sum_t(float v, double* sh) { return block_sum_f(v, sh); }
__device__ inline double block_sum_t(double v, double* sh) { return block_sum(v, sh); }

// Sum of part[i*stride + off], i < n, by warp 0 of the calling block: each lane
// issues eight loads before adding them, then a fixed shuffle tree.  The
// result is valid in warp 0 (thread 0); the other warps return 0.
__device__ inline double reduce_parts(const double* part, int n, int stride, int off, double* sh) {
    (void)sh;
    if (threadIdx.x >= 32) return 0.0;
    const int l = threadIdx.x;
    double s = 0.0;
    for (int base = 0; base < n; base += 256) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = base + u * 32 + l;
            v[u] = i < n ? __ldcg(part + (size_t)i * stride + off) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * 32 + l < n) s += v[u];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

// The two interleaved sums part[2i], part[2i+1] (i < n), by warp 0 as above.
__device__ inline void reduce_parts2(const double* part, int n, double* sh, double& out0, double& out1) {
    (void)sh;
    out0 = out1 = 0.0;
    if (threadIdx.x >= 32) return;
    const int l = threadIdx.x;
    const double2* p2 = reinterpret_cast<const double2*>(part);
    double s0 = 0.0, s1 = 0.0;
    for (int base = 0; base < n; base += 256) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = base + u * 32 + l;
            v[u] = i < n ? __ldcg(p2 + i) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * 32 + l < n) { s0 += v[u].x; s1 += v[u].y; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    out0 = s0;
    out1 = s1;
}

// Block-wide forms of the two sums above, for the last block of a large grid:
// every one of the NT threads of the block must call them (they hold block
// barriers).  Thread t loads entries t, t + NT, ... (eight in flight), so a
// grid of up to 8 NT blocks is read in one round trip instead of one per 256
// entries; each warp adds its lanes by a fixed shuffle tree and thread 0 adds
// the warp sums in warp order.  Fixed order; the result is valid in thread 0.
template <int NT>
__device__ inline double reduce_parts_blk(const double* part, int n, int stride, int off, double* sh) {
    static_assert(NT % 32 == 0 && NT / 32 <= 32, "sh holds one double per warp");
    double s = 0.0;
    for (int base = 0; base < n; base += 8 * NT) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = base + u * NT + (int)threadIdx.x;
            v[u] = i < n ? __ldcg(part + (size_t)i * stride + off) : 0.0;
        }
        // only the loaded entries are added (adding the zeros changes no
        // sum, and FP64 adds are scarce on this GPU)
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * NT + (int)threadIdx.x < n) s += v[u];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __syncthreads();  // sh may still be read by an earlier block sum
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; ++w) t += sh[w];
    return t;
}

template <int NT>
__device__ inline void reduce_parts2_blk(const double* part, int n, double* sh, double& out0, double& out1) {
    static_assert(NT % 32 == 0 && NT / 16 <= 32, "sh holds two doubles per warp");
    const double2* p2 = reinterpret_cast<const double2*>(part);
    double s0 = 0.0, s1 = 0.0;
    for (int base = 0; base < n; base += 8 * NT) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = base + u * NT + (int)threadIdx.x;
            v[u] = i < n ? __ldcg(p2 + i) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * NT + (int)threadIdx.x < n) { s0 += v[u].x; s1 += v[u].y; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) { sh[2 * (threadIdx.x >> 5)] = s0; sh[2 * (threadIdx.x >> 5) + 1] = s1; }
    __syncthreads();
    out0 = out1 = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; ++w) { out0 += sh[2 * w]; out1 += sh[2 * w + 1]; }
}

// Double-float counterparts of reduce_parts_blk / reduce_parts2_blk for
// partial sums stored as (hi, lo) float pairs (block_sum_df): the same
// loads (eight in flight per thread), df adds on the FP32 pipe where those
// use FP64 (GB300 runs FP64 at 1/64 of the FP32 rate, and these sums sit in
// the serial tail of every CG kernel).  sh: 32 doubles of shared memory,
// reused as 32 df.  Fixed order; the result (rounded to FP64) is valid in
// thread 0.
__device__ inline df warp_sum_df(df s) {
    for (int o = 16; o > 0; o >>= 1) {
        const df u = {__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)};
        s = df_add_acc(s, u);
    }
    return s;
}

__device__ inline double df_value(df a) { return (double)a.hi + (double)a.lo; }

// Sum of the (hi, lo) pairs part[i], i < n, by warp 0 (the double-float
// counterpart of reduce_parts): eight loads in flight per lane, df adds,
// a fixed butterfly.  Valid in warp 0.
__device__ inline double reduce_parts_df(const float2* part, int n) {
    if (threadIdx.x >= 32) return 0.0;
    const int l = threadIdx.x;
    df s = {0.f, 0.f};
    for (int base = 0; base < n; base += 256) {
        float2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = base + u * 32 + l;
            v[u] = i < n ? __ldcg(part + i) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * 32 + l < n) s = df_add_acc(s, df{v[u].x, v[u].y});
    }
    return df_value(warp_sum_df(s));
}

template <int NT>
__device__ inline double reduce_parts_df_blk(const float2* part, int n, double* sh) {
    static_assert(NT % 32 == 0 && NT / 32 <= 32, "sh holds one df per warp");
    df* shd = reinterpret_cast<df*>(sh);
    df s = {0.f, 0.f};
    for (int base = 0; base < n; base += 8 * NT) {
        float2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = base + u * NT + (int)threadIdx.x;
            v[u] = i < n ? __ldcg(part + i) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * NT + (int)threadIdx.x < n) s = df_add_acc(s, df{v[u].x, v[u].y});
    }
    s = warp_sum_df(s);
    __syncthreads();  // sh may still be read by an earlier block sum
    if ((threadIdx.x & 31) == 0) shd[threadIdx.x >> 5] = s;
    __syncthreads();
    df t = {0.f, 0.f};
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; ++w) t = df_add_acc(t, shd[w]);
    return df_value(t);
}

template <int NT>
__device__ inline void reduce_parts2_df_blk(const float4* part, int n, double* sh, double& out0, double& out1) {
    static_assert(NT % 32 == 0 && NT / 16 <= 32, "sh holds two df per warp");
    df* shd = reinterpret_cast<df*>(sh);
    df s0 = {0.f, 0.f}, s1 = {0.f, 0.f};
    for (int base = 0; base < n; base += 8 * NT) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = base + u * NT + (int)threadIdx.x;
            v[u] = i < n ? __ldcg(part + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * NT + (int)threadIdx.x < n) {
                s0 = df_add_acc(s0, df{v[u].x, v[u].y});
                s1 = df_add_acc(s1, df{v[u].z, v[u].w});
            }
    }
    s0 = warp_sum_df(s0);
    s1 = warp_sum_df(s1);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) { shd[2 * (threadIdx.x >> 5)] = s0; shd[2 * (threadIdx.x >> 5) + 1] = s1; }
    __syncthreads();
    out0 = out1 = 0.0;
    if (threadIdx.x == 0) {
        df t0 = {0.f, 0.f}, t1 = {0.f, 0.f};
        for (int w = 0; w < NT / 32; ++w) { t0 = df_add_acc(t0, shd[2 * w]); t1 = df_add_acc(t1, shd[2 * w + 1]); }
        out0 = df_value(t0);
        out1 = df_value(t1);
    }
}

}  // namespace isl
