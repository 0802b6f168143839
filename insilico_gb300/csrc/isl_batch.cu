// Batched Krylov solve: many independent instances (disjoint row ranges of
// one block-diagonal system) each run their own Jacobi-preconditioned CG with
// their own scalars, convergence test and iteration count, in the same
// kernel launches.  Thread blocks are assigned to row ranges of a single
// instance; each instance's reductions are summed by the last of its blocks
// (per-instance ticket), in a fixed order.  CHUNK iterations are captured
// into one CUDA graph and replayed until every instance is done.  The
// iteration kernels run on a fixed grid that loops over a device list of the
// row blocks of unfinished instances; the list is rebuilt at the start of
// every replay (kb_compact), so the launches shrink with the set of
// instances still iterating instead of sweeping every row block of the batch.
//
// Mixed method: FP32 CG with FP64 reliable updates per instance, inside the
// graph: an instance whose iterated residual dropped 10x (or met the
// tolerance) folds its FP32 increment into the FP64 iterate, recomputes its
// FP64 residual b - A64 x and resumes; it finishes when the FP64 residual
// meets the tolerance.
#include <cmath>
#include <functional>
#include <type_traits>
#include <vector>

#include "isl_device.cuh"
#include "isl_internal.h"

namespace isl {

namespace {

constexpr int BBS = 256;
constexpr int BCHUNK = 32;
constexpr int ROWS_PER_BLOCK = 2048;
// the reliable-update kernels split every row block of a listed instance into
// SUB row ranges, one CTA each, so that an instance's FP64 residual spreads
// over many SMs (FP64 runs at about 2 operations per clock per SM)
constexpr int SUB = 8;

// per-instance scalar slots in dbs [slot][ninst]
enum { S_ABSNEW, S_ABSOLD, S_ALPHA, S_BETA, S_RR, S_THRESH, S_RHS2, S_RRLAST, S_NS };
// per-instance int slots in dbi [slot][ninst]
enum { I_DONE, I_ITERS, I_BAD, I_UPDATE, I_RESET, I_NI };
// ticket slots in dbt [slot][ninst]; slot 3 element 0 counts remaining instances
enum { T_SPMV, T_UPD, T_RES, T_NT };

struct BArgs {
    int ninst;
    int nblk;             // row blocks of the batch (partial-sum slots per sum)
    const int* act;       // act[0]: listed row blocks, act[1..]: their ids (unfinished instances)
    const int* blk_inst;
    const int* blk_r0;
    const int* blk_r1;
    const int* inst_blk;  // [ninst+1]
    double* s;            // [S_NS][ninst]
    int* iv;              // [I_NI][ninst]
    unsigned* t;          // [T_NT][ninst]
    int* remaining;
    double* part;         // [SUB][nblocks]
    int* wl;              // [ninst] instances that need a reliable update this iteration
    int* wl_n;            // appends of the current iteration
    int* wl_cur;          // entries of the list being processed
    int* wl_cum;          // [ninst+1] row blocks of the listed instances before each entry
    int max_iter;
    double tol;
    double trig2;         // reliable update when r.r has dropped by this factor since the last one
    const int* blk_s0;    // batched sliced-ELL copy: slices of every row block
    const int* blk_s1;
};

__device__ inline double& SS(const BArgs& a, int slot, int k) { return a.s[(size_t)slot * a.ninst + k]; }
__device__ inline int& II(const BArgs& a, int slot, int k) { return a.iv[(size_t)slot * a.ninst + k]; }

__device__ inline void finish(const BArgs& a, int k, int code) {
    if (II(a, I_DONE, k) == 0) {
        II(a, I_DONE, k) = code;
        atomicSub(a.remaining, 1);
    }
}

__device__ inline double inst_sum(const BArgs& a, int k, int off, double* sh) {
    const int b0 = a.inst_blk[k], b1 = a.inst_blk[k + 1];
    return reduce_parts(a.part + (size_t)off * a.nblk + b0, b1 - b0, 1, 0, sh);
}

// FP32 vectors: a row block's partial sum as a double-float pair in its part
// slot, and an instance's total summed in double-float (the serial tails of
// the iteration kernels stay off the FP64 pipe)
__device__ inline void put_part_df(const BArgs& a, int off, int blk, float v, double* sh) {
    const df s = block_sum_df(v, reinterpret_cast<float*>(sh));
    if (threadIdx.x == 0) reinterpret_cast<float2*>(a.part)[(size_t)off * a.nblk + blk] = make_float2(s.hi, s.lo);
}
__device__ inline void put_part_df2(const BArgs& a, int blk, float v0, float v1, double* sh) {
    df s0, s1;
    block_sum_df2(v0, v1, reinterpret_cast<float*>(sh), s0, s1);
    if (threadIdx.x == 0) {
        reinterpret_cast<float2*>(a.part)[blk] = make_float2(s0.hi, s0.lo);
        reinterpret_cast<float2*>(a.part)[(size_t)a.nblk + blk] = make_float2(s1.hi, s1.lo);
    }
}
__device__ inline double inst_sum_df(const BArgs& a, int k, int off) {
    const int b0 = a.inst_blk[k], b1 = a.inst_blk[k + 1];
    return reduce_parts_df(reinterpret_cast<const float2*>(a.part) + (size_t)off * a.nblk + b0, b1 - b0);
}

// The listed row blocks, one per loop trip of a CTA: w-th entry of the list.
// Every thread of a CTA takes the same trips, so block barriers inside the
// body stay uniform.
#define FOR_LISTED_BLOCKS(a, blk)                                                   \
    for (int _w = blockIdx.x, _n = (a).act[0]; _w < _n; _w += gridDim.x)             \
        if (const int blk = (a).act[1 + _w]; true)

// The row blocks of every unfinished instance, in block order (one CTA; a
// block-wide scan over the instances' block counts).
__global__ void __launch_bounds__(1024) kb_compact(BArgs a, int* __restrict__ act) {
    __shared__ int sums[1024];
    const int per = (a.ninst + 1023) / 1024;
    const int k0 = min(a.ninst, (int)threadIdx.x * per), k1 = min(a.ninst, k0 + per);
    int cnt = 0;
    for (int k = k0; k < k1; ++k)
        if (!II(a, I_DONE, k)) cnt += a.inst_blk[k + 1] - a.inst_blk[k];
    sums[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // inclusive Hillis-Steele scan
        const int v = threadIdx.x >= o ? sums[threadIdx.x - o] : 0;
        __syncthreads();
        sums[threadIdx.x] += v;
        __syncthreads();
    }
    int pos = sums[threadIdx.x] - cnt;
    for (int k = k0; k < k1; ++k)
        if (!II(a, I_DONE, k))
            for (int b = a.inst_blk[k]; b < a.inst_blk[k + 1]; ++b) act[1 + pos++] = b;
    if (threadIdx.x == 1023) act[0] = sums[1023];
}

template <typename TB, typename TX>
__global__ void __launch_bounds__(BBS) kb_init(BArgs a, const TB* __restrict__ b, TX* __restrict__ x, TX* __restrict__ r,
                                               TX* __restrict__ p, const TX* __restrict__ dinv) {
    __shared__ double sh[32];
    const int k = a.blk_inst[blockIdx.x], r0 = a.blk_r0[blockIdx.x], r1 = a.blk_r1[blockIdx.x];
    double bb = 0.0, bz = 0.0;
    for (int i = r0 + threadIdx.x; i < r1; i += BBS) {
        const TB bi = b[i];
        const TX ri = (TX)bi;
        x[i] = TX(0);
        r[i] = ri;
        p[i] = TX(0);
        bb += (double)bi * (double)bi;
        bz += (double)ri * (double)(dinv[i] * ri);
    }
    const double s1 = block_sum(bb, sh), s2 = block_sum(bz, sh);
    if (threadIdx.x == 0) { a.part[blockIdx.x] = s1; a.part[a.nblk + blockIdx.x] = s2; }
    const unsigned cnt = a.inst_blk[k + 1] - a.inst_blk[k];
    if (last_of(&a.t[T_UPD * a.ninst + k], cnt)) {
        const double tbb = inst_sum(a, k, 0, sh), tbz = inst_sum(a, k, 1, sh);
        if (threadIdx.x == 0) {
            SS(a, S_RHS2, k) = tbb;
            SS(a, S_THRESH, k) = a.tol * a.tol * tbb;
            SS(a, S_ABSNEW, k) = tbz;
            SS(a, S_ABSOLD, k) = tbz;
            SS(a, S_BETA, k) = 0.0;
            SS(a, S_RR, k) = tbb;
            SS(a, S_RRLAST, k) = tbb;
            II(a, I_ITERS, k) = 0;
            II(a, I_UPDATE, k) = 0;
            II(a, I_BAD, k) = !(tbb == tbb);
            if (tbb == 0.0 || !(tbb == tbb)) finish(a, k, 1);
            a.t[T_UPD * a.ninst + k] = 0;
        }
    }
}

template <typename TX>
__global__ void __launch_bounds__(BBS) kb_dir(BArgs a, const TX* __restrict__ r, const TX* __restrict__ dinv, TX* __restrict__ p) {
    FOR_LISTED_BLOCKS(a, blk) {
        const int k = a.blk_inst[blk];
        if (II(a, I_DONE, k)) continue;
        const int r0 = a.blk_r0[blk], r1 = a.blk_r1[blk];
        const TX beta = (TX)SS(a, S_BETA, k);
        for (int i = r0 + threadIdx.x; i < r1; i += BBS) p[i] = dinv[i] * r[i] + beta * p[i];
    }
}

template <typename TV, typename TX, int LPR>
__global__ void __launch_bounds__(BBS) kb_spmv(BArgs a, const int* __restrict__ rowptr, const int* __restrict__ colind,
                                               const TV* __restrict__ val, const TX* __restrict__ p, TX* __restrict__ q) {
    __shared__ double sh[32];
    FOR_LISTED_BLOCKS(a, blk) {
    const int k = a.blk_inst[blk];
    if (II(a, I_DONE, k)) continue;
    const int r0 = a.blk_r0[blk], r1 = a.blk_r1[blk];
    const int lane = threadIdx.x % LPR, grp = threadIdx.x / LPR;
    const int wgrp = grp - grp % (32 / LPR);  // warp-uniform loop (full-mask shuffles)
    TX loc = TX(0);  // in the vectors' precision; warp sums are added in FP64
    // RU rows per lane group at a time: their index, value and p loads are
    // issued together, so a block keeps RU times more rows in flight (the
    // sums of each row keep the order of a one-row loop)
    constexpr int RU = 4;
    const int stride = BBS / LPR;
    for (int base = r0 + wgrp; base < r1; base += RU * stride) {
        int j[RU], e[RU];
        TX acc[RU];
#pragma unroll
        for (int u = 0; u < RU; ++u) {
            const int row = base + (grp - wgrp) + u * stride;
            const bool act = row < r1;
            j[u] = act ? __ldg(rowptr + row) + lane : 0;
            e[u] = act ? __ldg(rowptr + row + 1) : 0;
            acc[u] = TX(0);
        }
        for (;;) {
            int cj[RU];
            TV vv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (j[u] < e[u]) { cj[u] = __ldg(colind + j[u]); vv[u] = __ldg(val + j[u]); }
            bool more = false;
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (j[u] < e[u]) {
                    acc[u] += (TX)vv[u] * __ldg(p + cj[u]);
                    j[u] += LPR;
                    more |= j[u] < e[u];
                }
            if (!more) break;
        }
#pragma unroll
        for (int u = 0; u < RU; ++u) {
#pragma unroll
            for (int o = LPR / 2; o > 0; o >>= 1) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o, LPR);
            const int row = base + (grp - wgrp) + u * stride;
            if (row < r1 && lane == 0) {
                q[row] = acc[u];
                loc += p[row] * acc[u];
            }
        }
    }
    constexpr bool F32 = std::is_same<TX, float>::value;
    if constexpr (F32) {
        put_part_df(a, 0, blk, loc, sh);
    } else {
        const double s1 = block_sum_t(loc, sh);
        if (threadIdx.x == 0) a.part[blk] = s1;
    }
    const unsigned cnt = a.inst_blk[k + 1] - a.inst_blk[k];
    if (last_of(&a.t[T_SPMV * a.ninst + k], cnt)) {
        const double tot = F32 ? inst_sum_df(a, k, 0) : inst_sum(a, k, 0, sh);
        if (threadIdx.x == 0) {
            SS(a, S_ALPHA, k) = SS(a, S_ABSNEW, k) / tot;
            a.t[T_SPMV * a.ninst + k] = 0;
        }
    }
    }
}

// q = A p on the batched sliced-ELL copy: a row block's rows are sorted by
// length into slices of 32 (one lane per row); the block's 8 warps take its
// slices in turn and keep the loads of U slots in flight per lane.  The
// instance's p.q follows as in kb_spmv.
// TC = short: 16-bit column offsets from each lane's row (row 0 for a
// padding lane)
template <int U, int MINB, typename TC>
__global__ void __launch_bounds__(BBS, MINB) kb_sspmv(BArgs a, const int* __restrict__ soff, const int* __restrict__ swid,
                                                   const int* __restrict__ srow, const TC* __restrict__ scol,
                                                   const float* __restrict__ sv, const float* __restrict__ p,
                                                   float* __restrict__ q) {
    __shared__ double sh[32];
    FOR_LISTED_BLOCKS(a, blk) {
    const int k = a.blk_inst[blk];
    if (II(a, I_DONE, k)) continue;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sl0 = a.blk_s0[blk], sl1 = a.blk_s1[blk];
    float loc = 0.f;
    for (int s = sl0 + warp; s < sl1; s += BBS / 32) {
        const int o = soff[s] + lane, w = swid[s];
        const int row = srow[s * 32 + lane];
        const int base = sizeof(TC) == 2 ? max(row, 0) : 0;
        float acc = 0.f;
        for (int kk = 0; kk < w; kk += U) {
            int j[U];
            float v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (kk + u < w) {
                    j[u] = ld_stream(scol + o + (kk + u) * 32) + base;
                    v[u] = ld_stream(sv + o + (kk + u) * 32);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (kk + u < w) acc += v[u] * __ldg(p + j[u]);
        }
        if (row >= 0) {
            q[row] = acc;
            loc += p[row] * acc;
        }
    }
    put_part_df(a, 0, blk, loc, sh);
    const unsigned cnt = a.inst_blk[k + 1] - a.inst_blk[k];
    if (last_of(&a.t[T_SPMV * a.ninst + k], cnt)) {
        const double tot = inst_sum_df(a, k, 0);
        if (threadIdx.x == 0) {
            SS(a, S_ALPHA, k) = SS(a, S_ABSNEW, k) / tot;
            a.t[T_SPMV * a.ninst + k] = 0;
        }
    }
    }
}

// mixed = 1: convergence or a 10x drop of the iterated residual requests a
// reliable update instead of finishing
template <typename TX>
__global__ void __launch_bounds__(BBS) kb_update(BArgs a, TX* __restrict__ x, TX* __restrict__ r, const TX* __restrict__ p,
                                                 const TX* __restrict__ q, const TX* __restrict__ dinv, int mixed) {
    __shared__ double sh[32];
    FOR_LISTED_BLOCKS(a, blk) {
    const int k = a.blk_inst[blk];
    if (II(a, I_DONE, k)) continue;
    const int r0 = a.blk_r0[blk], r1 = a.blk_r1[blk];
    const TX alpha = (TX)SS(a, S_ALPHA, k);
    TX rr = TX(0), rz = TX(0);
    for (int i = r0 + threadIdx.x; i < r1; i += BBS) {
        x[i] += alpha * p[i];
        const TX ri = r[i] - alpha * q[i];
        r[i] = ri;
        rr += ri * ri;
        rz += ri * (dinv[i] * ri);
    }
    constexpr bool F32 = std::is_same<TX, float>::value;
    if constexpr (F32) {
        put_part_df2(a, blk, rr, rz, sh);
    } else {
        const double s1 = block_sum_t(rr, sh), s2 = block_sum_t(rz, sh);
        if (threadIdx.x == 0) { a.part[blk] = s1; a.part[a.nblk + blk] = s2; }
    }
    const unsigned cnt = a.inst_blk[k + 1] - a.inst_blk[k];
    if (last_of(&a.t[T_UPD * a.ninst + k], cnt)) {
        const double trr = F32 ? inst_sum_df(a, k, 0) : inst_sum(a, k, 0, sh);
        const double trz = F32 ? inst_sum_df(a, k, 1) : inst_sum(a, k, 1, sh);
        if (threadIdx.x == 0) {
            SS(a, S_RR, k) = trr;
            const int it = ++II(a, I_ITERS, k);
            SS(a, S_ABSOLD, k) = SS(a, S_ABSNEW, k);
            SS(a, S_BETA, k) = trz / SS(a, S_ABSNEW, k);
            SS(a, S_ABSNEW, k) = trz;
            if (!(trr == trr) || !(trz == trz)) { II(a, I_BAD, k) = 1; finish(a, k, 3); }
            else if (!mixed) {
                if (trr < SS(a, S_THRESH, k)) finish(a, k, 1);
                else if (it >= a.max_iter) finish(a, k, 2);
            } else if (trr < SS(a, S_THRESH, k) || trr < a.trig2 * SS(a, S_RRLAST, k) || it >= a.max_iter) {
                II(a, I_UPDATE, k) = 1;
                a.wl[atomicAdd(a.wl_n, 1)] = k;  // list order varies; each instance's sums do not
            }
            a.t[T_UPD * a.ninst + k] = 0;
        }
    }
    }
}

// The reliable updates of the listed instances.  kb_wl_scan turns the list
// into row-block offsets (one block); the kernels below run on a small fixed
// grid over (listed row block, sub-range) items, so an iteration in which no
// instance updates costs almost nothing.
__global__ void __launch_bounds__(BBS) kb_wl_scan(BArgs a) {
    __shared__ int sums[BBS];
    const int n = *a.wl_n;
    const int per = (n + BBS - 1) / BBS, i0 = min(n, (int)threadIdx.x * per), i1 = min(n, i0 + per);
    int loc = 0;
    for (int i = i0; i < i1; ++i) {
        const int k = a.wl[i];
        loc += a.inst_blk[k + 1] - a.inst_blk[k];
    }
    sums[threadIdx.x] = loc;
    __syncthreads();
    if (threadIdx.x == 0) {  // exclusive scan of the 256 segment sums
        int acc = 0;
        for (int t = 0; t < BBS; ++t) { const int v = sums[t]; sums[t] = acc; acc += v; }
        a.wl_cum[n] = acc;
        *a.wl_cur = n;
        *a.wl_n = 0;
    }
    __syncthreads();
    int acc = sums[threadIdx.x];
    for (int i = i0; i < i1; ++i) {
        a.wl_cum[i] = acc;
        const int k = a.wl[i];
        acc += a.inst_blk[k + 1] - a.inst_blk[k];
    }
}

// item w: listed row block w / SUB, sub-range w % SUB; false past the end
__device__ inline bool wl_item(const BArgs& a, int w, int& k, int& blk, int& r0, int& r1) {
    const int n = *a.wl_cur;
    if (n == 0 || w >= a.wl_cum[n] * SUB) return false;
    const int li = w / SUB, sub = w % SUB;
    int lo = 0, hi = n;  // largest lo with wl_cum[lo] <= li
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (a.wl_cum[mid] <= li) lo = mid; else hi = mid;
    }
    k = a.wl[lo];
    blk = a.inst_blk[k] + (li - a.wl_cum[lo]);
    const int b0 = a.blk_r0[blk], len = a.blk_r1[blk] - b0;
    r0 = b0 + (int)((long long)len * sub / SUB);
    r1 = b0 + (int)((long long)len * (sub + 1) / SUB);
    return true;
}

__global__ void __launch_bounds__(BBS) kb_fold_w(BArgs a, float* __restrict__ x32, double* __restrict__ x64) {
    int k, blk, r0, r1;
    for (int w = blockIdx.x; wl_item(a, w, k, blk, r0, r1); w += gridDim.x)
        for (int i = r0 + threadIdx.x; i < r1; i += BBS) {
            x64[i] += (double)x32[i];
            x32[i] = 0.0f;
        }
}

// r = b - A64 x on the listed instances (one thread per row); the last item of
// an instance sums its items' partials in order and decides: converged,
// iteration limit, or restart
__global__ void __launch_bounds__(BBS) kb_residual_w(BArgs a, const int* __restrict__ rowptr, const int* __restrict__ colind,
                                                     const double* __restrict__ val, const double* __restrict__ x,
                                                     const double* __restrict__ b, double* __restrict__ r) {
    __shared__ double sh[32];
    int k, blk, r0, r1;
    for (int w = blockIdx.x; wl_item(a, w, k, blk, r0, r1); w += gridDim.x) {
        double loc = 0.0;
        for (int row = r0 + threadIdx.x; row < r1; row += BBS) {
            double acc = 0.0;
            for (int j = rowptr[row]; j < rowptr[row + 1]; ++j) acc += __ldg(val + j) * x[__ldg(colind + j)];
            const double ri = b[row] - acc;
            r[row] = ri;
            loc += ri * ri;
        }
        const double s1 = block_sum(loc, sh);
        if (threadIdx.x == 0) a.part[(size_t)blk * SUB + (w % SUB)] = s1;
        const unsigned cnt = (unsigned)(a.inst_blk[k + 1] - a.inst_blk[k]) * SUB;
        if (last_of(&a.t[T_RES * a.ninst + k], cnt)) {
            const double tot = reduce_parts(a.part + (size_t)a.inst_blk[k] * SUB, (int)cnt, 1, 0, sh);
            if (threadIdx.x == 0) {
                // a true residual that has not dropped since the last update
                // means the FP32 directions have lost conjugacy: restart them
                const double prev = SS(a, S_RRLAST, k);
                II(a, I_RESET, k) = (prev > 0.0 && tot >= prev) ? 1 : 0;
                SS(a, S_RRLAST, k) = tot;
                SS(a, S_RR, k) = tot;
                if (!(tot == tot)) { II(a, I_BAD, k) = 1; finish(a, k, 3); }
                else if (tot <= a.tol * a.tol * SS(a, S_RHS2, k)) finish(a, k, 1);
                else if (II(a, I_ITERS, k) >= a.max_iter) finish(a, k, 2);
                a.t[T_RES * a.ninst + k] = 0;
            }
        }
    }
}

// restart of the listed instances that did not finish: r32 = r64, r.z, beta
__global__ void __launch_bounds__(BBS) kb_restart_w(BArgs a, const double* __restrict__ r64, float* __restrict__ r32,
                                                    const float* __restrict__ dinv) {
    __shared__ double sh[32];
    int k, blk, r0, r1;
    for (int w = blockIdx.x; wl_item(a, w, k, blk, r0, r1); w += gridDim.x) {
        if (II(a, I_DONE, k)) continue;  // decided by the residual kernel, the same for all its items
        double rz = 0.0;
        for (int i = r0 + threadIdx.x; i < r1; i += BBS) {
            const float ri = (float)r64[i];
            r32[i] = ri;
            rz += (double)ri * (double)(dinv[i] * ri);
        }
        const double s1 = block_sum(rz, sh);
        if (threadIdx.x == 0) a.part[(size_t)blk * SUB + (w % SUB)] = s1;
        const unsigned cnt = (unsigned)(a.inst_blk[k + 1] - a.inst_blk[k]) * SUB;
        if (last_of(&a.t[T_SPMV * a.ninst + k], cnt)) {
            const double tot = reduce_parts(a.part + (size_t)a.inst_blk[k] * SUB, (int)cnt, 1, 0, sh);
            if (threadIdx.x == 0) {
                SS(a, S_BETA, k) = II(a, I_RESET, k) ? 0.0 : tot / SS(a, S_ABSOLD, k);
                SS(a, S_ABSNEW, k) = tot;
                II(a, I_UPDATE, k) = 0;
                a.t[T_SPMV * a.ninst + k] = 0;
            }
        }
    }
}

template <typename TV, typename TX>
__global__ void kb_dinv(int n, const int* __restrict__ diag, const TV* __restrict__ val, TX* __restrict__ dinv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const TV d = val[diag[i]];
        dinv[i] = (d != TV(0)) ? TX(1) / (TX)d : TX(1);
    }
}

__global__ void kb_copy(int n, const double* __restrict__ a, double* __restrict__ b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}

__global__ void kb_f2d(int n, const float* __restrict__ a, double* __restrict__ b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = (double)a[i];
}

// sum of squares of v over each row block (grid = the batch's row blocks)
__global__ void __launch_bounds__(BBS) kb_sumsq(BArgs a, const double* __restrict__ v) {
    __shared__ double sh[32];
    const int r0 = a.blk_r0[blockIdx.x], r1 = a.blk_r1[blockIdx.x];
    double s = 0.0;
    for (int i = r0 + threadIdx.x; i < r1; i += BBS) s += v[i] * v[i];
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) a.part[blockIdx.x] = t;
}

// ||v_k|| / N_k per instance (Eigen3::norm of each instance's system): one
// thread per instance adds its row blocks' sums in block order
__global__ void kb_inst_norm(BArgs a, double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.ninst) return;
    const int b0 = a.inst_blk[k], b1 = a.inst_blk[k + 1];
    double s = 0.0;
    for (int b = b0; b < b1; ++b) s += a.part[b];
    const int nk = a.blk_r1[b1 - 1] - a.blk_r0[b0];
    out[k] = nk > 0 ? sqrt(s) / (double)nk : 0.0;
}

// clears the right-hand side of the instances the mask leaves out
__global__ void __launch_bounds__(BBS) kb_mask_rhs(BArgs a, const int* __restrict__ keep, double* __restrict__ b) {
    if (keep[a.blk_inst[blockIdx.x]]) return;
    for (int i = a.blk_r0[blockIdx.x] + threadIdx.x; i < a.blk_r1[blockIdx.x]; i += BBS) b[i] = 0.0;
}

// setDoFsFromSolver / addToDoFsFromSolver restricted to the instances the
// mask keeps (DOF objects of instance k: [inst_dof[k], inst_dof[k+1]))
__global__ void kb_distribute_masked(int64_t ndc, int ncomp, const int32_t* __restrict__ eq,
                                     const uint8_t* __restrict__ status, const double* __restrict__ cval,
                                     const double* __restrict__ x, double* __restrict__ u, int add,
                                     const int* __restrict__ keep, const int* __restrict__ inst_dof, int ninst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ndc; i += (int64_t)gridDim.x * blockDim.x) {
        const int obj = (int)(i / ncomp);
        int lo = 0, hi = ninst;  // largest lo with inst_dof[lo] <= obj
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (inst_dof[mid] <= obj) lo = mid; else hi = mid;
        }
        if (!keep[lo]) continue;
        if (status[i] == 0) u[i] = add ? u[i] + x[eq[i]] : x[eq[i]];
        else u[i] = cval[i];
    }
}

template <typename TV, typename TX>
void launch_kb_spmv(int lpr, unsigned grid, cudaStream_t st, const BArgs& a, const int* rp, const int* ci, const TV* v,
                    const TX* p, TX* q) {
    switch (lpr) {
        case 2: kb_spmv<TV, TX, 2><<<grid, BBS, 0, st>>>(a, rp, ci, v, p, q); break;
        case 4: kb_spmv<TV, TX, 4><<<grid, BBS, 0, st>>>(a, rp, ci, v, p, q); break;
        case 8: kb_spmv<TV, TX, 8><<<grid, BBS, 0, st>>>(a, rp, ci, v, p, q); break;
        case 16: kb_spmv<TV, TX, 16><<<grid, BBS, 0, st>>>(a, rp, ci, v, p, q); break;
        default: kb_spmv<TV, TX, 32><<<grid, BBS, 0, st>>>(a, rp, ci, v, p, q); break;
    }
}

// FP32 SpMV of the batched mixed solve: kind 2..32 CSR lanes per row,
// 100 + U the batched sliced-ELL copy
void launch_kb_spmv32(isl_ctx* c, int kind, unsigned grid, cudaStream_t st, const BArgs& a, const float* p, float* q) {
    const bool s16 = c->ss16 && c->use_scol16;  // 16-bit column offsets
    switch (kind) {
        case 102:
            if (s16) kb_sspmv<2, 8, short><<<grid, BBS, 0, st>>>(a, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col16.p, c->dss_val.p, p, q);
            else kb_sspmv<2, 8, int><<<grid, BBS, 0, st>>>(a, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col.p, c->dss_val.p, p, q);
            break;
        case 104:
            if (s16) kb_sspmv<4, 8, short><<<grid, BBS, 0, st>>>(a, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col16.p, c->dss_val.p, p, q);
            else kb_sspmv<4, 8, int><<<grid, BBS, 0, st>>>(a, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col.p, c->dss_val.p, p, q);
            break;
        case 108:
            if (s16) kb_sspmv<8, 6, short><<<grid, BBS, 0, st>>>(a, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col16.p, c->dss_val.p, p, q);
            else kb_sspmv<8, 6, int><<<grid, BBS, 0, st>>>(a, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col.p, c->dss_val.p, p, q);
            break;
        default: launch_kb_spmv<float, float>(kind, grid, st, a, c->drowptr.p, c->dcolind.p, c->dval32.p, p, q); break;
    }
}

int pick_lpr(isl_ctx* c) {
    const double avg = (double)c->nnz / (double)c->neq;
    int l = 2;
    while (l < 32 && l < avg / 2) l *= 2;
    return l;
}

// block -> (instance, row range) map and per-instance state buffers
int ensure_batch_state(isl_ctx* c) {
    if (c->nbblocks > 0 && (int64_t)c->inst_iters.size() == c->ninst) return ISL_OK;
    std::vector<int32_t> bi, b0, b1, ib(c->ninst + 1, 0);
    for (int64_t k = 0; k < c->ninst; ++k) {
        const int64_t r0 = c->inst_eq_off[k], r1 = c->inst_eq_off[k + 1];
        ib[k] = (int32_t)bi.size();
        if (r1 <= r0) {  // an instance with no active DOF still owns one (empty) block
            bi.push_back((int32_t)k); b0.push_back((int32_t)r0); b1.push_back((int32_t)r0);
            continue;
        }
        for (int64_t r = r0; r < r1; r += ROWS_PER_BLOCK) {
            bi.push_back((int32_t)k);
            b0.push_back((int32_t)r);
            b1.push_back((int32_t)std::min<int64_t>(r + ROWS_PER_BLOCK, r1));
        }
    }
    ib[c->ninst] = (int32_t)bi.size();
    c->nbblocks = (int64_t)bi.size();
    ISL_CHECK_CUDA(c, c->dblk_inst.alloc(bi.size()));
    ISL_CHECK_CUDA(c, c->dblk_row0.alloc(bi.size()));
    ISL_CHECK_CUDA(c, c->dblk_row1.alloc(bi.size()));
    ISL_CHECK_CUDA(c, c->dinst_blk.alloc(ib.size()));
    ISL_CHECK_CUDA(c, c->dbs.alloc((size_t)S_NS * c->ninst));
    ISL_CHECK_CUDA(c, c->dbi.alloc((size_t)I_NI * c->ninst + 1));
    ISL_CHECK_CUDA(c, c->dbt.alloc((size_t)T_NT * c->ninst));
    ISL_CHECK_CUDA(c, c->dbpart.alloc((size_t)SUB * bi.size()));
    ISL_CHECK_CUDA(c, c->dbwl.alloc((size_t)2 * c->ninst + 3));
    ISL_CHECK_CUDA(c, c->dbact.alloc(bi.size() + 1));
    ISL_CHECK_CUDA(c, c->dinst_dof.alloc((size_t)c->ninst + 1));
    ISL_CHECK_CUDA(c, c->dinst_norm.alloc((size_t)c->ninst));
    cudaStream_t st = c->stream;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dblk_inst.p, bi.data(), bi.size() * 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dblk_row0.p, b0.data(), b0.size() * 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dblk_row1.p, b1.data(), b1.size() * 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dinst_blk.p, ib.data(), ib.size() * 4, cudaMemcpyHostToDevice, st));
    std::vector<int32_t> idof(c->ninst + 1);
    for (int64_t k = 0; k <= c->ninst; ++k) idof[k] = (int32_t)c->inst_dof_off[k];
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dinst_dof.p, idof.data(), idof.size() * 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    c->inst_iters.assign(c->ninst, 0);
    c->inst_relres.assign(c->ninst, 0.0);
    return ISL_OK;
}

BArgs batch_args(isl_ctx* c, int64_t max_iter, double tol) {
    const int ni = (int)c->ninst;
    BArgs a;
    a.ninst = ni;
    a.nblk = (int)c->nbblocks;
    a.act = c->dbact.p;
    a.blk_inst = c->dblk_inst.p;
    a.blk_r0 = c->dblk_row0.p;
    a.blk_r1 = c->dblk_row1.p;
    a.inst_blk = c->dinst_blk.p;
    a.s = c->dbs.p;
    a.iv = c->dbi.p;
    a.t = c->dbt.p;
    a.remaining = c->dbi.p + (size_t)I_NI * ni;
    a.part = c->dbpart.p;
    a.wl = c->dbwl.p;
    a.wl_n = c->dbwl.p + ni;
    a.wl_cur = c->dbwl.p + ni + 1;
    a.wl_cum = c->dbwl.p + ni + 2;
    a.max_iter = (int)std::min<int64_t>(max_iter, INT32_MAX - 1);
    a.trig2 = c->ru_drop2;
    a.tol = tol;
    a.blk_s0 = nullptr;
    a.blk_s1 = nullptr;
    return a;
}

}  // namespace

// Average device time of one batched SpMV launch with every instance active
// (the kernel and grid the batched solve uses: FP32 = the autotuned kind of
// the last mixed solve, FP64 = CSR with the solve's lanes per row).
int time_spmv_batched(isl_ctx* c, int precision, int nrep, double* ms) {
    int rc = ensure_batch_state(c);
    if (rc != ISL_OK) return rc;
    const size_t n = (size_t)c->neq;
    if (c->w64.n < 6 * n) ISL_CHECK_CUDA(c, c->w64.alloc(6 * n));
    if (c->w32.n < 6 * n) ISL_CHECK_CUDA(c, c->w32.alloc(6 * n));
    cudaStream_t st = c->stream;
    const int ni = (int)c->ninst;
    BArgs a = batch_args(c, 1, 0.0);
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dbs.p, 0, (size_t)S_NS * ni * 8, st));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dbi.p, 0, ((size_t)I_NI * ni + 1) * 4, st));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dbt.p, 0, (size_t)T_NT * ni * 4, st));
    kb_compact<<<1, 1024, 0, st>>>(a, c->dbact.p);
    const unsigned lgrid = (unsigned)std::min<int64_t>(c->nbblocks, (int64_t)c->sm_count * 8);
    const unsigned sgrid = (unsigned)std::min<int64_t>(c->nbblocks, (int64_t)c->sm_count * 6);
    std::function<void()> launch;
    if (precision == ISL_PREC_FP32) {
        if (!c->have32) ISL_FAIL(c, ISL_ERR_ARG, "no FP32 matrix");
        rc = ensure_ssell(c);
        if (rc != ISL_OK) return rc;
        int kind = c->bspmv32 ? c->bspmv32 : pick_lpr(c);
        if (kind >= 100 && c->bsell_built && c->ss_nslice > 0) {
            a.blk_s0 = c->dblk_s0.p;
            a.blk_s1 = c->dblk_s1.p;
        } else if (kind >= 100) {
            kind = pick_lpr(c);
        }
        float* V = c->w32.p;
        ISL_CHECK_CUDA(c, cudaMemsetAsync(V + 2 * n, 0, n * 4, st));
        const unsigned g = kind >= 100 ? sgrid : lgrid;
        launch = [=] { launch_kb_spmv32(c, kind, g, st, a, V + 2 * n, V + 3 * n); };
    } else {
        if (!c->have64) ISL_FAIL(c, ISL_ERR_ARG, "no FP64 matrix");
        double* W = c->w64.p;
        ISL_CHECK_CUDA(c, cudaMemsetAsync(W + 2 * n, 0, n * 8, st));
        const int lpr = pick_lpr(c);
        launch = [=] { launch_kb_spmv<double, double>(lpr, lgrid, st, a, c->drowptr.p, c->dcolind.p, c->dval64.p, W + 2 * n, W + 3 * n); };
    }
    launch();
    cudaEventRecord(c->ev[2], st);
    for (int r = 0; r < nrep; ++r) launch();
    cudaEventRecord(c->ev[3], st);
    c->launches += nrep + 2;
    ISL_CHECK_CUDA(c, cudaEventSynchronize(c->ev[3]));
    float t = 0.f;
    cudaEventElapsedTime(&t, c->ev[2], c->ev[3]);
    *ms = t / nrep;
    ISL_CHECK_CUDA(c, cudaGetLastError());
    return ISL_OK;
}

// ||v_k|| / N_k of every instance, v = the solution after a solve, else the
// right-hand side (Eigen3::norm, base/solver/Eigen3.hpp:128-138, per
// instance), reduced on the device; out: ninst host doubles.
int inst_norms_device(isl_ctx* c, double* out) {
    int rc = ensure_batch_state(c);
    if (rc != ISL_OK) return rc;
    cudaStream_t st = c->stream;
    BArgs a = batch_args(c, 1, 0.0);
    const double* v = c->solved ? c->dsol.p : c->drhs.p;
    kb_sumsq<<<(unsigned)c->nbblocks, BBS, 0, st>>>(a, v);
    kb_inst_norm<<<(unsigned)((c->ninst + 255) / 256), 256, 0, st>>>(a, c->dinst_norm.p);
    c->launches += 2;
    ISL_CHECK_CUDA(c, cudaGetLastError());
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(out, c->dinst_norm.p, (size_t)c->ninst * 8, cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    return ISL_OK;
}

// distribute restricted to the instances of the mask (isl_batch_set_mask)
int distribute_masked(isl_ctx* c, int add) {
    int rc = ensure_batch_state(c);
    if (rc != ISL_OK) return rc;
    const int64_t ndc = c->ndofobj * c->ncomp;
    kb_distribute_masked<<<(unsigned)c->sm_count * 8, BBS, 0, c->stream>>>(
        ndc, c->ncomp, c->deq.p, c->dstatus.p, c->dcval.p, c->dsol.p, c->du.p, add, c->dinst_mask.p, c->dinst_dof.p,
        (int)c->ninst);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
}

int solve_batched(isl_ctx* c, int method, double tol, int64_t max_iter, int64_t* iters, double* relres) {
    int rc = ensure_batch_state(c);
    if (rc != ISL_OK) return rc;
    const size_t n = (size_t)c->neq;
    if (c->w64.n < 6 * n) ISL_CHECK_CUDA(c, c->w64.alloc(6 * n));
    if (c->w32.n < 6 * n) ISL_CHECK_CUDA(c, c->w32.alloc(6 * n));
    cudaStream_t st = c->stream;
    const unsigned grid = (unsigned)c->nbblocks;
    const int ni = (int)c->ninst;
    BArgs a = batch_args(c, max_iter, tol);
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dbs.p, 0, (size_t)S_NS * ni * 8, st));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dbi.p, 0, ((size_t)I_NI * ni + 1) * 4, st));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dbt.p, 0, (size_t)T_NT * ni * 4, st));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dbwl.p, 0, ((size_t)2 * ni + 3) * 4, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(a.remaining, &ni, 4, cudaMemcpyHostToDevice, st));
    const int lpr = pick_lpr(c);
    const unsigned vg = (unsigned)c->sm_count * 8;
    // the iteration kernels' fixed grids over the listed row blocks: as many
    // CTAs as fit on the GPU at once (never more than the batch's blocks)
    const unsigned lgrid = (unsigned)std::min<int64_t>(c->nbblocks, (int64_t)c->sm_count * 8);
    const unsigned sgrid = (unsigned)std::min<int64_t>(c->nbblocks, (int64_t)c->sm_count * 6);
    const unsigned wgrid = (unsigned)c->sm_count * 4;  // the reliable-update worklist kernels
    const bool mixed = (method == ISL_SOLVE_CG_FP32_IR);
    // FP32 iterations with FP64 reliable updates when the FP64 matrix exists;
    // after an ISL_PREC_FP32 assembly a plain FP32 CG on the iterated residual
    const bool refine = mixed && c->have64;
    if (mixed && !c->have32) ISL_FAIL(c, ISL_ERR_ARG, "batched FP32 solve needs an FP32 matrix");
    if (!mixed && !c->have64) ISL_FAIL(c, ISL_ERR_ARG, "batched FP64 solve needs the FP64 matrix");
    if (c->mask_on) {
        kb_mask_rhs<<<grid, BBS, 0, st>>>(a, c->dinst_mask.p, c->drhs.p);
        c->launches += 1;
    }
    double* W = c->w64.p;
    float* V = c->w32.p;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    if (!mixed) {
        double *x = W, *r = W + n, *p = W + 2 * n, *q = W + 3 * n, *dinv = W + 4 * n;
        kb_dinv<double, double><<<vg, BBS, 0, st>>>((int)n, c->ddiag.p, c->dval64.p, dinv);
        kb_init<double, double><<<grid, BBS, 0, st>>>(a, c->drhs.p, x, r, p, dinv);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        ISL_CHECK_CUDA(c, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        kb_compact<<<1, 1024, 0, st>>>(a, c->dbact.p);
        for (int k = 0; k < BCHUNK; ++k) {
            kb_dir<double><<<lgrid, BBS, 0, st>>>(a, r, dinv, p);
            launch_kb_spmv<double, double>(lpr, lgrid, st, a, c->drowptr.p, c->dcolind.p, c->dval64.p, p, q);
            kb_update<double><<<lgrid, BBS, 0, st>>>(a, x, r, p, q, dinv, 0);
        }
        ISL_CHECK_CUDA(c, cudaStreamEndCapture(st, &graph));
    } else {
        double *x64 = W, *r64 = W + n;
        float *x32 = V, *r32 = V + n, *p32 = V + 2 * n, *q32 = V + 3 * n, *d32 = V + 4 * n;
        if (refine) ISL_CHECK_CUDA(c, cudaMemsetAsync(x64, 0, n * 8, st));
        kb_dinv<float, float><<<vg, BBS, 0, st>>>((int)n, c->ddiag.p, c->dval32.p, d32);
        kb_init<double, float><<<grid, BBS, 0, st>>>(a, c->drhs.p, x32, r32, p32, d32);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        if (!c->bsell_built) {  // the batched sliced-ELL copy, once per pattern
            std::vector<int32_t> b0((size_t)c->nbblocks), b1((size_t)c->nbblocks), s0, s1;
            ISL_CHECK_CUDA(c, cudaMemcpyAsync(b0.data(), c->dblk_row0.p, b0.size() * 4, cudaMemcpyDeviceToHost, st));
            ISL_CHECK_CUDA(c, cudaMemcpyAsync(b1.data(), c->dblk_row1.p, b1.size() * 4, cudaMemcpyDeviceToHost, st));
            ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
            rc = batch_sell_pattern(c, b0, b1, s0, s1);
            if (rc != ISL_OK) return rc;
            if (c->ss_nslice > 0) {
                ISL_CHECK_CUDA(c, c->dblk_s0.alloc(s0.size()));
                ISL_CHECK_CUDA(c, c->dblk_s1.alloc(s1.size()));
                ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dblk_s0.p, s0.data(), s0.size() * 4, cudaMemcpyHostToDevice, st));
                ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dblk_s1.p, s1.data(), s1.size() * 4, cudaMemcpyHostToDevice, st));
                ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
            }
            c->bsell_built = true;
            c->bspmv32 = 0;
        }
        rc = ensure_ssell(c);
        if (rc != ISL_OK) return rc;
        if (c->ss_nslice > 0) {
            a.blk_s0 = c->dblk_s0.p;
            a.blk_s1 = c->dblk_s1.p;
        }
        kb_compact<<<1, 1024, 0, st>>>(a, c->dbact.p);
        c->launches += 1;
        if (c->spmv32_forced > 0 && (c->spmv32_forced < 100 || c->ss_nslice > 0)) {
            c->bspmv32 = c->spmv32_forced;
        } else if (!c->bspmv32) {
            // autotune: each candidate over 5 launches on the freshly started
            // iteration (they only write q and the instances' alpha, which the
            // first iteration recomputes)
            const int cand[4] = {lpr, 102, 104, 108};
            const int ncand = c->ss_nslice > 0 ? 4 : 1;
            int best = lpr, cached = 0;
            if (ncand > 1 && tune_lookup(c, "bspmv_batch", &cached) &&
                (cached == lpr || cached == 102 || cached == 104 || cached == 108))
                c->bspmv32 = cached;
            float bestms = 1e30f;
            for (int k2 = 0; k2 < ncand && ncand > 1 && !c->bspmv32; ++k2) {
                const unsigned g2 = cand[k2] >= 100 ? sgrid : lgrid;
                launch_kb_spmv32(c, cand[k2], g2, st, a, p32, q32);
                cudaEventRecord(c->ev[2], st);
                for (int r = 0; r < 5; ++r) launch_kb_spmv32(c, cand[k2], g2, st, a, p32, q32);
                cudaEventRecord(c->ev[3], st);
                cudaEventSynchronize(c->ev[3]);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
                if (ms < bestms) { bestms = ms; best = cand[k2]; }
            }
            if (!c->bspmv32) {
                c->launches += 6 * ncand;
                c->bspmv32 = best;
                if (ncand > 1) tune_store(c, "bspmv_batch", best);
            }
        }
        c->spmv_lpr32 = c->bspmv32;
        const unsigned g32 = c->bspmv32 >= 100 ? sgrid : lgrid;
        ISL_CHECK_CUDA(c, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        kb_compact<<<1, 1024, 0, st>>>(a, c->dbact.p);
        for (int k = 0; k < BCHUNK; ++k) {
            kb_dir<float><<<lgrid, BBS, 0, st>>>(a, r32, d32, p32);
            launch_kb_spmv32(c, c->bspmv32, g32, st, a, p32, q32);
            kb_update<float><<<lgrid, BBS, 0, st>>>(a, x32, r32, p32, q32, d32, refine ? 1 : 0);
            if (refine) {
                // reliable updates of the instances kb_update listed
                kb_wl_scan<<<1, BBS, 0, st>>>(a);
                kb_fold_w<<<wgrid, BBS, 0, st>>>(a, x32, x64);
                kb_residual_w<<<wgrid, BBS, 0, st>>>(a, c->drowptr.p, c->dcolind.p, c->dval64.p, x64, c->drhs.p, r64);
                kb_restart_w<<<wgrid, BBS, 0, st>>>(a, r64, r32, d32);
            }
        }
        ISL_CHECK_CUDA(c, cudaStreamEndCapture(st, &graph));
    }
    c->launches += 2;
    {
        cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        ISL_CHECK_CUDA(c, e);
    }
    const int per_iter = refine ? 7 : 3;  // plus the list rebuild once per replay
    const int64_t max_replays = (int64_t)a.max_iter / BCHUNK + 8;
    int remaining = ni;
    int64_t replays = 0;
    rc = ISL_OK;
    for (;;) {
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(&remaining, a.remaining, 4, cudaMemcpyDeviceToHost, st));
        ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
        if (remaining <= 0) break;
        if (++replays > max_replays) { rc = ISL_ERR_TIMEOUT; c->err = "batched CG made no progress"; break; }
        if (cudaGraphLaunch(exec, st) != cudaSuccess) { rc = ISL_ERR_CUDA; c->err = "graph launch failed"; break; }
        c->launches += (int64_t)per_iter * BCHUNK + 1;
    }
    cudaGraphExecDestroy(exec);
    if (rc != ISL_OK) return rc;
    if (mixed && !refine) kb_f2d<<<vg, BBS, 0, st>>>((int)n, V, c->dsol.p);  // the FP32 iterate
    else kb_copy<<<vg, BBS, 0, st>>>((int)n, W, c->dsol.p);  // x (plain) or x64 (mixed) both live at W
    c->launches += 1;
    std::vector<int> hi((size_t)I_NI * ni);
    std::vector<double> hs((size_t)S_NS * ni);
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(hi.data(), c->dbi.p, hi.size() * 4, cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(hs.data(), c->dbs.p, hs.size() * 8, cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    int64_t itmax = 0;
    double relmax = 0.0;
    bool nc = false, bad = false;
    for (int k = 0; k < ni; ++k) {
        const int done = hi[(size_t)I_DONE * ni + k];
        c->inst_iters[k] = hi[(size_t)I_ITERS * ni + k];
        const double rhs2 = hs[(size_t)S_RHS2 * ni + k];
        c->inst_relres[k] = rhs2 > 0 ? std::sqrt(hs[(size_t)S_RR * ni + k] / rhs2) : 0.0;
        itmax = std::max<int64_t>(itmax, c->inst_iters[k]);
        relmax = std::max(relmax, c->inst_relres[k]);
        nc |= (done == 2);
        bad |= (done == 3) || hi[(size_t)I_BAD * ni + k];
    }
    if (iters) *iters = itmax;
    if (relres) *relres = relmax;
    c->solved = true;
    if (bad) ISL_FAIL(c, ISL_ERR_NAN, "batched CG breakdown in an instance");
    if (nc) ISL_FAIL(c, ISL_ERR_NOT_CONVERGED, "an instance did not reach the tolerance");
    return ISL_OK;
}

}  // namespace isl
