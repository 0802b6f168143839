// BiCGSTAB for the non-symmetric systems (heat::Static tangents), in FP64.
//
// The recurrences of Eigen 3.2's BiCGSTAB, which the reference's
// Eigen3::biCGStabSolve calls (base/solver/Eigen3.hpp:277-289), after the
// published algorithm (van der Vorst 1992, right-preconditioned form):
//   r = b, r0 = r, rho = alpha = w = 1, v = p = 0                (x0 = 0)
//   loop while |r|^2 > tol^2 |b|^2:
//     rho_old = rho, rho = r0.r     (|rho| < eps^2 |r0|^2: restart with r0 = r)
//     beta = (rho / rho_old) (alpha / w)
//     p = r + beta (p - w v),  y = M^-1 p,  v = A y,  alpha = rho / (r0.v)
//     s = r - alpha v,  z = M^-1 s,  t = A z,  w = (t.s) / (t.t)  (0 if t = 0)
//     x += alpha y + w z,  r = s - w t
// The reference preconditions with IncompleteLUT; here M is the diagonal
// (Jacobi), the preconditioner of the reference's CG.
//
// One iteration is five kernels on the context stream; every scalar lives in
// device memory and is produced by the last block of the kernel that reduces
// it (ticket counter, fixed order), so the iteration needs no host round trip
// and is reproducible bit for bit.  Chunks of iterations are captured in a
// CUDA graph and replayed until the device-side done flag is set.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "isl_device.cuh"
#include "isl_internal.h"

namespace isl {

namespace {

constexpr int KB = 256;
constexpr int BI_CHUNK = 16;

struct BiScal {
    double rho, rho_old, alpha, w, beta, rr, rhs2, r0sq, tol2, eps2;
    int done;      // 1 converged, 2 restart needed, 3 iteration limit
    int iters, maxit, bad;
    unsigned ticket;
};

// y = dinv p after p = r + beta (p - w v)
__global__ void __launch_bounds__(KB) k_bi_dir(int n, const double* __restrict__ r, const double* __restrict__ v,
                                               const double* __restrict__ dinv, double* __restrict__ p,
                                               double* __restrict__ y, const BiScal* S) {
    if (S->done) return;
    const double beta = S->beta, w = S->w;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double pi = r[i] + beta * (p[i] - w * v[i]);
        p[i] = pi;
        y[i] = dinv[i] * pi;
    }
}

// s = r - alpha v, z = dinv s
__global__ void __launch_bounds__(KB) k_bi_s(int n, const double* __restrict__ r, const double* __restrict__ v,
                                             const double* __restrict__ dinv, double* __restrict__ s_,
                                             double* __restrict__ z, const BiScal* S) {
    if (S->done) return;
    const double alpha = S->alpha;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double si = r[i] - alpha * v[i];
        s_[i] = si;
        z[i] = dinv[i] * si;
    }
}

// out = A in, with the row products d1 = a.out (a = null: out.out) and
// d2 = b.out; the last block turns them into alpha (mode 0: rho / r0.v) or
// w (mode 1: (t.s) / (t.t))
template <int LPR>
__global__ void __launch_bounds__(KB) k_bi_spmv(int n, const int* __restrict__ rowptr, const int* __restrict__ colind,
                                                const double* __restrict__ val, const double* __restrict__ in,
                                                double* __restrict__ out, const double* __restrict__ a,
                                                const double* __restrict__ b, int mode, BiScal* S, double* part) {
    if (S->done) return;
    __shared__ double sh[32];
    const int lane = threadIdx.x % LPR;
    const int grp = (blockIdx.x * KB + threadIdx.x) / LPR, ngrp = gridDim.x * KB / LPR;
    const int wgrp = grp - grp % (32 / LPR);
    double d1 = 0.0, d2 = 0.0;
    for (int base = wgrp; base < n; base += ngrp) {
        const int row = base + (grp - wgrp);
        const bool act = row < n;
        const double acc = row_dot<double, double, LPR>(row, act, rowptr, colind, val, in, lane);
        if (act && lane == 0) {
            out[row] = acc;
            d1 += (a ? a[row] : acc) * acc;
            if (b) d2 += b[row] * acc;
        }
    }
    const double b1 = block_sum(d1, sh);
    const double b2 = block_sum(d2, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = b1; part[2 * blockIdx.x + 1] = b2; }
    if (last_block(&S->ticket)) {
        double t1, t2;
        reduce_parts2_blk<KB>(part, gridDim.x, sh, t1, t2);
        if (threadIdx.x == 0) {
            if (mode == 0) {
                S->alpha = S->rho / t1;
                if (!(S->alpha == S->alpha) || isinf(S->alpha)) { S->bad = 1; S->done = 1; }
            } else {
                S->w = t1 > 0.0 ? t2 / t1 : 0.0;
            }
            S->ticket = 0;
        }
    }
}

// The same product on the scalar sliced-ELL copy (rows length-sorted within
// windows of 2048, one lane per row, slots column-major) with FP64 values: the
// loads of U slots are issued before their gathers, so each lane keeps 12U
// bytes of the stream in flight.
template <int U, int MINB>
__global__ void __launch_bounds__(KB, MINB) k_bi_sspmv(int nslice, const int* __restrict__ soff, const int* __restrict__ swid,
                                                    const int* __restrict__ srow, const int* __restrict__ scol,
                                                    const double* __restrict__ sv, const double* __restrict__ in,
                                                    double* __restrict__ out, const double* __restrict__ a,
                                                    const double* __restrict__ b, int mode, BiScal* S, double* part) {
    if (S->done) return;
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * KB + threadIdx.x) >> 5, nwarps = gridDim.x * (KB / 32);
    double d1 = 0.0, d2 = 0.0;
    for (int s = warp; s < nslice; s += nwarps) {
        const int o = soff[s] + lane, w = swid[s];
        double acc = 0.0;
        for (int k = 0; k < w; k += U) {
            int j[U];
            double v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (k + u < w) {
                    j[u] = ld_stream(scol + o + (k + u) * 32);
                    v[u] = __ldcs(sv + o + (k + u) * 32);
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (k + u < w) acc += v[u] * __ldg(in + j[u]);
        }
        const int row = srow[s * 32 + lane];
        if (row >= 0) {
            out[row] = acc;
            d1 += (a ? a[row] : acc) * acc;
            if (b) d2 += b[row] * acc;
        }
    }
    const double b1 = block_sum(d1, sh);
    const double b2 = block_sum(d2, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = b1; part[2 * blockIdx.x + 1] = b2; }
    if (last_block(&S->ticket)) {
        double t1, t2;
        reduce_parts2_blk<KB>(part, gridDim.x, sh, t1, t2);
        if (threadIdx.x == 0) {
            if (mode == 0) {
                S->alpha = S->rho / t1;
                if (!(S->alpha == S->alpha) || isinf(S->alpha)) { S->bad = 1; S->done = 1; }
            } else {
                S->w = t1 > 0.0 ? t2 / t1 : 0.0;
            }
            S->ticket = 0;
        }
    }
}

// FP64 values into the sliced-ELL slots (padding slots stay zero)
__global__ void k_ssell_values64(int n, const int* __restrict__ rowptr, const int* __restrict__ spos,
                                 const double* __restrict__ val, double* __restrict__ sv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int lo = rowptr[i], hi = rowptr[i + 1], s0 = spos[i];
        for (int k = lo; k < hi; ++k) sv[s0 + (k - lo) * 32] = val[k];
    }
}

// x += alpha y + w z, r = s - w t; r.r and r0.r; the last block: convergence,
// the next rho and beta, or a restart request
__global__ void __launch_bounds__(KB) k_bi_update(int n, double* __restrict__ x, double* __restrict__ r,
                                                  const double* __restrict__ r0, const double* __restrict__ y,
                                                  const double* __restrict__ z, const double* __restrict__ s_,
                                                  const double* __restrict__ t, BiScal* S, double* part) {
    if (S->done) return;
    __shared__ double sh[32];
    const double alpha = S->alpha, w = S->w;
    double rr = 0.0, r0r = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * y[i] + w * z[i];
        const double ri = s_[i] - w * t[i];
        r[i] = ri;
        rr += ri * ri;
        r0r += r0[i] * ri;
    }
    const double b1 = block_sum(rr, sh);
    const double b2 = block_sum(r0r, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = b1; part[2 * blockIdx.x + 1] = b2; }
    if (last_block(&S->ticket)) {
        double trr, trho;
        reduce_parts2_blk<KB>(part, gridDim.x, sh, trr, trho);
        if (threadIdx.x == 0) {
            S->rr = trr;
            S->iters += 1;
            if (!(trr == trr)) { S->bad = 1; S->done = 1; }
            else if (trr <= S->tol2) S->done = 1;
            else if (S->iters >= S->maxit) S->done = 3;
            else if (fabs(trho) < S->eps2 * S->r0sq) S->done = 2;
            else {
                S->rho_old = S->rho;
                S->rho = trho;
                S->beta = (S->rho / S->rho_old) * (S->alpha / S->w);
                if (!(S->beta == S->beta) || isinf(S->beta)) { S->bad = 1; S->done = 1; }
            }
            S->ticket = 0;
        }
    }
}

// start (x = 0, r = r0 = b) or restart (r = b - A x, r0 = r): |r|^2, rho
template <int LPR>
__global__ void __launch_bounds__(KB) k_bi_start(int n, const int* __restrict__ rowptr, const int* __restrict__ colind,
                                                 const double* __restrict__ val, const double* __restrict__ bvec,
                                                 const double* __restrict__ x, double* __restrict__ r,
                                                 double* __restrict__ r0, double* __restrict__ p,
                                                 double* __restrict__ v, int restart, BiScal* S, double* part) {
    __shared__ double sh[32];
    const int lane = threadIdx.x % LPR;
    const int grp = (blockIdx.x * KB + threadIdx.x) / LPR, ngrp = gridDim.x * KB / LPR;
    const int wgrp = grp - grp % (32 / LPR);
    double rr = 0.0, bb = 0.0;
    for (int base = wgrp; base < n; base += ngrp) {
        const int row = base + (grp - wgrp);
        const bool act = row < n;
        const double ax = restart ? row_dot<double, double, LPR>(row, act, rowptr, colind, val, x, lane) : 0.0;
        if (act && lane == 0) {
            const double ri = bvec[row] - ax;
            r[row] = ri;
            r0[row] = ri;
            p[row] = 0.0;
            v[row] = 0.0;
            rr += ri * ri;
            bb += bvec[row] * bvec[row];
        }
    }
    const double b1 = block_sum(rr, sh);
    const double b2 = block_sum(bb, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = b1; part[2 * blockIdx.x + 1] = b2; }
    if (last_block(&S->ticket)) {
        double trr, tbb;
        reduce_parts2_blk<KB>(part, gridDim.x, sh, trr, tbb);
        if (threadIdx.x == 0) {
            if (!restart) {
                S->rhs2 = tbb;
                S->iters = 0;
            }
            S->rr = trr;
            S->r0sq = trr;
            S->rho = trr;
            S->rho_old = 1.0;
            S->alpha = 1.0;
            S->w = 1.0;
            S->beta = 0.0;  // p = r on the first pass after a (re)start
            S->done = (trr <= S->tol2 || tbb == 0.0) ? 1 : 0;
            S->ticket = 0;
        }
    }
}

__global__ void k_bi_dinv(int n, const int* __restrict__ diag, const double* __restrict__ val, double* __restrict__ dinv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double d = val[diag[i]];
        dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
    }
}

__global__ void k_bi_zero(int n, double* __restrict__ x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = 0.0;
}

// the SpMV of BiCGSTAB: kind 2..16 = CSR with that many lanes per row,
// 100 + U = the sliced-ELL copy with U slots in flight
void launch_bi_spmv(const isl_ctx* c, int kind, unsigned grid, const double* in, double* out, const double* a,
                    const double* b, int mode, BiScal* S, double* part) {
    cudaStream_t st = c->stream;
    const int n = (int)c->neq;
    const int* rp = c->drowptr.p;
    const int* ci = c->dcolind.p;
    const double* val = c->dval64.p;
    auto gs = [&](long long per_sm) {
        return (unsigned)std::max<long long>(1, std::min<long long>((c->ss_nslice + 7) / 8, per_sm * c->sm_count));
    };
    switch (kind) {
        case 2: k_bi_spmv<2><<<grid, KB, 0, st>>>(n, rp, ci, val, in, out, a, b, mode, S, part); break;
        case 4: k_bi_spmv<4><<<grid, KB, 0, st>>>(n, rp, ci, val, in, out, a, b, mode, S, part); break;
        case 8: k_bi_spmv<8><<<grid, KB, 0, st>>>(n, rp, ci, val, in, out, a, b, mode, S, part); break;
        case 16: k_bi_spmv<16><<<grid, KB, 0, st>>>(n, rp, ci, val, in, out, a, b, mode, S, part); break;
        case 102: k_bi_sspmv<2, 6><<<gs(6), KB, 0, st>>>((int)c->ss_nslice, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col.p, c->dss_val64.p, in, out, a, b, mode, S, part); break;
        case 104: k_bi_sspmv<4, 6><<<gs(6), KB, 0, st>>>((int)c->ss_nslice, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col.p, c->dss_val64.p, in, out, a, b, mode, S, part); break;
        default: k_bi_sspmv<8, 4><<<gs(4), KB, 0, st>>>((int)c->ss_nslice, c->dss_off.p, c->dss_wid.p, c->dss_row.p, c->dss_col.p, c->dss_val64.p, in, out, a, b, mode, S, part); break;
    }
}

void launch_iter(cudaStream_t st, unsigned grid, int n, const isl_ctx* c, int kind, double* const* V, BiScal* S,
                 double* part) {
    double *x = V[0], *r = V[1], *r0 = V[2], *p = V[3], *v = V[4], *y = V[5], *s_ = V[6], *z = V[7], *t = V[8],
           *dinv = V[9];
    k_bi_dir<<<grid, KB, 0, st>>>(n, r, v, dinv, p, y, S);
    launch_bi_spmv(c, kind, grid, y, v, r0, nullptr, 0, S, part);
    k_bi_s<<<grid, KB, 0, st>>>(n, r, v, dinv, s_, z, S);
    launch_bi_spmv(c, kind, grid, z, t, nullptr, s_, 1, S, part);
    k_bi_update<<<grid, KB, 0, st>>>(n, x, r, r0, y, z, s_, t, S, part);
}

int run_bicgstab(isl_ctx* c, int kind, double tol, int64_t max_iter, int64_t* iters, double* rel, bool* nc) {
    cudaStream_t st = c->stream;
    const int n = (int)c->neq;
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>((n + KB - 1) / KB, 4LL * c->sm_count));
    if (c->wbi.n < (size_t)10 * n) ISL_CHECK_CUDA(c, c->wbi.alloc((size_t)10 * n));
    if (c->dbis.n < 16) ISL_CHECK_CUDA(c, c->dbis.alloc(16));
    static_assert(sizeof(BiScal) <= 16 * sizeof(double), "BiCGSTAB scalars exceed their buffer");
    BiScal* S = reinterpret_cast<BiScal*>(c->dbis.p);
    double* part = c->dpart.p;
    double* V[10];
    for (int k = 0; k < 10; ++k) V[k] = c->wbi.p + (size_t)k * n;
    BiScal h;
    std::memset(&h, 0, sizeof h);
    h.tol2 = tol * tol;  // scaled by |b|^2 once the start kernel has it
    h.eps2 = 2.220446049250313e-16 * 2.220446049250313e-16;
    h.maxit = (int)std::min<int64_t>(max_iter, INT32_MAX - 1);
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(S, &h, sizeof h, cudaMemcpyHostToDevice, st));
    k_bi_dinv<<<grid, KB, 0, st>>>(n, c->ddiag.p, c->dval64.p, V[9]);
    k_bi_zero<<<grid, KB, 0, st>>>(n, V[0]);
    // |b|^2 first, then the start with the absolute threshold tol^2 |b|^2
    k_bi_start<4><<<grid, KB, 0, st>>>(n, c->drowptr.p, c->dcolind.p, c->dval64.p, c->drhs.p, V[0], V[1], V[2], V[3],
                                       V[4], 0, S, part);
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(&h, S, sizeof h, cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    c->launches += 3;
    const double rhs2 = h.rhs2;
    h.tol2 = tol * tol * rhs2;
    h.done = (h.rr <= h.tol2 || rhs2 == 0.0) ? 1 : 0;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(S, &h, sizeof h, cudaMemcpyHostToDevice, st));
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    ISL_CHECK_CUDA(c, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < BI_CHUNK; ++k) launch_iter(st, grid, n, c, kind, V, S, part);
    ISL_CHECK_CUDA(c, cudaStreamEndCapture(st, &graph));
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    ISL_CHECK_CUDA(c, e);
    int rc = ISL_OK;
    const int64_t max_replays = h.maxit / BI_CHUNK + 64;
    int restarts = 0;
    for (int64_t rep = 0; rc == ISL_OK && !h.done; ++rep) {
        if (rep > max_replays + 8 * restarts) { rc = ISL_ERR_TIMEOUT; c->err = "BiCGSTAB made no progress"; break; }
        if (cudaGraphLaunch(exec, st) != cudaSuccess) { rc = ISL_ERR_CUDA; c->err = "graph launch failed"; break; }
        c->launches += 5 * BI_CHUNK;
        if (cudaMemcpyAsync(&h, S, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) { rc = ISL_ERR_CUDA; c->err = "BiCGSTAB scalars"; break; }
        if (h.bad) { rc = ISL_ERR_NAN; c->err = "BiCGSTAB breakdown (non-finite scalar)"; break; }
        if (h.done == 2) {  // r0.r vanished: restart from the true residual
            ++restarts;
            k_bi_start<4><<<grid, KB, 0, st>>>(n, c->drowptr.p, c->dcolind.p, c->dval64.p, c->drhs.p, V[0], V[1],
                                               V[2], V[3], V[4], 1, S, part);
            c->launches += 1;
            if (cudaMemcpyAsync(&h, S, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) { rc = ISL_ERR_CUDA; c->err = "BiCGSTAB scalars"; break; }
        }
    }
    cudaGraphExecDestroy(exec);
    if (rc != ISL_OK) return rc;
    *iters = h.iters;
    *rel = rhs2 > 0.0 ? std::sqrt(h.rr / rhs2) : 0.0;
    *nc = (h.done == 3);
    ISL_CHECK_CUDA(c, c->dsol.alloc(n));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dsol.p, V[0], (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    return ISL_OK;
}

// time the SpMV candidates on the current matrix (20 launches each, CUDA
// events): CSR with 2, 4, 8, 16 lanes per row and, where the sliced-ELL copy
// exists, its batch depths 2, 4, 8; keep the fastest
int tune_kind(isl_ctx* c) {
    const int n = (int)c->neq;
    if (n < 20000) {
        const double avg = (double)c->nnz / (double)std::max<int64_t>(1, c->neq);
        int lpr = 2;
        while (lpr < 16 && lpr < avg / 4) lpr *= 2;
        return lpr;
    }
    int cached = 0;
    if (tune_lookup(c, "bicg", &cached) && cached != 0 && bicgstab_kind_valid(c, cached)) return cached;
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>((n + KB - 1) / KB, 4LL * c->sm_count));
    if (c->wbi.n < (size_t)10 * n && c->wbi.alloc((size_t)10 * n) != cudaSuccess) return 4;
    if (c->dbis.n < 16 && c->dbis.alloc(16) != cudaSuccess) return 4;
    BiScal* S = reinterpret_cast<BiScal*>(c->dbis.p);
    cudaMemsetAsync(S, 0, sizeof(BiScal), c->stream);
    cudaMemsetAsync(c->wbi.p, 0, (size_t)n * 8, c->stream);
    const double* in = c->wbi.p;
    double* out = c->wbi.p + n;
    const int cand[7] = {2, 4, 8, 16, 102, 104, 108};
    const int ncand = c->ss_nslice > 0 ? 7 : 4;
    int best = 4;
    float bestms = 1e30f;
    for (int k = 0; k < ncand; ++k) {
        launch_bi_spmv(c, cand[k], grid, in, out, nullptr, nullptr, 1, S, c->dpart.p);
        cudaEventRecord(c->ev[2], c->stream);
        for (int r = 0; r < 20; ++r) launch_bi_spmv(c, cand[k], grid, in, out, nullptr, nullptr, 1, S, c->dpart.p);
        cudaEventRecord(c->ev[3], c->stream);
        cudaEventSynchronize(c->ev[3]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
        if (ms < bestms) { bestms = ms; best = cand[k]; }
    }
    c->launches += 21 * ncand;
    tune_store(c, "bicg", best);
    return best;
}

}  // namespace

bool bicgstab_kind_valid(const isl_ctx* c, int kind) {
    if (kind == 0 || kind == 2 || kind == 4 || kind == 8 || kind == 16) return true;
    return (kind == 102 || kind == 104 || kind == 108) && c->ss_nslice > 0;
}

int solve_bicgstab(isl_ctx* c, double tol, int64_t max_iter, int64_t* iters, double* rel, bool* nc) {
    if (c->ss_nslice > 0 && c->ss_serial64 != c->asm_serial) {  // FP64 values of the sliced-ELL copy
        ISL_CHECK_CUDA(c, c->dss_val64.alloc(c->ss_nslot));
        if (c->ss_val64_pattern != c->pattern_serial) {
            ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dss_val64.p, 0, (size_t)c->ss_nslot * 8, c->stream));
            c->ss_val64_pattern = c->pattern_serial;
        }
        k_ssell_values64<<<(unsigned)c->sm_count * 8, KB, 0, c->stream>>>((int)c->neq, c->drowptr.p, c->dss_pos.p,
                                                                           c->dval64.p, c->dss_val64.p);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        c->launches += 1;
        c->ss_serial64 = c->asm_serial;
    }
    if (c->bicg_forced && bicgstab_kind_valid(c, c->bicg_forced)) {
        c->bicg_lpr = c->bicg_forced;
    } else if (!c->bicg_lpr || c->bicg_serial != c->pattern_serial) {
        c->bicg_lpr = tune_kind(c);
        c->bicg_serial = c->pattern_serial;
    }
    return run_bicgstab(c, c->bicg_lpr, tol, max_iter, iters, rel, nc);
}

}  // namespace isl
