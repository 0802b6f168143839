// Krylov solve of the assembled system on the GB300.
//
// Jacobi-preconditioned CG with the semantics of Eigen 3.2's
// ConjugateGradient<SparseMatrix<double>> as the reference calls it
// (base/solver/Eigen3.hpp:265-275): x0 = 0, z = D^{-1} r, stop when
// ||r||^2 < tol^2 ||b||^2 or after max_iter iterations.
//
// One iteration = three kernels, all on the context stream:
//   k_spmv_pap : q = A p and p.q             (last block: alpha)
//   k_cg_update: x += alpha p, r -= alpha q,  r.r and r.D^{-1}r
//                                            (last block: convergence, beta)
//   k_cg_dir   : p = D^{-1} r + beta p
// Block partial sums are reduced by the last block to finish (a ticket
// counter, not an atomic on the data), in a fixed order, so results are
// bit-reproducible.  Iterations are captured into a CUDA graph of CHUNK
// iterations that is replayed until the device-side done flag is set.
//
// The mixed method runs the same kernels in FP32 (dot products accumulated in
// FP64) inside FP64 iterative refinement: r64 = b - A64 x64 in FP64, inner
// FP32 CG on A32 d = r64/||r64||, x64 += ||r64|| d.
#include <cmath>
#include <vector>

#include "isl_internal.h"

namespace isl {

constexpr int BS = 256;
constexpr int CHUNK = 32;

template <typename T>
__device__ inline T ld(const T* p) { return __ldg(p); }

// fixed-order block reduction of a double (deterministic)
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
    return t;  // valid in thread 0
}

// the last block to arrive reduces part[0..gridDim.x) for each of nv values
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

__device__ inline double reduce_parts(const double* part, int n, int stride, int off, double* sh) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(part + (size_t)i * stride + off);
    return block_sum(s, sh);
}

template <typename TV, typename TX, int LPR>
__device__ inline TX row_dot(int row, const int* __restrict__ rowptr, const int* __restrict__ colind,
                             const TV* __restrict__ val, const TX* __restrict__ p, int lane) {
    TX acc = TX(0);
    const int lo = rowptr[row], hi = rowptr[row + 1];
    for (int k = lo + lane; k < hi; k += LPR) acc += (TX)ld(val + k) * ld(p + ld(colind + k));
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, LPR);
    return acc;
}

// q = A p; partial p.q; last block computes alpha = absNew / p.q
template <typename TV, typename TX, int LPR>
__global__ void __launch_bounds__(BS) k_spmv_pap(int n, const int* __restrict__ rowptr, const int* __restrict__ colind,
                                                 const TV* __restrict__ val, const TX* __restrict__ p, TX* __restrict__ q,
                                                 CGScal* S, double* part) {
    if (S->done) return;
    __shared__ double sh[32];
    const int lane = threadIdx.x % LPR;
    const int grp = (blockIdx.x * BS + threadIdx.x) / LPR, ngrp = gridDim.x * BS / LPR;
    double loc = 0.0;
    for (int row = grp; row < n; row += ngrp) {
        const TX acc = row_dot<TV, TX, LPR>(row, rowptr, colind, val, p, lane);
        if (lane == 0) {
            q[row] = acc;
            loc += (double)(p[row] * acc);
        }
    }
    const double bs = block_sum(loc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (last_block(&S->ticket1)) {
        const double tot = reduce_parts(part, gridDim.x, 1, 0, sh);
        if (threadIdx.x == 0) {
            S->pAp = tot;
            S->alpha = S->absNew / tot;
            S->ticket1 = 0;
        }
    }
}

// x += alpha p; r -= alpha q; partial r.r, r.z; last block: convergence + beta
template <typename TX>
__global__ void __launch_bounds__(BS) k_cg_update(int n, TX* __restrict__ x, TX* __restrict__ r, const TX* __restrict__ p,
                                                  const TX* __restrict__ q, const TX* __restrict__ dinv, CGScal* S,
                                                  double* part, int max_iter) {
    if (S->done) return;
    __shared__ double sh[32];
    const TX alpha = (TX)S->alpha;
    TX rr = TX(0), rz = TX(0);
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
        x[i] += alpha * p[i];
        const TX ri = r[i] - alpha * q[i];
        r[i] = ri;
        rr += ri * ri;
        rz += ri * (dinv[i] * ri);
    }
    const double b1 = block_sum((double)rr, sh);
    const double b2 = block_sum((double)rz, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = b1; part[2 * blockIdx.x + 1] = b2; }
    if (last_block(&S->ticket2)) {
        const double trr = reduce_parts(part, gridDim.x, 2, 0, sh);
        const double trz = reduce_parts(part, gridDim.x, 2, 1, sh);
        if (threadIdx.x == 0) {
            S->rr = trr;
            S->iters += 1;
            if (!(trr == trr) || !(trz == trz)) { S->bad = 1; S->done = 1; }
            else if (trr < S->threshold) S->done = 1;
            else if (S->iters >= max_iter) S->done = 2;
            else {
                S->beta = trz / S->absNew;
                S->absNew = trz;
            }
            S->ticket2 = 0;
        }
    }
}

template <typename TX>
__global__ void __launch_bounds__(BS) k_cg_dir(int n, const TX* __restrict__ r, const TX* __restrict__ dinv, TX* __restrict__ p,
                                               const CGScal* S) {
    if (S->done) return;
    const TX beta = (TX)S->beta;
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) p[i] = dinv[i] * r[i] + beta * p[i];
}

// setup: x = 0, r = b, p = D^{-1} b, absNew = r.p, rhsNorm2 = b.b
template <typename TX>
__global__ void __launch_bounds__(BS) k_cg_init(int n, const TX* __restrict__ b, TX* __restrict__ x, TX* __restrict__ r,
                                                TX* __restrict__ p, const TX* __restrict__ dinv, CGScal* S, double* part, double tol) {
    __shared__ double sh[32];
    double bb = 0.0, bz = 0.0;
    for (int i = blockIdx.x * BS + threadIdx.x; i < n; i += gridDim.x * BS) {
        const TX bi = b[i];
        x[i] = TX(0);
        r[i] = bi;
        const TX zi = dinv[i] * bi;
        p[i] = zi;
        bb += (double)bi * (double)bi;
        bz += (double)bi * (double)zi;
    }
    const double b1 = block_sum(bb, sh);
    const double b2 = block_sum(bz, sh);
    if (threadIdx.x == 0) { part[2 * blockIdx.x] = b1; part[2 * blockIdx.x + 1] = b2; }
    if (last_block(&S->ticket2)) {
        const double tbb = reduce_parts(part, gridDim.x, 2, 0, sh);
        const double tbz = reduce_parts(part, gridDim.x, 2, 1, sh);
        if (threadIdx.x == 0) {
            S->rhsNorm2 = tbb;
            S->threshold = tol * tol * tbb;
            S->absNew = tbz;
            S->rr = tbb;
            S->iters = 0;
            S->bad = !(tbb == tbb);
            S->done = (tbb == 0.0 || tbb < S->threshold || S->bad) ? 1 : 0;
            S->ticket1 = 0;
            S->ticket2 = 0;
        }
    }
}

template <typename TV, typename TX>
__global__ void k_dinv(int n, const int* __restrict__ diag, const TV* __restrict__ val, TX* __restrict__ dinv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const TV d = val[diag[i]];
        dinv[i] = (d != TV(0)) ? TX(1) / (TX)d : TX(1);
    }
}

// r64 = b - A64 x64 ; partial ||r||^2
template <int LPR>
__global__ void __launch_bounds__(BS) k_residual64(int n, const int* __restrict__ rowptr, const int* __restrict__ colind,
                                                   const double* __restrict__ val, const double* __restrict__ x,
                                                   const double* __restrict__ b, double* __restrict__ r, double* part,
                                                   unsigned int* ticket, double* out) {
    __shared__ double sh[32];
    const int lane = threadIdx.x % LPR;
    const int grp = (blockIdx.x * BS + threadIdx.x) / LPR, ngrp = gridDim.x * BS / LPR;
    double loc = 0.0;
    for (int row = grp; row < n; row += ngrp) {
        const double ax = row_dot<double, double, LPR>(row, rowptr, colind, val, x, lane);
        if (lane == 0) {
            const double ri = b[row] - ax;
            r[row] = ri;
            loc += ri * ri;
        }
    }
    const double bs = block_sum(loc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (last_block(ticket)) {
        const double tot = reduce_parts(part, gridDim.x, 1, 0, sh);
        if (threadIdx.x == 0) { *out = tot; *ticket = 0; }
    }
}

__global__ void k_scale_to32(int n, const double* __restrict__ r, double s, float* __restrict__ r32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) r32[i] = (float)(r[i] * s);
}

__global__ void k_axpy32to64(int n, double a, const float* __restrict__ d, double* __restrict__ x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += a * (double)d[i];
}

__global__ void k_copy64(int n, const double* __restrict__ a, double* __restrict__ b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}

// ---------------------------------------------------------------------------
struct Launch {
    unsigned grid;
};

static unsigned vec_grid(isl_ctx* c) { return (unsigned)c->sm_count * (2048 / BS); }

template <typename TV, typename TX>
static void launch_spmv(int lpr, unsigned grid, cudaStream_t st, int n, const int* rp, const int* ci, const TV* v, const TX* p,
                        TX* q, CGScal* S, double* part) {
    switch (lpr) {
        case 2: k_spmv_pap<TV, TX, 2><<<grid, BS, 0, st>>>(n, rp, ci, v, p, q, S, part); break;
        case 4: k_spmv_pap<TV, TX, 4><<<grid, BS, 0, st>>>(n, rp, ci, v, p, q, S, part); break;
        case 8: k_spmv_pap<TV, TX, 8><<<grid, BS, 0, st>>>(n, rp, ci, v, p, q, S, part); break;
        case 16: k_spmv_pap<TV, TX, 16><<<grid, BS, 0, st>>>(n, rp, ci, v, p, q, S, part); break;
        default: k_spmv_pap<TV, TX, 32><<<grid, BS, 0, st>>>(n, rp, ci, v, p, q, S, part); break;
    }
}

static void launch_residual(int lpr, unsigned grid, cudaStream_t st, int n, const int* rp, const int* ci, const double* v,
                            const double* x, const double* b, double* r, double* part, unsigned* ticket, double* out) {
    switch (lpr) {
        case 2: k_residual64<2><<<grid, BS, 0, st>>>(n, rp, ci, v, x, b, r, part, ticket, out); break;
        case 4: k_residual64<4><<<grid, BS, 0, st>>>(n, rp, ci, v, x, b, r, part, ticket, out); break;
        case 8: k_residual64<8><<<grid, BS, 0, st>>>(n, rp, ci, v, x, b, r, part, ticket, out); break;
        case 16: k_residual64<16><<<grid, BS, 0, st>>>(n, rp, ci, v, x, b, r, part, ticket, out); break;
        default: k_residual64<32><<<grid, BS, 0, st>>>(n, rp, ci, v, x, b, r, part, ticket, out); break;
    }
}

// Autotune of the SpMV row mapping (lanes per row): time each candidate on the
// current matrix, keep the fastest.  Chosen once per context and precision.
template <typename TV, typename TX>
static int autotune_lpr(isl_ctx* c, const TV* val, const TX* p, TX* q, CGScal* S, double* part) {
    const double avg = (double)c->nnz / (double)c->neq;
    int best = 2;
    while (best < 32 && best < avg / 2) best *= 2;
    if (c->neq < 20000) return best;  // too small to time meaningfully
    const int cand[4] = {4, 8, 16, 32};
    float bestms = 1e30f;
    cudaMemsetAsync(S, 0, sizeof(CGScal), c->stream);
    for (int k = 0; k < 4; ++k) {
        const int lpr = cand[k];
        launch_spmv<TV, TX>(lpr, vec_grid(c), c->stream, (int)c->neq, c->drowptr.p, c->dcolind.p, val, p, q, S, part);
        cudaEventRecord(c->ev[2], c->stream);
        for (int r = 0; r < 5; ++r)
            launch_spmv<TV, TX>(lpr, vec_grid(c), c->stream, (int)c->neq, c->drowptr.p, c->dcolind.p, val, p, q, S, part);
        cudaEventRecord(c->ev[3], c->stream);
        cudaEventSynchronize(c->ev[3]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
        if (ms < bestms) { bestms = ms; best = lpr; }
    }
    return best;
}

// Run CG on (val, b) of type TV/TX with workspace vectors; returns status.
template <typename TV, typename TX>
static int run_cg(isl_ctx* c, const TV* val, const TX* b, TX* x, TX* r, TX* p, TX* q, TX* dinv, double tol, int64_t max_iter,
                  int lpr, int64_t* iters, double* rr_out, double* rhs2_out, bool* not_converged) {
    cudaStream_t st = c->stream;
    const int n = (int)c->neq;
    CGScal* S = c->dscal.p;
    double* part = c->dpart.p;
    const unsigned grid = vec_grid(c);
    const int mi = (int)std::min<int64_t>(max_iter, INT32_MAX - 1);
    k_dinv<TV, TX><<<grid, BS, 0, st>>>(n, c->ddiag.p, val, dinv);
    ISL_CHECK_CUDA(c, cudaMemsetAsync(S, 0, sizeof(CGScal), st));
    k_cg_init<TX><<<grid, BS, 0, st>>>(n, b, x, r, p, dinv, S, part, tol);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    // capture one chunk of iterations
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    ISL_CHECK_CUDA(c, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < CHUNK; ++k) {
        launch_spmv<TV, TX>(lpr, grid, st, n, c->drowptr.p, c->dcolind.p, val, p, q, S, part);
        k_cg_update<TX><<<grid, BS, 0, st>>>(n, x, r, p, q, dinv, S, part, mi);
        k_cg_dir<TX><<<grid, BS, 0, st>>>(n, r, dinv, p, S);
    }
    ISL_CHECK_CUDA(c, cudaStreamEndCapture(st, &graph));
    ISL_CHECK_CUDA(c, cudaGraphInstantiate(&exec, graph, 0));
    int rc = ISL_OK;
    for (;;) {
        ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->hscal, S, sizeof(CGScal), cudaMemcpyDeviceToHost, st));
        ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
        if (c->hscal->done) break;
        if (cudaGraphLaunch(exec, st) != cudaSuccess) { rc = ISL_ERR_CUDA; break; }
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (rc != ISL_OK) ISL_FAIL(c, rc, "graph launch failed");
    const CGScal& h = *c->hscal;
    if (iters) *iters = h.iters;
    if (rr_out) *rr_out = h.rr;
    if (rhs2_out) *rhs2_out = h.rhsNorm2;
    if (not_converged) *not_converged = (h.done == 2);
    if (h.bad) ISL_FAIL(c, ISL_ERR_NAN, "CG breakdown (non-finite reduction)");
    return ISL_OK;
}

static int ensure_work(isl_ctx* c) {
    const size_t n = (size_t)c->neq;
    if (c->w64.n < 6 * n) ISL_CHECK_CUDA(c, c->w64.alloc(6 * n));
    if (c->w32.n < 6 * n) ISL_CHECK_CUDA(c, c->w32.alloc(6 * n));
    if (!c->dpart.p) ISL_CHECK_CUDA(c, c->dpart.alloc((size_t)2 * vec_grid(c) + 64));
    if (!c->dscal.p) ISL_CHECK_CUDA(c, c->dscal.alloc(2));
    return ISL_OK;
}

int solve_device(isl_ctx* c, int method, double tol, int64_t max_iter, int64_t* iters, double* relres) {
    int st_ = ensure_work(c);
    if (st_ != ISL_OK) return st_;
    cudaStream_t st = c->stream;
    const size_t n = (size_t)c->neq;
    if (max_iter <= 0) max_iter = 2 * (int64_t)n;
    if (c->timing) cudaEventRecord(c->ev[0], st);
    double* W = c->w64.p;
    double *x = W, *r = W + n, *p = W + 2 * n, *q = W + 3 * n, *dinv = W + 4 * n, *r64 = W + 5 * n;
    int rc = ISL_OK;
    int64_t total_it = 0;
    double rel = 0.0;
    bool nc = false;
    if (method == ISL_SOLVE_CG_FP64) {
        if (!c->spmv_lpr64) c->spmv_lpr64 = autotune_lpr<double, double>(c, c->dval64.p, c->drhs.p, q, c->dscal.p, c->dpart.p);
        double rr = 0, b2 = 0;
        rc = run_cg<double, double>(c, c->dval64.p, c->drhs.p, x, r, p, q, dinv, tol, max_iter, c->spmv_lpr64, &total_it, &rr, &b2, &nc);
        if (rc != ISL_OK) return rc;
        rel = b2 > 0 ? std::sqrt(rr / b2) : 0.0;
        k_copy64<<<vec_grid(c), BS, 0, st>>>((int)n, x, c->dsol.p);
    } else {
        // FP64 iterative refinement around FP32 CG
        float* V = c->w32.p;
        float *x32 = V, *r32 = V + n, *p32 = V + 2 * n, *q32 = V + 3 * n, *d32 = V + 4 * n, *b32 = V + 5 * n;
        if (!c->spmv_lpr32) c->spmv_lpr32 = autotune_lpr<float, float>(c, c->dval32.p, b32, q32, c->dscal.p, c->dpart.p);
        if (!c->spmv_lpr64 && c->have64)
            c->spmv_lpr64 = autotune_lpr<double, double>(c, c->dval64.p, c->drhs.p, q, c->dscal.p, c->dpart.p);
        const bool exact64 = c->have64;  // FP64 residual operator available
        ISL_CHECK_CUDA(c, cudaMemsetAsync(x, 0, n * 8, st));
        double* dres = (double*)(c->dscal.p + 1);  // scratch scalar slot
        unsigned* ticket = &(c->dscal.p + 1)->ticket1;
        ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dscal.p + 1, 0, sizeof(CGScal), st));
        // b norm
        k_copy64<<<vec_grid(c), BS, 0, st>>>((int)n, c->drhs.p, r64);
        double bnorm2 = 0.0;
        {
            std::vector<double> hb(n);
            ISL_CHECK_CUDA(c, cudaMemcpyAsync(hb.data(), c->drhs.p, n * 8, cudaMemcpyDeviceToHost, st));
            ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
            for (double v : hb) bnorm2 += v * v;
        }
        double rnorm2 = bnorm2;
        const double eta = 1e-4;  // inner relative tolerance
        const int max_outer = 60;
        if (bnorm2 == 0.0) {
            ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dsol.p, 0, n * 8, st));
        } else {
            for (int outer = 0; outer < max_outer; ++outer) {
                if (rnorm2 <= tol * tol * bnorm2) break;
                if (total_it >= max_iter) { nc = true; break; }
                const double rn = std::sqrt(rnorm2);
                k_scale_to32<<<vec_grid(c), BS, 0, st>>>((int)n, r64, 1.0 / rn, b32);
                int64_t it = 0;
                bool inc = false;
                rc = run_cg<float, float>(c, c->dval32.p, b32, d32, r32, p32, q32, x32 /*dinv*/, eta, max_iter - total_it,
                                          c->spmv_lpr32, &it, nullptr, nullptr, &inc);
                if (rc != ISL_OK) return rc;
                total_it += it;
                k_axpy32to64<<<vec_grid(c), BS, 0, st>>>((int)n, rn, d32, x);
                if (!exact64) {
                    // no FP64 operator: refinement residual from the FP32 matrix is not
                    // FP64-accurate; stop after one inner solve
                    rnorm2 = 0.0;
                    break;
                }
                launch_residual(c->spmv_lpr64, vec_grid(c), st, (int)n, c->drowptr.p, c->dcolind.p, c->dval64.p, x, c->drhs.p, r64,
                                c->dpart.p, ticket, dres);
                ISL_CHECK_CUDA(c, cudaMemcpyAsync(&rnorm2, dres, 8, cudaMemcpyDeviceToHost, st));
                ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
                if (!(rnorm2 == rnorm2)) ISL_FAIL(c, ISL_ERR_NAN, "refinement residual is not finite");
            }
        }
        rel = bnorm2 > 0 ? std::sqrt(rnorm2 / bnorm2) : 0.0;
        if (rel > tol && exact64) nc = true;
        k_copy64<<<vec_grid(c), BS, 0, st>>>((int)n, x, c->dsol.p);
    }
    ISL_CHECK_CUDA(c, cudaGetLastError());
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    if (c->timing) {
        cudaEventRecord(c->ev[1], st);
        cudaEventSynchronize(c->ev[1]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        c->tms[ISL_T_SOLVE] += ms;
        c->tcount[ISL_T_SOLVE]++;
    }
    c->solved = true;
    if (iters) *iters = total_it;
    if (relres) *relres = rel;
    if (nc) ISL_FAIL(c, ISL_ERR_NOT_CONVERGED, "solver did not reach the tolerance");
    return ISL_OK;
}

__global__ void k_distribute(int64_t ndc, const int32_t* __restrict__ eq, const uint8_t* __restrict__ status,
                             const double* __restrict__ cval, const double* __restrict__ x, double* __restrict__ u, int add) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ndc; k += (int64_t)gridDim.x * blockDim.x) {
        if (status[k] == 0) u[k] = add ? u[k] + x[eq[k]] : x[eq[k]];
        else u[k] = cval[k];
    }
}

int distribute_device(isl_ctx* c, int add) {
    const int64_t ndc = c->ndofobj * c->ncomp;
    k_distribute<<<vec_grid(c), BS, 0, c->stream>>>(ndc, c->deq.p, c->dstatus.p, c->dcval.p, c->dsol.p, c->du.p, add);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
}

int time_spmv(isl_ctx* c, int precision, int nrep, double* ms) {
    int rc = ensure_work(c);
    if (rc != ISL_OK) return rc;
    const size_t n = (size_t)c->neq;
    CGScal* S = c->dscal.p;
    cudaStream_t st = c->stream;
    ISL_CHECK_CUDA(c, cudaMemsetAsync(S, 0, sizeof(CGScal), st));
    if (precision == ISL_PREC_FP32) {
        if (!c->have32) ISL_FAIL(c, ISL_ERR_ARG, "no FP32 matrix");
        float* V = c->w32.p;
        if (!c->spmv_lpr32) c->spmv_lpr32 = autotune_lpr<float, float>(c, c->dval32.p, V + 2 * n, V + 3 * n, S, c->dpart.p);
        launch_spmv<float, float>(c->spmv_lpr32, vec_grid(c), st, (int)n, c->drowptr.p, c->dcolind.p, c->dval32.p, V + 2 * n, V + 3 * n, S, c->dpart.p);
        cudaEventRecord(c->ev[2], st);
        for (int r = 0; r < nrep; ++r)
            launch_spmv<float, float>(c->spmv_lpr32, vec_grid(c), st, (int)n, c->drowptr.p, c->dcolind.p, c->dval32.p, V + 2 * n, V + 3 * n, S, c->dpart.p);
        cudaEventRecord(c->ev[3], st);
    } else {
        if (!c->have64) ISL_FAIL(c, ISL_ERR_ARG, "no FP64 matrix");
        double* W = c->w64.p;
        if (!c->spmv_lpr64) c->spmv_lpr64 = autotune_lpr<double, double>(c, c->dval64.p, W + 2 * n, W + 3 * n, S, c->dpart.p);
        launch_spmv<double, double>(c->spmv_lpr64, vec_grid(c), st, (int)n, c->drowptr.p, c->dcolind.p, c->dval64.p, W + 2 * n, W + 3 * n, S, c->dpart.p);
        cudaEventRecord(c->ev[2], st);
        for (int r = 0; r < nrep; ++r)
            launch_spmv<double, double>(c->spmv_lpr64, vec_grid(c), st, (int)n, c->drowptr.p, c->dcolind.p, c->dval64.p, W + 2 * n, W + 3 * n, S, c->dpart.p);
        cudaEventRecord(c->ev[3], st);
    }
    ISL_CHECK_CUDA(c, cudaEventSynchronize(c->ev[3]));
    float t = 0.f;
    cudaEventElapsedTime(&t, c->ev[2], c->ev[3]);
    *ms = t / nrep;
    ISL_CHECK_CUDA(c, cudaGetLastError());
    return ISL_OK;
}

}  // namespace isl
