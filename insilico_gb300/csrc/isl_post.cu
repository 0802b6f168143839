// Post-processing on the GPU: the physical coordinates of the quadrature
// points, and the error of the FE field against a reference solution in the
// L2 norm or the H1 semi-norm (base::post::errorComputation<ORDER>,
// base/post/ErrorNorm.hpp:84-123 and the ErrorNorm functor :300-330).
//
// The reference solution is a host function in the reference (a
// boost::function of x).  A device cannot call it, so the caller evaluates it
// at the points isl_quadrature_points returns and hands the table over, the
// same way conductivities and materials are tabulated per element.
//
// Per quadrature point, as the reference: x = sum_i N_i(xi) X_i (geometry
// functions), detJ signed, error = ref - u_h (u_h and its gradient from the
// field's current values), errorSquared += (error . error) detJ w; the result
// is sqrt of the sum over elements.  One thread per element; element sums are
// added per block in FP64 and the blocks' sums by the last block in a fixed
// order, so the result is reproducible bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "isl_device.cuh"
#include "isl_internal.h"

namespace isl {

namespace {

constexpr int PB = 128;

template <int D>
__device__ inline double det_inv_t(const double J[D][D], double Ji[D][D]) {
    if (D == 2) {
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const double id = 1.0 / det;
        Ji[0][0] = J[1][1] * id;  Ji[0][1] = -J[1][0] * id;
        Ji[1][0] = -J[0][1] * id; Ji[1][1] = J[0][0] * id;
        return det;
    } else {
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const double id = 1.0 / det;
        Ji[0][0] = c00 * id; Ji[0][1] = c01 * id; Ji[0][2] = c02 * id;
        Ji[1][0] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        Ji[1][2] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        Ji[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        Ji[2][1] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
        return det;
    }
}

template <int SHAPE, int FDEG, int NQ>
using PTab = Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ>;

template <int SHAPE, int FDEG, int NQ>
__global__ void __launch_bounds__(PB) k_qpoints(int E, const double* __restrict__ X, const int32_t* __restrict__ conn,
                                                const PTab<SHAPE, FDEG, NQ> T, double* __restrict__ xq) {
    constexpr int D = ET<SHAPE, FDEG>::D, NG = ET<SHAPE, FDEG>::NG;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        double Xe[NG][D];
#pragma unroll
        for (int i = 0; i < NG; ++i) {
            const int nd = conn[i * E + e];
#pragma unroll
            for (int d = 0; d < D; ++d) Xe[i][d] = X[(size_t)nd * D + d];
        }
        for (int q = 0; q < NQ; ++q)
#pragma unroll
            for (int d = 0; d < D; ++d) {
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < NG; ++i) s += T.N[q][i] * Xe[i][d];
                xq[((size_t)e * NQ + q) * D + d] = s;
            }
    }
}

// sum over the elements of (ref - u_h)^2 detJ w (order 0) or of
// |grad ref - grad u_h|^2 detJ w (order 1); ncomp <= 3
template <int SHAPE, int FDEG, int NQ>
__global__ void __launch_bounds__(PB) k_error(int E, int ncomp, int order, const double* __restrict__ X,
                                              const int32_t* __restrict__ conn, const int32_t* __restrict__ edof,
                                              const double* __restrict__ u, const PTab<SHAPE, FDEG, NQ> T,
                                              const double* __restrict__ ref, double* part, unsigned* ticket,
                                              double* out) {
    constexpr int D = ET<SHAPE, FDEG>::D, NG = ET<SHAPE, FDEG>::NG, NF = ET<SHAPE, FDEG>::NF;
    __shared__ double sh[32];
    double loc = 0.0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        double Xe[NG][D];
#pragma unroll
        for (int i = 0; i < NG; ++i) {
            const int nd = conn[i * E + e];
#pragma unroll
            for (int d = 0; d < D; ++d) Xe[i][d] = X[(size_t)nd * D + d];
        }
        double ue[3][NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const int o = edof[f * E + e];
#pragma unroll
            for (int c = 0; c < 3; ++c) ue[c][f] = c < ncomp ? u[(size_t)o * ncomp + c] : 0.0;
        }
        double esum = 0.0;
        for (int q = 0; q < NQ; ++q) {
            double J[D][D], Ji[D][D];
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b = 0; b < D; ++b) {
                    double s = 0.0;
#pragma unroll
                    for (int i = 0; i < NG; ++i) s += Xe[i][a] * T.dN[q][i][b];
                    J[a][b] = s;
                }
            const double detJ = det_inv_t<D>(J, Ji);
            double s2 = 0.0;
            if (order == 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    if (c >= ncomp) break;
                    double uh = 0.0;
#pragma unroll
                    for (int f = 0; f < NF; ++f) uh += T.phi[q][f] * ue[c][f];
                    const double d = ref[((size_t)e * NQ + q) * ncomp + c] - uh;
                    s2 += d * d;
                }
            } else {
                double g[NF][D];
#pragma unroll
                for (int f = 0; f < NF; ++f)
#pragma unroll
                    for (int a = 0; a < D; ++a) {
                        double s = 0.0;
#pragma unroll
                        for (int b = 0; b < D; ++b) s += Ji[a][b] * T.dphi[q][f][b];
                        g[f][a] = s;
                    }
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    if (c >= ncomp) break;
#pragma unroll
                    for (int a = 0; a < D; ++a) {
                        double gh = 0.0;
#pragma unroll
                        for (int f = 0; f < NF; ++f) gh += g[f][a] * ue[c][f];
                        const double d = ref[(((size_t)e * NQ + q) * ncomp + c) * D + a] - gh;
                        s2 += d * d;
                    }
                }
            }
            esum += s2 * detJ * T.w[q];
        }
        loc += esum;
    }
    const double bs = block_sum(loc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = bs;
    if (last_block(ticket)) {
        const double tot = reduce_parts_blk<PB>(part, gridDim.x, 1, 0, sh);
        if (threadIdx.x == 0) { *out = tot; *ticket = 0; }
    }
}

template <int SHAPE, int FDEG, int NQ>
void fill(PTab<SHAPE, FDEG, NQ>& T, const HostTab& h) {
    constexpr int D = ET<SHAPE, FDEG>::D, NG = ET<SHAPE, FDEG>::NG, NF = ET<SHAPE, FDEG>::NF;
    for (int q = 0; q < NQ; ++q) {
        T.w[q] = h.w[q];
        for (int f = 0; f < NF; ++f) {
            T.phi[q][f] = h.phi[q * NF + f];
            for (int d = 0; d < D; ++d) T.dphi[q][f][d] = h.dphi[(q * NF + f) * D + d];
        }
        for (int i = 0; i < NG; ++i) {
            T.N[q][i] = h.N[q * NG + i];
            for (int d = 0; d < D; ++d) T.dN[q][i][d] = h.dN[(q * NG + i) * D + d];
        }
    }
}

unsigned post_grid(const isl_ctx* c) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((c->nelem + PB - 1) / PB, (int64_t)8 * c->sm_count));
}

// qpoints (error == nullptr) or the squared error sum into *dout
template <int SHAPE, int FDEG, int NQ>
int run(isl_ctx* c, const HostTab& h, double* dxq, int order, const double* dref, double* dpart, unsigned* dticket,
        double* dout) {
    PTab<SHAPE, FDEG, NQ> T;
    fill<SHAPE, FDEG, NQ>(T, h);
    const unsigned g = post_grid(c);
    if (dxq)
        k_qpoints<SHAPE, FDEG, NQ><<<g, PB, 0, c->stream>>>((int)c->nelem, c->dX.p, c->dconn.p, T, dxq);
    else
        k_error<SHAPE, FDEG, NQ><<<g, PB, 0, c->stream>>>((int)c->nelem, c->ncomp, order, c->dX.p, c->dconn.p,
                                                         c->dedof.p, c->du.p, T, dref, dpart, dticket, dout);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

int dispatch(isl_ctx* c, const HostTab& h, double* dxq, int order, const double* dref, double* dpart,
             unsigned* dticket, double* dout) {
    const int s = c->shape, k = c->fedeg, nq = h.nq;
#define ISL_POST_CASE(S, K, N) \
    if (s == S && k == K && nq == N) return run<S, K, N>(c, h, dxq, order, dref, dpart, dticket, dout);
    ISL_POST_CASE(ISL_QUAD, 1, 1) ISL_POST_CASE(ISL_QUAD, 1, 4) ISL_POST_CASE(ISL_QUAD, 1, 9)
    ISL_POST_CASE(ISL_QUAD, 2, 1) ISL_POST_CASE(ISL_QUAD, 2, 4) ISL_POST_CASE(ISL_QUAD, 2, 9)
    ISL_POST_CASE(ISL_HEX, 1, 1) ISL_POST_CASE(ISL_HEX, 1, 8) ISL_POST_CASE(ISL_HEX, 1, 27)
    ISL_POST_CASE(ISL_TET, 1, 1) ISL_POST_CASE(ISL_TET, 1, 4) ISL_POST_CASE(ISL_TET, 2, 1)
    ISL_POST_CASE(ISL_TET, 2, 4) ISL_POST_CASE(ISL_TET, 2, 11)
#undef ISL_POST_CASE
    ISL_FAIL(c, ISL_ERR_ARG, "post-processing: unsupported element / quadrature combination");
}

}  // namespace

int quadrature_points_device(isl_ctx* c, int qdeg, int64_t* n, double* x) {
    HostTab h;
    if (!make_host_tables(c->shape, c->fedeg, qdeg, h)) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    const int64_t np = c->nelem * h.nq;
    *n = np;
    if (!x) return ISL_OK;
    DBuf<double> dxq;
    ISL_CHECK_CUDA(c, dxq.alloc((size_t)np * c->dim));
    int rc = dispatch(c, h, dxq.p, 0, nullptr, nullptr, nullptr, nullptr);
    if (rc != ISL_OK) return rc;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(x, dxq.p, (size_t)np * c->dim * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    return ISL_OK;
}

int error_norm_device(isl_ctx* c, int order, int qdeg, const double* ref, double* err) {
    HostTab h;
    if (!make_host_tables(c->shape, c->fedeg, qdeg, h)) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    const size_t per = (size_t)c->ncomp * (order == 1 ? c->dim : 1);
    const size_t nref = (size_t)c->nelem * h.nq * per;
    DBuf<double> dref, dpart, dout;
    DBuf<unsigned> dticket;
    ISL_CHECK_CUDA(c, dref.alloc(nref));
    ISL_CHECK_CUDA(c, dpart.alloc(post_grid(c)));
    ISL_CHECK_CUDA(c, dout.alloc(1));
    ISL_CHECK_CUDA(c, dticket.alloc(1));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(dticket.p, 0, sizeof(unsigned), c->stream));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(dref.p, ref, nref * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = dispatch(c, h, nullptr, order, dref.p, dpart.p, dticket.p, dout.p);
    if (rc != ISL_OK) {
        cudaStreamSynchronize(c->stream);
        return rc;
    }
    double sum = 0.0;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(&sum, dout.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(c->stream));
    *err = std::sqrt(sum);
    return ISL_OK;
}

}  // namespace isl
