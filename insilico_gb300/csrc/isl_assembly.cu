// Device assembly for the GB300 (sm_103a) inSilico hot path.
//
//  * pattern_build: the CSR pattern of active DOF pairs (the reference's
//    pre-structured triplet pattern, base/solver/TripletContainer.hpp:158-301)
//    is built on the device by a stable radix sort of (row, col) keys of every
//    element's active local pairs.  The sorted order doubles as the
//    element-to-slot contribution list: slot s sums the staged element entries
//    src[seg[s] .. seg[s+1]) in element order, the order in which the
//    reference's serial element loop adds into a triplet
//    (TripletContainer::insert, :305-352).  No atomics are used.
//  * element kernels stage the packed upper triangle of every element matrix
//    (element-major: stage[e * nup + u], so that the contributions a CSR row
//    gathers from one element lie together) and the element force vector
//    (entry-major); a gather kernel then forms CSR values and the RHS.
//  * Dirichlet columns move to the RHS per element (b -= K[:,c] g_c,
//    base/asmb/assembleMatrix.hpp:56-130) in a kernel over the elements that
//    own a constrained DOF.
#include <cub/cub.cuh>

#include <cmath>
#include <cstdio>
#include <type_traits>
#include <vector>

#include "isl_df.cuh"
#include "isl_elem.cuh"
#include "isl_internal.h"

namespace isl {

// ---------------------------------------------------------------------------
// heat::Laplace element kernel, one thread per element.
//   K[M][N] += (grad phi_M . grad phi_N) (kappa detJ w)   base/kernel/Laplace.hpp:131-148
//   F[i]    -= kappa grad u . grad phi_i detJ w           heat/Laplace.hpp:150-183 (x -1)
//   F[s]    += f(x) phi_s w detJ                          base/asmb/BodyForce.hpp:172-205
// TI: the time-integration terms (mass matrix, weighted history, residual
// forces at past states) are compiled in; the plain assembly runs without them.
// DF (mixed precision): the stiffness sum runs in double-float on the FP32 pipe
// (isl_df.cuh: about 48 significant bits; FP32 runs at about 64 times the
// FP64 rate here), from the FP64 Jacobian and the double-float shape-function
// gradients TD.dphi; one FP64 addition per entry forms the staged FP64 value.
// The forces stay in FP64.
template <int D, int NF, int NQ>
struct TabDF {
    df dphi[NQ][NF][D];
};

template <int SHAPE, int FDEG, int NQ, typename R, bool TI, bool DF = false>
__global__ void __launch_bounds__(128) k_laplace(const ElemArgs A, const Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ> T,
                                                 const TabDF<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NF, NQ> TD) {
    constexpr int D = ET<SHAPE, FDEG>::D, NG = ET<SHAPE, FDEG>::NG, NF = ET<SHAPE, FDEG>::NF;
    constexpr int NUP = NF * (NF + 1) / 2;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.nelem) return;
    const int E = A.nelem;
    double X[NG][D];
    int nodes[NG];
#pragma unroll
    for (int i = 0; i < NG; ++i) {
        nodes[i] = A.conn[i * E + e];
#pragma unroll
        for (int d = 0; d < D; ++d) X[i][d] = A.X[(size_t)nodes[i] * D + d];
    }
    const double kap = A.coef[e];
    double uloc[NF];
    if (A.with_residual) {
#pragma unroll
        for (int f = 0; f < NF; ++f) uloc[f] = A.u[A.edof[f * E + e]];
    }
    const bool aff = affine<SHAPE, NG, D>(X);
    double Ji[D][D], detJ = 0.0;
    if (aff) detJ = jac<NG, D>(X, T.dN[0], Ji);
    double hloc[NF];
    const double rho = (TI && A.rho) ? A.rho[e] : 0.0;
    if (TI && A.rho) {
#pragma unroll
        for (int f = 0; f < NF; ++f) hloc[f] = A.hvec[A.edof[f * E + e]];
    }
    constexpr int NACC = DF ? 1 : NUP;
    R acc[NACC];
#pragma unroll
    for (int u = 0; u < NACC; ++u) acc[u] = R(0);
    constexpr int NACCD = DF ? NUP : 1;
    df accd[NACCD];
#pragma unroll
    for (int u = 0; u < NACCD; ++u) accd[u] = df{0.f, 0.f};
    double fe[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) fe[f] = 0.0;
    bool bad = false;
    // the FP64 gradients feed the forces (and the FP64 / FP32 stiffness)
    const bool need_g = !DF || A.fnodal || A.with_residual || TI;
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        if (!aff) detJ = jac<NG, D>(X, T.dN[q], Ji);
        bad |= !(detJ > 0.0);
        double g[NF][D];
        if (need_g) {
#pragma unroll
            for (int M = 0; M < NF; ++M)
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    double s = 0.0;
#pragma unroll
                    for (int b = 0; b < D; ++b) s += Ji[a][b] * T.dphi[q][M][b];
                    g[M][a] = s;
                }
        }
        const double kq = A.kqp ? A.kqp[(size_t)q * E + e] : kap;
        const double c = kq * detJ * T.w[q];
        if constexpr (DF) {
            df Jd[D][D];
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b = 0; b < D; ++b) Jd[a][b] = df_from_double(Ji[a][b]);
            df gd[NF][D];
#pragma unroll
            for (int M = 0; M < NF; ++M)
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    df s = df_mul(Jd[a][0], TD.dphi[q][M][0]);
#pragma unroll
                    for (int b = 1; b < D; ++b) s = df_add(s, df_mul(Jd[a][b], TD.dphi[q][M][b]));
                    gd[M][a] = s;
                }
            const df cd = df_from_double(c);
#pragma unroll
            for (int M = 0; M < NF; ++M)
#pragma unroll
                for (int N = M; N < NF; ++N) {
                    df dot = df_mul(gd[M][0], gd[N][0]);
#pragma unroll
                    for (int k = 1; k < D; ++k) dot = df_add(dot, df_mul(gd[M][k], gd[N][k]));
                    accd[upidx(M, N, NF)] = df_add_acc(accd[upidx(M, N, NF)], df_mul(dot, cd));
                }
        } else {
            const R cr = R(c);
#pragma unroll
            for (int M = 0; M < NF; ++M)
#pragma unroll
                for (int N = M; N < NF; ++N) {
                    R dot = R(0);
#pragma unroll
                    for (int k = 0; k < D; ++k) dot += R(g[M][k]) * R(g[N][k]);
                    acc[upidx(M, N, NF)] += dot * cr;
                }
        }
        if (A.fnodal) {
            double f = 0.0;
#pragma unroll
            for (int i = 0; i < NG; ++i) f += T.N[q][i] * A.fnodal[nodes[i]];
#pragma unroll
            for (int s = 0; s < NF; ++s) fe[s] += f * T.phi[q][s] * T.w[q] * detJ;
        }
        if (TI && A.rho) {  // base/kernel/Mass.hpp: M[i][j] += rho phi_i phi_j detJ w
            const double m = rho * detJ * T.w[q];
            double hq = 0.0;
#pragma unroll
            for (int f = 0; f < NF; ++f) hq += T.phi[q][f] * hloc[f];
#pragma unroll
            for (int M = 0; M < NF; ++M) {
#pragma unroll
                for (int N = M; N < NF; ++N) {
                    const double mv = A.mass_w * m * T.phi[q][M] * T.phi[q][N];
                    if constexpr (DF) accd[upidx(M, N, NF)] = df_add_acc(accd[upidx(M, N, NF)], df_from_double(mv));
                    else acc[upidx(M, N, NF)] += R(mv);
                }
                fe[M] += m * T.phi[q][M] * hq;
            }
        }
        if (A.with_residual) {
            double gu[D];
#pragma unroll
            for (int k = 0; k < D; ++k) {
                double s = 0.0;
#pragma unroll
                for (int f = 0; f < NF; ++f) s += g[f][k] * uloc[f];
                gu[k] = kq * s;
            }
#pragma unroll
            for (int i = 0; i < NF; ++i) {
                double dp = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) dp += gu[k] * g[i][k];
                fe[i] -= dp * detJ * T.w[q];
            }
        }
        for (int sidx = 0; TI && sidx < A.nfw; ++sidx) {  // heat/Laplace.hpp:150-183 at a past state
            double gu[D];
#pragma unroll
            for (int k = 0; k < D; ++k) gu[k] = 0.0;
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const double hf = A.hist[(size_t)sidx * A.hstride + A.edof[f * E + e]];
#pragma unroll
                for (int k = 0; k < D; ++k) gu[k] += g[f][k] * hf;
            }
#pragma unroll
            for (int i = 0; i < NF; ++i) {
                double dp = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) dp += kq * gu[k] * g[i][k];
                fe[i] -= A.fw[sidx] * dp * detJ * T.w[q];
            }
        }
    }
    if (bad) atomicOr(A.flags, 1);
    R* SK = (R*)A.stageK;
    if constexpr (DF) {
#pragma unroll
        for (int u = 0; u < NUP; ++u) SK[(size_t)e * NUP + u] = R(df_to_double(accd[u]));
    } else {
#pragma unroll
        for (int u = 0; u < NUP; ++u) SK[(size_t)e * NUP + u] = acc[u];
    }
#pragma unroll
    for (int s = 0; s < NF; ++s) A.stageF[(size_t)s * E + e] = fe[s];
}

// ---------------------------------------------------------------------------
// Weighted DOF history of a multi-step method (ReactionTerms.hpp,
// CollectWeightedHistory): h = w0 x^(0) + w1 x^(1) + ... with x^(0) the
// current values and x^(s) = hist[s - 1] the values s steps back.
__global__ void k_hist_combine(int64_t n, const double* __restrict__ u, const double* __restrict__ hist, int nw,
                               double w0, double w1, double w2, double w3, double w4, double* __restrict__ h) {
    const double w[5] = {w0, w1, w2, w3, w4};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = nw > 0 ? w[0] * u[i] : 0.0;
        for (int k = 1; k < nw; ++k) s += w[k] * hist[(size_t)(k - 1) * n + i];
        h[i] = s;
    }
}

// history shift (base::dof::pushHistory): hist[s] = hist[s - 1], hist[0] = u
__global__ void k_hist_push(int64_t n, int nhist, const double* __restrict__ u, double* __restrict__ hist) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        for (int s = nhist - 1; s > 0; --s) hist[(size_t)s * n + i] = hist[(size_t)(s - 1) * n + i];
        hist[i] = u[i];
    }
}

int push_history_device(isl_ctx* c) {
    const int64_t n = c->ndofobj * c->ncomp;
    k_hist_push<<<(unsigned)c->sm_count * 8, 256, 0, c->stream>>>(n, c->nhist, c->du.p, c->dhist.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

// ---------------------------------------------------------------------------
// heat::Static element kernel (heat/Static.hpp:98-225), one thread per element,
// with the isotropic materials of mat/thermal: IsotropicConstant (K = k I,
// K' = 0) and FenicsTest (K = (1 + u)^m I, K' = m (1 + u)^(m-1) I,
// mat/thermal/FenicsTest.hpp:47-60).  The tangent is not symmetric, so the
// whole NF x NF matrix is staged (element-major, stage[e NF^2 + i NF + j]):
//   K[i][j] += detJ w sum_K (g_iK k g_jK + g_iK k' gu_K phi_j)
//   F[i]    -= detJ w sum_K g_iK k gu_K                (residual, x -1)
//   F[s]    += f(x) phi_s w detJ                        (body force)
template <int SHAPE, int FDEG, int NQ>
__global__ void __launch_bounds__(128) k_heat_static(const ElemArgs A, const Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ> T) {
    constexpr int D = ET<SHAPE, FDEG>::D, NG = ET<SHAPE, FDEG>::NG, NF = ET<SHAPE, FDEG>::NF;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.nelem) return;
    const int E = A.nelem;
    double X[NG][D];
    int nodes[NG];
#pragma unroll
    for (int i = 0; i < NG; ++i) {
        nodes[i] = A.conn[i * E + e];
#pragma unroll
        for (int d = 0; d < D; ++d) X[i][d] = A.X[(size_t)nodes[i] * D + d];
    }
    const double prm = A.coef[e];
    double uloc[NF], hloc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        uloc[f] = A.u[A.edof[f * E + e]];
        hloc[f] = A.rho ? A.hvec[A.edof[f * E + e]] : 0.0;
    }
    const double rho = A.rho ? A.rho[e] : 0.0;
    double K[NF][NF];
#pragma unroll
    for (int i = 0; i < NF; ++i)
#pragma unroll
        for (int j = 0; j < NF; ++j) K[i][j] = 0.0;
    double fe[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) fe[f] = 0.0;
    bool bad = false;
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        double Ji[D][D];
        const double detJ = jac<NG, D>(X, T.dN[q], Ji);
        bad |= !(detJ > 0.0);
        double g[NF][D];
#pragma unroll
        for (int M = 0; M < NF; ++M)
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double s = 0.0;
#pragma unroll
                for (int b = 0; b < D; ++b) s += Ji[a][b] * T.dphi[q][M][b];
                g[M][a] = s;
            }
        double u = 0.0, gu[D];
#pragma unroll
        for (int k = 0; k < D; ++k) gu[k] = 0.0;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            u += T.phi[q][f] * uloc[f];
#pragma unroll
            for (int k = 0; k < D; ++k) gu[k] += g[f][k] * uloc[f];
        }
        double k0, k1;
        if (A.material == ISL_THERMAL_FENICS) {
            k0 = pow(1.0 + u, prm);
            k1 = prm * pow(1.0 + u, prm - 1.0);
        } else {
            k0 = prm;
            k1 = 0.0;
        }
        const double dw = detJ * T.w[q];
#pragma unroll
        for (int i = 0; i < NF; ++i)
#pragma unroll
            for (int j = 0; j < NF; ++j) {
                double entry = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    entry += g[i][k] * k0 * g[j][k];
                    entry += g[i][k] * k1 * gu[k] * T.phi[q][j];
                }
                K[i][j] += dw * entry;
            }
        if (A.with_residual) {
#pragma unroll
            for (int i = 0; i < NF; ++i) {
                double sum = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) sum += g[i][k] * k0 * gu[k];
                fe[i] -= sum * dw;
            }
        }
        if (A.fnodal) {
            double f = 0.0;
#pragma unroll
            for (int i = 0; i < NG; ++i) f += T.N[q][i] * A.fnodal[nodes[i]];
#pragma unroll
            for (int s = 0; s < NF; ++s) fe[s] += f * T.phi[q][s] * T.w[q] * detJ;
        }
        for (int sidx = 0; sidx < A.nfw; ++sidx) {  // residualForceHistory at a past state
            double us = 0.0, gus[D];
#pragma unroll
            for (int k = 0; k < D; ++k) gus[k] = 0.0;
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const double hf = A.hist[(size_t)sidx * A.hstride + A.edof[f * E + e]];
                us += T.phi[q][f] * hf;
#pragma unroll
                for (int k = 0; k < D; ++k) gus[k] += g[f][k] * hf;
            }
            const double ks = A.material == ISL_THERMAL_FENICS ? pow(1.0 + us, prm) : prm;
#pragma unroll
            for (int i = 0; i < NF; ++i) {
                double sum = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) sum += g[i][k] * ks * gus[k];
                fe[i] -= A.fw[sidx] * sum * dw;
            }
        }
        if (A.rho) {  // base/kernel/Mass.hpp: M[i][j] += rho phi_i phi_j detJ w
            const double m = rho * dw;
            double hq = 0.0;
#pragma unroll
            for (int f = 0; f < NF; ++f) hq += T.phi[q][f] * hloc[f];
#pragma unroll
            for (int i = 0; i < NF; ++i) {
#pragma unroll
                for (int j = 0; j < NF; ++j) K[i][j] += A.mass_w * m * T.phi[q][i] * T.phi[q][j];
                fe[i] += m * T.phi[q][i] * hq;
            }
        }
    }
    if (bad) atomicOr(A.flags, 1);
    double* SK = (double*)A.stageK;
#pragma unroll
    for (int i = 0; i < NF; ++i)
#pragma unroll
        for (int j = 0; j < NF; ++j) SK[((size_t)e * NF + i) * NF + j] = K[i][j];
#pragma unroll
    for (int s = 0; s < NF; ++s) A.stageF[(size_t)s * E + e] = fe[s];
}

// ---------------------------------------------------------------------------
// solid::HyperElastic on trilinear hexahedra, 2x2x2 quadrature.
// 8 threads per element: in phase 1 thread q evaluates quadrature point q
// (geometry, deformation, stress, effective elasticity), in phase 2 thread M
// accumulates row-node M's 3x3 blocks K_MN (N >= M) over the quadrature points.
//   K[Md+i, Nd+k] += sum_JL phi_M,J (d_ik S_JL + F_iA C_AJBL F_kB) phi_N,L detJ w
//                                           solid/HyperElastic.hpp:110-179,282-310
//   F[Md+i] -= sum_J (F S)_iJ phi_M,J detJ w  solid/HyperElastic.hpp:209-257 (x -1)
// Materials: StVenant mat/hypel/StVenant.hpp:77-114,
//            NeoHookeanCompressible mat/hypel/NeoHookeanCompressible.hpp:77-172.
// At u == 0 (F = I, S = 0) both reduce to isotropic linear elasticity and the
// kernel uses  K_MN = c (lam g_M g_N^T + mu g_N g_M^T + mu (g_M.g_N) I).
// TI compiles in the time-integration terms of a vector field (the plain
// assembly runs without them):
//   K[Md+i, Nd+i] += mass_w rho phi_M phi_N detJ w    base/kernel/Mass.hpp:72-101
//   F[Md+i]       += sum_N (rho phi_M phi_N detJ w) h[Nd+i]   ReactionTerms.hpp
//   F[Md+i]       -= sum_s fw_s (F_s S_s)_iJ phi_M,J detJ w at the past state s
//                                           base/time/ResidualForceHistory.hpp
// The host runs the finite-strain path (general) whenever past-state forces
// are asked for, so that their contributions have the shared staging.
template <typename R, int EPB, bool TI>
__global__ void __launch_bounds__(EPB * 8) k_hyper_hex8(const ElemArgs A, const Tab<3, 8, 8, 8> T) {
    constexpr int NLOC = 24;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // shared layout (element index fastest to keep banks distinct)
    double* sX = (double*)smem_raw;                 // [8][3][EPB]
    double* su = sX + 8 * 3 * EPB;                  // [8][3][EPB]
    double* sfq = su + 8 * 3 * EPB;                 // [8 q][8 node][3][EPB] residual contributions
    R* sg = (R*)(sfq + (A.general ? 8 * 8 * 3 * EPB : 0));  // [8 q][8 node][3][EPB]
    R* sc = sg + 8 * 8 * 3 * EPB;                   // [8][EPB]
    R* sA = sc + 8 * EPB;                           // [8 q][81][EPB] (general only)

    const int el = threadIdx.x % EPB, role = threadIdx.x / EPB;
    const int E = A.nelem;
    const int e = blockIdx.x * EPB + el;
    const bool valid = e < E;
    const int ec = valid ? e : E - 1;
    {
        const int node = A.conn[role * E + ec];
#pragma unroll
        for (int d = 0; d < 3; ++d) sX[(role * 3 + d) * EPB + el] = A.X[(size_t)node * 3 + d];
        if (A.general) {
            const int obj = A.edof[role * E + ec];
#pragma unroll
            for (int d = 0; d < 3; ++d) su[(role * 3 + d) * EPB + el] = A.u[(size_t)obj * 3 + d];
        }
    }
    __syncthreads();
    // affine elements (parallelepipeds): one FP64 Jacobian per element, by role 0
    __shared__ double sJi[10][EPB];
    __shared__ int saff[EPB];
    if (role == 0) {
        double X[8][3];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d) X[i][d] = sX[(i * 3 + d) * EPB + el];
        const bool aff = affine<ISL_HEX, 8, 3>(X);
        saff[el] = aff;
        if (aff) {
            double Ji[3][3];
            sJi[9][el] = jac<8, 3>(X, T.dN[0], Ji);
#pragma unroll
            for (int a = 0; a < 9; ++a) sJi[a][el] = Ji[a / 3][a % 3];
        }
    }
    __syncthreads();
    const double lam = A.coef[ec], mu = A.coef[E + ec];
    // ---- phase 1: quadrature point q = role
    {
        const int q = role;
        double Ji[3][3], detJ;
        if (saff[el]) {
#pragma unroll
            for (int a = 0; a < 9; ++a) Ji[a / 3][a % 3] = sJi[a][el];
            detJ = sJi[9][el];
        } else {
            double X[8][3];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int d = 0; d < 3; ++d) X[i][d] = sX[(i * 3 + d) * EPB + el];
            detJ = jac<8, 3>(X, T.dN[q], Ji);
        }
        if (valid && !(detJ > 0.0)) atomicOr(A.flags, 1);
        const double c = detJ * T.w[q];
        sc[q * EPB + el] = R(c);
        if (!A.general) {
            // small-strain path: gradients only needed in R
            R Jr[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) Jr[a][b] = R(Ji[a][b]);
#pragma unroll
            for (int M = 0; M < 8; ++M)
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    sg[((q * 8 + M) * 3 + a) * EPB + el] =
                        Jr[a][0] * R(T.dphi[q][M][0]) + Jr[a][1] * R(T.dphi[q][M][1]) + Jr[a][2] * R(T.dphi[q][M][2]);
        }
        if (A.general) {
            double g[8][3];
#pragma unroll
            for (int M = 0; M < 8; ++M)
#pragma unroll
                for (int a = 0; a < 3; ++a) g[M][a] = Ji[a][0] * T.dphi[q][M][0] + Ji[a][1] * T.dphi[q][M][1] + Ji[a][2] * T.dphi[q][M][2];
#pragma unroll
            for (int M = 0; M < 8; ++M)
#pragma unroll
                for (int a = 0; a < 3; ++a) sg[((q * 8 + M) * 3 + a) * EPB + el] = R(g[M][a]);
            double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
            for (int f = 0; f < 8; ++f)
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const double uf = su[(f * 3 + i) * EPB + el];
#pragma unroll
                    for (int J = 0; J < 3; ++J) F[i][J] += g[f][J] * uf;
                }
            double S[3][3], C[6][6];
            material_eval(A.material, lam, mu, F, S, C);
            bool nan = false;
            // residual contribution of this quadrature point: c (F S)_iJ g_N,J
            double P[3][3];
            for (int i = 0; i < 3; ++i)
                for (int J = 0; J < 3; ++J) P[i][J] = F[i][0] * S[0][J] + F[i][1] * S[1][J] + F[i][2] * S[2][J];
#pragma unroll
            for (int N = 0; N < 8; ++N)
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const double v = (P[i][0] * g[N][0] + P[i][1] * g[N][1] + P[i][2] * g[N][2]) * c;
                    nan |= !(v == v);
                    sfq[((q * 8 + N) * 3 + i) * EPB + el] = (TI && !A.with_residual) ? 0.0 : v;
                }
            if (TI) {
                // residual forces at the past states, weighted (x -1 when summed)
                for (int sidx = 0; sidx < A.nfw; ++sidx) {
                    double Fh[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
                    for (int f = 0; f < 8; ++f) {
                        const size_t obj = (size_t)A.edof[f * E + ec];
                        for (int i = 0; i < 3; ++i) {
                            const double uf = A.hist[(size_t)sidx * A.hstride + obj * 3 + i];
                            for (int J = 0; J < 3; ++J) Fh[i][J] += g[f][J] * uf;
                        }
                    }
                    double Sh[3][3], Ch[6][6];
                    material_eval(A.material, lam, mu, Fh, Sh, Ch);
                    double Ph[3][3];
                    for (int i = 0; i < 3; ++i)
                        for (int J = 0; J < 3; ++J) Ph[i][J] = Fh[i][0] * Sh[0][J] + Fh[i][1] * Sh[1][J] + Fh[i][2] * Sh[2][J];
                    for (int N = 0; N < 8; ++N)
                        for (int i = 0; i < 3; ++i) {
                            const double v = A.fw[sidx] * (Ph[i][0] * g[N][0] + Ph[i][1] * g[N][1] + Ph[i][2] * g[N][2]) * c;
                            nan |= !(v == v);
                            sfq[((q * 8 + N) * 3 + i) * EPB + el] += v;
                        }
                }
            }
            if (valid && nan) atomicOr(A.flags, 2);
            // effective elasticity A[iJ][kL] = d_ik S_JL + F_iA C_V(A,J)V(B,L) F_kB
            for (int i = 0; i < 3; ++i)
                for (int J = 0; J < 3; ++J)
                    for (int k = 0; k < 3; ++k)
                        for (int L = 0; L < 3; ++L) {
                            double s = (i == k) ? S[J][L] : 0.0;
                            for (int Aa = 0; Aa < 3; ++Aa) {
                                const int v1 = voigt(Aa, J);
                                double t = 0.0;
                                for (int B = 0; B < 3; ++B) t += C[v1][voigt(B, L)] * F[k][B];
                                s += F[i][Aa] * t;
                            }
                            sA[((q * 81) + ((i * 3 + J) * 9 + k * 3 + L)) * EPB + el] = R(s);
                        }
        }
    }
    __syncthreads();
    // ---- phase 2: row node M = role
    const int M = role;
    R acc[8][9];
#pragma unroll
    for (int N = 0; N < 8; ++N)
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[N][t] = R(0);
#pragma unroll 1
    for (int q = 0; q < 8; ++q) {
        const R c = sc[q * EPB + el];
        R gM[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) gM[a] = sg[((q * 8 + M) * 3 + a) * EPB + el];
        if (!A.general) {
            const R cl = c * R(lam), cm = c * R(mu);
            R a_[3], b_[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) { a_[i] = cl * gM[i]; b_[i] = cm * gM[i]; }
#pragma unroll
            for (int N = 0; N < 8; ++N) {
                if (N < M) continue;
                R gN[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) gN[a] = sg[((q * 8 + N) * 3 + a) * EPB + el];
                const R db = b_[0] * gN[0] + b_[1] * gN[1] + b_[2] * gN[2];
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k) acc[N][i * 3 + k] += a_[i] * gN[k] + b_[k] * gN[i] + (i == k ? db : R(0));
            }
        } else {
            // h[i][k][L] = c sum_J gM_J A[iJ][kL]
            R h[3][3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k)
#pragma unroll
                    for (int L = 0; L < 3; ++L) {
                        R s = R(0);
#pragma unroll
                        for (int J = 0; J < 3; ++J) s += gM[J] * sA[((q * 81) + ((i * 3 + J) * 9 + k * 3 + L)) * EPB + el];
                        h[i][k][L] = s * c;
                    }
#pragma unroll
            for (int N = 0; N < 8; ++N) {
                if (N < M) continue;
                R gN[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) gN[a] = sg[((q * 8 + N) * 3 + a) * EPB + el];
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int k = 0; k < 3; ++k) acc[N][i * 3 + k] += h[i][k][0] * gN[0] + h[i][k][1] * gN[1] + h[i][k][2] * gN[2];
            }
        }
        if (TI && A.rho) {  // mass per component: the diagonal of each 3x3 block
            const R mM = R(A.mass_w * A.rho[ec] * T.phi[q][M]) * c;
#pragma unroll
            for (int N = 0; N < 8; ++N) {
                if (N < M) continue;
                const R v = mM * R(T.phi[q][N]);
                acc[N][0] += v;
                acc[N][4] += v;
                acc[N][8] += v;
            }
        }
    }
    if (!valid) return;
    R* SK = (R*)A.stageK;
#pragma unroll
    for (int N = 0; N < 8; ++N) {
        if (N < M) continue;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int a = 3 * M + i, b = 3 * N + k;
                if (a <= b) SK[(size_t)e * (NLOC * (NLOC + 1) / 2) + upidx(a, b, NLOC)] = acc[N][i * 3 + k];
            }
    }
    // forces of row node M: -(internal) + body
    double fe[3] = {0.0, 0.0, 0.0};
    if (A.general && (A.with_residual || (TI && A.nfw > 0))) {
        for (int q = 0; q < 8; ++q)
#pragma unroll
            for (int i = 0; i < 3; ++i) fe[i] -= sfq[((q * 8 + M) * 3 + i) * EPB + el];
    }
    if (TI && A.rho) {
        // F[Md+i] += sum_q rho phi_M(q) detJ w (sum_N phi_N(q) h[Nd+i]), in FP64
        double hN[8][3];
        for (int N = 0; N < 8; ++N) {
            const size_t obj = (size_t)A.edof[N * E + e];
            for (int i = 0; i < 3; ++i) hN[N][i] = A.hvec[obj * 3 + i];
        }
        double X[8][3], Ji[3][3];
        for (int i = 0; i < 8; ++i)
            for (int d = 0; d < 3; ++d) X[i][d] = sX[(i * 3 + d) * EPB + el];
        const double rho = A.rho[e];
        for (int q = 0; q < 8; ++q) {
            const double m = rho * jac<8, 3>(X, T.dN[q], Ji) * T.w[q];
            for (int i = 0; i < 3; ++i) {
                double hq = 0.0;
                for (int N = 0; N < 8; ++N) hq += T.phi[q][N] * hN[N][i];
                fe[i] += m * T.phi[q][M] * hq;
            }
        }
    }
    if (A.fnodal) {
        for (int q = 0; q < 8; ++q) {
            double f[3] = {0, 0, 0};
            for (int i = 0; i < 8; ++i) {
                const int node = A.conn[i * E + e];
                for (int d = 0; d < 3; ++d) f[d] += T.N[q][i] * A.fnodal[(size_t)node * 3 + d];
            }
            // detJ w = c (recomputed in FP64 from the geometry)
            double X[8][3], Ji[3][3];
            for (int i = 0; i < 8; ++i)
                for (int d = 0; d < 3; ++d) X[i][d] = sX[(i * 3 + d) * EPB + el];
            const double c = jac<8, 3>(X, T.dN[q], Ji) * T.w[q];
            for (int d = 0; d < 3; ++d) fe[d] += f[d] * T.phi[q][M] * c;
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) A.stageF[(size_t)(3 * M + i) * E + e] = fe[i];
}


// ---------------------------------------------------------------------------
// Linear elasticity (HyperElastic<StVenant> at u = 0) on affine hexahedra,
// one thread per element.  With a constant Jacobian the quadrature sum of
// k_hyper_hex8 factors:
//   W_ik^{MN} = sum_q w_q detJ g_M,i(q) g_N,k(q)
//             = detJ sum_ab Ji[i][a] I_ab^{MN} Ji[k][b],
//   I_ab^{MN} = sum_q w_q dphi_q,M,a dphi_q,N,b   (the reference rule, FP64),
//   K[3M+i][3N+k] = lam W_ik + mu (W_ki + delta_ik tr W)
// -- the same sum in another order: about 2.9k FP64 operations per element
// instead of 7.5k (FP64 runs at 2 operations per clock per SM here).
struct AffineHexTab {
    double I[36][9];  // (M <= N) pairs in row order, [a][b]
    double dN0[8][3];
};

template <typename R>
__global__ void __launch_bounds__(128) k_elast_affine_hex8(const ElemArgs A, const AffineHexTab T) {
    constexpr int NLOC = 24;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int E = A.nelem;
    if (e >= E) return;
    double X[8][3];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int node = A.conn[i * E + e];
#pragma unroll
        for (int d = 0; d < 3; ++d) X[i][d] = A.X[(size_t)node * 3 + d];
    }
    double Ji[3][3];
    const double detJ = jac<8, 3>(X, T.dN0, Ji);
    if (!(detJ > 0.0)) atomicOr(A.flags, 1);
    const double lam = A.coef[e], mu = A.coef[E + e];
    R* SK = (R*)A.stageK;
    int pr = 0;
#pragma unroll 1
    for (int M = 0; M < 8; ++M) {
#pragma unroll 1
        for (int N = M; N < 8; ++N, ++pr) {
            const double* I = T.I[pr];
            double T1[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int b = 0; b < 3; ++b) T1[i][b] = Ji[i][0] * I[b] + Ji[i][1] * I[3 + b] + Ji[i][2] * I[6 + b];
            double W[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) W[i][k] = detJ * (T1[i][0] * Ji[k][0] + T1[i][1] * Ji[k][1] + T1[i][2] * Ji[k][2]);
            const double tr = W[0][0] + W[1][1] + W[2][2];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const int a = 3 * M + i, b = 3 * N + k;
                    if (a <= b) SK[(size_t)e * (NLOC * (NLOC + 1) / 2) + upidx(a, b, NLOC)] = R(lam * W[i][k] + mu * (W[k][i] + (i == k ? tr : 0.0)));
                }
        }
    }
#pragma unroll
    for (int f = 0; f < NLOC; ++f) A.stageF[(size_t)f * E + e] = 0.0;
}

// every hexahedron a parallelepiped (the test of affine<ISL_HEX> on the host)
static bool mesh_is_affine_hex(const isl_ctx* c) {
    const int64_t E = c->nelem;
    for (int64_t e = 0; e < E; ++e) {
        const int64_t* v = &c->hconn[(size_t)e * 8];
        double dev = 0.0, scale = 0.0;
        for (int d = 0; d < 3; ++d) {
            double x[8];
            for (int i = 0; i < 8; ++i) x[i] = c->hX[(size_t)v[i] * 3 + d];
            const double xy = x[0] - x[1] + x[2] - x[3];
            const double xz = x[0] - x[1] - x[4] + x[5];
            const double yz = x[0] - x[3] - x[4] + x[7];
            const double xyz = -x[0] + x[1] - x[2] + x[3] + x[4] - x[5] + x[6] - x[7];
            dev = std::max(dev, std::max(std::max(std::fabs(xy), std::fabs(xz)), std::max(std::fabs(yz), std::fabs(xyz))));
            scale = std::max(scale, std::fabs(x[1] - x[0]) + std::fabs(x[3] - x[0]) + std::fabs(x[4] - x[0]));
        }
        if (!(dev <= 1e-13 * scale)) return false;
    }
    return true;
}

// every element a translate of the first: its three edge vectors from the
// first vertex (hierarchic order 0->1, 0->3, 0->4) equal the first
// element's within 1e-13 of their length, so all the parallelepipeds share
// one Jacobian
static bool mesh_is_uniform_hex(const isl_ctx* c) {
    const int64_t E = c->nelem;
    if (E == 0) return false;
    auto edges = [&](int64_t e, double r[3][3]) {
        const int64_t* v = &c->hconn[(size_t)e * 8];
        const int idx[3] = {1, 3, 4};
        for (int k = 0; k < 3; ++k)
            for (int d = 0; d < 3; ++d) r[k][d] = c->hX[(size_t)v[idx[k]] * 3 + d] - c->hX[(size_t)v[0] * 3 + d];
    };
    double r0[3][3], scale = 0.0;
    edges(0, r0);
    for (int k = 0; k < 3; ++k)
        for (int d = 0; d < 3; ++d) scale = std::max(scale, std::fabs(r0[k][d]));
    for (int64_t e = 1; e < E; ++e) {
        double r[3][3];
        edges(e, r);
        for (int k = 0; k < 3; ++k)
            for (int d = 0; d < 3; ++d)
                if (!(std::fabs(r[k][d] - r0[k][d]) <= 1e-13 * scale)) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Neumann tractions (base/asmb/NeumannForce.hpp:132-174): one thread per
// element owning Neumann faces; f_s += t phi_s(xi(eta)) w |J_s|.
template <int NF, int NCOMP>
struct FaceArgs {
    int nelem, n_neu, nfaces, nsq, nfv, dim;
    const double* X;
    const int32_t* conn;
    const int32_t* neu_elem;
    const int32_t* neu_off;
    const int32_t* neu_face;
    const double* trac;     // [n][NCOMP] per face, or [n][nfv][NCOMP] per face vertex (vert)
    int vert;
    double* stageF;
    int fv[6][4];
    double w[9];
    double S[9][4];         // face geometry functions at the surface points
    double dS[9][4][2];
    double phi[6][9][NF];
};

template <int NF, int NCOMP, int NG, int D>
__global__ void k_neumann(const FaceArgs<NF, NCOMP> A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= A.n_neu) return;
    const int e = A.neu_elem[k];
    const int E = A.nelem;
    double fe[NF][NCOMP];
    for (int s = 0; s < NF; ++s)
        for (int c = 0; c < NCOMP; ++c) fe[s][c] = 0.0;
    for (int j = A.neu_off[k]; j < A.neu_off[k + 1]; ++j) {
        const int f = A.neu_face[j];
        double Xv[4][3];
        for (int v = 0; v < A.nfv; ++v) {
            const int node = A.conn[A.fv[f][v] * E + e];
            for (int d = 0; d < D; ++d) Xv[v][d] = A.X[(size_t)node * D + d];
        }
        for (int q = 0; q < A.nsq; ++q) {
            double Tg[3][2] = {{0, 0}, {0, 0}, {0, 0}};
            for (int v = 0; v < A.nfv; ++v)
                for (int d = 0; d < D; ++d)
                    for (int a = 0; a < D - 1; ++a) Tg[d][a] += Xv[v][d] * A.dS[q][v][a];
            double len;
            if (D == 2) len = sqrt(Tg[0][0] * Tg[0][0] + Tg[1][0] * Tg[1][0]);
            else {
                const double n0 = Tg[1][0] * Tg[2][1] - Tg[2][0] * Tg[1][1];
                const double n1 = Tg[2][0] * Tg[0][1] - Tg[0][0] * Tg[2][1];
                const double n2 = Tg[0][0] * Tg[1][1] - Tg[1][0] * Tg[0][1];
                len = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
            }
            // traction at the point: constant per face, or interpolated from
            // the face vertices by the face geometry functions (exact for a
            // traction linear along a straight face)
            double t[NCOMP];
            for (int c = 0; c < NCOMP; ++c) {
                if (A.vert) {
                    double s = 0.0;
                    for (int v = 0; v < A.nfv; ++v) s += A.S[q][v] * A.trac[((size_t)j * A.nfv + v) * NCOMP + c];
                    t[c] = s;
                } else {
                    t[c] = A.trac[j * NCOMP + c];
                }
            }
            for (int s = 0; s < NF; ++s) {
                const double wgt = A.phi[f][q][s] * A.w[q] * len;
                for (int c = 0; c < NCOMP; ++c) fe[s][c] += t[c] * wgt;
            }
        }
    }
    for (int s = 0; s < NF; ++s)
        for (int c = 0; c < NCOMP; ++c) A.stageF[(size_t)(s * NCOMP + c) * E + e] += fe[s][c];
}

// ---------------------------------------------------------------------------
// Dirichlet lift over elements that own constrained DOFs:
//   F[a] -= sum_c K[a][c] g_c,  g_c = constraint (- current value if incremental)
template <typename R>
__global__ void k_lift(int nlift, const int32_t* lift_elem, int nelem, int nfun, int ncomp, const int32_t* edof,
                       const uint8_t* status, const double* cval, const double* u, int incremental, const R* stageK,
                       double* stageF, int full) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlift) return;
    const int e = lift_elem[k];
    const int nloc = nfun * ncomp;  // <= 30, checked by the host
    if (nloc > 30) return;
    double g[30];
    bool act[30];
    bool any = false;
    for (int a = 0; a < nloc; ++a) {
        const size_t kk = (size_t)edof[(a / ncomp) * nelem + e] * ncomp + a % ncomp;
        act[a] = status[kk] == 0;
        g[a] = act[a] ? 0.0 : (incremental ? cval[kk] - u[kk] : cval[kk]);
        any |= (g[a] != 0.0);
    }
    if (!any) return;
    for (int a = 0; a < nloc; ++a) {
        if (!act[a]) continue;
        double s = 0.0;
        for (int b = 0; b < nloc; ++b) {
            if (act[b] || g[b] == 0.0) continue;
            const size_t kidx = full ? ((size_t)e * nloc + a) * nloc + b
                                     : (size_t)e * (nloc * (nloc + 1) / 2) + (a <= b ? upidx(a, b, nloc) : upidx(b, a, nloc));
            s += (double)stageK[kidx] * g[b];
        }
        stageF[(size_t)a * nelem + e] -= s;
    }
}

// ---------------------------------------------------------------------------
// gather: CSR value of slot s = sum of its staged contributions, in element order
template <typename RS>
__global__ void k_gather_mat(int nnz, const int32_t* __restrict__ seg, const int32_t* __restrict__ src,
                             const RS* __restrict__ stage, double* __restrict__ v64, float* __restrict__ v32) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nnz; s += gridDim.x * blockDim.x) {
        const int lo = seg[s], hi = seg[s + 1];
        RS acc = RS(0);
        for (int k = lo; k < hi; ++k) acc += stage[src[k]];
        if (v64) v64[s] = (double)acc;
        if (v32) v32[s] = (float)acc;
    }
}

__global__ void k_gather_vec(int neq, const int32_t* __restrict__ seg, const int32_t* __restrict__ src,
                             const double* __restrict__ stageF, double* __restrict__ rhs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < neq; i += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int k = seg[i]; k < seg[i + 1]; ++k) acc += stageF[src[k]];
        rhs[i] = acc;
    }
}

// ---------------------------------------------------------------------------
// pattern build kernels
__device__ inline int local_eq(const int32_t* edof, const int32_t* eq, int nelem, int ncomp, int e, int a) {
    return eq[(size_t)edof[(a / ncomp) * nelem + e] * ncomp + a % ncomp];
}

// full: the element stage holds whole nloc x nloc matrices (non-symmetric
// kernels), else packed upper triangles
__global__ void k_gen_pairs(int nelem, int ncomp, int nloc, const int32_t* edof, const int32_t* eq, uint64_t* keys,
                            int32_t* vals, unsigned long long* nvalid, int full) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nelem * nloc) return;
    const int e = (int)(t / nloc), a = (int)(t % nloc);
    const int qa = local_eq(edof, eq, nelem, ncomp, e, a);
    int cnt = 0;
    for (int b = 0; b < nloc; ++b) {
        const int qb = local_eq(edof, eq, nelem, ncomp, e, b);
        const size_t idx = ((size_t)e * nloc + a) * nloc + b;  // element-major: stable sort keeps element order
        if (qa >= 0 && qb >= 0) {
            keys[idx] = ((uint64_t)(uint32_t)qa << 32) | (uint32_t)qb;
            vals[idx] = full ? (int32_t)idx : e * (nloc * (nloc + 1) / 2) + (a <= b ? upidx(a, b, nloc) : upidx(b, a, nloc));
            ++cnt;
        } else {
            keys[idx] = ~0ull;
            vals[idx] = -1;
        }
    }
    if (cnt) atomicAdd(nvalid, (unsigned long long)cnt);
}

__global__ void k_heads(long long n, const uint64_t* keys, int32_t* flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_fill_csr(long long n, const uint64_t* keys, const int32_t* flag, const int32_t* slot, int32_t* colind,
                           int32_t* seg, int32_t* rowptr, int32_t* diag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    const int s = slot[i];
    const uint32_t row = (uint32_t)(keys[i] >> 32), col = (uint32_t)(keys[i] & 0xffffffffu);
    colind[s] = (int32_t)col;
    seg[s] = (int32_t)i;
    if (i == 0 || (uint32_t)(keys[i - 1] >> 32) != row) rowptr[row] = s;
    if (row == col) diag[row] = s;
}

__global__ void k_gen_vec(int nelem, int ncomp, int nloc, const int32_t* edof, const int32_t* eq, uint32_t* keys,
                          int32_t* vals) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nelem * nloc) return;
    const int e = (int)(t / nloc), a = (int)(t % nloc);
    const int q = local_eq(edof, eq, nelem, ncomp, e, a);
    keys[t] = q >= 0 ? (uint32_t)q : 0xffffffffu;
    vals[t] = a * nelem + e;
}

__global__ void k_seg_vec(long long n, const uint32_t* keys, int32_t* seg) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (keys[i] == 0xffffffffu) return;
    if (i == 0 || keys[i] != keys[i - 1]) seg[keys[i]] = (int32_t)i;
}

static int bits_for(uint64_t v) {
    int b = 1;
    while ((1ull << b) <= v) ++b;
    return b;
}

static inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int pattern_build(isl_ctx* c) {
    cudaStream_t st = c->stream;
    cudaEvent_t t0 = c->ev[0], t1 = c->ev[1];
    cudaEventRecord(t0, st);
    const int E = (int)c->nelem, nloc = c->nloc;
    const long long npairs = (long long)E * nloc * nloc;
    if (npairs >= (1ll << 31)) ISL_FAIL(c, ISL_ERR_ARG, "mesh too large for 32-bit contribution lists");
    if ((long long)c->nup * E >= (1ll << 31)) ISL_FAIL(c, ISL_ERR_ARG, "mesh too large for 32-bit staging");
    DBuf<uint64_t> kin, kout;
    DBuf<int32_t> vin;
    DBuf<unsigned long long> dcount;
    ISL_CHECK_CUDA(c, kin.alloc(npairs));
    ISL_CHECK_CUDA(c, kout.alloc(npairs));
    ISL_CHECK_CUDA(c, vin.alloc(npairs));
    ISL_CHECK_CUDA(c, c->dsrc.alloc(npairs));
    ISL_CHECK_CUDA(c, dcount.alloc(1));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(dcount.p, 0, 8, st));
    k_gen_pairs<<<nblk((long long)E * nloc, 256), 256, 0, st>>>(E, c->ncomp, nloc, c->dedof.p, c->deq.p, kin.p, vin.p, dcount.p,
                                                                c->stage_full ? 1 : 0);
    c->pattern_full = c->stage_full;
    c->pattern_serial++;
    ISL_CHECK_CUDA(c, cudaGetLastError());
    const int end_bit = 32 + bits_for((uint64_t)c->neq);
    size_t tmp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, kin.p, kout.p, vin.p, c->dsrc.p, (int)npairs, 0, end_bit, st);
    DBuf<unsigned char> tmp;
    ISL_CHECK_CUDA(c, tmp.alloc(tmp_bytes));
    ISL_CHECK_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, kin.p, kout.p, vin.p, c->dsrc.p, (int)npairs, 0, end_bit, st));
    unsigned long long nvalid = 0;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(&nvalid, dcount.p, 8, cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    kin.release();
    vin.release();
    c->ncontrib = (int64_t)nvalid;
    // heads + exclusive scan -> slot ids
    DBuf<int32_t> flag, slot;
    ISL_CHECK_CUDA(c, flag.alloc(nvalid));
    ISL_CHECK_CUDA(c, slot.alloc(nvalid));
    k_heads<<<nblk(nvalid, 256), 256, 0, st>>>((long long)nvalid, kout.p, flag.p);
    size_t sb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, sb, flag.p, slot.p, (int)nvalid, st);
    if (sb > tmp.n) { ISL_CHECK_CUDA(c, tmp.alloc(sb)); }
    ISL_CHECK_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, sb, flag.p, slot.p, (int)nvalid, st));
    int32_t last_slot = 0, last_flag = 0;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(&last_slot, slot.p + nvalid - 1, 4, cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(&last_flag, flag.p + nvalid - 1, 4, cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    const int64_t nnz = (int64_t)last_slot + last_flag;
    c->nnz = nnz;
    ISL_CHECK_CUDA(c, c->dcolind.alloc(nnz));
    ISL_CHECK_CUDA(c, c->dseg.alloc(nnz + 1));
    ISL_CHECK_CUDA(c, c->drowptr.alloc(c->neq + 1));
    ISL_CHECK_CUDA(c, c->ddiag.alloc(c->neq));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->ddiag.p, 0, c->neq * 4, st));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->drowptr.p, 0xff, (c->neq + 1) * 4, st));
    k_fill_csr<<<nblk(nvalid, 256), 256, 0, st>>>((long long)nvalid, kout.p, flag.p, slot.p, c->dcolind.p, c->dseg.p,
                                                   c->drowptr.p, c->ddiag.p);
    const int32_t tail_seg = (int32_t)nvalid, tail_row = (int32_t)nnz;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dseg.p + nnz, &tail_seg, 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->drowptr.p + c->neq, &tail_row, 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    {
        // every active row owns its diagonal, so every row pointer is set; check
        // monotonicity before any kernel indexes with them
        std::vector<int32_t> rp(c->neq + 1);
        ISL_CHECK_CUDA(c, cudaMemcpy(rp.data(), c->drowptr.p, rp.size() * 4, cudaMemcpyDeviceToHost));
        bool ok = rp[0] == 0 && rp[c->neq] == nnz;
        for (int64_t i = 0; ok && i < c->neq; ++i) ok = rp[i] >= 0 && rp[i] < rp[i + 1];
        if (!ok) ISL_FAIL(c, ISL_ERR_ARG, "pattern build: inconsistent row pointers");
        // kept for sizing the one-cluster solve of small systems
        c->hrp_small.clear();
        if (c->neq <= 65536) c->hrp_small = rp;
        const int brc = block_pattern(c, rp);
        if (brc != ISL_OK) return brc;
        const int src = scalar_sell_pattern(c, rp);
        if (src != ISL_OK) return src;
    }
    kout.release();
    flag.release();
    slot.release();
    // vector contributions (eq <- element local entries), element order within an equation
    const long long nv = (long long)E * nloc;
    DBuf<uint32_t> vk_in, vk_out;
    DBuf<int32_t> vv_in;
    ISL_CHECK_CUDA(c, vk_in.alloc(nv));
    ISL_CHECK_CUDA(c, vk_out.alloc(nv));
    ISL_CHECK_CUDA(c, vv_in.alloc(nv));
    ISL_CHECK_CUDA(c, c->dsrcF.alloc(nv));
    ISL_CHECK_CUDA(c, c->dsegF.alloc(c->neq + 1));
    k_gen_vec<<<nblk(nv, 256), 256, 0, st>>>(E, c->ncomp, nloc, c->dedof.p, c->deq.p, vk_in.p, vv_in.p);
    size_t vb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, vb, vk_in.p, vk_out.p, vv_in.p, c->dsrcF.p, (int)nv, 0, 32, st);
    if (vb > tmp.n) { ISL_CHECK_CUDA(c, tmp.alloc(vb)); }
    ISL_CHECK_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, vb, vk_in.p, vk_out.p, vv_in.p, c->dsrcF.p, (int)nv, 0, 32, st));
    k_seg_vec<<<nblk(nv, 256), 256, 0, st>>>(nv, vk_out.p, c->dsegF.p);
    // number of valid vector contributions = position of the first invalid key
    int64_t nvF = 0;
    {
        std::vector<int32_t> dummy;
        // count on host via the total of active local entries
        std::vector<int32_t> heq = c->heq;
        for (int64_t e = 0; e < c->nelem; ++e)
            for (int a = 0; a < nloc; ++a)
                if (heq[(size_t)c->hedof[e * c->nfun + a / c->ncomp] * c->ncomp + a % c->ncomp] >= 0) ++nvF;
    }
    c->ncontribF = nvF;
    const int32_t tailF = (int32_t)nvF;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dsegF.p + c->neq, &tailF, 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaGetLastError());
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    cudaEventRecord(t1, st);
    cudaEventSynchronize(t1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    c->tms[ISL_T_PATTERN] = ms;
    c->tcount[ISL_T_PATTERN] = 1;
    // staging + system buffers
    ISL_CHECK_CUDA(c, c->dstageF.alloc((size_t)nloc * E));
    ISL_CHECK_CUDA(c, c->drhs.alloc(c->neq));
    ISL_CHECK_CUDA(c, c->dsol.alloc(c->neq));
    c->have64 = c->have32 = false;
    c->solved = false;
    return ISL_OK;
}

// ---------------------------------------------------------------------------

// Autotune of an element kernel's launch shape: on the first assembly of a
// problem class every candidate runs once (each writes the same staged
// values: the per-element arithmetic does not depend on the launch shape),
// timed with CUDA events; the first candidate within 2 % of the fastest, in
// the given preference order, is kept in the tuning cache.  Problems too small
// to time take the first candidate.
template <typename LAUNCH>
static int tune_elem(isl_ctx* c, const char* tuner, const int* cand, int ncand, LAUNCH launch) {
    int v = 0;
    if (tune_lookup(c, tuner, &v))
        for (int k = 0; k < ncand; ++k)
            if (cand[k] == v) return v;
    if (c->nelem < 20000) return cand[0];
    float ms_of[8], best = 1e30f;
    for (int k = 0; k < ncand && k < 8; ++k) {
        cudaEventRecord(c->ev[2], c->stream);
        launch(cand[k]);
        cudaEventRecord(c->ev[3], c->stream);
        cudaEventSynchronize(c->ev[3]);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
        ms_of[k] = ms;
        best = std::min(best, ms);
    }
    c->launches += ncand;
    v = cand[0];
    for (int k = 0; k < ncand && k < 8; ++k)
        if (ms_of[k] <= 1.02f * best) { v = cand[k]; break; }
    tune_store(c, tuner, v);
    return v;
}

template <int SHAPE, int FDEG, int NQ, typename R>
static int launch_laplace(isl_ctx* c, const ElemArgs& A) {
    HostTab h;
    if (!make_host_tables(SHAPE, FDEG, c->qdeg, h) || h.nq != NQ) ISL_FAIL(c, ISL_ERR_ARG, "quadrature");
    Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ> T;
    fill_tab<SHAPE, FDEG, NQ>(T, h);
    const bool ti = A.rho || A.nfw > 0;
    constexpr int D = ET<SHAPE, FDEG>::D, NF = ET<SHAPE, FDEG>::NF;
    TabDF<D, NF, NQ> TD;
    for (int q = 0; q < NQ; ++q)
        for (int f = 0; f < NF; ++f)
            for (int d = 0; d < D; ++d) TD.dphi[q][f][d] = df_from_double(T.dphi[q][f][d]);
    // the mixed assembly (FP64 stage from double-float sums; its FP64 values
    // feed the FP32 copy and the reliable updates); the plain FP64 path keeps
    // FP64 arithmetic
    constexpr bool R64 = std::is_same<R, double>::value;
    const bool dfm = R64 && c->asm_precision == ISL_PREC_MIXED;
    // one thread per element: the threads per block decide the occupancy and
    // the width of the element-major loads
    auto launch = [&](int bs) {
        const unsigned g = nblk(c->nelem, bs);
        if (ti) k_laplace<SHAPE, FDEG, NQ, R, true><<<g, bs, 0, c->stream>>>(A, T, TD);
        else if (dfm) k_laplace<SHAPE, FDEG, NQ, R, false, R64><<<g, bs, 0, c->stream>>>(A, T, TD);
        else k_laplace<SHAPE, FDEG, NQ, R, false><<<g, bs, 0, c->stream>>>(A, T, TD);
    };
    static const int cand[3] = {128, 64, 32};
    char tuner[48];
    std::snprintf(tuner, sizeof tuner, "elem_laplace_q%d_r%d_t%d_d%d", NQ, (int)sizeof(R), ti ? 1 : 0, dfm ? 1 : 0);
    const int bs = tune_elem(c, tuner, cand, 3, launch);
    launch(bs);
    c->elem_variant = bs;
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

template <typename R>
static int dispatch_laplace(isl_ctx* c, const ElemArgs& A) {
    HostTab h;
    if (!make_host_tables(c->shape, c->fedeg, c->qdeg, h)) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    const int nq = h.nq;
    if (c->shape == ISL_QUAD && c->fedeg == 1 && nq == 4) return launch_laplace<ISL_QUAD, 1, 4, R>(c, A);
    if (c->shape == ISL_QUAD && c->fedeg == 1 && nq == 9) return launch_laplace<ISL_QUAD, 1, 9, R>(c, A);
    if (c->shape == ISL_QUAD && c->fedeg == 2 && nq == 9) return launch_laplace<ISL_QUAD, 2, 9, R>(c, A);
    if (c->shape == ISL_QUAD && c->fedeg == 2 && nq == 4) return launch_laplace<ISL_QUAD, 2, 4, R>(c, A);
    if (c->shape == ISL_HEX && c->fedeg == 1 && nq == 8) return launch_laplace<ISL_HEX, 1, 8, R>(c, A);
    if (c->shape == ISL_TET && c->fedeg == 2 && nq == 4) return launch_laplace<ISL_TET, 2, 4, R>(c, A);
    // 11 points: Quadrature<4,TET>, the drivers' 2 x fieldDeg for P2
    if (c->shape == ISL_TET && c->fedeg == 2 && nq == 11) return launch_laplace<ISL_TET, 2, 11, R>(c, A);
    if (c->shape == ISL_TET && c->fedeg == 1 && nq == 1) return launch_laplace<ISL_TET, 1, 1, R>(c, A);
    if (c->shape == ISL_TET && c->fedeg == 1 && nq == 4) return launch_laplace<ISL_TET, 1, 4, R>(c, A);
    ISL_FAIL(c, ISL_ERR_ARG, "Laplace: unsupported element / quadrature combination");
}

template <int SHAPE, int FDEG, int NQ>
static int launch_heat_static(isl_ctx* c, const ElemArgs& A) {
    HostTab h;
    if (!make_host_tables(SHAPE, FDEG, c->qdeg, h) || h.nq != NQ) ISL_FAIL(c, ISL_ERR_ARG, "quadrature");
    Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ> T;
    fill_tab<SHAPE, FDEG, NQ>(T, h);
    k_heat_static<SHAPE, FDEG, NQ><<<nblk(c->nelem, 128), 128, 0, c->stream>>>(A, T);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

static int dispatch_heat_static(isl_ctx* c, ElemArgs A, int with_residual) {
    HostTab h;
    if (!make_host_tables(c->shape, c->fedeg, c->qdeg, h)) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    A.with_residual = with_residual;  // the tangent depends on u even where the residual vanishes
    const int nq = h.nq;
    if (c->shape == ISL_QUAD && c->fedeg == 1 && nq == 4) return launch_heat_static<ISL_QUAD, 1, 4>(c, A);
    if (c->shape == ISL_QUAD && c->fedeg == 1 && nq == 9) return launch_heat_static<ISL_QUAD, 1, 9>(c, A);
    if (c->shape == ISL_QUAD && c->fedeg == 2 && nq == 4) return launch_heat_static<ISL_QUAD, 2, 4>(c, A);
    if (c->shape == ISL_QUAD && c->fedeg == 2 && nq == 9) return launch_heat_static<ISL_QUAD, 2, 9>(c, A);
    if (c->shape == ISL_HEX && c->fedeg == 1 && nq == 8) return launch_heat_static<ISL_HEX, 1, 8>(c, A);
    if (c->shape == ISL_TET && c->fedeg == 1 && nq == 1) return launch_heat_static<ISL_TET, 1, 1>(c, A);
    if (c->shape == ISL_TET && c->fedeg == 2 && nq == 4) return launch_heat_static<ISL_TET, 2, 4>(c, A);
    if (c->shape == ISL_TET && c->fedeg == 2 && nq == 11) return launch_heat_static<ISL_TET, 2, 11>(c, A);
    ISL_FAIL(c, ISL_ERR_ARG, "heat::Static: unsupported element / quadrature combination");
}

template <typename R>
static int dispatch_hyper(isl_ctx* c, const ElemArgs& A) {
    if (!(c->shape == ISL_HEX && c->fedeg == 1)) return hyper_generic(c, A, sizeof(R) == 4);
    HostTab h;
    if (!make_host_tables(ISL_HEX, 1, c->qdeg, h)) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    if (h.nq != 8) return hyper_generic(c, A, sizeof(R) == 4);  // the fast path is written for 2x2x2
    Tab<3, 8, 8, 8> T;
    fill_tab<ISL_HEX, 1, 8>(T, h);
    if (c->mesh_affine < 0) {
        c->mesh_affine = mesh_is_affine_hex(c) ? 1 : 0;
        c->mesh_uniform = (c->mesh_affine == 1 && mesh_is_uniform_hex(c)) ? 1 : 0;
    }
    const bool ti = A.rho || A.nfw > 0;
    if (!A.general && !A.fnodal && !ti && c->mesh_affine == 1) {
        // small strain on parallelepipeds: reference integrals times the constant Jacobian
        AffineHexTab AT;
        int pr = 0;
        for (int M = 0; M < 8; ++M)
            for (int N = M; N < 8; ++N, ++pr)
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        double s = 0.0;
                        for (int q = 0; q < 8; ++q) s += T.w[q] * T.dphi[q][M][a] * T.dphi[q][N][b];
                        AT.I[pr][a * 3 + b] = s;
                    }
        for (int i = 0; i < 8; ++i)
            for (int d = 0; d < 3; ++d) AT.dN0[i][d] = T.dN[0][i][d];
        k_elast_affine_hex8<R><<<nblk(c->nelem, 128), 128, 0, c->stream>>>(A, AT);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        c->launches += 1;
        return ISL_OK;
    }
    // shared memory of a block of epb elements (8 threads each)
    auto smem_of = [&](int epb) {
        return (size_t)8 * 3 * epb * 8 * 2 + (A.general ? (size_t)8 * 8 * 3 * epb * 8 : 0) +
               (size_t)8 * 8 * 3 * epb * sizeof(R) + (size_t)8 * epb * sizeof(R) +
               (A.general ? (size_t)8 * 81 * epb * sizeof(R) : 0);
    };
    auto launch = [&](int epb) {
        const size_t smem = smem_of(epb);
        if (epb == 32) {
            auto kern = ti ? k_hyper_hex8<R, 32, true> : k_hyper_hex8<R, 32, false>;
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<nblk(c->nelem, 32), 32 * 8, smem, c->stream>>>(A, T);
        } else if (epb == 16) {
            auto kern = ti ? k_hyper_hex8<R, 16, true> : k_hyper_hex8<R, 16, false>;
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<nblk(c->nelem, 16), 16 * 8, smem, c->stream>>>(A, T);
        } else {
            auto kern = ti ? k_hyper_hex8<R, 8, true> : k_hyper_hex8<R, 8, false>;
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<nblk(c->nelem, 8), 8 * 8, smem, c->stream>>>(A, T);
        }
    };
    // elements per block: the candidates whose shared memory fits
    int cand[3], ncand = 0;
    for (int epb : {32, 16, 8})
        if (smem_of(epb) <= 200 * 1024) cand[ncand++] = epb;
    char tuner[48];
    std::snprintf(tuner, sizeof tuner, "elem_hex8_r%d_g%d_t%d", (int)sizeof(R), A.general ? 1 : 0, ti ? 1 : 0);
    const int epb = tune_elem(c, tuner, cand, ncand, launch);
    launch(epb);
    c->elem_variant = epb;
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

template <int NF, int NCOMP, int NG, int D>
static int launch_neumann(isl_ctx* c) {
    FaceTab ft;
    if (!make_face_tables(c->shape, c->fedeg, c->sqdeg, ft) || ft.nf != NF || ft.nsq > 9)
        ISL_FAIL(c, ISL_ERR_ARG, "Neumann tables");
    FaceArgs<NF, NCOMP> A;
    memset(&A, 0, sizeof(A));
    A.nelem = (int)c->nelem; A.n_neu = (int)c->n_neu_elem; A.nfaces = ft.nfaces; A.nsq = ft.nsq; A.nfv = ft.nfv; A.dim = D;
    A.X = c->dX.p; A.conn = c->dconn.p; A.neu_elem = c->dneu_elem.p; A.neu_off = c->dneu_off.p; A.neu_face = c->dneu_face.p;
    A.trac = c->dneu_trac.p; A.vert = c->neu_vertex ? 1 : 0; A.stageF = c->dstageF.p;
    for (int f = 0; f < ft.nfaces; ++f)
        for (int v = 0; v < ft.nfv; ++v) A.fv[f][v] = ft.fv[f * ft.nfv + v];
    for (int q = 0; q < ft.nsq; ++q) {
        A.w[q] = ft.w[q];
        for (int v = 0; v < ft.nfv; ++v) A.S[q][v] = ft.S[q * ft.nfv + v];
        for (int v = 0; v < ft.nfv; ++v)
            for (int a = 0; a < D - 1; ++a) A.dS[q][v][a] = ft.dS[(q * ft.nfv + v) * (D - 1) + a];
    }
    for (int f = 0; f < ft.nfaces; ++f)
        for (int q = 0; q < ft.nsq; ++q)
            for (int s = 0; s < NF; ++s) A.phi[f][q][s] = ft.phi[(f * ft.nsq + q) * NF + s];
    k_neumann<NF, NCOMP, NG, D><<<nblk(c->n_neu_elem, 64), 64, 0, c->stream>>>(A);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

static int dispatch_neumann(isl_ctx* c) {
    if (c->shape == ISL_QUAD && c->fedeg == 1 && c->ncomp == 1) return launch_neumann<4, 1, 4, 2>(c);
    if (c->shape == ISL_QUAD && c->fedeg == 1 && c->ncomp == 2) return launch_neumann<4, 2, 4, 2>(c);
    if (c->shape == ISL_QUAD && c->fedeg == 2 && c->ncomp == 1) return launch_neumann<9, 1, 4, 2>(c);
    if (c->shape == ISL_QUAD && c->fedeg == 2 && c->ncomp == 2) return launch_neumann<9, 2, 4, 2>(c);
    if (c->shape == ISL_HEX && c->fedeg == 1 && c->ncomp == 1) return launch_neumann<8, 1, 8, 3>(c);
    if (c->shape == ISL_HEX && c->fedeg == 1 && c->ncomp == 3) return launch_neumann<8, 3, 8, 3>(c);
    if (c->shape == ISL_TET && c->fedeg == 1 && c->ncomp == 1) return launch_neumann<4, 1, 4, 3>(c);
    if (c->shape == ISL_TET && c->fedeg == 1 && c->ncomp == 3) return launch_neumann<4, 3, 4, 3>(c);
    if (c->shape == ISL_TET && c->fedeg == 2 && c->ncomp == 1) return launch_neumann<10, 1, 4, 3>(c);
    if (c->shape == ISL_TET && c->fedeg == 2 && c->ncomp == 3) return launch_neumann<10, 3, 4, 3>(c);
    ISL_FAIL(c, ISL_ERR_ARG, "Neumann: unsupported element");
}

int assemble_device(isl_ctx* c, int precision, int incremental, int with_residual) {
    cudaStream_t st = c->stream;
    c->asm_precision = precision;
    const int E = (int)c->nelem;
    // the tangent (stiffness) is staged in FP32 only for ISL_PREC_FP32 (not for
    // heat::Static, whose kernel runs in FP64 only)
    const bool k32 = (precision == ISL_PREC_FP32) && c->kernel != ISL_KERNEL_HEAT_STATIC;
    const size_t nstage = c->stage_full ? (size_t)c->nloc * c->nloc : (size_t)c->nup;
    if (precision != ISL_PREC_FP32) ISL_CHECK_CUDA(c, c->dval64.alloc(c->nnz));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dflags.p, 0, sizeof(int), st));
    if (c->timing) cudaEventRecord(c->ev[0], st);
    ElemArgs A;
    A.nelem = E;
    A.X = c->dX.p;
    A.conn = c->dconn.p;
    A.edof = c->dedof.p;
    A.coef = c->dcoef.p;
    A.u = c->du.p;
    A.fnodal = c->has_body ? c->dfnodal.p : nullptr;
    A.with_residual = with_residual && c->u_nonzero;
    A.general = c->u_nonzero ? 1 : 0;
    A.material = c->material;
    A.stageK = k32 ? (void*)c->dstageK32.p : (void*)c->dstageK64.p;
    A.stageF = c->dstageF.p;
    A.flags = c->dflags.p;
    A.rho = nullptr;
    A.mass_w = 0.0;
    A.hvec = nullptr;
    A.hist = c->dhist.p;
    A.hstride = c->ndofobj * c->ncomp;
    A.nfw = c->nforce_w;
    for (int k = 0; k < 4; ++k) A.fw[k] = k < c->nforce_w ? c->force_w[k] : 0.0;
    A.kqp = (c->kernel == ISL_KERNEL_LAPLACE && c->has_kqp) ? c->dkqp.p : nullptr;
    // k_lift holds one element's constraint values in fixed arrays of 30
    if (c->n_lift > 0 && c->nloc > 30)
        ISL_FAIL(c, ISL_ERR_ARG, "Dirichlet values on elements with more than 30 local DOFs are not supported");
    // the weights may not reach past the stored history (isl_set_history can
    // shrink it after the weights were set)
    if (c->nforce_w > c->nhist || (c->inertia && c->nhist_w > c->nhist + 1))
        ISL_FAIL(c, ISL_ERR_ARG, "time-integration weights reach past the stored history");
    // past-state forces of HyperElastic go through the finite-strain path
    if (c->nforce_w > 0 && c->kernel == ISL_KERNEL_HYPERELASTIC) A.general = 1;
    if (c->inertia) {
        // h = sum_s w_s x^(s): x^(0) the current values, x^(s) the s-th stored step
        const int64_t ndc = c->ndofobj * c->ncomp;
        ISL_CHECK_CUDA(c, c->dhvec.alloc(ndc));
        k_hist_combine<<<(unsigned)c->sm_count * 8, 256, 0, st>>>(ndc, c->du.p, c->dhist.p, c->nhist_w, c->hist_w[0],
                                                                 c->hist_w[1], c->hist_w[2], c->hist_w[3], c->hist_w[4],
                                                                 c->dhvec.p);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        c->launches += 1;
        A.rho = c->drho.p;
        A.mass_w = c->mass_w;
        A.hvec = c->dhvec.p;
    }
    int rc;
    // mixed precision on parallelepiped hexahedra (small strain, node-blocked):
    // element blocks straight into the FP64 CSR and the FP32 block copies
    if (c->kernel == ISL_KERNEL_HYPERELASTIC && c->mesh_affine < 0 && c->shape == ISL_HEX && c->fedeg == 1) {
        c->mesh_affine = mesh_is_affine_hex(c) ? 1 : 0;
        c->mesh_uniform = (c->mesh_affine == 1 && mesh_is_uniform_hex(c)) ? 1 : 0;
    }
    const bool direct = precision == ISL_PREC_MIXED && c->qdeg == 3 && !c->stage_full && affine_blocks_eligible(c, A);
    if (!direct) {
        if (k32) ISL_CHECK_CUDA(c, c->dstageK32.alloc(nstage * E));
        else ISL_CHECK_CUDA(c, c->dstageK64.alloc(nstage * E));
        if (precision != ISL_PREC_FP64) ISL_CHECK_CUDA(c, c->dval32.alloc(c->nnz));
        A.stageK = k32 ? (void*)c->dstageK32.p : (void*)c->dstageK64.p;
    }
    if (direct) rc = assemble_affine_blocks(c, A);
    else if (c->kernel == ISL_KERNEL_LAPLACE) rc = k32 ? dispatch_laplace<float>(c, A) : dispatch_laplace<double>(c, A);
    else if (c->kernel == ISL_KERNEL_HEAT_STATIC) rc = dispatch_heat_static(c, A, with_residual);
    else rc = k32 ? dispatch_hyper<float>(c, A) : dispatch_hyper<double>(c, A);
    if (rc != ISL_OK) return rc;
    if (c->n_neu_elem > 0) {
        rc = dispatch_neumann(c);
        if (rc != ISL_OK) return rc;
    }
    if (c->n_lift > 0 && direct) {
        rc = affine_lift(c, incremental);
        if (rc != ISL_OK) return rc;
    } else if (c->n_lift > 0) {
        if (k32)
            k_lift<float><<<nblk(c->n_lift, 64), 64, 0, st>>>((int)c->n_lift, c->dlift_elem.p, E, c->nfun, c->ncomp, c->dedof.p,
                                                              c->dstatus.p, c->dcval.p, c->du.p, incremental, c->dstageK32.p, c->dstageF.p,
                                                              c->stage_full ? 1 : 0);
        else
            k_lift<double><<<nblk(c->n_lift, 64), 64, 0, st>>>((int)c->n_lift, c->dlift_elem.p, E, c->nfun, c->ncomp, c->dedof.p,
                                                               c->dstatus.p, c->dcval.p, c->du.p, incremental, c->dstageK64.p, c->dstageF.p,
                                                               c->stage_full ? 1 : 0);
        ISL_CHECK_CUDA(c, cudaGetLastError());
        c->launches += 1;
    }
    if (c->timing) cudaEventRecord(c->ev[1], st);
    const unsigned gblocks = (unsigned)std::min<long long>(nblk(c->nnz, 256), (long long)c->sm_count * 8);
    if (direct) {
        // the values are in place
    } else if (k32) {
        k_gather_mat<float><<<gblocks, 256, 0, st>>>((int)c->nnz, c->dseg.p, c->dsrc.p, c->dstageK32.p, nullptr, c->dval32.p);
        c->launches += 1;
    } else {
        k_gather_mat<double><<<gblocks, 256, 0, st>>>((int)c->nnz, c->dseg.p, c->dsrc.p, c->dstageK64.p, c->dval64.p,
                                                      precision == ISL_PREC_MIXED ? c->dval32.p : nullptr);
        c->launches += 1;
    }
    const unsigned vblocks = (unsigned)std::min<long long>(nblk(c->neq, 256), (long long)c->sm_count * 8);
    k_gather_vec<<<vblocks, 256, 0, st>>>((int)c->neq, c->dsegF.p, c->dsrcF.p, c->dstageF.p, c->drhs.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    if (c->timing) cudaEventRecord(c->ev[2], st);
    int flags = 0;
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(&flags, c->dflags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    if (c->timing) {
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
        c->tms[ISL_T_ELEMENT] += a; c->tcount[ISL_T_ELEMENT]++;
        c->tms[ISL_T_GATHER] += b; c->tcount[ISL_T_GATHER]++;
    }
    c->have64 = (precision != ISL_PREC_FP32);
    c->have32 = (precision != ISL_PREC_FP64);
    c->asm_serial++;
    // the direct path writes the FP32 block copies, not the scalar FP32 CSR
    // values (derived on demand from the FP64 ones)
    if (direct) c->bvals_serial = c->asm_serial;
    else if (c->have32) c->val32_serial = c->asm_serial;
    c->last_direct = direct;
    c->solved = false;
    if (flags & 2) ISL_FAIL(c, ISL_ERR_NAN, "non-finite stress (det F <= 0?)");
    if (flags & 1) ISL_FAIL(c, ISL_ERR_DEGENERATE, "element with det J <= 0");
    return ISL_OK;
}

}  // namespace isl
