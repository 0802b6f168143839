// solid::HyperElastic element kernels outside the trilinear-hexahedron fast
// path of isl_assembly.cu (k_hyper_hex8): quadrilaterals Q1 / Q2 in plane
// strain, tetrahedra Q1 / Q2 (P1 / P2) and trilinear hexahedra with rules
// other than 2x2x2.  These serve the reference's 2-D examples and meshes of
// other shapes; they are parity paths, not throughput paths.
#include "isl_elem.cuh"

namespace isl {

// ---------------------------------------------------------------------------
// One thread per element, FP64 throughout.  In D = 2 the 2x2 displacement
// gradient sits in a 3x3 deformation gradient with F_33 = 1 (plane strain,
// solid/Deformation.hpp:25-46) and the materials are evaluated in 3-D; the
// tangent and residual then use the in-plane indices only.
//   K[Md+i, Nd+k] += sum_JL g_M,J (d_ik S_JL + F_iA C_AJBL F_kB) g_N,L detJ w
//                                        solid/HyperElastic.hpp:110-179,282-310
//   F[Md+i]       -= sum_J (F S)_iJ g_M,J detJ w   solid/HyperElastic.hpp:209-257
//   F[Md+i]       += f_i(x) phi_M detJ w           base/asmb/BodyForce.hpp:172-205
// TI adds the time-integration terms of a vector field:
//   K[Md+i, Nd+i] += mass_w rho phi_M phi_N detJ w       base/kernel/Mass.hpp:72-101
//   F[Md+i]       += rho phi_M detJ w sum_N phi_N h[Nd+i] base/time/ReactionTerms.hpp
//   F[Md+i]       -= sum_s fw_s (F_s S_s)_iJ g_M,J detJ w at the past state s
//                                        base/time/ResidualForceHistory.hpp
// The element matrix is accumulated in the element's own staging slice
// (upper triangle, element-major) instead of registers: a P2 tetrahedron
// has 465 entries.  The function also runs on the host, which is how its
// arithmetic was checked against the oracle before its first device run.
template <int SHAPE, int FDEG, int NQ, typename R, bool TI>
__host__ __device__ inline void hyper_element(
    const ElemArgs& A, const Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ>& T, int e) {
    constexpr int D = ET<SHAPE, FDEG>::D, NG = ET<SHAPE, FDEG>::NG, NF = ET<SHAPE, FDEG>::NF;
    constexpr int NLOC = D * NF, NUP = NLOC * (NLOC + 1) / 2;
    const int E = A.nelem;
    double X[NG][D];
    int nodes[NG];
    for (int i = 0; i < NG; ++i) {
        nodes[i] = A.conn[i * E + e];
        for (int d = 0; d < D; ++d) X[i][d] = A.X[(size_t)nodes[i] * D + d];
    }
    int obj[NF];
    double uloc[NF][D];
    for (int f = 0; f < NF; ++f) {
        obj[f] = A.edof[f * E + e];
        for (int i = 0; i < D; ++i) uloc[f][i] = A.u[(size_t)obj[f] * D + i];
    }
    const double lam = A.coef[e], mu = A.coef[E + e];
    const bool mass = TI && A.rho;
    const double rho = mass ? A.rho[e] : 0.0;
    R* SK = (R*)A.stageK + (size_t)e * NUP;
    for (int u = 0; u < NUP; ++u) SK[u] = R(0);
    double fe[NLOC];
    for (int a = 0; a < NLOC; ++a) fe[a] = 0.0;
    bool bad = false, nan = false;
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        double Ji[D][D];
        const double detJ = jac<NG, D>(X, T.dN[q], Ji);
        bad |= !(detJ > 0.0);
        const double c = detJ * T.w[q];
        double g[NF][D];
        for (int M = 0; M < NF; ++M)
            for (int a = 0; a < D; ++a) {
                double s = 0.0;
                for (int b = 0; b < D; ++b) s += Ji[a][b] * T.dphi[q][M][b];
                g[M][a] = s;
            }
        double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int f = 0; f < NF; ++f)
            for (int i = 0; i < D; ++i)
                for (int J = 0; J < D; ++J) F[i][J] += g[f][J] * uloc[f][i];
        double S[3][3], C[6][6];
        material_eval(A.material, lam, mu, F, S, C);
        // effective elasticity Ae[i][J][k][L] = d_ik S_JL + F_iA C_V(A,J)V(B,L) F_kB
        double Ae[D][D][D][D];
        for (int i = 0; i < D; ++i)
            for (int J = 0; J < D; ++J)
                for (int k = 0; k < D; ++k)
                    for (int L = 0; L < D; ++L) {
                        double v = (i == k) ? S[J][L] : 0.0;
                        for (int Aa = 0; Aa < D; ++Aa) {
                            double t = 0.0;
                            for (int B = 0; B < D; ++B) t += C[voigt(Aa, J)][voigt(B, L)] * F[k][B];
                            v += F[i][Aa] * t;
                        }
                        Ae[i][J][k][L] = v;
                    }
#pragma unroll 1
        for (int M = 0; M < NF; ++M)
            for (int i = 0; i < D; ++i) {
                const int a = D * M + i;
                double h[D][D];  // c sum_J g_M,J Ae[i][J][k][L]
                for (int k = 0; k < D; ++k)
                    for (int L = 0; L < D; ++L) {
                        double s = 0.0;
                        for (int J = 0; J < D; ++J) s += g[M][J] * Ae[i][J][k][L];
                        h[k][L] = c * s;
                    }
                const double mM = mass ? A.mass_w * rho * c * T.phi[q][M] : 0.0;
#pragma unroll 1
                for (int N = M; N < NF; ++N)
                    for (int k = 0; k < D; ++k) {
                        const int b = D * N + k;
                        if (b < a) continue;
                        double v = 0.0;
                        for (int L = 0; L < D; ++L) v += h[k][L] * g[N][L];
                        if (mass && i == k) v += mM * T.phi[q][N];
                        SK[upidx(a, b, NLOC)] += R(v);
                    }
            }
        if (A.with_residual) {
            for (int M = 0; M < NF; ++M)
                for (int i = 0; i < D; ++i) {
                    double v = 0.0;
                    for (int J = 0; J < D; ++J) v += (F[i][0] * S[0][J] + F[i][1] * S[1][J] + F[i][2] * S[2][J]) * g[M][J];
                    v *= c;
                    nan |= !(v == v);
                    fe[D * M + i] -= v;
                }
        }
        if (TI) {
            for (int sidx = 0; sidx < A.nfw; ++sidx) {  // residual force at a past state
                double Fh[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
                for (int f = 0; f < NF; ++f)
                    for (int i = 0; i < D; ++i) {
                        const double uf = A.hist[(size_t)sidx * A.hstride + (size_t)obj[f] * D + i];
                        for (int J = 0; J < D; ++J) Fh[i][J] += g[f][J] * uf;
                    }
                double Sh[3][3], Ch[6][6];
                material_eval(A.material, lam, mu, Fh, Sh, Ch);
                for (int M = 0; M < NF; ++M)
                    for (int i = 0; i < D; ++i) {
                        double v = 0.0;
                        for (int J = 0; J < D; ++J)
                            v += (Fh[i][0] * Sh[0][J] + Fh[i][1] * Sh[1][J] + Fh[i][2] * Sh[2][J]) * g[M][J];
                        v *= A.fw[sidx] * c;
                        nan |= !(v == v);
                        fe[D * M + i] -= v;
                    }
            }
            if (mass) {  // M h, h the weighted history
                double hq[D];
                for (int i = 0; i < D; ++i) hq[i] = 0.0;
                for (int f = 0; f < NF; ++f)
                    for (int i = 0; i < D; ++i) hq[i] += T.phi[q][f] * A.hvec[(size_t)obj[f] * D + i];
                for (int M = 0; M < NF; ++M)
                    for (int i = 0; i < D; ++i) fe[D * M + i] += rho * c * T.phi[q][M] * hq[i];
            }
        }
        if (A.fnodal) {
            double fx[D];
            for (int d = 0; d < D; ++d) fx[d] = 0.0;
            for (int i = 0; i < NG; ++i)
                for (int d = 0; d < D; ++d) fx[d] += T.N[q][i] * A.fnodal[(size_t)nodes[i] * D + d];
            for (int M = 0; M < NF; ++M)
                for (int d = 0; d < D; ++d) fe[D * M + d] += fx[d] * T.phi[q][M] * c;
        }
    }
    if (bad) flag_or(A.flags, 1);
    if (nan) flag_or(A.flags, 2);
    for (int a = 0; a < NLOC; ++a) A.stageF[(size_t)a * E + e] = fe[a];
}

template <int SHAPE, int FDEG, int NQ, typename R, bool TI>
__global__ void __launch_bounds__(128)
    k_hyper_elem(const ElemArgs A, const Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ> T) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < A.nelem) hyper_element<SHAPE, FDEG, NQ, R, TI>(A, T, e);
}

namespace {

template <int SHAPE, int FDEG, int NQ, typename R>
int launch(isl_ctx* c, const ElemArgs& A, const HostTab& h) {
    Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ> T;
    fill_tab<SHAPE, FDEG, NQ>(T, h);
    const unsigned grid = (unsigned)((c->nelem + 127) / 128);
    if (A.rho || A.nfw > 0)
        k_hyper_elem<SHAPE, FDEG, NQ, R, true><<<grid, 128, 0, c->stream>>>(A, T);
    else
        k_hyper_elem<SHAPE, FDEG, NQ, R, false><<<grid, 128, 0, c->stream>>>(A, T);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

template <typename R>
int dispatch(isl_ctx* c, const ElemArgs& A) {
    HostTab h;
    if (!make_host_tables(c->shape, c->fedeg, c->qdeg, h)) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    const int s = c->shape, k = c->fedeg, nq = h.nq;
    if (s == ISL_QUAD && k == 1 && nq == 4) return launch<ISL_QUAD, 1, 4, R>(c, A, h);
    if (s == ISL_QUAD && k == 1 && nq == 9) return launch<ISL_QUAD, 1, 9, R>(c, A, h);
    if (s == ISL_QUAD && k == 2 && nq == 4) return launch<ISL_QUAD, 2, 4, R>(c, A, h);
    if (s == ISL_QUAD && k == 2 && nq == 9) return launch<ISL_QUAD, 2, 9, R>(c, A, h);
    if (s == ISL_TET && k == 1 && nq == 1) return launch<ISL_TET, 1, 1, R>(c, A, h);
    if (s == ISL_TET && k == 1 && nq == 4) return launch<ISL_TET, 1, 4, R>(c, A, h);
    if (s == ISL_TET && k == 2 && nq == 1) return launch<ISL_TET, 2, 1, R>(c, A, h);
    if (s == ISL_TET && k == 2 && nq == 4) return launch<ISL_TET, 2, 4, R>(c, A, h);
    if (s == ISL_TET && k == 2 && nq == 11) return launch<ISL_TET, 2, 11, R>(c, A, h);
    if (s == ISL_HEX && k == 1 && nq == 27) return launch<ISL_HEX, 1, 27, R>(c, A, h);
    ISL_FAIL(c, ISL_ERR_ARG,
             "HyperElastic: Q1 / Q2 quadrilaterals (2x2, 3x3), P1 / P2 tetrahedra (1, 4 points; 11 for P2) or "
             "trilinear hexahedra (2x2x2, 3x3x3) on the device");
}

}  // namespace

int hyper_generic(isl_ctx* c, const ElemArgs& A, bool k32) { return k32 ? dispatch<float>(c, A) : dispatch<double>(c, A); }

}  // namespace isl
