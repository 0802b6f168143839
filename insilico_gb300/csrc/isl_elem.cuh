// Element-kernel helpers shared by the assembly translation units: the
// geometry map (Jacobian, inverse transpose, affinity test), the packed
// upper-triangle index, the kernel argument block, the hyperelastic
// material laws and the reference-table upload.  Functions used by element
// math that is also run on the host are __host__ __device__.
#pragma once

#include <cmath>

#include "isl_internal.h"

namespace isl {

// ---------------------------------------------------------------------------
// small helpers
__host__ __device__ inline int upidx(int a, int b, int n) {  // packed upper, row-major, a <= b
    return a * n - (a * (a - 1)) / 2 + (b - a);
}

template <int D>
__host__ __device__ inline double inv_t(const double J[D][D], double Ji[D][D]) {
    // Ji = J^{-T}; returns det J  (signed, as the reference)
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
        // (J^{-1})^T = cofactor(J) / det
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

// Is the geometry map affine (constant Jacobian)?  Tetrahedra always are;
// quads/hexes when their bilinear/trilinear coefficients vanish.
template <int SHAPE, int NG, int D>
__device__ inline bool affine(const double X[NG][D]) {
    if (SHAPE == ISL_TET) return true;
    double scale = 0.0, dev = 0.0;
    for (int d = 0; d < D; ++d) {
        if (SHAPE == ISL_QUAD) {
            const double t = X[0][d] - X[1][d] + X[2][d] - X[3][d];
            dev = fmax(dev, fabs(t));
            scale = fmax(scale, fabs(X[1][d] - X[0][d]) + fabs(X[3][d] - X[0][d]));
        } else {
            // hierarchic hex vertices: 0 c000, 1 c100, 2 c110, 3 c010, 4 c001, 5 c101, 6 c111, 7 c011
            const double xy = X[0][d] - X[1][d] + X[2][d] - X[3][d];
            const double xz = X[0][d] - X[1][d] - X[4][d] + X[5][d];
            const double yz = X[0][d] - X[3][d] - X[4][d] + X[7][d];
            const double xyz = -X[0][d] + X[1][d] - X[2][d] + X[3][d] + X[4][d] - X[5][d] + X[6][d] - X[7][d];
            dev = fmax(dev, fmax(fmax(fabs(xy), fabs(xz)), fmax(fabs(yz), fabs(xyz))));
            scale = fmax(scale, fabs(X[1][d] - X[0][d]) + fabs(X[3][d] - X[0][d]) + fabs(X[4][d] - X[0][d]));
        }
    }
    return dev <= 1e-13 * scale;
}

template <int NG, int D>
__host__ __device__ inline double jac(const double X[NG][D], const double dN[NG][D], double Ji[D][D]) {
    double J[D][D];
    for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) {
            double s = 0.0;
            for (int i = 0; i < NG; ++i) s += X[i][a] * dN[i][b];
            J[a][b] = s;
        }
    return inv_t<D>(J, Ji);
}

struct ElemArgs {
    int nelem;
    const double* X;        // [nnodes][D]
    const int32_t* conn;    // [NG][nelem]
    const int32_t* edof;    // [NF][nelem]
    const double* coef;     // [ncoef][nelem]
    const double* u;        // per dofobj comp
    const double* fnodal;   // [nnodes][ncomp] or null
    int with_residual;
    int general;            // hyperelastic: 1 = finite strain path, 0 = small-strain at u = 0
    int material;
    void* stageK;           // [nup][nelem] (R)
    double* stageF;         // [nloc][nelem]
    int* flags;
    // inertia terms of a multi-step method (base/time/ReactionTerms.hpp):
    // K += mass_w rho M, F += rho M h, h = the weighted DOF history; rho null: none
    const double* rho;      // [nelem]
    double mass_w;
    const double* hvec;     // per dofobj comp
    // residual forces at past states (base/time/ResidualForceHistory.hpp):
    // F -= sum_s fw[s] F_int(x^(s+1)), x^(s+1) = hist[s * hstride + .]
    const double* hist;
    int64_t hstride;
    int nfw;
    double fw[4];
    // heat::Laplace conductivity per quadrature point [nq][nelem] (the
    // conductivity function at the point, heat/Laplace.hpp:119-120); null:
    // one value per element (coef)
    const double* kqp;
};

// direct block assembly of small-strain elasticity on parallelepipeds (isl_blocks.cu)
bool affine_blocks_eligible(const isl_ctx* c, const ElemArgs& A);
int assemble_affine_blocks(isl_ctx* c, const ElemArgs& A);

__host__ __device__ inline int voigt(int i, int j) {  // mat/TensorAlgebra.hpp:141-164
    const int m = (i + 1) * (j + 1);
    return m == 1 ? 0 : m == 4 ? 1 : m == 9 ? 2 : m == 2 ? 3 : m == 3 ? 4 : 5;
}

__host__ __device__ inline void material_eval(int mat, double lam, double mu, const double F[3][3], double S[3][3], double C[6][6]) {
    double Cg[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) Cg[a][b] = F[0][a] * F[0][b] + F[1][a] * F[1][b] + F[2][a] * F[2][b];
    if (mat == ISL_MAT_STVENANT) {
        double E[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) E[a][b] = 0.5 * (Cg[a][b] - (a == b ? 1.0 : 0.0));
        const double tr = E[0][0] + E[1][1] + E[2][2];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) S[a][b] = lam * tr * (a == b ? 1.0 : 0.0) + 2.0 * mu * E[a][b];
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b) C[a][b] = (a < 3 && b < 3) ? lam : 0.0;
        for (int i = 0; i < 3; ++i) C[i][i] += 2.0 * mu;
        for (int i = 3; i < 6; ++i) C[i][i] += mu;
        return;
    }
    double Ci[3][3];
    const double detC = inv_t<3>(Cg, Ci);  // Cg symmetric, so Ci = Cg^{-T} = Cg^{-1}
    (void)detC;
    const double J = F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) - F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
                     F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
    const double lj = log(J);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) S[a][b] = (lam * lj - mu) * Ci[a][b] + mu * (a == b ? 1.0 : 0.0);
    const double f2 = mu - lam * lj;
    for (int A = 0; A < 3; ++A)
        for (int B = A; B < 3; ++B)
            for (int Cc = 0; Cc < 3; ++Cc)
                for (int Dd = Cc; Dd < 3; ++Dd)
                    C[voigt(A, B)][voigt(Cc, Dd)] =
                        lam * Ci[A][B] * Ci[Cc][Dd] + f2 * (Ci[A][Cc] * Ci[B][Dd] + Ci[A][Dd] * Ci[B][Cc]);
}

// status bits of an element kernel (1: det J <= 0, 2: non-finite value)
__host__ __device__ inline void flag_or(int* flags, int v) {
#ifdef __CUDA_ARCH__
    atomicOr(flags, v);
#else
    *flags |= v;
#endif
}

// reference tables (any size) into the fixed-size table of a kernel
template <int SHAPE, int FDEG, int NQ>
inline void fill_tab(Tab<ET<SHAPE, FDEG>::D, ET<SHAPE, FDEG>::NG, ET<SHAPE, FDEG>::NF, NQ>& T, const HostTab& h) {
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

// HyperElastic element kernels outside the trilinear-hexahedron fast path:
// quadrilaterals (plane strain), tetrahedra, hexahedra with other rules
// (isl_hyper.cu).  k32: FP32 staging.
int hyper_generic(isl_ctx* c, const ElemArgs& A, bool k32);

}  // namespace isl
