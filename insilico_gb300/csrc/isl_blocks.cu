// Small-strain elasticity on parallelepiped hexahedra, assembled straight
// into the node-blocked matrix: the mixed-precision assembly of
// solid::HyperElastic<StVenant> at u = 0 (solid/HyperElastic.hpp:110-179,
// mat/hypel/StVenant.hpp:77-114; = mat::Lame linear elasticity).
//
// With a constant Jacobian the quadrature sum of an element block factors
// into reference integrals (the same factorisation as k_elast_affine_hex8):
//   W^{MN}_ik = detJ sum_ab Ji[i][a] I^{MN}_ab Ji[k][b],
//   I^{MN}_ab = sum_q w_q dphi_q,M,a dphi_q,N,b   (the reference rule),
//   K[3M+i][3N+k] = lam W_ik + mu (W_ki + delta_ik tr W).
// Instead of staging every element matrix and gathering the CSR values from
// element-to-slot lists, one thread owns one stored 3x3 block (o, c) of the
// matrix: it walks the elements shared by DOF objects o and c in increasing
// element order (the order in which the reference's triplet store adds them,
// base/solver/TripletContainer.hpp:305-352), adds their blocks K^{MN} and
// writes the block once: FP64 CSR values and the FP32 block copies the
// solver reads.  The arithmetic is double-float on the FP32 pipe (about 48
// significant bits; GB300 runs FP32 at about 64 times its FP64 rate), and one
// FP64 addition per value forms the FP64 entry.  Threads follow the slots of
// the sliced-ELL block copy, so its writes are coalesced.
//
// The Dirichlet lift (base/asmb/assembleMatrix.hpp:91-96) needs the columns
// of constrained DOFs, which have no stored block: k_affine_lift recomputes
// them in FP64 on the elements that own constrained DOFs.
#include <algorithm>
#include <vector>

#include "isl_df.cuh"
#include "isl_elem.cuh"
#include "isl_internal.h"

namespace isl {

namespace {

constexpr int GEO_F4 = 10;  // per element: G = detJ Ji (9 df), Ji (9 df), lam, mu -> 20 df = 10 float4

// reference integrals of the 2x2x2 rule for every (M, N), double-float and FP64
struct AffinePairs {
    df I[64][9];
    double I64[64][9];
    double dN0[8][3];
};

__device__ __forceinline__ df ldf(const float4* p, int k) {  // k-th double-float of a float4 array
    const float4 v = p[k >> 1];
    return (k & 1) ? df{v.z, v.w} : df{v.x, v.y};
}

// per element: the Jacobian at the first quadrature point (constant on a
// parallelepiped), its inverse transpose and det J in FP64, stored as
// double-float with the element's Lame parameters
__global__ void k_affine_geo(int E, int nel, const double* __restrict__ X, const int32_t* __restrict__ conn,
                             const double* __restrict__ coef, AffinePairs T, float4* __restrict__ geo, int* flags) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // the first nel of the E elements
    if (e >= nel) return;
    double Xe[8][3];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int node = conn[i * E + e];
#pragma unroll
        for (int d = 0; d < 3; ++d) Xe[i][d] = X[(size_t)node * 3 + d];
    }
    double Ji[3][3];
    const double detJ = jac<8, 3>(Xe, T.dN0, Ji);
    if (!(detJ > 0.0)) atomicOr(flags, 1);
    df v[20];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            v[i * 3 + a] = df_from_double(detJ * Ji[i][a]);
            v[9 + i * 3 + a] = df_from_double(Ji[i][a]);
        }
    v[18] = df_from_double(coef[e]);
    v[19] = df_from_double(coef[E + e]);
    float4* g = geo + (size_t)e * GEO_F4;
#pragma unroll
    for (int k = 0; k < GEO_F4; ++k) g[k] = make_float4(v[2 * k].hi, v[2 * k].lo, v[2 * k + 1].hi, v[2 * k + 1].lo);
}

// per element: lam and mu as double-float (lam.hi, lam.lo, mu.hi, mu.lo), the
// values k_affine_geo stores in the last float4 of its record; on a mesh of
// translates of one element the geometry record of element 0 is all the
// block kernel reads besides these
__global__ void k_affine_lame(int E, const double* __restrict__ coef, float4* __restrict__ lame) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
        const df lam = df_from_double(coef[e]), mu = df_from_double(coef[E + e]);
        lame[e] = make_float4(lam.hi, lam.lo, mu.hi, mu.lo);
    }
}

struct BlockArgs {
    int nslot, nblk;
    const int* sblk;      // block of every sliced-ELL slot, -1 for padding
    const int* brow;
    const int* bptr;
    const int* bcol;
    const int* brobj;     // DOF object of every block row
    const int* adj_off;   // DOF object -> its elements: (element << 3 | local vertex), by element
    const int* adj;
    const int* rowptr;
    const float4* geo;
    const float4* lame;   // per element lam, mu (k_affine_blocks_u)
    double* v64;
    float* sv;            // [slot/32][9][32]
    float* bv;            // [9][nblk] block-row copy, or null
};

__global__ void __launch_bounds__(256) k_affine_blocks(BlockArgs P, AffinePairs T) {
    __shared__ df sI[64][9];
    for (int k = threadIdx.x; k < 64 * 9; k += blockDim.x) sI[k / 9][k % 9] = T.I[k / 9][k % 9];
    __syncthreads();
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < P.nslot; s += gridDim.x * blockDim.x) {
        const int b = P.sblk[s];
        if (b < 0) continue;  // padding slot: its values stay 0
        const int br = P.brow[b], bc = P.bcol[b], j = b - P.bptr[br];
        const int o = P.brobj[br], c = P.brobj[bc];
        int ia = P.adj_off[o];
        const int ea = P.adj_off[o + 1];
        int ib = P.adj_off[c];
        const int eb = P.adj_off[c + 1];
        df acc[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] = df{0.f, 0.f};
        while (ia < ea && ib < eb) {
            const int va = P.adj[ia], vb = P.adj[ib];
            const int e1 = va >> 3, e2 = vb >> 3;
            if (e1 != e2) {
                if (e1 < e2) ++ia; else ++ib;
                continue;
            }
            ++ia;
            ++ib;
            const int pr = (va & 7) * 8 + (vb & 7);
            const float4* g = P.geo + (size_t)e1 * GEO_F4;
            df G[9], Ji[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) { G[k] = ldf(g, k); Ji[k] = ldf(g, 9 + k); }
            const df lam = ldf(g, 18), mu = ldf(g, 19);
            // T1 = G I, W = T1 Ji^T
            df T1[9];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int bb = 0; bb < 3; ++bb)
                    T1[i * 3 + bb] = df_add(df_add(df_mul(G[i * 3], sI[pr][bb]), df_mul(G[i * 3 + 1], sI[pr][3 + bb])),
                                            df_mul(G[i * 3 + 2], sI[pr][6 + bb]));
            df W[9];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    W[i * 3 + k] = df_add(df_add(df_mul(T1[i * 3], Ji[k * 3]), df_mul(T1[i * 3 + 1], Ji[k * 3 + 1])),
                                          df_mul(T1[i * 3 + 2], Ji[k * 3 + 2]));
            const df tr = df_add(df_add(W[0], W[4]), W[8]);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    df m = W[k * 3 + i];
                    if (i == k) m = df_add(m, tr);
                    acc[i * 3 + k] = df_add_acc(acc[i * 3 + k], df_add(df_mul(lam, W[i * 3 + k]), df_mul(mu, m)));
                }
        }
        const size_t g = (size_t)s >> 5, l = (size_t)s & 31;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double* out = P.v64 + P.rowptr[3 * br + r] + 3 * j;
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                const df v = acc[r * 3 + cc];
                out[cc] = df_to_double(v);
                P.sv[(g * 9 + r * 3 + cc) * 32 + l] = v.hi;
                if (P.bv) P.bv[(size_t)(r * 3 + cc) * P.nblk + b] = v.hi;
            }
        }
    }
}

// The same blocks on a mesh whose elements all share the first element's
// geometry (translates of one parallelepiped): the 64 local pairs' Lame
// blocks W_ab (the lambda part) and W_ab^T + tr(W_ab) I (the mu part) are
// formed once per CTA in shared memory, from the first element's G and Ji,
// and each (block, element) pair adds lam_e WL + mu_e WM in double-float
// (36 operations instead of about 130).  Element order and the final
// expression per entry are those of k_affine_blocks.
__global__ void __launch_bounds__(256) k_affine_blocks_u(BlockArgs P, AffinePairs T) {
    __shared__ df sL[64][9], sM[64][9];
    if (threadIdx.x < 64) {
        const int pr = threadIdx.x;
        df G[9], Ji[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) { G[k] = ldf(P.geo, k); Ji[k] = ldf(P.geo, 9 + k); }
        df T1[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int bb = 0; bb < 3; ++bb)
                T1[i * 3 + bb] = df_add(df_add(df_mul(G[i * 3], T.I[pr][bb]), df_mul(G[i * 3 + 1], T.I[pr][3 + bb])),
                                        df_mul(G[i * 3 + 2], T.I[pr][6 + bb]));
        df W[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                W[i * 3 + k] = df_add(df_add(df_mul(T1[i * 3], Ji[k * 3]), df_mul(T1[i * 3 + 1], Ji[k * 3 + 1])),
                                      df_mul(T1[i * 3 + 2], Ji[k * 3 + 2]));
        const df tr = df_add(df_add(W[0], W[4]), W[8]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                df m = W[k * 3 + i];
                if (i == k) m = df_add(m, tr);
                sL[pr][i * 3 + k] = W[i * 3 + k];
                sM[pr][i * 3 + k] = m;
            }
    }
    __syncthreads();
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < P.nslot; s += gridDim.x * blockDim.x) {
        const int b = P.sblk[s];
        if (b < 0) continue;  // padding slot: its values stay 0
        const int br = P.brow[b], bc = P.bcol[b], j = b - P.bptr[br];
        const int o = P.brobj[br], c = P.brobj[bc];
        int ia = P.adj_off[o];
        const int ea = P.adj_off[o + 1];
        int ib = P.adj_off[c];
        const int eb = P.adj_off[c + 1];
        df acc[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] = df{0.f, 0.f};
        while (ia < ea && ib < eb) {
            const int va = P.adj[ia], vb = P.adj[ib];
            const int e1 = va >> 3, e2 = vb >> 3;
            if (e1 != e2) {
                if (e1 < e2) ++ia; else ++ib;
                continue;
            }
            ++ia;
            ++ib;
            const int pr = (va & 7) * 8 + (vb & 7);
            const float4 lm = __ldg(P.lame + e1);
            const df lam = {lm.x, lm.y}, mu = {lm.z, lm.w};
#pragma unroll
            for (int k = 0; k < 9; ++k)
                acc[k] = df_add_acc(acc[k], df_add(df_mul(lam, sL[pr][k]), df_mul(mu, sM[pr][k])));
        }
        const size_t g = (size_t)s >> 5, l = (size_t)s & 31;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double* out = P.v64 + P.rowptr[3 * br + r] + 3 * j;
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) {
                const df v = acc[r * 3 + cc];
                out[cc] = df_to_double(v);
                P.sv[(g * 9 + r * 3 + cc) * 32 + l] = v.hi;
                if (P.bv) P.bv[(size_t)(r * 3 + cc) * P.nblk + b] = v.hi;
            }
        }
    }
}

// Dirichlet lift of the listed elements (those owning constrained DOFs):
// F[a] -= sum_c K[a][c] g_c over active a and constrained c, with
// g_c = constraint (- current value when incremental); K in FP64 from the
// same factorisation.
__global__ void k_affine_lift(int nlift, const int32_t* __restrict__ lift_elem, int E, const double* __restrict__ X,
                              const int32_t* __restrict__ conn, const int32_t* __restrict__ edof,
                              const uint8_t* __restrict__ status, const double* __restrict__ cval,
                              const double* __restrict__ u, int incremental, const double* __restrict__ coef,
                              AffinePairs T, double* __restrict__ stageF) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nlift) return;
    const int e = lift_elem[k];
    double g[24];
    bool act[24];
    bool any = false;
    for (int a = 0; a < 24; ++a) {
        const size_t kk = (size_t)edof[(a / 3) * E + e] * 3 + a % 3;
        act[a] = status[kk] == 0;
        g[a] = act[a] ? 0.0 : (incremental ? cval[kk] - u[kk] : cval[kk]);
        any |= (g[a] != 0.0);
    }
    if (!any) return;
    double Xe[8][3], Ji[3][3];
    for (int i = 0; i < 8; ++i) {
        const int node = conn[i * E + e];
        for (int d = 0; d < 3; ++d) Xe[i][d] = X[(size_t)node * 3 + d];
    }
    const double detJ = jac<8, 3>(Xe, T.dN0, Ji);
    const double lam = coef[e], mu = coef[E + e];
    for (int M = 0; M < 8; ++M)
        for (int N = 0; N < 8; ++N) {
            bool need = false;
            for (int kk = 0; kk < 3; ++kk) need |= !act[3 * N + kk] && g[3 * N + kk] != 0.0;
            if (!need) continue;
            const double* I = T.I64[M * 8 + N];
            double T1[3][3], W[3][3];
            for (int i = 0; i < 3; ++i)
                for (int bb = 0; bb < 3; ++bb) T1[i][bb] = Ji[i][0] * I[bb] + Ji[i][1] * I[3 + bb] + Ji[i][2] * I[6 + bb];
            for (int i = 0; i < 3; ++i)
                for (int kk = 0; kk < 3; ++kk)
                    W[i][kk] = detJ * (T1[i][0] * Ji[kk][0] + T1[i][1] * Ji[kk][1] + T1[i][2] * Ji[kk][2]);
            const double tr = W[0][0] + W[1][1] + W[2][2];
            for (int i = 0; i < 3; ++i) {
                const int a = 3 * M + i;
                if (!act[a]) continue;
                double s = 0.0;
                for (int kk = 0; kk < 3; ++kk) {
                    const int cidx = 3 * N + kk;
                    if (act[cidx] || g[cidx] == 0.0) continue;
                    s += (lam * W[i][kk] + mu * (W[kk][i] + (i == kk ? tr : 0.0))) * g[cidx];
                }
                stageF[(size_t)a * E + e] -= s;
            }
        }
}

__global__ void k_slot_block(int nblk, const int* __restrict__ sdst, int* __restrict__ sblk) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nblk; b += gridDim.x * blockDim.x) sblk[sdst[b]] = b;
}

__global__ void k_d2f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

int fill_pairs(isl_ctx* c, AffinePairs& T) {
    HostTab h;
    if (!make_host_tables(ISL_HEX, 1, c->qdeg, h) || h.nq != 8) ISL_FAIL(c, ISL_ERR_ARG, "quadrature degree");
    for (int M = 0; M < 8; ++M)
        for (int N = 0; N < 8; ++N)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    double s = 0.0;
                    for (int q = 0; q < 8; ++q) s += h.w[q] * h.dphi[((size_t)q * 8 + M) * 3 + a] * h.dphi[((size_t)q * 8 + N) * 3 + b];
                    T.I64[M * 8 + N][a * 3 + b] = s;
                    T.I[M * 8 + N][a * 3 + b] = df_from_double(s);
                }
    for (int i = 0; i < 8; ++i)
        for (int d = 0; d < 3; ++d) T.dN0[i][d] = h.dN[(size_t)i * 3 + d];
    return ISL_OK;
}

// once per numbering: DOF object of every block row, the DOF objects'
// element lists, and the block of every sliced-ELL slot
int ensure_block_maps(isl_ctx* c) {
    if (c->bmap_serial == c->pattern_serial) return ISL_OK;
    const int64_t nobj = c->ndofobj, E = c->nelem;
    std::vector<int32_t> brobj((size_t)c->nbr, -1);
    for (int64_t o = 0; o < nobj; ++o) {
        const int32_t q = c->heq[(size_t)o * 3];
        if (q >= 0) brobj[q / 3] = (int32_t)o;
    }
    std::vector<int32_t> off((size_t)nobj + 1, 0), adj((size_t)E * 8);
    for (int64_t e = 0; e < E; ++e)
        for (int a = 0; a < 8; ++a) off[(size_t)c->hedof[(size_t)e * 8 + a] + 1]++;
    for (int64_t o = 0; o < nobj; ++o) off[o + 1] += off[o];
    std::vector<int32_t> pos(off.begin(), off.end() - 1);
    for (int64_t e = 0; e < E; ++e)  // elements in increasing order: each list is sorted
        for (int a = 0; a < 8; ++a) adj[pos[(size_t)c->hedof[(size_t)e * 8 + a]]++] = (int32_t)((e << 3) | a);
    cudaStream_t st = c->stream;
    ISL_CHECK_CUDA(c, c->dbrobj.alloc(brobj.size()));
    ISL_CHECK_CUDA(c, c->dadj_off.alloc(off.size()));
    ISL_CHECK_CUDA(c, c->dadj.alloc(adj.size()));
    ISL_CHECK_CUDA(c, c->dsblk.alloc((size_t)c->nslot));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dbrobj.p, brobj.data(), brobj.size() * 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dadj_off.p, off.data(), off.size() * 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaMemcpyAsync(c->dadj.p, adj.data(), adj.size() * 4, cudaMemcpyHostToDevice, st));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dsblk.p, 0xFF, (size_t)c->nslot * 4, st));
    k_slot_block<<<(unsigned)c->sm_count * 8, 256, 0, st>>>((int)c->nblk, c->dsdst.p, c->dsblk.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    ISL_CHECK_CUDA(c, cudaStreamSynchronize(st));
    c->launches += 1;
    c->bmap_serial = c->pattern_serial;
    return ISL_OK;
}

}  // namespace

// The path applies to node-blocked systems of trilinear parallelepipeds with
// the small-strain StVenant kernel at u = 0 (no body force, no
// time-integration terms), 2x2x2 points, when the block solver is in use.
bool affine_blocks_eligible(const isl_ctx* c, const ElemArgs& A) {
    return c->kernel == ISL_KERNEL_HYPERELASTIC && c->shape == ISL_HEX && c->fedeg == 1 && c->ncomp == 3 &&
           c->blocked && !c->bpad && c->use_block && c->ninst == 1 && !A.general && !A.fnodal && !A.rho && A.nfw == 0 &&
           c->mesh_affine == 1 && c->nfun == 8 && c->nelem < (1 << 28) && c->nslot < INT32_MAX;
}

// Element blocks straight into the FP64 CSR and the FP32 block copies; the
// element forces are zeroed (Neumann, lift and the force gather follow).
int assemble_affine_blocks(isl_ctx* c, const ElemArgs& A) {
    AffinePairs T;
    int rc = fill_pairs(c, T);
    if (rc != ISL_OK) return rc;
    rc = ensure_block_maps(c);
    if (rc != ISL_OK) return rc;
    cudaStream_t st = c->stream;
    const int E = (int)c->nelem;
    c->last_shared_geo = c->use_shared_geo && c->mesh_uniform == 1;
    ISL_CHECK_CUDA(c, c->dgeo.alloc((size_t)(c->last_shared_geo ? 1 : E) * GEO_F4));
    ISL_CHECK_CUDA(c, c->dbval.alloc((size_t)9 * c->nblk));
    ISL_CHECK_CUDA(c, cudaMemsetAsync(c->dstageF.p, 0, (size_t)c->nloc * E * 8, st));
    if (c->last_shared_geo) {
        // translates of element 0: its geometry record (their Jacobians, and with them the
        // sign of det J, are element 0's), and lam, mu of every element
        ISL_CHECK_CUDA(c, c->dlame.alloc((size_t)E));
        k_affine_geo<<<1, 32, 0, st>>>(E, 1, c->dX.p, c->dconn.p, c->dcoef.p, T, c->dgeo.p, A.flags);
        k_affine_lame<<<(unsigned)std::min<int64_t>((E + 255) / 256, (int64_t)c->sm_count * 8), 256, 0, st>>>(
            E, c->dcoef.p, c->dlame.p);
        c->launches += 1;
    } else {
        k_affine_geo<<<(unsigned)((E + 127) / 128), 128, 0, st>>>(E, E, c->dX.p, c->dconn.p, c->dcoef.p, T, c->dgeo.p,
                                                                  A.flags);
    }
    BlockArgs P;
    P.nslot = (int)c->nslot;
    P.nblk = (int)c->nblk;
    P.sblk = c->dsblk.p;
    P.brow = c->dbrow.p;
    P.bptr = c->dbptr.p;
    P.bcol = c->dbcol.p;
    P.brobj = c->dbrobj.p;
    P.adj_off = c->dadj_off.p;
    P.adj = c->dadj.p;
    P.rowptr = c->drowptr.p;
    P.geo = c->dgeo.p;
    P.lame = c->last_shared_geo ? c->dlame.p : nullptr;
    P.v64 = c->dval64.p;
    P.sv = c->dsval.p;
    // the block-row copy only feeds the block-row SpMV variants (and their
    // autotune, before a variant is chosen)
    const bool need_bv = c->bspmv_lpb == 0 || c->bspmv_lpb == 4 || c->bspmv_lpb == 8 || c->bspmv_lpb == 16;
    P.bv = need_bv ? c->dbval.p : nullptr;
    const unsigned grid = (unsigned)std::min<int64_t>((c->nslot + 255) / 256, (int64_t)c->sm_count * 8);
    if (c->last_shared_geo) k_affine_blocks_u<<<grid, 256, 0, st>>>(P, T);
    else k_affine_blocks<<<grid, 256, 0, st>>>(P, T);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 2;
    return ISL_OK;
}

int affine_lift(isl_ctx* c, int incremental) {
    if (c->n_lift == 0) return ISL_OK;
    AffinePairs T;
    int rc = fill_pairs(c, T);
    if (rc != ISL_OK) return rc;
    k_affine_lift<<<(unsigned)((c->n_lift + 63) / 64), 64, 0, c->stream>>>(
        (int)c->n_lift, c->dlift_elem.p, (int)c->nelem, c->dX.p, c->dconn.p, c->dedof.p, c->dstatus.p, c->dcval.p,
        c->du.p, incremental, c->dcoef.p, T, c->dstageF.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    return ISL_OK;
}

// The scalar FP32 CSR values, derived from the FP64 ones when the last
// assembly wrote only the block copies.
int ensure_val32(isl_ctx* c) {
    if (!c->have64 || c->val32_serial == c->asm_serial) return ISL_OK;
    ISL_CHECK_CUDA(c, c->dval32.alloc(c->nnz));
    k_d2f<<<(unsigned)c->sm_count * 8, 256, 0, c->stream>>>(c->nnz, c->dval64.p, c->dval32.p);
    ISL_CHECK_CUDA(c, cudaGetLastError());
    c->launches += 1;
    c->val32_serial = c->asm_serial;
    return ISL_OK;
}

}  // namespace isl
