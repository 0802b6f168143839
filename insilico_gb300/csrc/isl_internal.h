// Internal state of an isl_ctx and helpers shared by the host and device
// translation units of the GB300 assembly + Krylov library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/isl_gpu.h"

namespace isl {

// ---------------------------------------------------------------------------
// Element traits (geometry degree 1, field degree FDEG)
template <int SHAPE, int FDEG>
struct ET;
template <> struct ET<ISL_QUAD, 1> { static constexpr int D = 2, NG = 4, NF = 4; };
template <> struct ET<ISL_QUAD, 2> { static constexpr int D = 2, NG = 4, NF = 9; };
template <> struct ET<ISL_HEX, 1> { static constexpr int D = 3, NG = 8, NF = 8; };
template <> struct ET<ISL_TET, 1> { static constexpr int D = 3, NG = 4, NF = 4; };
template <> struct ET<ISL_TET, 2> { static constexpr int D = 3, NG = 4, NF = 10; };

// Reference-element tables handed to the element kernels by value.
template <int D, int NG, int NF, int NQ>
struct Tab {
    double w[NQ];
    double phi[NQ][NF];
    double dphi[NQ][NF][D];
    double N[NQ][NG];
    double dN[NQ][NG][D];
};

// Host-side reference tables (any size), filled by shape tables code.
struct HostTab {
    int dim = 0, nq = 0, nf = 0, ng = 0;
    std::vector<double> w, xi, phi, dphi, N, dN;
};
bool make_host_tables(int shape, int fedeg, int qdeg, HostTab& t);
// surface (face) tables for Neumann integration: per local face, per surface qp:
// FE values of the domain element at the mapped point, weights, and the face
// geometry function gradients (for the metric)
struct FaceTab {
    int nfaces = 0, nsq = 0, nfv = 0, nf = 0, dim = 0;
    std::vector<int> fv;        // [nfaces][nfv] local vertex ids of the face
    std::vector<double> w;      // [nsq]
    std::vector<double> S;      // [nsq][nfv] face geometry function values
    std::vector<double> phi;    // [nfaces][nsq][nf]
    std::vector<double> dS;     // [nsq][nfv][dim-1] face geometry gradients
};
bool make_face_tables(int shape, int fedeg, int sqdeg, FaceTab& t);

// ---------------------------------------------------------------------------
// Device buffer with RAII.  Memory comes from the stream-ordered pool
// (cudaMallocAsync / cudaFreeAsync on the per-thread stream), so allocating or
// freeing never synchronises the device: contexts serving concurrent requests
// keep overlapping.  Buffers are only released after the owning context's
// stream has been synchronised.
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFreeAsync(p, cudaStreamPerThread);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count) {
        if (count == n && p) return cudaSuccess;
        release();
        if (count == 0) return cudaSuccess;
        cudaError_t e = cudaMallocAsync((void**)&p, count * sizeof(T), cudaStreamPerThread);
        if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamPerThread);
        if (e == cudaSuccess) n = count;
        else p = nullptr;
        return e;
    }
};

// CG workspace for one precision
struct CGWork {
    void* x = nullptr;  // solution (T)
    void* r = nullptr;
    void* p = nullptr;
    void* q = nullptr;  // A p
    void* dinv = nullptr;
    size_t n = 0;
};

// scalar block shared by the CG kernels (device)
struct CGScal {
    double absNew, absOld, pAp, alpha, beta, rr, rz, threshold, rhsNorm2;
    double rrtrig;  // mixed CG: stop for a reliable update when rr falls below (0 = never)
    int done;
    int iters;
    int bad;
    int fault;   // persistent CG: a grid barrier timed out
    unsigned int ticket1, ticket2;
};

}  // namespace isl

struct isl_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int sm_count = 0;

    // instances: a context holds one mesh or a batch of independent meshes
    // (disjoint node/element ranges); DOF objects and equations are numbered
    // per instance and concatenated
    int64_t ninst = 1;
    std::vector<int64_t> inst_node_off, inst_elem_off, inst_dof_off, inst_eq_off;

    // mesh
    int shape = 0, dim = 0, ngeom = 0;
    int64_t nnodes = 0, nelem = 0;
    std::vector<double> hX;
    std::vector<int64_t> hconn;  // [nelem][ngeom]
    isl::DBuf<double> dX;        // [nnodes][dim]
    isl::DBuf<int32_t> dconn;    // SoA [ngeom][nelem]

    // field
    int fedeg = 0, ncomp = 0, nfun = 0, nloc = 0, nup = 0;
    int64_t ndofobj = 0;
    std::vector<int64_t> hedof;  // [nelem][nfun]
    std::vector<std::pair<int64_t, int>> bf_cache;  // boundary (element, face) list of the current mesh
    bool bf_valid = false;
    bool host_setup = false;     // DOF numbering and boundary detection on the host even with a device
    isl::DBuf<int32_t> dedof;    // SoA [nfun][nelem]
    std::vector<uint8_t> status; // per dofobj comp: 0 active, 1 constrained
    std::vector<double> cval;
    std::vector<double> hu;      // host mirror of values (valid when u_on_host)
    std::vector<int32_t> heq;
    int64_t neq = 0;
    bool numbered = false;
    isl::DBuf<int32_t> deq;      // per dofobj comp
    isl::DBuf<uint8_t> dstatus;
    isl::DBuf<double> dcval;
    isl::DBuf<double> du;        // current values per dofobj comp
    bool u_nonzero = false;

    // kernel data
    int kernel = -1, material = 0, qdeg = 2, sqdeg = 2;
    bool stage_full = false;     // the kernel's element matrices are not symmetric: staged whole
    // inertia terms of a multi-step method (isl_set_inertia) and the DOF history
    bool inertia = false;
    double mass_w = 0.0;         // LHS weight of the mass matrix (a0 / (b0 dt))
    int nhist_w = 0;             // history weights in use (index 0: current values)
    double hist_w[5] = {0, 0, 0, 0, 0};
    int nhist = 0;               // stored past steps
    int nforce_w = 0;            // residual-force history weights in use (x^(1), x^(2), ...)
    double force_w[4] = {0, 0, 0, 0};
    isl::DBuf<double> drho, dhist, dhvec;  // density per element, [nhist][ndofobj*ncomp], weighted history
    bool pattern_full = false;   // the contribution lists index whole element matrices
    isl::DBuf<double> dcoef;     // SoA [ncoef][nelem]
    isl::DBuf<double> dkqp;      // Laplace conductivity per quadrature point, SoA [nq][nelem]
    bool has_kqp = false;
    bool has_body = false;
    isl::DBuf<double> dfnodal;   // [nnodes][ncomp]
    // Neumann: faces grouped by element
    int64_t n_neu_elem = 0;
    isl::DBuf<int32_t> dneu_elem, dneu_off, dneu_face;
    isl::DBuf<double> dneu_trac;
    bool neu_vertex = false;     // dneu_trac holds values per face vertex (isl_set_neumann_vertex)
    // elements with at least one constrained local DOF (for the Dirichlet lift)
    int64_t n_lift = 0;
    isl::DBuf<int32_t> dlift_elem;

    // pattern
    bool pattern_ready = false;  // true after isl_register_pattern (also for an empty system)
    int64_t nnz = 0, ncontrib = 0, ncontribF = 0;
    isl::DBuf<int32_t> drowptr, dcolind, ddiag, dseg, dsrc, dsegF, dsrcF;
    // staged element matrices/vectors (SoA)
    isl::DBuf<double> dstageK64;
    isl::DBuf<float> dstageK32;
    isl::DBuf<double> dstageF;
    // assembled system
    isl::DBuf<double> dval64;
    isl::DBuf<float> dval32;
    bool have64 = false, have32 = false;
    isl::DBuf<double> drhs;      // b (FP64)
    isl::DBuf<double> dsol;      // x (FP64)
    bool solved = false;

    // node-blocked (3x3) FP32 copy of the matrix for the mixed solver: used
    // when every DOF object has all three components active or all constrained
    bool blocked = false;
    bool use_block = true;
    std::vector<int32_t> hrp_small;  // host row pointers of a system small enough for the one-cluster solve
    int mesh_affine = -1;        // every element a parallelepiped / parallelogram (-1: not yet checked)
    int mesh_uniform = -1;       // every hexahedron a translate of the first (set with mesh_affine)
    bool use_shared_geo = true;  // ISL_OPT_SHARED_GEOMETRY
    bool last_shared_geo = false;  // the last direct block assembly formed its blocks from shared tables
    int use_persist = 1;         // one-launch CG kernels: 0 never, 1 for small systems, 2 always where supported
    int cluster_size = -1;       // CTAs of the small-system cluster solve (-1: not yet probed, 0: unavailable)
    int persist_grid = -1;       // blocks of the persistent kernel (-1: not yet probed, 0: unavailable)
    bool barrier_test = false;   // test hook: the next persistent launch finds its grid barrier pre-armed (never completes)
    isl::DBuf<unsigned int> dbar; // grid barrier of the persistent kernel: arrivals, generation
    int64_t nbr = 0, nblk = 0;
    isl::DBuf<int32_t> dbptr, dbcol, dbrow;
    // sliced-ELL copy of the blocks for the SpMV: block rows in slices of 32,
    // each slice padded to its longest row, stored column-major (slot =
    // slice_off + k*32 + lane) so a warp reads every block position coalesced
    int64_t nslice = 0, nslot = 0;
    isl::DBuf<int32_t> dsoff, dswid, dscol, dsdst;
    isl::DBuf<float> dsval;      // [slot/32][9][32]: the 9 values of a group of 32 slots contiguous
    isl::DBuf<float> dbval;      // block-row CSR copy: SoA [9][nblk]
    int bspmv_kind = 0;          // autotuned: 1..3 sliced-ELL (unroll 1,2,4), 4/8/16 block-row CSR lanes per row
    isl::DBuf<float> dbinv;      // SoA [9][nbr] inverse diagonal blocks
    int64_t asm_serial = 0, bsr_serial = -1;
    int64_t val32_serial = -1;   // assembly whose values dval32 holds
    int64_t bvals_serial = -1;   // assembly that wrote the FP32 block copies directly
    // direct block assembly of small-strain elasticity on parallelepipeds (isl_blocks.cu)
    isl::DBuf<float4> dgeo;      // per element: detJ Ji, Ji, lam, mu as double-float (element 0 only on a mesh of translates)
    isl::DBuf<float4> dlame;     // per element lam, mu as double-float (mesh of translates)
    isl::DBuf<int32_t> dbrobj, dadj_off, dadj, dsblk;
    int64_t bmap_serial = -1;
    int asm_precision = 0;       // precision of the assembly in progress
    bool last_direct = false;    // the last assembly wrote the blocks directly (ISL_OPT_DIRECT_BLOCKS)
    int64_t tune_runs = 0;       // autotunes that timed candidates (the others came from the tuning cache)
    int elem_variant = 0;        // autotuned launch shape of the element kernel (0: not yet chosen)
    int64_t elem_variant_key = -1;
    int bspmv_lpb = 0;
    bool fuse_dir = true;  // fold the block-Jacobi direction update into the block SpMV
    double ru_drop2 = 1e-2;      // mixed CG: reliable update after r.r drops by this factor (ISL_OPT_RELIABLE_DROP)
    isl::DBuf<int16_t> dscol16;  // slot columns as 16-bit offsets from the slot's block row
    bool scol16 = false;         // every offset fits (dscol16 valid)
    bool use_scol16 = true;      // ISL_OPT_SHORT_COLUMNS
    isl::DBuf<int16_t> dss_col16;  // scalar sliced-ELL columns as 16-bit offsets from each lane's row
    bool ss16 = false;           // every offset fits (dss_col16 valid)
    int bupd_kind[2] = {0, 0};  // block CG update kernel (separate / folded direction), 0: not tuned yet
    // padded node blocks: DOF objects with some components constrained keep a
    // 3x3 block row; the solver vectors live in the padded space (3 nbr
    // entries, zero at constrained components) and map to equations here
    bool bpad = false;
    isl::DBuf<int32_t> dbaeq;    // [3 nbr] equation of each block-row component, -1 constrained
    isl::DBuf<int32_t> dbcb;     // [nblk] CSR position base: value (r, c) at rowptr[eq_r] + dbcb + eq_c

    // scalar sliced-ELL copy of the FP32 matrix for the mixed solver of a
    // system that is not node-blocked: rows sorted by length (longest first)
    // within windows of 2048 rows, slices of 32 sorted rows padded to their
    // longest row, slots column-major (slot = slice_off + k*32 + lane)
    int64_t ss_nslice = 0, ss_nslot = 0;
    isl::DBuf<int32_t> dss_off, dss_wid, dss_row, dss_col, dss_pos;
    isl::DBuf<float> dss_val;
    int64_t ss_serial = -1;      // assembly whose values the copy holds

    // batched CG (ninst > 1): row ranges of thread blocks and per-instance state
    isl::DBuf<int32_t> dinst_row, dblk_inst, dblk_row0, dblk_row1, dinst_blk;
    isl::DBuf<int32_t> dblk_s0, dblk_s1;  // slices of every row block in the batched sliced-ELL copy
    bool bsell_built = false;
    int bspmv32 = 0;             // FP32 SpMV kind of the batched mixed solve (autotuned once per pattern)
    isl::DBuf<double> dbs;        // per-instance scalars [16][ninst]
    isl::DBuf<int32_t> dbi;       // per-instance ints   [8][ninst]
    isl::DBuf<unsigned int> dbt;  // per-instance tickets [4][ninst]
    isl::DBuf<double> dbpart;     // per-block partials [8][nblocks]
    isl::DBuf<int32_t> dbwl;      // reliable-update worklist: instances, append count, count, block offsets
    isl::DBuf<int32_t> dbact;     // row blocks of unfinished instances: count, then the block ids
    isl::DBuf<int32_t> dinst_dof; // DOF-object offsets of the instances [ninst+1]
    isl::DBuf<double> dinst_norm; // per-instance norms (isl_batch_norms)
    isl::DBuf<int32_t> dinst_mask;// instances that take part in the next solves and distributes (isl_batch_set_mask)
    bool mask_on = false;
    bool force_batched = false;   // ISL_OPT_BATCHED_SOLVE: one instance through the batched solver
    int64_t nbblocks = 0;
    std::vector<int64_t> inst_iters;
    std::vector<double> inst_relres;

    // status word written by kernels (bit 0: det J <= 0, bit 1: NaN)
    isl::DBuf<int> dflags;

    // solver workspace
    isl::DBuf<double> w64;       // FP64 vectors
    isl::DBuf<float> w32;        // FP32 vectors
    isl::DBuf<double> dpart;     // block partial sums
    isl::DBuf<double> wbi;       // BiCGSTAB vectors (10 N)
    isl::DBuf<double> dbis;      // BiCGSTAB scalars
    int bicg_lpr = 0;            // BiCGSTAB SpMV kind (autotuned per pattern): CSR lanes per row, 100 + U sliced-ELL
    int bicg_forced = 0;         // kind set through ISL_OPT_BICGSTAB_KIND (0: autotune)
    isl::DBuf<double> dss_val64; // FP64 values of the scalar sliced-ELL copy (BiCGSTAB)
    int64_t ss_serial64 = -1, ss_val64_pattern = -1;
    int64_t bicg_serial = -1, pattern_serial = 0;
    isl::DBuf<isl::CGScal> dscal;
    isl::CGScal* hscal = nullptr;  // pinned host mirror
    int spmv_lpr64 = 0, spmv_lpr32 = 0;  // autotuned lanes per row (FP32: 100 + U = sliced-ELL, U slots in flight)
    int spmv32_forced = 0;               // FP32 SpMV kind set through ISL_OPT_SPMV32_KIND (0: autotune)

    // timing
    bool timing = false;
    double tms[ISL_NTIMERS] = {0};
    int64_t tcount[ISL_NTIMERS] = {0};
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t mark[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int64_t launches = 0;  // kernels launched (graph nodes included)
};

// status helpers
#define ISL_CHECK_CUDA(ctx, call)                                                        \
    do {                                                                                 \
        cudaError_t _e = (call);                                                         \
        if (_e != cudaSuccess) {                                                         \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(_e);             \
            return (_e == cudaErrorMemoryAllocation) ? ISL_ERR_NOMEM : ISL_ERR_CUDA;     \
        }                                                                                \
    } while (0)

#define ISL_FAIL(ctx, code, msg) \
    do {                         \
        (ctx)->err = (msg);      \
        return (code);           \
    } while (0)

namespace isl {
// Status for a C++ exception caught at the C ABI: the message goes to the
// context when there is one (the assignment itself may fail under memory
// pressure, which leaves the old message).
inline int fail_exception(isl_ctx* c, int code, const char* what) noexcept {
    if (c) {
        try {
            c->err = what;
        } catch (...) {
        }
    }
    return code;
}
}  // namespace isl

// Every extern "C" entry point with host allocations runs its body inside
// ISL_TRY .. ISL_CATCH(ctx): no exception crosses the C ABI.  Allocation
// failures (std::bad_alloc, or a container size above max_size) return
// ISL_ERR_NOMEM, anything else ISL_ERR_ARG.
#define ISL_TRY try {
#define ISL_CATCH(ctx)                                                                          \
    }                                                                                           \
    catch (const std::bad_alloc&) {                                                             \
        return isl::fail_exception((ctx), ISL_ERR_NOMEM, "host allocation failed");             \
    }                                                                                           \
    catch (const std::length_error&) {                                                          \
        return isl::fail_exception((ctx), ISL_ERR_NOMEM, "host allocation larger than max_size"); \
    }                                                                                           \
    catch (const std::exception& _x) {                                                          \
        return isl::fail_exception((ctx), ISL_ERR_ARG, _x.what());                              \
    }                                                                                           \
    catch (...) {                                                                               \
        return isl::fail_exception((ctx), ISL_ERR_ARG, "unknown exception");                    \
    }

namespace isl {
// Tuning cache: autotuned kernel variants per (tuner, problem class), kept
// in memory and, when a file is set (isl_tune_cache or ISL_TUNE_CACHE), in
// that file, so that later contexts and processes skip the timing.
bool tune_lookup(const isl_ctx* c, const char* tuner, int* value);
bool update_kind_valid(int kind);  // ISL_OPT_BLOCK_UPDATE values other than 0
void tune_store(isl_ctx* c, const char* tuner, int value);
// device-side entry points implemented in the .cu files
int pattern_build(isl_ctx* c);
int push_history_device(isl_ctx* c);
int assemble_device(isl_ctx* c, int precision, int incremental, int with_residual);
int solve_device(isl_ctx* c, int method, double tol, int64_t max_iter, int64_t* iters, double* relres);
int distribute_device(isl_ctx* c, int add);
int time_spmv(isl_ctx* c, int precision, int nrep, double* ms);
int time_kernels(isl_ctx* c, int nrep, double* ms);
int block_pattern(isl_ctx* c, const std::vector<int32_t>& rowptr);
int scalar_sell_pattern(isl_ctx* c, const std::vector<int32_t>& rowptr);
int batch_sell_pattern(isl_ctx* c, const std::vector<int32_t>& b0, const std::vector<int32_t>& b1,
                       std::vector<int32_t>& s0, std::vector<int32_t>& s1);
int ensure_ssell(isl_ctx* c);
// One level of n-faces for the device DOF numbering: nfc faces per element of
// w vertices each (w = 0: the cell itself, not grouped), `stride` DOFs per
// face starting at local DOF position `begin`.
struct DeviceLevel {
    int nfc = 0, w = 0, stride = 0, begin = 0;
    int v[12][4] = {};
};
bool device_setup_fits(const isl_ctx* c, int nfc);
int quadrature_points_device(isl_ctx* c, int qdeg, int64_t* n, double* x);
int error_norm_device(isl_ctx* c, int order, int qdeg, const double* ref, double* err);
int device_dofobj_numbering(isl_ctx* c, const std::vector<DeviceLevel>& levels, int nf);
int device_boundary_slots(isl_ctx* c, const DeviceLevel& lv, std::vector<int64_t>& slots);
bool spmv32_kind_valid(const isl_ctx* c, int kind);
int solve_batched(isl_ctx* c, int method, double tol, int64_t max_iter, int64_t* iters, double* relres);
int time_spmv_batched(isl_ctx* c, int precision, int nrep, double* ms);
int ensure_val32(isl_ctx* c);
int affine_lift(isl_ctx* c, int incremental);
int inst_norms_device(isl_ctx* c, double* out);
int distribute_masked(isl_ctx* c, int add);
int solve_bicgstab(isl_ctx* c, double tol, int64_t max_iter, int64_t* iters, double* rel, bool* nc);
bool bicgstab_kind_valid(const isl_ctx* c, int kind);
}  // namespace isl
