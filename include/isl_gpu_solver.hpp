// isl_gpu_solver.hpp — header-only C++ adapter over the C-ABI (isl_gpu.h)
// that satisfies the duck-typed SOLVER interface of the reference
// (base::solver::Eigen3, base/solver/Eigen3.hpp:64-342) for the operations the
// hot path needs, plus the asmb entry points as member calls:
//
//   reference                                         adapter
//   Eigen3(size_t N)                         base/solver/Eigen3.hpp:71-77    Gb300Solver(ctx) after numberDoFs()
//   registerFields<FTB>(fb)                  :332-336                         registerFields()
//   stiffnessMatrixComputation<FTB>(...)     base/asmb/StiffnessMatrix.hpp:49-87   assemble(...)
//   computeResidualForces<FTB>(...)          base/asmb/ForceIntegrator.hpp:37-71   assemble(..., with_residual)
//   finishAssembly()                         :142-153                         finishAssembly() (no-op)
//   int cgSolve()                            :265-275                         cgSolve()
//   int biCGStabSolve()                      :277-289                         biCGStabSolve() (Jacobi, not ILUT)
//   smf::readMesh / writeMesh                base/io/smf/Reader.hpp, Writer.hpp     readSMF(path, shape), writeSMF(path)
//   vtk::LegacyWriter + writePointData       base/io/vtk/LegacyWriter.hpp          writeVTK(path, name)
//   post::errorComputation<ORDER>            base/post/ErrorNorm.hpp:84-123        errorComputation(order, qdeg, f)
//   heat::Static<Material>                   heat/Static.hpp:98-225                heatStatic(material, param, qdeg)
//   time::computeInertiaTerms<FTB,MSM>       base/time/ReactionTerms.hpp:62-79     inertia(density, lhs_w, weights)
//   time::computeResidualForceHistory        base/time/ResidualForceHistory.hpp    forceHistory(weights)
//   dof::pushHistory                         base/dof/DegreeOfFreedom.hpp:185-190  history(n), pushHistory()
//   number getValue(i)                       :293-296                         getValue(i)
//   double norm(), norm(first, last)         :128-138                         norm() (device-reduced), norm(first, last)
//   CompressibleDriver::solve per request    solid/CompressibleDriver.hpp:156-214  Gb300Server::submit / wait / result
//   insertToLHS / insertToRHS                :81-124                          not offered: assembly runs on the device
//
// Errors: the reference aborts through VERIFY_MSG (base/verify.hpp:63-65);
// the adapter throws isl::gpu_error carrying the isl_status code instead.
#pragma once

#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "isl_gpu.h"

namespace isl {

struct gpu_error : std::runtime_error {
    int code;
    gpu_error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// base::Quadrature<DEG,SHAPE> as the element kernels use it: weights and
// reference points ([n][dim]), for tabulating functors at the points
struct QuadratureRule {
    std::vector<double> w, xi;
};
inline QuadratureRule quadratureRule(int shape, int degree) {
    int n = 0;
    if (isl_quadrature_rule(shape, degree, &n, nullptr, nullptr) != ISL_OK)
        throw std::runtime_error("isl_quadrature_rule: no rule for this shape and degree");
    QuadratureRule r;
    r.w.resize(n);
    r.xi.resize((size_t)n * (shape == ISL_QUAD ? 2 : 3));
    isl_quadrature_rule(shape, degree, &n, r.w.data(), r.xi.data());
    return r;
}

inline void check(isl_ctx* ctx, int st, const char* what) {
    if (st != ISL_OK) throw gpu_error(st, std::string(what) + ": " + isl_last_error(ctx));
}

// Owns one isl_ctx: mesh, field, DOF state, pattern, system and solution on one GPU.
class Gb300Solver {
public:
    explicit Gb300Solver(int device = 0, void* stream = nullptr) {
        int st = isl_ctx_create(&ctx_, device, stream);
        if (st != ISL_OK) throw gpu_error(st, "isl_ctx_create");
    }
    ~Gb300Solver() { if (ctx_) isl_ctx_destroy(ctx_); }
    Gb300Solver(const Gb300Solver&) = delete;
    Gb300Solver& operator=(const Gb300Solver&) = delete;

    isl_ctx* ctx() { return ctx_; }

    // ---- mesh / field / DOFs (base::Unstructured, base::dof::generate, ...)
    void readSMF(const std::string& path, int shape) {
        check(ctx_, isl_mesh_read_smf(ctx_, path.c_str(), shape), "isl_mesh_read_smf");
    }
    void writeSMF(const std::string& path) { check(ctx_, isl_mesh_write_smf(ctx_, path.c_str()), "isl_mesh_write_smf"); }
    // the field's values at the mesh nodes as POINT_DATA, optional per-cell data
    void writeVTK(const std::string& path, const char* point_name, const char* cell_name = nullptr, int rows = 0,
                  int cols = 0, const std::vector<double>& cell_values = {}) {
        check(ctx_, isl_write_vtk(ctx_, path.c_str(), point_name, cell_name, rows, cols,
                                  cell_values.empty() ? nullptr : cell_values.data()), "isl_write_vtk");
    }
    void mesh(int shape, int dim, const std::vector<double>& X, const std::vector<int64_t>& conn, int nv) {
        check(ctx_, isl_mesh_upload(ctx_, shape, dim, (int64_t)X.size() / dim, X.data(), (int64_t)conn.size() / nv, conn.data()),
              "isl_mesh_upload");
    }
    int64_t field(int fe_degree, int ncomp) {
        int64_t n = 0;
        int nf = 0;
        check(ctx_, isl_field_create(ctx_, fe_degree, ncomp, &n, &nf), "isl_field_create");
        ncomp_ = ncomp;
        return n;
    }
    // constrainBoundary with a functor f(const double* x, int comp, double& value) -> bool
    template <typename DIRIFUN>
    void constrainBoundary(int dim, DIRIFUN f) {
        int64_t n = 0;
        check(ctx_, isl_boundary_points(ctx_, &n, nullptr, nullptr), "isl_boundary_points");
        std::vector<double> x((size_t)n * dim);
        std::vector<int64_t> dof(n);
        check(ctx_, isl_boundary_points(ctx_, &n, x.data(), dof.data()), "isl_boundary_points");
        std::vector<int64_t> d;
        std::vector<int> c;
        std::vector<double> v;
        for (int64_t i = 0; i < n; ++i)
            for (int k = 0; k < ncomp_; ++k) {
                double val = 0.0;
                if (f(&x[(size_t)i * dim], k, val)) { d.push_back(dof[i]); c.push_back(k); v.push_back(val); }
            }
        check(ctx_, isl_constrain(ctx_, (int64_t)d.size(), d.data(), c.data(), v.data()), "isl_constrain");
    }
    std::size_t numberDoFs() {
        int64_t n = 0;
        check(ctx_, isl_number_dofs(ctx_, &n), "isl_number_dofs");
        n_ = (std::size_t)n;
        return n_;
    }
    void registerFields() {
        int64_t nnz = 0;
        check(ctx_, isl_register_pattern(ctx_, &nnz), "isl_register_pattern");
    }
    // base::mesh::MeshBoundary: the (element, local face) pairs seen once
    void boundaryFaces(std::vector<int64_t>& elem, std::vector<int>& face) {
        int64_t n = 0;
        check(ctx_, isl_boundary_faces(ctx_, &n, nullptr, nullptr), "isl_boundary_faces");
        elem.resize(n);
        face.resize(n);
        check(ctx_, isl_boundary_faces(ctx_, &n, elem.data(), face.data()), "isl_boundary_faces");
    }

    // ---- kernels (per-element tabulated coefficients)
    void laplace(const std::vector<double>& kappa, int quad_degree) {
        check(ctx_, isl_set_laplace(ctx_, kappa.data(), quad_degree), "isl_set_laplace");
    }
    void hyperElastic(int material, const std::vector<double>& lam, const std::vector<double>& mu, int quad_degree) {
        check(ctx_, isl_set_hyperelastic(ctx_, material, lam.data(), mu.data(), quad_degree), "isl_set_hyperelastic");
    }
    void heatStatic(int material, const std::vector<double>& param, int quad_degree) {
        check(ctx_, isl_set_heat_static(ctx_, material, param.data(), quad_degree), "isl_set_heat_static");
    }
    // time integration: keep n past steps; inertia terms for the next assemblies
    void history(int n) { check(ctx_, isl_set_history(ctx_, n), "isl_set_history"); }
    void pushHistory() { check(ctx_, isl_push_history(ctx_), "isl_push_history"); }
    void inertia(const std::vector<double>& density, double lhs_weight, const std::vector<double>& weights) {
        check(ctx_, isl_set_inertia(ctx_, density.data(), lhs_weight, (int)weights.size(), weights.data()),
              "isl_set_inertia");
    }
    // computeResidualForceHistory: weights[s-1] of the residual force at x^(s)
    void forceHistory(const std::vector<double>& weights) {
        check(ctx_, isl_set_force_history(ctx_, (int)weights.size(), weights.empty() ? nullptr : weights.data()),
              "isl_set_force_history");
    }
    void bodyForceNodal(const std::vector<double>& f) {
        check(ctx_, isl_set_body_force_nodal(ctx_, f.data()), "isl_set_body_force_nodal");
    }
    // neumannForceComputation over the given boundary faces: a traction per
    // face ([n][ncomp]) or per face vertex ([n][nfv][ncomp], vertex = true)
    void neumann(const std::vector<int64_t>& elem, const std::vector<int>& face, const std::vector<double>& traction,
                 int squad_degree, bool vertex = false) {
        const int64_t n = (int64_t)elem.size();
        const int st = vertex ? isl_set_neumann_vertex(ctx_, n, elem.data(), face.data(), traction.data(), squad_degree)
                              : isl_set_neumann(ctx_, n, elem.data(), face.data(), traction.data(), squad_degree);
        check(ctx_, st, vertex ? "isl_set_neumann_vertex" : "isl_set_neumann");
    }

    // ---- assembly + solve (SOLVER duck type)
    void assemble(int precision = ISL_PREC_FP64, bool incremental = true, bool with_residual = false) {
        check(ctx_, isl_assemble(ctx_, precision, incremental, with_residual), "isl_assemble");
        cache_.clear();
    }
    void finishAssembly(bool = true) {}
    int cgSolve(double tol = 2.220446049250313e-16) {
        int64_t it = 0;
        double rr = 0.0;
        const int st = isl_solve(ctx_, ISL_SOLVE_CG_FP64, tol, 0, &it, &rr);
        if (st != ISL_OK && st != ISL_ERR_NOT_CONVERGED) check(ctx_, st, "isl_solve");
        cache_.clear();
        return (int)it;
    }
    int cgSolveMixed(double tol) {
        int64_t it = 0;
        double rr = 0.0;
        check(ctx_, isl_solve(ctx_, ISL_SOLVE_CG_FP32_IR, tol, 0, &it, &rr), "isl_solve");
        cache_.clear();
        return (int)it;
    }
    int biCGStabSolve(double tol = 2.220446049250313e-16) {
        int64_t it = 0;
        double rr = 0.0;
        const int st = isl_solve(ctx_, ISL_SOLVE_BICGSTAB, tol, 0, &it, &rr);
        if (st != ISL_OK && st != ISL_ERR_NOT_CONVERGED) check(ctx_, st, "isl_solve");
        cache_.clear();
        return (int)it;
    }
    // errorComputation<order>: f(x, out) writes the reference value (order 0:
    // ncomp values) or gradient (order 1: ncomp x dim) at a quadrature point
    template <typename FUN>
    double errorComputation(int order, int quad_degree, int dim, FUN f) {
        int64_t n = 0;
        check(ctx_, isl_quadrature_points(ctx_, quad_degree, &n, nullptr), "isl_quadrature_points");
        std::vector<double> x((size_t)n * dim);
        check(ctx_, isl_quadrature_points(ctx_, quad_degree, &n, x.data()), "isl_quadrature_points");
        const int per = ncomp_ * (order == 1 ? dim : 1);
        std::vector<double> ref((size_t)n * per);
        for (int64_t i = 0; i < n; ++i) f(&x[(size_t)i * dim], &ref[(size_t)i * per]);
        double err = 0.0;
        check(ctx_, isl_error_norm(ctx_, order, quad_degree, ref.data(), &err), "isl_error_norm");
        return err;
    }
    double getValue(std::size_t i) {
        fill();
        return cache_.at(i);
    }
    // ||b|| / N after an assembly, ||x|| / N after a solve (Eigen3's b_ holds
    // x), reduced on the device
    double norm() {
        double v = 0.0;
        check(ctx_, isl_norm(ctx_, &v), "isl_norm");
        return v;
    }
    double norm(std::size_t first, std::size_t last) {
        fill();
        double s = 0.0;
        for (std::size_t i = first; i < last; ++i) s += cache_[i] * cache_[i];
        return std::sqrt(s) / (double)(last - first);
    }
    void setDoFsFromSolver() { check(ctx_, isl_distribute(ctx_, 0), "isl_distribute"); }
    void addToDoFsFromSolver() { check(ctx_, isl_distribute(ctx_, 1), "isl_distribute"); }

private:
    void fill() {
        if (cache_.size() == n_) return;
        cache_.resize(n_);
        check(ctx_, isl_get_solution(ctx_, cache_.data()), "isl_get_solution");
    }
    isl_ctx* ctx_ = nullptr;
    int ncomp_ = 1;
    std::size_t n_ = 0;
    std::vector<double> cache_;
};

// The served path: many CompressibleDriver runs on one GPU, batched by the
// native server (isl_serve_*).  submit copies the request's arrays.
class Gb300Server {
public:
    explicit Gb300Server(int device = 0, int precision = ISL_PREC_FP32, int max_batch = 64, int max_batches = 4,
                         int64_t reserve_bytes = 0, int64_t batch_window_us = 0, double size_ratio = 0.0) {
        isl_serve_config cfg{};
        cfg.max_batch = max_batch;
        cfg.max_batches = max_batches;
        cfg.precision = precision;
        cfg.reserve_bytes = reserve_bytes;
        cfg.batch_window_us = batch_window_us;
        cfg.size_ratio = size_ratio;
        const int st = isl_serve_create(&s_, device, &cfg);
        if (st != ISL_OK) throw gpu_error(st, "isl_serve_create");
    }
    ~Gb300Server() { if (s_) isl_serve_destroy(s_); }
    Gb300Server(const Gb300Server&) = delete;
    Gb300Server& operator=(const Gb300Server&) = delete;

    int64_t submit(const isl_serve_request& r) {
        int64_t t = 0;
        const int st = isl_serve_submit(s_, &r, &t);
        if (st != ISL_OK) throw gpu_error(st, "isl_serve_submit");
        return t;
    }
    // blocks until the request has finished; its DOF values and statistics
    std::vector<double> result(int64_t ticket, std::size_t ndof, isl_serve_stats* stats = nullptr) {
        int state = 0;
        int st = isl_serve_wait(s_, ticket, 1e9, &state);
        if (st != ISL_OK) throw gpu_error(st, "isl_serve_wait");
        std::vector<double> u(ndof);
        isl_serve_stats local{};
        st = isl_serve_result(s_, ticket, u.data(), stats ? stats : &local);
        if (st != ISL_OK) throw gpu_error(st, std::string("served request failed: ") + isl_serve_error(s_, ticket));
        isl_serve_release(s_, ticket);
        return u;
    }

private:
    isl_server* s_ = nullptr;
};

}  // namespace isl
