/*
 * isl_gpu.h — C-ABI of the GB300 (sm_103a) assembly + Krylov library for the
 * inSilico finite-element hot path.
 *
 * The reference (thrueberg/inSilico) is a header-only C++ template library
 * with no FFI: its "plugin interface" is the duck-typed SOLVER template
 * parameter (base::solver::Eigen3) plus the asmb call surface and the kernel
 * functors.  Each entry point below replaces one step of that call surface;
 * the reference file:line it stands in for is cited beside it.  A C++ adapter
 * that satisfies the SOLVER duck type on top of this ABI is
 * include/isl_gpu_solver.hpp.
 *
 * Conventions
 *   - every function returns an isl_status (ISL_OK == 0); isl_last_error()
 *     returns a message for the last failure on a context;
 *   - plain pointers and sizes only; host buffers unless the name says _dev;
 *   - a context owns all device memory it allocates and runs all work on the
 *     stream given at creation (NULL = a stream the context creates);
 *   - one host thread per context (not re-entrant); several contexts may
 *     share a device;
 *   - local element DOF order is node-major, component-minor (a = M*ncomp + i),
 *     as in solid/HyperElastic.hpp:171 (matrix(M*nDoFs+i, N*nDoFs+k)).
 */
#ifndef ISL_GPU_H
#define ISL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    ISL_OK = 0,
    ISL_ERR_ARG = 1,            /* invalid argument or call order */
    ISL_ERR_NOMEM = 2,          /* device or host allocation failed */
    ISL_ERR_DEGENERATE = 3,     /* an element had det J <= 0 (results still written) */
    ISL_ERR_NOT_CONVERGED = 4,  /* solver hit max_iter before the tolerance */
    ISL_ERR_TIMEOUT = 5,        /* a bounded device wait expired */
    ISL_ERR_CUDA = 6,           /* CUDA runtime error */
    ISL_ERR_NAN = 7,            /* non-finite value in a reduction */
    ISL_ERR_CAPACITY = 8        /* input larger than a fixed capacity (isl_cg_solve_noalloc) */
} isl_status;

/* element shapes (geometry degree 1, hierarchic vertex order of
 * base/mesh/HierarchicOrder.hpp) */
enum { ISL_QUAD = 3, ISL_TET = 4, ISL_HEX = 5 };
/* ISL_TRI: the faces of tetrahedra; a shape of isl_quadrature_rule only (the
 * surface rules of Neumann tractions on tetrahedra) */
enum { ISL_TRI = 2 };
/* kernel functors */
enum { ISL_KERNEL_LAPLACE = 0, ISL_KERNEL_HYPERELASTIC = 1, ISL_KERNEL_HEAT_STATIC = 2 };
/* materials of solid::HyperElastic */
enum { ISL_MAT_STVENANT = 0, ISL_MAT_NEOHOOKE = 1 };
/* mat::thermal materials of heat::Static: IsotropicConstant, FenicsTest */
enum { ISL_THERMAL_CONSTANT = 0, ISL_THERMAL_FENICS = 1 };
/* arithmetic of the element kernels and of the stored matrix */
enum { ISL_PREC_FP64 = 0, ISL_PREC_FP32 = 1, ISL_PREC_MIXED = 2 };
/* solve methods */
enum { ISL_SOLVE_CG_FP64 = 0, ISL_SOLVE_CG_FP32_IR = 1, ISL_SOLVE_BICGSTAB = 2 };
/* phase timers reported by isl_timings (milliseconds, CUDA events) */
enum { ISL_T_ELEMENT = 0, ISL_T_GATHER = 1, ISL_T_SOLVE = 2, ISL_T_SPMV = 3, ISL_T_PATTERN = 4, ISL_NTIMERS = 8 };

typedef struct isl_ctx isl_ctx;

/* Context lifetime.  stream: a cudaStream_t (NULL = create one). */
int isl_ctx_create(isl_ctx** out, int device, void* stream);
int isl_ctx_destroy(isl_ctx* ctx);
const char* isl_last_error(const isl_ctx* ctx);

/* Mesh: coordinates [n_nodes][dim], connectivity [n_elem][n_vertices]
 * (int64 node ids, hierarchic order).
 * Replaces base::io::smf::readMesh / base::Unstructured construction
 * (base/io/smf/Reader.hpp:275-307). */
int isl_mesh_upload(isl_ctx* ctx, int shape, int dim, int64_t n_nodes, const double* coords, int64_t n_elem,
                    const int64_t* conn);

/* Batch of independent meshes in one context (the batched-instances path):
 * node_off / elem_off [n_inst+1] delimit each instance's nodes and elements
 * in the concatenated coords / conn (conn holds global node ids; an element
 * only uses nodes of its own instance).  DOF objects and equations are
 * numbered per instance exactly as for a single mesh and concatenated; the
 * assembly runs over all instances in the same launches, and isl_solve runs
 * one CG per instance (own scalars, own convergence) in the same launches.
 * No reference counterpart: the reference assembles one mesh at a time. */
int isl_batch_mesh_upload(isl_ctx* ctx, int shape, int dim, int64_t n_inst, const int64_t* node_off, const double* coords,
                          const int64_t* elem_off, const int64_t* conn);
/* n_inst, equation offsets [n_inst+1] and DOF-object offsets [n_inst+1] of the
 * instances (any of the three may be NULL). */
int isl_batch_info(isl_ctx* ctx, int64_t* n_inst, int64_t* eq_off, int64_t* dofobj_off);
/* Per-instance CG iterations and final relative residuals of the last solve. */
int isl_batch_solve_stats(isl_ctx* ctx, int64_t* iters, double* rel_res);
/* Eigen3::norm (base/solver/Eigen3.hpp:128-138) of every instance's own
 * system: ||v_k|| / N_k with v the solution after a solve, else the
 * right-hand side; reduced on the device, out [n_inst].  The batched form of
 * the convergence test of solid/CompressibleDriver.hpp:190-210. */
int isl_batch_norms(isl_ctx* ctx, double* out);
/* base::dof::scaleConstraints (base/dof/Distribute.hpp:75-81) with one factor
 * per instance (factors [n_inst]): instances at different load steps. */
int isl_batch_scale_constraints(isl_ctx* ctx, const double* factors);
/* Instances that take part in the next solves and distributes (keep
 * [n_inst], nonzero = take part; NULL: all).  A solve clears the right-hand
 * side of the others, which then finish at once with x = 0, and
 * isl_distribute leaves their DOF values as they are.  Kept until the next
 * call or renumbering.  No reference counterpart: it lets instances whose
 * Newton loops are at different points share one batched solve. */
int isl_batch_set_mask(isl_ctx* ctx, const uint8_t* keep);

/* Field of Lagrange degree fe_degree with ncomp components per DOF object;
 * generates the DOF-object ids per element.
 * Replaces base::dof::generate (base/dof/generate.hpp:65-115 ->
 * base/dof/IndexMap.hpp:221-280). */
int isl_field_create(isl_ctx* ctx, int fe_degree, int ncomp, int64_t* n_dofobj, int* n_fun);
int isl_field_elem_dofobj(isl_ctx* ctx, int64_t* out /* [n_elem][n_fun] */);

/* Boundary = faces seen once, sorted by vertex key.  Call with NULL arrays to
 * get the count.  Replaces base::mesh::MeshBoundary::create
 * (base/mesh/createBoundaryFromUnstructured.hpp:51-109). */
int isl_boundary_faces(isl_ctx* ctx, int64_t* n, int64_t* elem, int* face);
/* Support points of every boundary face DOF with its DOF object, in the
 * order base::dof::constrainBoundary visits them
 * (base/dof/constrainBoundary.hpp:50-124); the caller evaluates its
 * Dirichlet functor on them and calls isl_constrain. */
int isl_boundary_points(isl_ctx* ctx, int64_t* n, double* x /* [n][dim] */, int64_t* dofobj);
/* DegreeOfFreedom::constrainValue (base/dof/DegreeOfFreedom.hpp:232-242) */
int isl_constrain(isl_ctx* ctx, int64_t n, const int64_t* dofobj, const int* comp, const double* value);
/* base::dof::scaleConstraints (base/dof/Distribute.hpp:75-81) */
int isl_scale_constraints(isl_ctx* ctx, double factor);
/* base::dof::numberDoFsConsecutively (base/dof/numbering.hpp:44-68) */
int isl_number_dofs(isl_ctx* ctx, int64_t* n_active);
/* equation index per DOF-object component (-1 if constrained) */
int isl_dof_index(isl_ctx* ctx, int64_t* out /* [n_dofobj*ncomp] */);

/* CSR pattern of active DOF pairs + element-to-slot contribution lists, built
 * on the device.  Replaces Eigen3::registerFields ->
 * TripletContainer::registerFields (base/solver/TripletContainer.hpp:158-301). */
int isl_register_pattern(isl_ctx* ctx, int64_t* nnz);

/* The quadrature rule the element kernels use for a shape and polynomial
 * degree (base::Quadrature<DEG,SHAPE>, base/Quadrature.hpp:28-80: tensor
 * Gauss-Legendre on [0,1] for quadrilaterals and hexahedra,
 * base/quad/GaussLegendre.hpp:115-134; the tetrahedron rules of degree 1 to 5,
 * base/quad/GaussTetrahedron.hpp:93-175), for callers that tabulate their
 * functors at the quadrature points.  Weights [n], reference points [n][dim];
 * NULL arrays give the count.  Host only, no context.  Rules exist for
 * degrees 1 to 5: Gauss-Legendre with 1, 2 or 3 points per direction
 * ((degree + 2) / 2, base/quad/GaussLegendre.hpp:33-37) on quadrilaterals and
 * hexahedra, 1, 4, 5, 11 or 15 points on tetrahedra, and 1, 3, 4, 6 or 7
 * points on triangles (ISL_TRI, the surface rules of tetrahedron faces,
 * base/quad/GaussTriangle.hpp:97-180); ISL_ERR_ARG for degree 0, degrees
 * above 5 and other shapes. */
int isl_quadrature_rule(int shape, int degree, int* n, double* w, double* xi);

/* Kernel functor tabulation (per element coefficients; the reference's
 * ConductivityFun / Material objects are evaluated per element by the caller):
 *   heat::Laplace (heat/Laplace.hpp:113-126, base/kernel/Laplace.hpp:100-151)
 *   solid::HyperElastic<StVenant|NeoHookeanCompressible>
 *     (solid/HyperElastic.hpp:110-257, mat/hypel/StVenant.hpp:77-114,
 *      mat/hypel/NeoHookeanCompressible.hpp:77-172); on the device for
 *     trilinear hexahedra (2x2x2 or 3x3x3 points), P1 / P2 tetrahedra and
 *     Q1 / Q2 quadrilaterals (plane strain, solid/Deformation.hpp:25-46)
 * quad_degree: base::Quadrature<DEG,SHAPE> degree (base/Quadrature.hpp:113-143). */
int isl_set_laplace(isl_ctx* ctx, const double* kappa /* [n_elem] */, int quad_degree);
/* heat::Laplace with a conductivity that varies inside the elements: the
 * value of the ConductivityFun at every quadrature point
 * (heat/Laplace.hpp:119-120 evaluates conductivityFun_(geomEp, xi) there),
 * kappa[e * nq + q] in the order of isl_quadrature_points for the same
 * quad_degree (nq from isl_quadrature_rule); the tangent and the residual
 * use it.  Replaces the per-element table of isl_set_laplace. */
int isl_set_laplace_qp(isl_ctx* ctx, const double* kappa, int quad_degree);
int isl_set_hyperelastic(isl_ctx* ctx, int material, const double* lambda, const double* mu, int quad_degree);
/* heat::Static (heat/Static.hpp:98-225), the nonlinear heat conduction kernel,
 * with an isotropic mat::thermal material per element: ISL_THERMAL_CONSTANT
 * (IsotropicConstant, param = conductivity) or ISL_THERMAL_FENICS
 * (FenicsTest, K(u) = (1 + u)^m, param = m; mat/thermal/FenicsTest.hpp).
 * Scalar fields.  Its tangent is not symmetric: the element matrices are
 * staged whole (the contribution lists are rebuilt once, at the next
 * isl_assemble) and the system is solved with ISL_SOLVE_BICGSTAB. */
int isl_set_heat_static(isl_ctx* ctx, int material, const double* param /* [n_elem] */, int quad_degree);
/* Time integration by a linear multi-step method: the inertia terms of
 * base::time::computeInertiaTerms (base/time/ReactionTerms.hpp:62-79,
 * ReactionTerms::operator() :185-254) and the DOF history
 * (DegreeOfFreedom::pushHistory, base/dof/DegreeOfFreedom.hpp:185-190).
 * isl_set_history: keep the DOF values of the last nhist (<= 4) steps, zeroed.
 * isl_push_history: shift them back one step and store the current values as
 * the latest.
 * isl_set_inertia: the next assemblies add lhs_weight * M to the matrix and
 * M h to the right-hand side, with M_ij = int density phi_i phi_j detJ w
 * (base/kernel/Mass.hpp, the kernel's quadrature) and h = sum_s weights[s]
 * x^(s), x^(0) the current values, x^(s) the values s steps back.  For a
 * MultiStep method at time step k: lhs_weight = systemMassWeight(k) / dt and
 * weights[s] = -reactionWeights(k)[s] / dt (incremental; weights[0] = 0
 * otherwise).  Laplace, heat::Static and HyperElastic (every element it
 * runs on), where the mass acts on each displacement component
 * (Mass.hpp:84-86); density NULL turns the terms off. */
int isl_set_history(isl_ctx* ctx, int nhist);
int isl_push_history(isl_ctx* ctx);
int isl_set_inertia(isl_ctx* ctx, const double* density /* [n_elem] */, double lhs_weight, int nweights,
                    const double* weights);
/* The residual-force history of a multi-step method with RHS weights
 * (Adams-Moulton; base::time::computeResidualForceHistory,
 * base/time/ResidualForceHistory.hpp): the next assemblies add
 * -sum_s weights[s-1] F(x^(s)) to the right-hand side, F the kernel's internal
 * force (residualForceHistory<s>) at the values s steps back, s = 1..nweights
 * (<= the stored history, <= 4).  For a MultiStep method at step k: weights =
 * forceWeights(k).  Laplace, heat::Static and HyperElastic (every element
 * it runs on); nweights 0 turns it off. */
int isl_set_force_history(isl_ctx* ctx, int nweights, const double* weights);
/* Body force interpolated from nodal values by the geometry functions
 * (base/asmb/BodyForce.hpp:172-205 with EvaluateViaElement); NULL clears it. */
int isl_set_body_force_nodal(isl_ctx* ctx, const double* f /* [n_nodes][ncomp] */);
/* Constant traction per boundary face (base/asmb/NeumannForce.hpp:132-174);
 * n == 0 clears it. */
int isl_set_neumann(isl_ctx* ctx, int64_t n, const int64_t* elem, const int* face, const double* traction,
                    int squad_degree);
/* Traction given at the vertices of each boundary face ([n][nfv][ncomp], nfv
 * = 2 on quadrilaterals, 4 on hexahedra, in the face's vertex order: element
 * vertices (0,1) (1,2) (2,3) (3,0) of a quadrilateral's faces 0-3, and
 * (0,3,2,1) (4,5,6,7) (0,1,5,4) (1,2,6,5) (2,3,7,6) (3,0,4,7) of a
 * hexahedron's faces 0-5, vertices in hierarchic order) and
 * interpolated by the face geometry functions: the caller's tabulation of a
 * traction function (base/asmb/NeumannForce.hpp:132-174 evaluates it at the
 * surface quadrature points), exact for tractions linear along straight faces
 * such as reference/06-elastic/PulledSheet.hpp:60-75.  Replaces the faces of
 * isl_set_neumann; n == 0 clears them. */
int isl_set_neumann_vertex(isl_ctx* ctx, int64_t n, const int64_t* elem, const int* face, const double* traction,
                           int squad_degree);

/* Current DOF values (DegreeOfFreedom values_[0]) [n_dofobj*ncomp]. */
int isl_set_values(isl_ctx* ctx, const double* u);
int isl_get_values(isl_ctx* ctx, double* u);

/* Assemble the system: stiffness with Dirichlet columns moved to the RHS,
 * body + Neumann forces and, if with_residual, the internal forces times -1.
 * Replaces stiffnessMatrixComputation (base/asmb/StiffnessMatrix.hpp:49-87)
 * + computeResidualForces (base/asmb/ForceIntegrator.hpp:37-71) +
 * bodyForceComputation + neumannForceComputation + Eigen3::finishAssembly
 * (base/solver/Eigen3.hpp:142-153).  precision: ISL_PREC_FP64 (FP64 element
 * kernels, FP64 matrix), ISL_PREC_FP32 (FP32 tangent, FP64 forces, FP32
 * matrix), ISL_PREC_MIXED (FP64 element kernels, FP64 + FP32 matrix copies). */
int isl_assemble(isl_ctx* ctx, int precision, int incremental, int with_residual);

/* Solve the assembled system (Eigen3::cgSolve base/solver/Eigen3.hpp:265-275:
 * Jacobi-preconditioned CG, ||r|| <= tol ||b||, x0 = 0).
 *   ISL_SOLVE_CG_FP64   : FP64 throughout (the plain path)
 *   ISL_SOLVE_CG_FP32_IR: FP32 CG (FP64 dot reductions) with FP64 reliable
 *                         updates: the FP64 residual b - A64 x replaces the
 *                         iterated one each time it has dropped 10x; ends
 *                         when the FP64 residual meets the tolerance.  After
 *                         an ISL_PREC_FP32 assembly (no FP64 matrix) it is a
 *                         plain FP32 CG on the iterated residual, the inexact
 *                         linear solve of a Newton step whose residual is FP64.
 *   ISL_SOLVE_BICGSTAB  : FP64 BiCGSTAB for non-symmetric systems (the
 *                         recurrences of Eigen 3.2's BiCGSTAB, which the
 *                         reference's biCGStabSolve calls,
 *                         base/solver/Eigen3.hpp:277-289), with a Jacobi
 *                         preconditioner instead of IncompleteLUT; x0 = 0,
 *                         ||r|| <= tol ||b||.
 * max_iter <= 0 means 2N.  iters/rel_res may be NULL. */
int isl_solve(isl_ctx* ctx, int method, double tol, int64_t max_iter, int64_t* iters, double* rel_res);

/* After a solve the solution replaces the right-hand side, as in Eigen3
 * (b_ holds x; Eigen3::getValue base/solver/Eigen3.hpp:293-296). */
int isl_get_solution(isl_ctx* ctx, double* x /* [n_active] */);
int isl_get_rhs(isl_ctx* ctx, double* b /* [n_active] */);
/* Eigen3::norm: ||b||_2 / N (base/solver/Eigen3.hpp:128-138), b the
 * right-hand side after an assembly and the solution after a solve (Eigen3's
 * b_ holds x), reduced on the device; one double comes back. */
int isl_norm(isl_ctx* ctx, double* out);
/* setDoFsFromSolver (add=0) / addToDoFsFromSolver (add=1)
 * (base/dof/Distribute.hpp:139-215) */
int isl_distribute(isl_ctx* ctx, int add);

/* Post-processing (base/post/ErrorNorm.hpp).  The reference evaluates a host
 * function of x at every quadrature point; here the caller evaluates it at the
 * points isl_quadrature_points returns and passes the table.
 * isl_quadrature_points: physical coordinates x[(e*nq + q)*dim + d] of the
 * points of Quadrature<quad_degree, SHAPE> (base/Quadrature.hpp:132-141) on
 * every element, x = sum_i N_i(xi_q) X_i; x NULL: only *n_points = nelem*nq.
 * isl_error_norm: base::post::errorComputation<order>
 * (base/post/ErrorNorm.hpp:84-123, functor :300-330) for the field's current
 * values (isl_set_values / isl_distribute):
 *   order 0: ref[(e*nq + q)*ncomp + c] = u_c(x_eq); *error = L2 norm of u - u_h
 *   order 1: ref[((e*nq + q)*ncomp + c)*dim + d] = d u_c / d x_d;
 *            *error = H1 semi-norm of u - u_h
 * i.e. sqrt(sum_e sum_q |ref - approx|^2 detJ w), detJ signed as the
 * reference.  Computed on the device; reproducible bit for bit. */
int isl_quadrature_points(isl_ctx* ctx, int quad_degree, int64_t* n_points, double* x);
int isl_error_norm(isl_ctx* ctx, int order, int quad_degree, const double* ref, double* error);

/* Mesh and field I/O with the reference's text layouts; every host thread
 * converts numbers (the file is cut at line boundaries).
 * isl_mesh_read_smf: base::io::smf::readMesh (base/io/smf/Reader.hpp:36-41,
 * 98-313) followed by isl_mesh_upload: the header must name the shape
 * ("! elementShape", matched as a lower-case substring) and its node count
 * ("! elementNumPoints"); "#" comment lines around the header; "!
 * externalNodes" / "! externalElements" files opened as given; per node line
 * the first dim numbers, per element line the 0-based node indices in file
 * order.  Errors: ISL_ERR_ARG with the reference's messages.
 * isl_mesh_get: counts and host copies of the mesh (either array may be NULL).
 * isl_mesh_write_smf: base::io::smf::writeMesh (base/io/smf/Writer.hpp:60-140).
 * isl_write_vtk: base::io::vtk::LegacyWriter (base/io/vtk/LegacyWriter.hpp)
 * writeUnstructuredGrid, then, when point_name is given, writePointData of
 * the field's current values at the geometry nodes, and, when cell_name is
 * given, writeCellData of cell_values: per cell a cell_rows x cell_cols
 * matrix (row-major, at most 3 x 3) or, with 0 x 0, one plain double. */
int isl_mesh_read_smf(isl_ctx* ctx, const char* path, int shape);
int isl_mesh_get(isl_ctx* ctx, int64_t* n_nodes, int64_t* n_elem, double* coords, int64_t* conn);
int isl_mesh_write_smf(isl_ctx* ctx, const char* path);
int isl_write_vtk(isl_ctx* ctx, const char* path, const char* point_name, const char* cell_name, int cell_rows,
                  int cell_cols, const double* cell_values);

/* Assembled CSR (int64 row pointers / column ids, FP64 values) for parity. */
int isl_get_csr(isl_ctx* ctx, int64_t* rowptr, int64_t* colind, double* values);

/* Synchronise the context stream; per-phase timings of the last assemble /
 * solve (ms) when timing is on. */
int isl_sync(isl_ctx* ctx);
int isl_set_timing(isl_ctx* ctx, int on);
int isl_timings(isl_ctx* ctx, double* ms /* [ISL_NTIMERS] */, int64_t* counts /* [ISL_NTIMERS] */);
/* Solver options.  ISL_OPT_BLOCK_SOLVER (default 1): the mixed solve (and
 * the FP32 solve of a system assembled in ISL_PREC_FP32 alone) of a single
 * 3-component field uses a 3x3 node-block copy of the FP32 matrix with
 * block-Jacobi preconditioning; 0 keeps the scalar CSR + Jacobi path.  DOF
 * objects with some components constrained keep padded blocks (zero rows
 * and columns at the constrained components, identity in their Jacobi
 * block; the solver vectors carry zeros there).  Read-only through
 * isl_get_option: ISL_OPT_BLOCKED (1: node-blocked, 2: node-blocked with
 * padded blocks, 0: scalar),
 * ISL_OPT_NBLOCKS (stored 3x3 blocks), ISL_OPT_NSLOTS (block slots of the
 * sliced-ELL copy, padding included).  ISL_OPT_PERSISTENT selects the
 * one-launch CG kernels of the mixed solve: 0 never (CUDA graphs of separate
 * kernels), 1 (default) for small systems, where launch latency dominates:
 * a scalar system of at most 65,536 equations is solved whole, FP64 reliable
 * updates included, by one thread-block cluster; a node-blocked system of at
 * most 32,768 nodes runs its iterations in a persistent cooperative kernel.
 * 2: the persistent block kernel at every size.  ISL_OPT_BARRIER_TEST (test
 * hook, write-only, one-shot): the next persistent launch starts with its grid
 * barrier armed so that it cannot complete; its bounded wait runs out and the
 * solve returns ISL_ERR_TIMEOUT with the context still usable.
 * ISL_OPT_SPMV32_KIND: the FP32 SpMV of the scalar mixed solve, 0 (default)
 * autotuned on the matrix, 2, 4, 8, 16 or 32 CSR with that many lanes per
 * row, 102, 104 or 108 the sliced-ELL copy with 2, 4 or 8 slots of loads in
 * flight per lane (only where the copy exists, or on a batch, which builds
 * its copy at its first mixed solve); read back, the kind in use (0 before
 * the first mixed solve).  ISL_OPT_SCALAR_SLOTS (read-only): slots
 * of the scalar sliced-ELL copy, padding included; 0 when there is none
 * (node-blocked, batched, or fewer than 20,000 equations).
 * ISL_OPT_HOST_SETUP (default 0): with a device, isl_field_create numbers the
 * DOF objects of fields of degree > 1 and isl_boundary_faces /
 * isl_boundary_points find the boundary on the GPU (sorts and scans, the
 * same ids and order as the host rules); 1 runs both on the host.
 * ISL_OPT_BICGSTAB_KIND: the FP64 SpMV of ISL_SOLVE_BICGSTAB, 0 (default)
 * autotuned per pattern, 2, 4, 8 or 16 CSR lanes per row, 102, 104 or 108
 * the sliced-ELL copy with FP64 values (where it exists); read back, the kind
 * of the last solve. */
enum { ISL_OPT_BLOCK_SOLVER = 0, ISL_OPT_BLOCKED = 1, ISL_OPT_NBLOCKS = 2, ISL_OPT_NSLOTS = 3, ISL_OPT_PERSISTENT = 4,
       ISL_OPT_BARRIER_TEST = 5, ISL_OPT_SPMV32_KIND = 6, ISL_OPT_SCALAR_SLOTS = 7, ISL_OPT_HOST_SETUP = 8,
       ISL_OPT_BICGSTAB_KIND = 9, ISL_OPT_BATCHED_SOLVE = 10, ISL_OPT_DIRECT_BLOCKS = 11, ISL_OPT_TUNE_RUNS = 12,
       ISL_OPT_ELEM_VARIANT = 13, ISL_OPT_FOLD_DIRECTION = 14, ISL_OPT_BLOCK_UPDATE = 15,
       ISL_OPT_SHORT_COLUMNS = 16, ISL_OPT_RELIABLE_DROP = 17, ISL_OPT_SHARED_GEOMETRY = 18 };
/* ISL_OPT_SHARED_GEOMETRY (default 1): the direct block assembly
 * (ISL_OPT_DIRECT_BLOCKS) of a mesh whose hexahedra are all translates of the
 * first (edge vectors equal within 1e-13) forms the 64 local pairs' Lame
 * blocks once from the first element's Jacobian and adds lam_e and mu_e
 * multiples of them per element; 0 forms every element's blocks from its own
 * Jacobian.  Read back: 1 when the last assembly used the shared blocks. */
/* ISL_OPT_RELIABLE_DROP (default 2): the mixed CG (one system on the graph
 * path, or each instance of a batch) takes an FP64 reliable update when its
 * FP32 r.r has dropped by 10^value since the last one (2: 100x in r.r, i.e.
 * 10x in ||r||); 1..8.  The one-launch solves of small systems keep 2. */
/* ISL_OPT_SHORT_COLUMNS (default 1): the block SpMV with the folded direction
 * update reads each slot's column as a 16-bit offset from its block row (2 B
 * per stored block instead of 4), and the FP32 scalar sliced-ELL SpMVs (one
 * system, or a batch) as an offset from the slot's row (6 B per stored entry
 * instead of 8), when every offset of the matrix fits; 0 keeps the 32-bit
 * columns.  Read back: 1 when the 16-bit columns are in use (the option on
 * and the offsets fitting). */
/* ISL_OPT_BLOCK_UPDATE: the update kernel of the graph path of the block CG
 * (x, r, z = B^-1 r, r.r, r.z): 1 one thread per node (what 0, the default,
 * selects), 2, 4 or 8 tiles of 256 nodes staged through shared memory with
 * that many blocks per SM.  Read back: the value set (0: the default). */
/* ISL_OPT_FOLD_DIRECTION (default 1): the graph path of the node-blocked
 * mixed solve forms the search direction p = B^-1 r + beta p inside the block
 * SpMV (the update kernel stores z = B^-1 r; each column block of p is formed
 * where the product reads it, and its owner row writes it to the second of
 * two direction buffers), two launches per iteration instead of three; 0
 * keeps the separate direction kernel.  Applies to the batched-load SpMV
 * variants the autotune prefers. */
/* ISL_OPT_TUNE_RUNS (read-only): autotunes of this context that timed their
 * candidates; the others took their choice from the tuning cache.
 * ISL_OPT_ELEM_VARIANT (read-only): the launch shape the element kernel
 * autotune chose (threads per block of the one-thread-per-element kernels,
 * elements per block of the eight-threads-per-element hexahedron kernel);
 * 0 before the first assembly. */
/* ISL_OPT_DIRECT_BLOCKS (read-only): 1 when the last assembly formed the
 * matrix blocks directly: ISL_PREC_MIXED small-strain HyperElastic<StVenant>
 * (u = 0, no body force or time-integration terms) on trilinear
 * parallelepipeds with 2x2x2 points and a node-blocked pattern, the block
 * solver on.  One thread per stored 3x3 block adds the blocks of the
 * elements its two DOF objects share, in element order, in double-float
 * arithmetic (about 48 bits), and writes the FP64 CSR values and the FP32
 * block copies; no element matrices are staged.  The scalar FP32 CSR values
 * are then derived from the FP64 ones when a scalar FP32 path needs them. */
/* ISL_OPT_BATCHED_SOLVE (default 0): 1 runs the CG of a context holding one
 * instance through the batched solver (per-instance scalars and reductions),
 * so that its result is bitwise the same as when it is solved inside a batch
 * of instances; batches always use it. */
int isl_set_option(isl_ctx* ctx, int key, int64_t value);
int isl_get_option(isl_ctx* ctx, int key, int64_t* value);

/* Device-side marks on the context stream (CUDA events, 8 slots) and the
 * elapsed time between two of them, for timing regions from the host. */
int isl_mark(isl_ctx* ctx, int slot);
int isl_elapsed(isl_ctx* ctx, int slot_a, int slot_b, double* ms);
/* Free and total device memory (cudaMemGetInfo) of a device, for admission
 * control of served requests. */
int isl_device_memory(int device, int64_t* free_bytes, int64_t* total_bytes);
/* Number of kernel launches (graph kernel nodes included) issued by the
 * context since creation. */
int isl_launch_count(isl_ctx* ctx, int64_t* n);
/* Average device time (ms) of one launch of the solver's SpMV kernel on the
 * current matrix, precision ISL_PREC_FP64 or ISL_PREC_FP32, over nrep launches
 * that follow one untimed launch; nrep < 0: over -nrep launches with no
 * launch before them (the first starts from whatever the caches hold).
 * On a batch: the batched SpMV of isl_solve with every instance active (the
 * FP32 kind the last mixed solve chose). */
int isl_time_spmv(isl_ctx* ctx, int precision, int nrep, double* ms_per_launch);

/* Warm per-kernel device time (ms per launch, CUDA events over nrep launches)
 * of the solver's kernels on the current system: ms[0] FP32 block SpMV,
 * ms[1] block-Jacobi update, ms[2] block-Jacobi direction, ms[3] FP64 CSR
 * SpMV, ms[4] FP64 update, ms[5] FP64 direction, ms[6] FP64 residual, ms[7]
 * the autotuned block SpMV variant (-1 entries: not applicable). */
int isl_time_kernels(isl_ctx* ctx, int nrep, double* ms /* [8] */);

/* Tuning cache of the autotuned kernel variants (the SpMV formats of the
 * solvers, the element kernels' launch shapes), keyed by the problem class:
 * tuner, shape, field degree, components, kernel, material, node-blocked,
 * batched, and floor(log2(equations)).  Kept in memory for the process; with
 * a path (or the environment variable ISL_TUNE_CACHE, read on first use) the
 * entries are read from and appended to that text file, so later processes
 * take the same variants without timing them.  path NULL: memory only.
 * No reference counterpart (the reference's only knob is the compile-time
 * thread count of its element loop, base/auxi/parallel.hpp:37-56). */
int isl_tune_cache(const char* path);

/* Served solves with continuous batching.  No single reference counterpart:
 * each request is one run of solid::CompressibleDriver's load stepping and
 * Newton loop (solid/CompressibleDriver.hpp:156-214) on its own mesh and
 * field, and the server runs many requests on one GPU at once.
 *
 * A request: an isoparametric field (geometry and field of degree 1, one DOF
 * object per node) on its own mesh; heat::Laplace (ncomp 1, coef0 = the
 * conductivity per element) or solid::HyperElastic (ncomp = dim, material
 * ISL_MAT_*, coef0 / coef1 = lambda / mu per element); an optional nodal body
 * force; Dirichlet values per (node, component) for the first load step,
 * scaled by (k+1)/k at load step k as the driver does (:164-172).  Per load
 * step, Newton: assemble tangent and residual (incremental), stop when
 * ||R||/N < tolerance, solve (CG to lin_tol), add the increment, stop when
 * ||dU||/N < tolerance or after max_newton iterations (:180-211).  The
 * request's arrays are copied at submit.
 *
 * The server forms batches from the queue in arrival order (same shape,
 * ncomp, kernel, material, quadrature and lin_tol; at most max_batch
 * requests; within the 32-bit contribution budget max_pairs and the free HBM
 * minus reserve_bytes; a partial batch waits up to batch_window_us after its
 * oldest request arrived, to take in requests submitted together; with
 * size_ratio > 1 only requests of similar element counts share a batch, so a
 * small request does not run at the pace of a large one) and runs
 * each batch as one context of instances on its own stream and host thread;
 * at most max_batches batches run at once,
 * so requests that arrive while others run are admitted as batches finish
 * and memory frees up.  A batch shares every launch of a Newton iteration
 * between its requests (assembly, norms, CG with per-request convergence,
 * distribute); each request follows its own Newton loop and completes as
 * soon as it finishes.  With max_batch > 1 every batch (a batch of one too)
 * runs the batched solver, so a request's result does not depend on its
 * batch; with max_batch = 1 each request runs the single-system solvers.
 * precision: ISL_PREC_FP64 (FP64 tangent and CG), ISL_PREC_FP32 (FP32
 * tangent and FP32 CG, FP64 residual: inexact Newton steps) or
 * ISL_PREC_MIXED (FP64 and FP32 matrices, FP32 CG with FP64 reliable
 * updates).  A failure inside a batch (for example a degenerate element)
 * fails every request of that batch with the status and message.
 * test_budget_bytes > 0 replaces the free-HBM figure by a fixed budget, and
 * test_fake_us_per_elem > 0 replaces the GPU work by a sleep of that many
 * microseconds per element (scheduler tests without a GPU). */
typedef struct isl_server isl_server;
typedef struct {
    int max_batch;            /* requests per batch */
    int max_batches;          /* batches running at once */
    int precision;            /* ISL_PREC_* */
    int64_t reserve_bytes;    /* HBM kept free */
    int64_t max_pairs;        /* element pairs (n_elem * nloc^2) per batch; <= 0: 1.3e9 */
    int64_t test_budget_bytes;
    double test_fake_us_per_elem;
    int64_t batch_window_us;  /* a partial batch waits this long after its oldest request arrived (0: none) */
    double size_ratio;        /* > 1: a batch takes only requests whose element count is within this factor of
                                 its first request's (requests of other sizes wait for a batch of their own);
                                 <= 1: any size */
    int persistent;           /* ISL_OPT_PERSISTENT of single-request batches' contexts: 0 (default) CUDA graphs
                                 of separate kernels, which overlap with the other batches' launches; 1 the
                                 library default (small systems solved in one launch: a cooperative grid over
                                 every SM, or one thread-block cluster) */
    int order;                /* 0 (default): batches start from the oldest queued request; 1: from the
                                 largest (elements; the oldest among equals), which shortens the time to
                                 finish a queue of requests submitted together */
} isl_serve_config;
typedef struct {
    int shape;                /* ISL_QUAD, ISL_TET, ISL_HEX */
    int64_t n_nodes;
    const double* coords;     /* [n_nodes][dim] */
    int64_t n_elem;
    const int64_t* conn;      /* [n_elem][n_vertices], hierarchic order, ids < n_nodes */
    int ncomp;
    int kernel;               /* ISL_KERNEL_LAPLACE or ISL_KERNEL_HYPERELASTIC */
    int material;             /* ISL_MAT_* (HyperElastic) */
    int quad_degree;
    const double* coef0;      /* [n_elem] */
    const double* coef1;      /* [n_elem] or NULL */
    const double* body;       /* [n_nodes][ncomp] or NULL */
    int64_t n_fixed;
    const int64_t* fixed_node;
    const int* fixed_comp;
    const double* fixed_value;
    int load_steps;
    int max_newton;
    double tolerance;         /* on ||R||/N and ||dU||/N */
    double lin_tol;           /* CG: ||r|| <= lin_tol ||b|| */
} isl_serve_request;
typedef struct {
    int64_t newton_iters, cg_iters, load_steps_done;
    int converged;            /* every load step met the tolerance within max_newton */
    int status;               /* ISL_OK or the failing isl_status */
    double t_submit, t_admit, t_finish;  /* seconds since isl_serve_create */
    int64_t batch_id;
    int batch_size;
} isl_serve_stats;
int isl_serve_create(isl_server** out, int device, const isl_serve_config* cfg);
/* queue a request; *ticket identifies it */
int isl_serve_submit(isl_server* s, const isl_serve_request* req, int64_t* ticket);
/* state: 0 queued, 1 running, 2 done, 3 failed */
int isl_serve_poll(isl_server* s, int64_t ticket, int* state);
/* wait up to timeout_s for the request to finish (ISL_ERR_TIMEOUT if it has not) */
int isl_serve_wait(isl_server* s, int64_t ticket, double timeout_s, int* state);
/* DOF values [n_nodes][ncomp] (u may be NULL) and statistics of a finished
 * request; returns its status */
int isl_serve_result(isl_server* s, int64_t ticket, double* u, isl_serve_stats* stats);
const char* isl_serve_error(isl_server* s, int64_t ticket);
/* forget a finished request */
int isl_serve_release(isl_server* s, int64_t ticket);
/* kernel launches of the finished batches and batches formed so far */
int isl_serve_counters(isl_server* s, int64_t* launches, int64_t* batches);
/* host wall time of the finished batches (any pointer may be NULL): context
 * setup, assembly with the residual norms, solve with the distribute and the
 * increment norms, whole batches; and the Newton iterations they ran */
int isl_serve_times(isl_server* s, double* setup_s, double* assemble_s, double* solve_s, double* batch_s,
                    int64_t* newton_ticks);
/* waits for the running batches; queued requests fail */
int isl_serve_destroy(isl_server* s);

/* Allocation-free FP64 CG.  This entry point has no counterpart in the
 * reference; it serves callers that must not allocate device memory while
 * they solve: an application that owns all device memory through its own
 * pool or arena (a cudaMalloc there fails or fragments the pool), and
 * time-stepping or control loops that solve every step, where cudaMalloc /
 * cudaFree would synchronise the device and stall the loop.
 *
 * Same algorithm as isl_solve(ISL_SOLVE_CG_FP64): Jacobi-preconditioned CG,
 * x0 = 0, stops when ||r|| <= tol ||b|| or after max_iter iterations
 * (max_iter <= 0 means 2n).  Every pointer is a caller-owned device pointer on
 * `device`: the n x n CSR matrix (rowptr[n+1], colind[nnz], val[nnz]), b[n]
 * and the output x[n].  `stream` is a cudaStream_t (NULL: the default
 * stream).  The call reads the CG scalars back to the host and waits on
 * `stream` after every round of 32 iterations, and returns once the solve has
 * finished.  iters/rel_res may be NULL; on every status after the solve has
 * started they hold the iterations and relative residual of the last scalar
 * record read back.
 *
 * The work vectors live in one scratch array compiled into the library's
 * device code: ISL_NOALLOC_MAX_N entries for each of its four vectors plus
 * the partial sums, about 2.1 MiB that every GPU loading the library holds
 * until the process exits.  n > ISL_NOALLOC_MAX_N returns ISL_ERR_CAPACITY
 * before any device work.  The call makes no cudaMalloc / cudaFree and no
 * other allocating call.
 *
 * The first call on a device looks the scratch array up on that device
 * (cudaGetSymbolAddress, with that device current), and looks it up again
 * when the device's context has changed (after cudaDeviceReset).  Every call
 * copies to the host and waits on `stream`, so no call may run while that
 * stream (or the legacy default stream) is being captured into a graph.
 * All calls on a device share the one array, and
 * it keeps the last call's contents: each call clears what has to start at
 * zero, but calls that overlap on the GPU (other streams or host threads)
 * race on it and must be serialised by the caller. */
#define ISL_NOALLOC_MAX_N 65536
int isl_cg_solve_noalloc(int device, void* stream, int n, const int32_t* rowptr, const int32_t* colind,
                         const double* val, const double* b, double* x, double tol, int64_t max_iter,
                         int64_t* iters, double* rel_res);

#ifdef __cplusplus
}
#endif
#endif /* ISL_GPU_H */
