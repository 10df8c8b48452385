/*
 * ikarus_gb300.h -- C ABI of the GB300-native Newton-Raphson / LoadControl path for Q1 hexahedral
 * Neo-Hookean solids (displacement-based and enhanced-assumed-strain), mirroring ikarus-project/ikarus v0.4.9.
 *
 * Plain pointers and sizes only.  Every function returns IKR_OK (0) or a negative IKR_ERR_* status; the
 * message of the last failure on the calling thread is available from ikr_last_error().  No function
 * throws or aborts.  Arrays passed in are host arrays and are copied; device storage belongs to the
 * library.  Handles are not thread-safe: use one handle set per host thread (or lock externally).
 *
 * Numbering: dof = 3 * node + component (FlatInterleaved, ikarus/utils/flatprebasis.hh:57-76).
 * Element corners in Dune reference-cube order (vertex v at (v&1, v>>1&1, v>>2&1)).
 * Element-local dofs are node-major (local k = 3*i + c, ikarus/finiteelements/fehelper.hh:145-153).
 * Element matrices are returned column-major (Eigen default, fetraits.hh:79-86).
 */
#ifndef IKARUS_GB300_H
#define IKARUS_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace DUNE_THROW / abort(): no exception crosses the C ABI) ----------------------- */
enum {
  IKR_OK = 0,
  IKR_ERR_ARG = -1,
  IKR_ERR_NOT_IMPLEMENTED = -2,   /* DUNE_THROW(Dune::NotImplemented), e.g. enhancedassumedstrains.hh:231-235 */
  IKR_ERR_INVALID_STATE = -3,     /* DUNE_THROW(Dune::InvalidStateException), e.g. assembler/interface.hh:187-193 */
  IKR_ERR_NONPOSITIVE_DETC = -4,  /* checkPositiveOrAbort, materials/materialhelpers.hh:119-126 (aborts there) */
  IKR_ERR_NOT_CONVERGED = -5,
  IKR_ERR_CG_BREAKDOWN = -6,
  IKR_ERR_CUDA = -7,
  IKR_ERR_SINGULAR = -8,
  IKR_ERR_NO_DEVICE = -9,
  IKR_ERR_TIMEOUT = -10           /* a bounded wait inside a kernel gave up (the context stays usable) */
};

/* ---- enums with the reference's values ------------------------------------------------------------------ */
/* DBCOption, ikarus/assembler/dirichletbcenforcement.hh:8 */
enum { IKR_DBC_RAW = 0, IKR_DBC_REDUCED = 1, IKR_DBC_FULL = 2 };
/* VectorAffordance / MatrixAffordance / ScalarAffordance, ikarus/finiteelements/ferequirements.hh:35-89 */
enum { IKR_VEC_NO_AFFORDANCE = 0, IKR_VEC_FORCES = 1 };
enum { IKR_MAT_NO_AFFORDANCE = 0, IKR_MAT_STIFFNESS = 1 };
enum { IKR_SCALAR_NO_AFFORDANCE = 0, IKR_SCALAR_MECHANICAL_POTENTIAL_ENERGY = 1 };
/* strain measure enhanced by EAS: none (NonLinearElastic only), EAS::GreenLagrangeStrain,
 * EAS::DisplacementGradient, EAS::DisplacementGradientTransposed (strainenhancements/easfunctions/) */
enum { IKR_EAS_NONE = 0, IKR_EAS_GREEN_LAGRANGE = 1, IKR_EAS_DISPLACEMENT_GRADIENT = 2,
       IKR_EAS_DISPLACEMENT_GRADIENT_TRANSPOSED = 3 };
/* SolverTypeTag (ikarus/solver/linearsolver/linearsolver.hh:28-31): all 19 names with the reference's values, then
 * the device solvers of this library.  What each reference tag runs on the device (tangents of this path are
 * symmetric, and nonsingular wherever the reference's solvers succeed, so every sparse tag has the same solution):
 *   si_ConjugateGradient, si_LeastSquaresConjugateGradient, si_BiCGSTAB (Eigen's iterative solvers with their
 *     default diagonal preconditioner): device CG with point-Jacobi preconditioning, tolerance as set (1e-10);
 *   sd_SimplicialLLT, sd_SimplicialLDLT (the reference's default SPD solver, controlroutines/common.hh:39-54),
 *     sd_SparseLU, sd_SparseQR, sd_CholmodSupernodalLLT, sd_UmfPackLU (the cantilever goldens' solver): a
 *     direct-accuracy solve -- FP64 block-Jacobi CG to ||r|| <= 1e-13 ||b|| (or the tolerance set, whichever is
 *     tighter, whatever the Newton's linear tolerance); an FP32 tangent needs the FP64 outer solve
 *     (ikr_linear_solver_set_fp64_outer), else IKR_ERR_NOT_IMPLEMENTED;
 *   sd_SuperLU: IKR_ERR_NOT_IMPLEMENTED at creation (the reference throws there, linearsolver.cpp:51-53);
 *   d_* (dense solvers): created, but factorize / compute on the sparse assembled tangent return
 *     IKR_ERR_NOT_IMPLEMENTED (the reference throws "does not support solving with sparse matrices",
 *     linearsolver.hh:139-144);
 *   none: created; factorize returns IKR_ERR_INVALID_STATE (no solver behind it). */
enum {
  IKR_SOLVER_NONE = 0,
  IKR_SOLVER_SI_CONJUGATE_GRADIENT = 1,
  IKR_SOLVER_SI_LEAST_SQUARES_CONJUGATE_GRADIENT = 2,
  IKR_SOLVER_SI_BICGSTAB = 3,
  IKR_SOLVER_SD_SIMPLICIAL_LLT = 4,
  IKR_SOLVER_SD_SIMPLICIAL_LDLT = 5,
  IKR_SOLVER_SD_SPARSE_LU = 6,
  IKR_SOLVER_SD_SPARSE_QR = 7,
  IKR_SOLVER_SD_CHOLMOD_SUPERNODAL_LLT = 8,
  IKR_SOLVER_SD_UMFPACK_LU = 9,
  IKR_SOLVER_SD_SUPER_LU = 10,
  IKR_SOLVER_D_PARTIAL_PIV_LU = 11,
  IKR_SOLVER_D_FULL_PIV_LU = 12,
  IKR_SOLVER_D_HOUSEHOLDER_QR = 13,
  IKR_SOLVER_D_COL_PIV_HOUSEHOLDER_QR = 14,
  IKR_SOLVER_D_FULL_PIV_HOUSEHOLDER_QR = 15,
  IKR_SOLVER_D_COMPLETE_ORTHOGONAL_DECOMPOSITION = 16,
  IKR_SOLVER_D_LLT = 17,
  IKR_SOLVER_D_LDLT = 18,
  IKR_SOLVER_GPU_PCG_BLOCK_JACOBI = 100,  /* FP64 or FP32 CG, 3x3 block-Jacobi, precision of the assembled K */
  IKR_SOLVER_GPU_PCG_BATCHED = 101,       /* one block-Jacobi CG per instance, all in one launch (see below) */
};
#define IKR_DIRECT_SOLVE_RTOL 1e-13
/* precision of the assembled tangent */
enum { IKR_PRECISION_FP64 = 0, IKR_PRECISION_FP32 = 1 };
/* messages, ikarus/utils/broadcaster/broadcastermessages.hh:18,23-24 (spelling of the reference kept) */
enum { IKR_CONTROL_STARTED = 0, IKR_CONTROL_ENDED, IKR_STEP_STARTED, IKR_STEP_ENDED, IKR_CONTROL_SOLUTION_CHANGED };
enum { IKR_NLS_INIT = 0, IKR_NLS_ITERATION_STARTED, IKR_NLS_ITERATION_ENDED, IKR_NLS_RESIDUALNORM_UPDATED,
       IKR_NLS_CORRECTIONNORM_UPDATED, IKR_NLS_CORRECTION_UPDATED, IKR_NLS_SOLUTION_CHANGED,
       IKR_NLS_FINISHED_SUCESSFULLY };

typedef struct ikr_fes_s* ikr_fes;   /* the bound finite elements of one mesh (the reference's std::vector<FE>) */
typedef struct ikr_req_s* ikr_req;   /* FERequirements: displacement (device, FP64) + load factor */
typedef struct ikr_asm_s* ikr_asm;   /* SparseFlatAssembler (+ AssemblerManipulator point loads) */
typedef struct ikr_ls_s* ikr_ls;     /* LinearSolver */
typedef struct ikr_nr_s* ikr_nr;     /* NewtonRaphson */
typedef struct ikr_lc_s* ikr_lc;     /* LoadControl */

/* ---- library ---------------------------------------------------------------------------------------------- */
int ikr_version(void);
/* copies the last error message of this thread (NUL-terminated, truncated to len) */
int ikr_last_error(char* buf, int32_t len);
/* number of kernels this library has launched (for launch-count reporting) */
int64_t ikr_kernel_launches(void);

/* ---- finite elements ----------------------------------------------------------------------------------------
 * Replaces: for (ge : elements(gridView)) { fes.emplace_back(makeFE(basis, skills(nonLinearElastic(NeoHooke(
 * {lambda, mu})), eas<ES>(n_alpha)))); fes.back().bind(ge); }  (fefactory.hh:67-72, febase.hh:77-161,
 * nonlinearelastic.hh:439-444, enhancedassumedstrains.hh:443-448, materials/hyperelastic/neohooke.hh:37-208).
 * conn: n_elems x 8 corner node ids (row-major), coords: n_nodes x 3. */
int ikr_fes_create(ikr_fes* out, int32_t n_nodes, const double* coords, int32_t n_elems, const int32_t* conn,
                   double lambda, double mu, int32_t eas_kind, int32_t n_alpha);
/* Replaces skills(neumannBoundaryLoad(patch, f)) (loads/traction.hh:21-33, 105-138): dead traction
 * lambda * t on each listed face (Dune face numbering 2d: xi_d = 0, 2d+1: xi_d = 1), t given per face as the
 * value of f at the face's single quadrature point (the face centre; rule order = order() = 1). */
int ikr_fes_add_neumann(ikr_fes fes, int32_t n_faces, const int32_t* face_elem, const int32_t* face_local,
                        const double* traction);
/* Loads given as functions of the position and the load factor, evaluated on the host:
 * out[3k .. 3k+2] = f(X[3k .. 3k+2], lambda) for k < n (the reference's std::function<Vector(FieldVector, double)>). */
typedef void (*ikr_point_fn)(int32_t n, const double* X, double lambda, double* out, void* user);
/* Replaces skills(neumannBoundaryLoad(patch, f)) with a general f(X, lambda) (loads/traction.hh:21-33, 105-138): the
 * traction f at each listed face's quadrature point (the face centre, rule order 1).  f is called whenever a force
 * vector or energy is assembled at a load factor other than the last one (one call per Neumann set with all its
 * face points); ikr_fes_add_neumann is the faster form for f(X, lambda) = lambda t(X). */
int ikr_fes_add_neumann_function(ikr_fes fes, int32_t n_faces, const int32_t* face_elem, const int32_t* face_local,
                                 ikr_point_fn f, void* user);
/* Replaces skills(volumeLoad<3>(f)) (loads/volume.hh:86-106): body force f(X, lambda) per unit reference volume on
 * every element, integrated with the element's 2x2x2 Gauss rule, f_I -= N_I b w detJ (and -u.b w detJ in the energy).
 * f is called with the 8 n_elems Gauss points (element-major; point q = x + 2y + 4z of the element, xi_d =
 * 1/2 -+ 1/(2 sqrt 3) for bit d of q clear / set) whenever the load factor changes.  Several volume loads add up. */
int ikr_fes_add_volume_load(ikr_fes fes, ikr_point_fn f, void* user);
int ikr_fes_clear_volume_loads(ikr_fes fes);
/* removes every Neumann load added so far (the element set keeps its mesh, material and state) */
int ikr_fes_clear_neumann(ikr_fes fes);
/* per-element Lame parameters (n_elems each) replacing the set's single NeoHooke material */
int ikr_fes_set_element_materials(ikr_fes fes, const double* lambda, const double* mu);
/* Declares the mesh a union of n_instances independent problems on the contiguous node ranges
 * [node_offsets[i], node_offsets[i+1]) (no element may connect two ranges).  With the solver tag
 * IKR_SOLVER_GPU_PCG_BATCHED every instance then runs its own Newton test (relative to its own initial
 * residual) and its own CG, all instances in one launch per Newton iteration (no reference counterpart). */
int ikr_fes_set_instances(ikr_fes fes, int32_t n_instances, const int32_t* node_offsets);
int ikr_fes_destroy(ikr_fes fes);
int ikr_fes_num_colours(ikr_fes fes, int32_t* n_colours);
/* EAS internal variables alpha_ (enhancedassumedstrains.hh:207, 364): n_elems x n_alpha, row-major */
int ikr_fes_get_alpha(ikr_fes fes, double* alpha);
int ikr_fes_set_alpha(ikr_fes fes, const double* alpha);

/* ---- element level: calculateVector / calculateMatrix / calculateScalar (mixin.hh:126-152) and
 * updateState (mixin.hh:284-287), batched over the element range [e_begin, e_end).  Results are written
 * (not added) to out: 24 (vector), 576 column-major (matrix) or 1 (scalar) values per element. ---------- */
int ikr_fe_calculate_vector(ikr_fes fes, ikr_req req, int32_t affordance, int32_t e_begin, int32_t e_end,
                            double* out);
int ikr_fe_calculate_matrix(ikr_fes fes, ikr_req req, int32_t affordance, int32_t e_begin, int32_t e_end,
                            double* out);
/* calculateAt<ResultType> (nonlinearelastic.hh:237-271, feresulttypes.hh:125-133): stress of every element in
 * [e_begin, e_end) at a local point of the reference cube [0,1]^3 (local: 3 values per element when
 * local_per_element != 0, else 3 for all); out: 6 Voigt values per element [11, 22, 33, 23, 13, 12] without shear
 * factors (toVoigt(S, false)).  EAS element sets use their stored alpha (enhancedassumedstrains.hh:127-188): GL
 * enhances the strain (F compatible), H9 / H9T the displacement gradient. */
enum { IKR_RESULT_PK2_STRESS = 0, IKR_RESULT_KIRCHHOFF_STRESS = 1, IKR_RESULT_CAUCHY_STRESS = 2 };
int ikr_fe_calculate_at(ikr_fes fes, ikr_req req, int32_t result_type, int32_t e_begin, int32_t e_end,
                        const double* local, int32_t local_per_element, double* out);
int ikr_fe_calculate_scalar(ikr_fes fes, ikr_req req, int32_t affordance, int32_t e_begin, int32_t e_end,
                            double* out);
/* EAS::updateStateImpl (enhancedassumedstrains.hh:225-248) on every element; correction has n dofs (a
 * reduced-size correction returns IKR_ERR_NOT_IMPLEMENTED like the reference). */
int ikr_fe_update_state(ikr_fes fes, ikr_req req, const double* correction, int32_t correction_size);

/* ---- FERequirements (ferequirements.hh:222-407) -------------------------------------------------------- */
int ikr_req_create(ikr_req* out, ikr_fes fes);
int ikr_req_destroy(ikr_req req);
int ikr_req_insert_global_solution(ikr_req req, const double* u);  /* copies n dofs to the device */
int ikr_req_global_solution(ikr_req req, double* u);               /* copies n dofs to the host */
int ikr_req_insert_parameter(ikr_req req, double load_factor);
int ikr_req_parameter(ikr_req req, double* load_factor);
/* device address of the displacement (valid for the lifetime of req) */
int ikr_req_solution_device(ikr_req req, double** dptr);
/* deep copy of solution and load factor, device to device (the FERequirements copy constructor,
 * ferequirements.hh:222-407); both requirements must belong to the same element set */
int ikr_req_copy(ikr_req dst, ikr_req src);

/* ---- SparseFlatAssembler (simpleassemblers.hh:108-177, assembler/interface.hh:28-266) --------------------
 * fixed: n dofs, 1 = constrained (DirichletValues flags, dirichletvalues.hh:110-131, 187-194).
 * precision: IKR_PRECISION_FP64 or IKR_PRECISION_FP32 for the stored tangent. */
int ikr_assembler_create(ikr_asm* out, ikr_fes fes, const uint8_t* fixed, int32_t precision);
int ikr_assembler_destroy(ikr_asm a);
/* AssemblerManipulator vector hook (assemblermanipulatorbuildingblocks.hh:94-121) of the form
 * vec[dof] += load_factor * value, applied after the Dirichlet treatment. */
int ikr_assembler_add_point_loads(ikr_asm a, int32_t n, const int32_t* dofs, const double* values);
/* AssemblerManipulator matrix hook (assemblermanipulatorbuildingblocks.hh:155-183) in the form of the reference's
 * springs (testassembler.cpp:212-219): after every matrix assembly and its Dirichlet treatment K(rows[k], cols[k])
 * += values[k] (full-system dof indices inside the sparsity pattern; repeated calls accumulate).  The Reduced
 * option keeps the entries of free rows and columns only. */
int ikr_assembler_add_matrix_entries(ikr_asm a, int32_t n, const int32_t* rows, const int32_t* cols,
                                     const double* values);
int ikr_assembler_bind(ikr_asm a, ikr_req req, int32_t dbc_option);                    /* interface.hh:150-175 */
int ikr_assembler_size(ikr_asm a, int32_t* size);
int ikr_assembler_reduced_size(ikr_asm a, int32_t* size);
int ikr_assembler_constraints_below(ikr_asm a, int32_t* out);   /* n dofs, interface.hh:50-62 */
/* vector(req, affordance, dbc) (interface.hh:355-365): assembles on the device; out (host, may be NULL)
 * receives size() or reducedSize() values. */
int ikr_assembler_vector(ikr_asm a, ikr_req req, int32_t affordance, int32_t dbc_option, double* out);
/* matrix(req, affordance, dbc) (interface.hh:430-440): assembles the 3x3-block CSR on the device. */
int ikr_assembler_matrix(ikr_asm a, ikr_req req, int32_t affordance, int32_t dbc_option);
/* scalar CSC export of the last assembled matrix for the given option (parity with Eigen's column-major
 * SparseMatrix): col_ptr (cols+1), row_idx (nnz), values (nnz); pass NULLs to query nnz. */
int ikr_assembler_matrix_nnz(ikr_asm a, int32_t dbc_option, int64_t* nnz);
int ikr_assembler_export_csc(ikr_asm a, int32_t dbc_option, int64_t* col_ptr, int32_t* row_idx, double* values);
/* inhomogeneous Dirichlet values (DirichletValues::storeInhomogeneousBoundaryCondition, dirichletvalues.hh:213-222,
 * for values linear in the load factor): u_D(lambda) = lambda * rate on constrained dofs (rate must vanish on free
 * dofs; NULL removes them).  NewtonRaphson then adds the IDBC forces K_raw rate * stepSize to its first residual
 * (newtonraphson.hh:212-215, functionhelper.hh:170-184) and sets the constrained entries to u_D(lambda) after
 * every update (nonlinearsolverfactory.hh:45-52); LoadControl also after a step that needed no iteration
 * (loadcontrol.inl:43-44).  Not available in batched solves. */
int ikr_assembler_set_dirichlet_values(ikr_asm a, const double* rate);
/* DirichletValues::storeInhomogeneousBoundaryCondition(f) with a general f(x, lambda) (dirichletvalues.hh:213-282):
 * value(X, lambda) is called on the host with every node position (ikr_point_fn, out: 3 values per node) at each
 * load factor the prescribed values are imposed at; its entries that are nonzero overwrite the displacement
 * (nonlinearsolverfactory.hh:45-52).  derivative(X, lambda) = d value / d lambda (the reference differentiates f with
 * autodiff) is evaluated once at lambda = 1: the IDBC forces K_raw du_D/dlambda stepSize (functionhelper.hh:
 * 170-184).  LoadControl / NewtonRaphson only: path following returns IKR_ERR_NOT_IMPLEMENTED. */
int ikr_assembler_set_dirichlet_function(ikr_asm a, ikr_point_fn value, ikr_point_fn derivative, void* user);
/* the block pattern itself: row_ptr (n_nodes+1), col (n_blocks) */
int ikr_assembler_block_pattern(ikr_asm a, int32_t* n_rows, int64_t* n_blocks, int32_t* row_ptr, int32_t* col);
/* ||R|| of the last assembled vector (FP64, deterministic device reduction) */
int ikr_assembler_vector_norm(ikr_asm a, double* norm);

/* ---- LinearSolver (linearsolver.hh:49-233) --------------------------------------------------------------- */
int ikr_linear_solver_create(ikr_ls* out, int32_t solver_type_tag);
int ikr_linear_solver_destroy(ikr_ls ls);
int ikr_linear_solver_set_tolerance(ikr_ls ls, double rtol, int32_t max_iter);
/* no reference counterpart: FP64 outer solve of an FP32 tangent (off while restart = 0, the default).  The tangent
 * is then assembled in FP64 and rounded to FP32 once; each solve runs flexible GMRES(restart) on the FP64 tangent,
 * right-preconditioned by the FP32 block-Jacobi CG on the FP32 one (relative tolerance inner_rtol, at most
 * inner_max_iter iterations per application), until ||b - K64 x|| <= rtol ||b|| or outer_max_iter Arnoldi steps.
 * For tangents whose FP32 rounding is too coarse for an FP32 Newton correction (cond(K) eps_32 > 1, e.g. nearly
 * incompressible EAS elements).  Newton and path-following solves with this solver assemble the FP64 twin
 * themselves; a direct caller of ikr_linear_solver_solve calls ikr_linear_solver_analyze_pattern before
 * assembling the matrix (a solve without the twin of the last assembly returns IKR_ERR_INVALID_STATE).
 * restart in [1, 63]; FP64 tangents are solved by the CG as before.  last_info then reports the inner CG iterations
 * and the achieved FP64 relative residual, outer_info the Arnoldi steps and restart cycles of the last solve. */
int ikr_linear_solver_set_fp64_outer(ikr_ls ls, int32_t restart, double inner_rtol, int32_t inner_max_iter,
                                     int32_t outer_max_iter);
int ikr_linear_solver_outer_info(ikr_ls ls, int32_t* outer_iterations, int32_t* cycles);
/* no reference counterpart; for tests of the bounded device waits: barrier_polls = polls of a grid barrier of the
 * persistent CG before it gives up (0 = the default, 2^24); withhold_first_arrival != 0 makes CTA 0 of the next
 * persistent CG launch skip its arrival at the first grid barrier, so every CTA's first wait runs out after
 * barrier_polls polls: that solve returns IKR_ERR_TIMEOUT (after its in-flight copies have been drained), the switch
 * clears itself, and the handle solves normally afterwards.  No fault and no unbounded wait are involved. */
int ikr_linear_solver_set_wait_test(ikr_ls ls, int32_t barrier_polls, int32_t withhold_first_arrival);
int ikr_linear_solver_analyze_pattern(ikr_ls ls, ikr_asm a);
int ikr_linear_solver_factorize(ikr_ls ls, ikr_asm a);       /* builds the preconditioner from the device K */
/* solve(x, b) with host arrays of size() (Full option system) */
int ikr_linear_solver_solve(ikr_ls ls, ikr_asm a, double* x, const double* b);
/* solve(x, B) with two right-hand-side columns (LinearSolver::solve on an n x 2 Eigen matrix, as the bordered
 * path-following solve calls it, newtonraphsonwithscalarsubsidiaryfunction.hh:265-267); host arrays */
int ikr_linear_solver_solve2(ikr_ls ls, ikr_asm a, double* x0, double* x1, const double* b0, const double* b1);
/* iterations and achieved relative residual of the last solve */
int ikr_linear_solver_last_info(ikr_ls ls, int32_t* iterations, double* rel_residual);
/* Measurement hooks (no reference counterpart): with profiling on, every CG SpMV launch is bracketed by
 * device events inside the CUDA graphs; read returns the summed SpMV device time and the launch count
 * since profiling was switched on. */
int ikr_linear_solver_profile(ikr_ls ls, int32_t on);
int ikr_linear_solver_profile_read(ikr_ls ls, double* spmv_ms_total, int64_t* spmv_launches);
/* Launch shape of the CG (no reference counterpart): iterations are issued in chunks of chunk_len
 * (1..256, default 16) between host convergence polls, captured as CUDA graphs when use_graphs != 0
 * (default) or launched kernel by kernel otherwise (for profilers that do not follow graph kernels). */
int ikr_linear_solver_set_launch(ikr_ls ls, int32_t use_graphs, int32_t chunk_len);
/* CG kernels (no reference counterpart).  spmv_kind 0 = two kernels per iteration with a direct-load SpMV,
 * 1..4 = two kernels with a bulk-copy staged SpMV (chunk size / pipeline depth / warps per block), 5..13 = the
 * whole solve in one persistent cooperative kernel (5..11: grid barriers for the two reductions of an iteration,
 * 12..13: one reduction per iteration; only where every warp's rows fit its registers), 14..15 = the persistent
 * kernel with the coarse correction in the same launch (needs ikr_linear_solver_set_coarse_space; at most 64
 * slabs), -1 = autotune (with a coarse space: a fused kind whenever one fits); l2_keep_fraction in [0, 1) = share of the
 * matrix the staged kernels keep in L2 across iterations, -1 = autotune.  The choice is made at the
 * next factorize from timed CG iterations on the assembled tangent and kept for that assembler.  info
 * returns the kind and keep fraction in use and the SpMV time per launch the tuner measured (0 if fixed). */
int ikr_linear_solver_set_kernel(ikr_ls ls, int32_t spmv_kind, double l2_keep_fraction);
/* the CG kind ranges of this build: out4 = {first staged kind, first persistent kind, first fused coarse kind,
 * number of kinds} (no reference counterpart) */
int ikr_cg_kind_ranges(int32_t* out4);
/* no reference counterpart: the kernel of the FP32 displacement-based tangent -- 1: coloured element kernel (8 lanes
 * per element, one read-modify-write launch per colour class), 2: row kernel (NeoHooke on a set without instances: a
 * thread per node row adds its row of every adjacent element's tangent, one launch, no colouring), 3: element blocks
 * + gather (one launch writes every element's 36 distinct FP32 blocks to a scratch array with coalesced stores, a
 * second sums each matrix block's contributions in a fixed order and writes every slice once, Dirichlet treatment
 * included; the scratch holds 1.3 KB per element), 0 (default): the fastest, timed at the first assembly.  All give
 * the same FP32 tangent up to the order of the FP32 additions. */
int ikr_assembler_set_tangent_kernel(ikr_asm a, int32_t path);
int ikr_assembler_tangent_kernel(ikr_asm a, int32_t* path);
/* no reference counterpart: solves with two right-hand sides and one tangent (path following's bordered
 * system) run both CGs in one persistent launch that streams the matrix once per iteration (on = 1, default)
 * or one after the other (0) */
int ikr_linear_solver_set_multi_rhs(ikr_ls ls, int32_t on);
int ikr_linear_solver_kernel_info(ikr_ls ls, int32_t* spmv_kind, double* l2_keep_fraction, double* spmv_us);
/* no reference counterpart: coarse correction of IKR_SOLVER_GPU_PCG_BLOCK_JACOBI (off by default, n_slabs = 0).
 * n_slabs in [1, 128] adds P A_c^-1 P^T to the block-Jacobi preconditioner, an additive two-level method: the
 * nodes are cut into n_slabs slabs of equal node count along the mesh's longest extent, P holds the six
 * rigid-body modes of every slab (zero at constrained dofs) and A_c = P^T K P is rebuilt at every factorize.
 * The CG then runs the two-kernel forms only.  Needs a Full-DBC tangent of an element set without instances;
 * slabs thinner than the elements (coupling more than 3 slabs apart) are rejected at factorize.  coarse_info
 * out4: slabs in use (0 = off), coarse dofs, modes dropped as linearly dependent, probe colours. */
int ikr_linear_solver_set_coarse_space(ikr_ls ls, int32_t n_slabs);
int ikr_linear_solver_coarse_info(ikr_ls ls, int32_t* out4);
/* rebuild A_c only at every n-th factorize (default 1: at every one); the others keep A_c of an earlier tangent of
 * the same assembler, which is still SPD, so the solution is unchanged and only the CG iterations can grow (no
 * reference counterpart) */
int ikr_linear_solver_set_coarse_refresh(ikr_ls ls, int32_t every);
/* material law of all elements (the reference's Material template argument of makeFE): NeoHooke (default,
 * neohooke.hh) or StVenantKirchhoff (svk.hh), both with the Lame parameters given at creation, or BlatzKo
 * (makeBlatzKo(mu), hyperelastic/factory.hh:34-39: deviatoric function on the total principal stretches, no
 * volumetric part) with the shear modulus given at creation (the first Lame parameter is not used) */
enum { IKR_MATERIAL_NEOHOOKE = 0, IKR_MATERIAL_SVK = 1, IKR_MATERIAL_BLATZKO = 2, IKR_MATERIAL_HYPERELASTIC = 3 };
int ikr_fes_set_material(ikr_fes fes, int32_t material);
/* Hyperelastic<Deviatoric<DF>, Volumetric<VF>> (materials/hyperelastic/interface.hh): a deviatoric function of the
 * principal stretches plus K U(J) with a volumetric function VF0..VF12 (volumetric/volumetricfunctions.hh).  The
 * factories of hyperelastic/factory.hh map onto it: makeBlatzKo(mu) = {BLATZKO, mu}; makeOgden<n, tag>(mu, alpha,
 * K, VF) = {OGDEN_TOTAL or OGDEN_DEVIATORIC, n, mu, alpha}; makeInvariantBased<n>(mu, p, q, K, VF) =
 * {INVARIANT_BASED, n, mu, p, q}, makeMooneyRivlin(mu) its p = {1, 0}, q = {0, 1} and makeYeoh(mu) its
 * p = {1, 2, 3}, q = {0, 0, 0}; makeArrudaBoyce({mu, lambdaM}) = {ARRUDA_BOYCE, mu[0], param = lambdaM};
 * makeGent({mu, Jm}) = {GENT, mu[0], param = Jm}; makePureVolumetric(VF, K) = {NONE}. */
enum {
  IKR_DEV_NONE = 0,
  IKR_DEV_BLATZKO = 1,
  IKR_DEV_OGDEN_TOTAL = 2,
  IKR_DEV_OGDEN_DEVIATORIC = 3,
  IKR_DEV_INVARIANT_BASED = 4,
  IKR_DEV_ARRUDA_BOYCE = 5,
  IKR_DEV_GENT = 6
};
#define IKR_HYPER_MAX_TERMS 4
typedef struct ikr_hyperelastic {
  int32_t deviatoric;                /* IKR_DEV_* */
  int32_t n_terms;                   /* Ogden / invariant-based terms, 1..IKR_HYPER_MAX_TERMS */
  double mu[IKR_HYPER_MAX_TERMS];    /* Ogden mu_n, invariant-based C_n, else mu[0] = shear modulus */
  double alpha[IKR_HYPER_MAX_TERMS]; /* Ogden exponents */
  int32_t p[IKR_HYPER_MAX_TERMS];    /* invariant-based exponents of (W1 - 3) */
  int32_t q[IKR_HYPER_MAX_TERMS];    /* invariant-based exponents of (W2 - 3) */
  double param;                      /* Arruda-Boyce lambdaM, Gent Jm */
  int32_t volumetric;                /* 0..12: VF0 (none) .. VF12 */
  int32_t reserved;
  double K;                          /* Volumetric(K, VF) */
  double beta;                       /* VF4 / VF7 / VF10 parameter */
} ikr_hyperelastic;
/* sets IKR_MATERIAL_HYPERELASTIC with these functions on every element (displacement-based and EAS): residual,
 * tangent (FP64 material point also under an FP32 tangent), energy and stresses.  IKR_ERR_ARG for an invalid
 * description (InvariantBased with p_i = q_i = 0 throws in the reference); a Gent element evaluated at
 * Jm <= W1 - 3 makes the call return IKR_ERR_INVALID_STATE (gent.hh checkJm throws InvalidStateException). */
int ikr_fes_set_hyperelastic(ikr_fes fes, const ikr_hyperelastic* h);
/* elements per block the displacement element kernel uses for residual / FP64 tangent / FP32 tangent
 * assembly (16, 32 or 64, chosen by timing at the first assembly of each kind; 0 = not assembled yet; no
 * reference counterpart) */
int ikr_fes_kernel_info(ikr_fes fes, int32_t* epb_residual, int32_t* epb_tangent64, int32_t* epb_tangent32);
/* the CUDA stream (cudaStream_t) all work on this element set is issued on */
int ikr_fes_stream(ikr_fes fes, void** stream);

/* Allocation-free solve of K x = b with the tangent the assembler last assembled (no counterpart in the
 * reference).  For callers that may not allocate device memory after start-up (a fixed device-memory
 * budget, or all allocations routed through their own allocator): it calls no cudaMalloc / cudaFree /
 * cudaMallocHost and no allocating library routine.  The CG vectors, the 3x3 block-Jacobi inverse and the
 * reduction slots live in one file-scope device array of the library (about 8.7 MB), so the system may have
 * at most IKR_NOALLOC_MAX_NODES nodes (3x as many dofs); larger systems return IKR_ERR_ARG.  The array's
 * device memory is committed when the library's device code is loaded on a GPU -- with CUDA's lazy module
 * loading (the default) at the first call of this entry point on that GPU -- and held until the process
 * exits; later calls change no device-memory figure.  b and x are device pointers of size() doubles; the CG runs in
 * the precision of the stored tangent with the same block-Jacobi preconditioner, tolerance rtol on
 * ||r|| / ||b|| and at most max_iter iterations (IKR_ERR_NOT_CONVERGED when that limit is hit).
 * The first call on a device looks up the array's device address; make that call before any stream
 * capture.  All calls share the one array, which keeps the last call's contents (every call re-initialises
 * what it reads), so calls whose GPU work overlaps -- e.g. from two element sets on different streams --
 * race on it: serialise them.  The looked-up address is kept for the process; after cudaDeviceReset (which
 * also frees every handle's device memory) no handle of this library, this entry point included, is valid. */
#define IKR_NOALLOC_MAX_NODES 32768
int ikr_linear_solver_solve_noalloc(ikr_asm a, const double* b_device, double* x_device, double rtol,
                                    int32_t max_iter, int32_t* iterations);

/* ---- assembled scalar and NonLinearOperator ----------------------------------------------------------------
 * scalar(req, affordance) (simpleassemblers.inl, scalarImpl): the sum over all elements, in element order, of
 * calculateScalar (mechanical potential energy: stored energy minus the work of the dead loads); EAS element sets
 * return IKR_ERR_NOT_IMPLEMENTED as the reference's EAS skill throws (enhancedassumedstrains.hh:305-309). */
int ikr_assembler_scalar(ikr_asm a, ikr_req req, int32_t affordance, double* out);
/* DifferentiableFunctionFactory::op(assembler, affordances, dbcOption) (utils/differentiablefunctionfactory.hh:
 * 24-51): the non-linear operator over the assembler.  With a scalar affordance (not IKR_SCALAR_NO_AFFORDANCE) the
 * function is the energy, its derivative the force vector and its second derivative the tangent; otherwise the
 * function is the force vector and its derivative the tangent.  evaluate(order): 0 = f(req), 1 = derivative(f)(req),
 * 2 = derivative(derivative(f))(req); kind returns 0 scalar, 1 vector, 2 matrix.  A scalar or vector result is
 * copied to out (1, size() or reducedSize() doubles; out may be NULL); a matrix stays in the assembler (the
 * reference returns a reference to the assembler's storage): export it with ikr_assembler_export_csc.  An order
 * above the operator's is IKR_ERR_ARG. */
typedef struct ikr_nlo_s* ikr_nlo;
int ikr_nonlinear_operator_create(ikr_nlo* out, ikr_asm a, int32_t scalar_affordance, int32_t vector_affordance,
                                  int32_t matrix_affordance, int32_t dbc_option);
int ikr_nonlinear_operator_destroy(ikr_nlo f);
int ikr_nonlinear_operator_evaluate(ikr_nlo f, int32_t order, ikr_req req, double* out, int32_t* kind);

/* ---- listeners: NonLinearSolverLogger (utils/listener/nonlinearsolverlogger.hh:22-95) and ControlLogger
 * (controllogger.hh:22-66, controllogger.cpp) write the reference's lines (spdlog's info level) through sink, or to
 * stdout as "[info] <line>" when sink is NULL.  The logger lives as long as the object it is subscribed to. ---- */
typedef void (*ikr_log_sink)(const char* line, void* user);

/* ---- NewtonRaphson (newtonraphson.hh:27-303, nonlinearsolverfactory.hh:110-122) -------------------------- */
typedef struct ikr_nr_settings {
  double tol;          /* NRSettings::tol (default 1e-8) */
  int32_t max_iter;    /* NRSettings::maxIter (default 20) */
  int32_t min_iter;    /* NRSettings::minIter (default 0) */
  /* additions of this library (defaults reproduce the reference) */
  int32_t tol_mode;    /* 0: ||R|| <= tol (reference); 1: ||R|| <= tol * ||R at solve start|| */
  int32_t forcing;     /* 0: fixed linear tolerance; 1: Eisenstat-Walker inexact Newton */
  double linear_rtol;  /* fixed linear relative tolerance (forcing = 0) / upper bound (forcing = 1) */
  double linear_rtol_min;
  int32_t linear_max_iter;
  int32_t refinements; /* FP64 iterative-refinement sweeps around an FP32 solve (0 = none) */
  int32_t max_backtracks; /* a correction that inverts an element (det C <= 0; the reference aborts) is halved up
                             to this many times before the error is returned (0 = reference behaviour); batched
                             solves halve the correction of the affected instances only, and an instance that still
                             inverts goes back once per solve to the state before that correction and takes its
                             next corrections with linear_rtol_min (inverting again takes it out) */
  int32_t step_graphs;    /* 1 (default): every Newton iteration after the first of a solver's life -- tangent
                             assembly, preconditioner, the persistent CG, update, residual assembly and norms -- runs
                             as one CUDA graph launch with one host synchronisation, where the configuration allows
                             it (displacement-based elements, persistent CG kind, no backtracking, refinement, coarse
                             correction, FP64 outer solve or inhomogeneous Dirichlet values); results are identical
                             to the launch-by-launch iteration; 0: launch by launch */
} ikr_nr_settings;
typedef struct ikr_nr_info {   /* NonLinearSolverInformation (solverinfos.hh:20-32) */
  int32_t success;
  double residual_norm;
  double correction_norm;
  int32_t iterations;
  int64_t linear_iterations;   /* addition: CG iterations spent in this solve */
} ikr_nr_info;
typedef struct ikr_nr_state {  /* NonlinearSolverState (nonlinearsolverstate.hh:22-31) */
  ikr_req domain;
  double residual_norm;
  double correction_norm;
  int32_t iterations;
  double load_factor;
} ikr_nr_state;
typedef void (*ikr_nr_observer)(int32_t message, const ikr_nr_state* state, void* user);

int ikr_nr_settings_default(ikr_nr_settings* s);
int ikr_newton_create(ikr_nr* out, ikr_asm a, ikr_ls ls, const ikr_nr_settings* settings);
int ikr_newton_destroy(ikr_nr nr);
/* Broadcaster::subscribe (broadcaster.hh:24-78) for NonLinearSolverMessages */
int ikr_newton_subscribe(ikr_nr nr, ikr_nr_observer cb, void* user);
/* the EAS skill's subscription (enhancedassumedstrains.hh:350-359): update alpha on CORRECTION_UPDATED */
int ikr_newton_subscribe_fe_state(ikr_nr nr, int32_t on);
/* solve(x, stepSize) (newtonraphson.hh:193-257) */
int ikr_newton_solve(ikr_nr nr, ikr_req req, double step_size, ikr_nr_info* info);
/* residual() / jacobian() / updateFunction() (newtonraphson.hh:260-287): the solver's residual function (force
 * vector with the Full Dirichlet treatment, out: size() doubles, may be NULL), its derivative (the tangent, kept in
 * the assembler) and the update x += dx of the requirement's displacement (dx: size() host doubles; inhomogeneous
 * Dirichlet values re-imposed afterwards, nonlinearsolverfactory.hh:45-52). */
int ikr_newton_residual(ikr_nr nr, ikr_req req, double* out);
int ikr_newton_jacobian(ikr_nr nr, ikr_req req);
int ikr_newton_update(ikr_nr nr, ikr_req req, const double* correction);
/* no reference counterpart: Newton iterations this solver ran as one CUDA graph launch each (step_graphs), since its
 * creation */
int ikr_newton_graph_iterations(ikr_nr nr, int64_t* n);
/* NonLinearSolverLogger::subscribeTo(nr) */
int ikr_newton_subscribe_logger(ikr_nr nr, ikr_log_sink sink, void* user);
/* per instance (batched solves): Newton iterations, final residual norm and convergence of the last solve
 * (1 converged, -1 taken out after its elements inverted, det C <= 0 -- the reference aborts there --, -2 taken out
 * because it was still above its tolerance after max_iter -- the reference's LoadControl stops there --, -3 kept out
 * by ikr_newton_exclude_instances, -4 taken out after its CG ran out of iterations (ikr_newton_set_batched_take_out);
 * here the
 * other instances go on and the solve succeeds when all instances not taken out converge).  Instances taken out
 * stay out for the rest of a LoadControl run. */
int ikr_newton_instance_info(ikr_nr nr, int32_t* iterations, double* residual_norms, int32_t* converged);
/* batched solves (no reference counterpart): instances whose mask entry is nonzero take no part in the following
 * solves (no corrections; their displacement stays as the requirement holds it; status -3 in instance_info), e.g.
 * to solve again in FP64 only the instances an FP32 run took out.  n = 0 clears the mask; otherwise n must equal
 * the number of instances. */
int ikr_newton_exclude_instances(ikr_nr nr, int32_t n, const uint8_t* mask);
/* batched solves (no reference counterpart): CG iterations per instance over the last solve (one value per
 * instance).  The batched solve notifies the solver's observers like the single-system one, with the largest
 * residual norm over the instances still in the solve. */
int ikr_newton_instance_linear_iterations(ikr_nr nr, int64_t* cg_iterations);
/* batched solves (no reference counterpart): the CG of a Newton iteration runs as launches of first_chunk (0: 128),
 * then twice as many iterations (at most 4096 unless first_chunk is larger), each re-planned over the instances
 * still running.  variant -1 lets the planner choose the kernel variant per launch (the first that fits of: in
 * FP32 one instance per 16-CTA thread-block cluster with vectors in distributed shared memory; sixteen (FP64 only),
 * eight or four threads per row with the matrix in shared memory; one row per thread; rows looped per thread); 0..5
 * keeps variant 0 (row loop), 1 (one row per thread), 2 (four threads per row), 3 (eight), 4 (clusters, FP32) or 5
 * (sixteen threads per row) where it fits, else the row loop.  For tests and tuning; the results agree to rounding.  batched_cg_launches: launches since creation. */
int ikr_newton_set_batched_cg(ikr_nr nr, int32_t variant, int32_t first_chunk);
int ikr_newton_batched_cg_launches(ikr_nr nr, int64_t* n);
/* the same per kernel variant 0..5 (six values) */
int ikr_newton_batched_cg_variant_launches(ikr_nr nr, int64_t* by_variant6);
/* the batched CG's planner on given capacities, without a device (tests): n running instances with their rows and
 * widest slice (blocks), the precision, a forced variant (-1: the planner's choice), the co-resident CTAs of each
 * variant 0..5 (caps6; entry 4 unused) and the co-resident 16-CTA clusters; gives the variant and the CTAs per
 * instance (16 per instance for the cluster variant) */
int ikr_batched_plan_preview(int32_t n, const int32_t* rows, const int32_t* widths, int32_t fp32, int32_t variant,
                             const int32_t* caps6, int32_t cluster_cap, int32_t* out_variant, int32_t* out_ctas);
/* batched solves (no reference counterpart): unsolved_linear = 1 takes out an instance whose CG ends above its
 * tolerance after linear_max_iter (status -4 in instance_info; in FP32 the attainable accuracy of the tangent can lie
 * above the tolerance, and the direction is then no Newton direction) */
int ikr_newton_set_batched_take_out(ikr_nr nr, int32_t unsolved_linear);
/* batched load control (no reference counterpart): precision escalation.  An instance the run's solver takes out in
 * a load step (-1 inverted, -2 above tolerance after max_iter, -4 CG unsolved) is solved again from the state at the
 * start of that step by nr64 on req64 -- a solver over a twin element set with the same instances, e.g. in FP64 --
 * and stays with nr64 for the rest of the run; its displacement is copied into the run's requirement at every step
 * end.  A step succeeds when every instance converged in one of the two solvers or was taken out by nr64 as well.
 * nr64 = req64 = NULL switches it off.  escalated: the instances escalated in the last run (one byte each). */
int ikr_load_control_set_escalation(ikr_lc lc, ikr_nr nr64, ikr_req req64);
int ikr_load_control_escalated(ikr_lc lc, int32_t n, uint8_t* mask);
/* on = 1: the instances escalated in earlier steps are solved by nr64 on a second host thread and its own stream
 * while the run's solver does the step (each batched CG plan then takes half of the co-resident CTAs); 0 (default):
 * one after the other, which measured faster (the halved plans cost more than the overlap gains).  instance_status: per instance the status of the solver that holds it at the end of the last run
 * (instance_info codes: 1 converged, -1, -2, -4 taken out). */
int ikr_load_control_set_escalation_concurrent(ikr_lc lc, int32_t on);
int ikr_load_control_instance_status(ikr_lc lc, int32_t n, int32_t* status);

/* ---- LoadControl (loadcontrol.hh:29-113, loadcontrol.inl:17-57, controlroutinefactory.hh:38-48) --------- */
typedef struct ikr_control_state {   /* ControlRoutineState (controlroutinestate.hh:21-31) */
  ikr_req domain;
  int32_t load_step;                 /* -1 during the initial equilibrium solve, as the reference's state */
  double step_size;
  double load_factor;
  int32_t total_iterations;          /* ControlInformation::totalIterations so far */
  const char* name;                  /* ControlInformation::name ("Load Control Method", "Path following with ...") */
} ikr_control_state;
typedef void (*ikr_control_observer)(int32_t message, const ikr_control_state* state, void* user);
typedef struct ikr_control_info {    /* ControlInformation (controlinfos.hh:22-32) */
  int32_t success;
  int32_t total_iterations;
  int32_t n_solver_infos;
  int64_t total_linear_iterations;
} ikr_control_info;
/* ControlRoutineFactory::create(LoadControlConfig{load_steps, t_begin, t_end}, nr, assembler): also
 * subscribes the elements' state update to the Newton solver. */
int ikr_load_control_create(ikr_lc* out, ikr_nr nr, int32_t load_steps, double t_begin, double t_end);
int ikr_load_control_destroy(ikr_lc lc);
int ikr_load_control_subscribe(ikr_lc lc, ikr_control_observer cb, void* user);
/* ControlLogger::subscribeTo(lc) */
int ikr_load_control_subscribe_logger(ikr_lc lc, ikr_log_sink sink, void* user);
/* run(req): info plus per-solve NonLinearSolverInformation (capacity entries; index 0 = the initial
 * equilibrium solve at the starting load factor). */
int ikr_load_control_run(ikr_lc lc, ikr_req req, ikr_control_info* info, ikr_nr_info* solver_infos,
                         int32_t capacity);

/* ---- PathFollowing (pathfollowing.hh:148-236, pathfollowing.inl:25-73) with NewtonRaphsonWithSubsidiaryFunction
 * (newtonraphsonwithscalarsubsidiaryfunction.hh:128-316) ---------------------------------------------------------
 * Each Newton iteration solves K dR = -R and K dL = Fext0 - F_idbc with the Newton object's linear solver and takes
 * dlambda = (-f - dfdDD.dR) / (dfdDD.dL + dfdDlambda), dD = dR + dlambda dL (Fext0 = -R(u = 0, lambda = 1)). */
typedef struct ikr_pf_s* ikr_pf;
enum { IKR_PF_ARC_LENGTH = 0,              /* ArcLength (pathfollowingfunctions.hh:88-203) */
       IKR_PF_LOAD_CONTROL = 1,            /* LoadControlSubsidiaryFunction (:217-281) */
       IKR_PF_DISPLACEMENT_CONTROL = 2 };  /* DisplacementControl (:295-368) */
/* PathFollowing(nr, steps, stepSize, pathFollowingType): the Newton object supplies the assembler (Full Dirichlet
 * handling), the linear solver and NewtonRaphsonWithSubsidiaryFunctionSettings{tol, maxIter} plus this library's
 * linear-tolerance additions.  controlled: DisplacementControl's dof indices (free, not repeated).  steps <= 0:
 * IKR_ERR_INVALID_STATE.  Also subscribes the elements' state update (EAS) to the solver. */
int ikr_path_following_create(ikr_pf* out, ikr_nr nr, int32_t steps, double step_size, int32_t kind,
                              int32_t n_controlled, const int32_t* controlled);
int ikr_path_following_destroy(ikr_pf pf);
/* kind 0: AdaptiveStepSizing::NoOp (default); 1: IterationBased with target_iterations (adaptivestepsizing.hh:36-57;
 * target 0 is IKR_ERR_INVALID_STATE as in setTargetIterations) */
int ikr_path_following_set_adaptive_step_sizing(ikr_pf pf, int32_t kind, int32_t target_iterations);
int ikr_path_following_subscribe(ikr_pf pf, ikr_control_observer cb, void* user);
/* ControlLogger::subscribeTo(pf) */
int ikr_path_following_subscribe_logger(ikr_pf pf, ikr_log_sink sink, void* user);
/* run(req): per-solve NonLinearSolverInformation, steps + 1 entries (the solve at load step -1 first).  Load-control
 * and displacement-control subsidiary functions with inhomogeneous Dirichlet values: IKR_ERR_NOT_IMPLEMENTED (the
 * reference rejects them at compile time, pathfollowingfunctions.hh:22-26). */
int ikr_path_following_run(ikr_pf pf, ikr_req req, ikr_control_info* info, ikr_nr_info* solver_infos,
                           int32_t capacity);
/* SubsidiaryArgs of the current state (pathfollowingfunctions.hh:30-41): out[0] stepSize, [1] Dlambda, [2] f,
 * [3] dfdDlambda, [4] the arc length's psi, [5] currentStep */
int ikr_path_following_subsidiary_args(ikr_pf pf, double* out6);
/* no reference counterpart: the load column K dL = Fext0 - F_idbc of every Newton iteration starts from the
 * previous dL and is solved for the change to the same relative accuracy (on = 1, default), or from zero (0, as
 * the reference's direct solve has no initial guess) */
int ikr_path_following_set_warm_start(ikr_pf pf, int32_t on);
/* no reference counterpart, last run: out[0] FP64 refinement sweeps of the arc length's initial prediction (FP32
 * tangent only), [1] its final relative FP64 residual, [2] its CG iterations, [3] load-column solves the warm start
 * made unnecessary */
int ikr_path_following_stats(ikr_pf pf, double* out4);
/* SubsidiaryArgs::DD, the solution increment of the current step (n doubles, host memory) */
int ikr_path_following_increment(ikr_pf pf, double* dd);

/* ---- Newton predictor of LoadControl (no counterpart in the reference, whose predictor only increments
 * the load factor, loadcontrol.inl:54-57) -------------------------------------------------------------------
 * kind 0: none (the reference's behaviour); 1: previous converged increment; 2: learned (predictor object);
 * 3: second-order extrapolation u + 2 du_{k-1} - du_{k-2}.  The learned and the second-order candidates are kept
 * only when their FP64 residual is below the previous-increment candidate's (their fallback); candidates that
 * invert an element are discarded; the relative Newton test of the step stays referenced to the unpredicted
 * residual.  record = 1 appends every converged increment (and params, the path's load parameters) to the
 * predictor's training snapshots. */
typedef struct ikr_pred_s* ikr_pred;
typedef struct ikr_mlp_s* ikr_mlp;
int ikr_load_control_set_predictor(ikr_lc lc, int32_t kind, ikr_pred pred, const double* params, int32_t record);
/* predictions kept / rejected by the residual test since the predictor was set */
int ikr_load_control_predictor_stats(ikr_lc lc, int32_t* accepted, int32_t* rejected);
/* per load step of the last run, 6 doubles: step, FP64 residual norm of the unpredicted state, of the
 * previous-increment candidate, of the learned candidate (-1 when not evaluated, inf when an element
 * inverted), the state kept (0 unpredicted, 1 previous increment, 2 learned, 3 second-order extrapolation) and
 * the residual norm of the second-order candidate (-1 when not evaluated).  n returns the number of steps; at
 * most capacity rows are written. */
int ikr_load_control_predictor_history(ikr_lc lc, int32_t capacity, double* out, int32_t* n);
/* gated != 0 (default): the learned candidate is kept only when its FP64 residual norm is below that of its
 * fallback (the previous increment, the unpredicted state on the first step); 0: kept whenever no element
 * inverts (no reference counterpart) */
int ikr_load_control_set_predictor_gate(ikr_lc lc, int32_t gated);
/* POD (n_modes) + MLP (depth hidden layers of width, GELU, BF16 weights, FP32 accumulation) over the
 * features [params, load factor, POD coordinates of the previous two increments]; snapshots: up to capacity
 * increments of the element set's dofs, held on the device in FP32. */
int ikr_predictor_create(ikr_pred* out, ikr_fes fes, int32_t n_params, int32_t n_modes, int32_t width,
                         int32_t depth, int64_t capacity, uint64_t seed);
int ikr_predictor_destroy(ikr_pred pred);
int ikr_predictor_num_snapshots(ikr_pred pred, int64_t* n);
/* builds the POD basis of the recorded increments (randomized range finder on the device) and trains the
 * network on the device with Adam; returns the last epoch's mean loss and the captured POD energy fraction */
int ikr_predictor_fit(ikr_pred pred, int32_t epochs, int32_t batch, float lr, float* final_loss,
                      double* pod_energy);

/* ---- the dense network on its own (gradient checks, stand-alone training); parameters are the FP32 master
 * copies, per layer W (out x in, row-major) then b (out); the forward pass uses their BF16 rounding -------- */
int ikr_mlp_create(ikr_mlp* out, int32_t n_in, int32_t width, int32_t depth, int32_t n_out, uint64_t seed);
int ikr_mlp_destroy(ikr_mlp mlp);
int ikr_mlp_num_params(ikr_mlp mlp, int64_t* n);
int ikr_mlp_get_params(ikr_mlp mlp, float* params);
int ikr_mlp_set_params(ikr_mlp mlp, const float* params);
int ikr_mlp_forward(ikr_mlp mlp, int32_t batch, const float* x, float* y);
/* mean-squared-error loss over batch x n_out outputs and its gradient w.r.t. all parameters */
int ikr_mlp_loss_grad(ikr_mlp mlp, int32_t batch, const float* x, const float* target, float* loss, float* grad);
int ikr_mlp_train(ikr_mlp mlp, int32_t n, const float* x, const float* target, int32_t epochs, int32_t batch,
                  float lr, uint64_t seed, float* final_loss);

#ifdef __cplusplus
}
#endif
#endif
