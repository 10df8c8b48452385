/*
 * ikarus_oracle.h -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * C interface of the CPU oracle: a plain-C++ FP64 restatement of the reference
 * (ikarus-project/ikarus v0.4.9) nonlinear-mechanics hot path for Q1 hexahedra:
 * NeoHooke material, displacement-based and EAS elements (GL-E9/E21, H9, H9T),
 * dead Neumann tractions, the flat sparse assembler with Raw/Full/Reduced
 * Dirichlet handling, a direct solve, Newton-Raphson and LoadControl.
 *
 * Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker / reported CPU baseline.
 * The GPU product (ikarus_gb300/) never links or calls it.
 *
 * All functions return 0 on success and a negative status on failure
 * (see ORC_* below).  Dof numbering is the reference's FlatInterleaved one:
 * global dof = 3*node + component.  Element-local dofs are node-major:
 * local k = 3*i + c (ikarus/finiteelements/fehelper.hh:145-153).
 */
#ifndef IKARUS_ORACLE_H
#define IKARUS_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_OK = 0,
  ORC_ERR_ARG = -1,
  ORC_ERR_NOT_IMPLEMENTED = -2,  /* mirrors DUNE_THROW(NotImplemented) */
  ORC_ERR_NONPOSITIVE_DETC = -3, /* mirrors checkPositiveOrAbort (materialhelpers.hh:119-126) */
  ORC_ERR_SINGULAR = -4,
  ORC_ERR_NOT_CONVERGED = -5
};

/* EAS kinds: 0 = none (NonLinearElastic), 1 = Green-Lagrange (E9/E21),
 * 2 = displacement gradient (H9), 3 = displacement gradient transposed (H9T). */
enum { ORC_EAS_NONE = 0, ORC_EAS_GL = 1, ORC_EAS_H = 2, ORC_EAS_HT = 3 };
/* DBCOption (ikarus/assembler/dirichletbcenforcement.hh:8) */
enum { ORC_DBC_RAW = 0, ORC_DBC_REDUCED = 1, ORC_DBC_FULL = 2 };
enum { ORC_MATERIAL_NEOHOOKE = 0, ORC_MATERIAL_SVK = 1, ORC_MATERIAL_BLATZKO = 2, ORC_MATERIAL_HYPERELASTIC = 3 };

/* Hyperelastic<Deviatoric<DF>, Volumetric<VF>> (materials/hyperelastic/interface.hh): a deviatoric function of the
 * principal stretches plus K U(J).  Deviatoric functions (hyperelastic/deviatoric/): NoDev, BlatzKo, Ogden with
 * total or deviatoric stretches, InvariantBased (Mooney-Rivlin, Yeoh), ArrudaBoyce, Gent.  Volumetric functions
 * VF0..VF12 (hyperelastic/volumetric/volumetricfunctions.hh). */
enum {
  ORC_DEV_NONE = 0,
  ORC_DEV_BLATZKO = 1,           /* mu[0] */
  ORC_DEV_OGDEN_TOTAL = 2,       /* mu[0..n), alpha[0..n) */
  ORC_DEV_OGDEN_DEVIATORIC = 3,  /* mu[0..n), alpha[0..n) */
  ORC_DEV_INVARIANT_BASED = 4,   /* mu[0..n) (the C_pq), p[0..n), q[0..n) */
  ORC_DEV_ARRUDA_BOYCE = 5,      /* mu[0], param = lambdaM */
  ORC_DEV_GENT = 6               /* mu[0], param = Jm */
};
#define ORC_HYPER_MAX_TERMS 4
typedef struct orc_hyper {
  int32_t deviatoric, n_terms;
  double mu[ORC_HYPER_MAX_TERMS], alpha[ORC_HYPER_MAX_TERMS];
  int32_t p[ORC_HYPER_MAX_TERMS], q[ORC_HYPER_MAX_TERMS];
  double param;
  int32_t volumetric, reserved; /* VF0..VF12 */
  double K, beta;               /* Volumetric(K, VF), beta of VF4 / VF7 / VF10 */
} orc_hyper;
/* linear solvers of the oracle */
enum { ORC_SOLVER_BANDED_LDLT = 0, ORC_SOLVER_CG_JACOBI = 1 };

typedef struct orc_problem orc_problem;

orc_problem* orc_problem_create(int n_nodes, const double* coords, int n_elems, const int32_t* conn,
                                double lambda, double mu, int eas_kind, int n_alpha);
void orc_problem_destroy(orc_problem* p);
/* material law of all elements: NeoHooke (default, neohooke.hh), StVenantKirchhoff (svk.hh) or BlatzKo
 * (makeBlatzKo(mu), hyperelastic/factory.hh:34-39; uses mu only) */
int orc_set_material(orc_problem* p, int material);
/* material law ORC_MATERIAL_HYPERELASTIC with these functions (ORC_ERR_ARG for an invalid description) */
int orc_set_hyperelastic(orc_problem* p, const orc_hyper* h);
/* deviatoric function at principal stretches lambda[3]: out = {W, dW/dlambda_i (3), secondDerivative (3x3 row-major)},
 * the three functions of each DF (storedEnergyImpl, firstDerivativeImpl, secondDerivativeImpl) */
int orc_hyper_deviatoric(const orc_hyper* h, const double* lambda, double* out13);
/* volumetric function (without K) at J: out = {U, U', U''} */
int orc_hyper_volumetric(int vf, double beta, double J, double* out3);
/* material point of any law at the right Cauchy-Green tensor C (3x3 row-major): out = {psi, S Voigt (6),
 * material moduli Voigt (6x6 row-major)}; ORC_ERR_NONPOSITIVE_DETC when det C fails the check */
int orc_material_point(int material, double lambda, double mu, const orc_hyper* h, const double* C, double* out43);
int orc_set_dirichlet(orc_problem* p, const uint8_t* fixed_dofs);
/* Dead Neumann load on element faces (Dune face numbering: 2d -> xi_d = 0, 2d+1 -> xi_d = 1).
 * traction: 3 values per face = t(X_face_center, lambda = 1); the applied load is lambda * t. */
/* inhomogeneous Dirichlet values u_D(lambda) = lambda * rate on constrained dofs (rate zero on free dofs;
 * NULL removes them); load_control then applies them like the reference's NR with its IDBC force function */
int orc_set_dirichlet_values(orc_problem* p, const double* rate);
int orc_add_neumann(orc_problem* p, int n_faces, const int32_t* face_elem, const int32_t* face_local,
                    const double* traction);
/* loads given as functions: out[3k..3k+2] = f(X[3k..3k+2], lambda) for k < n */
typedef void (*orc_point_fn)(int32_t n, const double* X, double lambda, double* out, void* user);
/* inhomogeneous Dirichlet values given as a function (storeInhomogeneousBoundaryCondition, dirichletvalues.hh:213-222):
 * u_D(lambda) = value(X_node, lambda) at every node (entries that are nonzero are imposed, nonlinearsolverfactory.hh:
 * 45-52), IDBC forces from derivative(X_node, 1) (functionhelper.hh:170-184); load_control only */
int orc_set_dirichlet_function(orc_problem* p, orc_point_fn value, orc_point_fn derivative, void* user);
/* VolumeLoad (loads/volume.hh:86-106): body force f(X, lambda) integrated with the element's Gauss rule */
int orc_add_volume_load(orc_problem* p, orc_point_fn f, void* user);
/* Neumann faces with a traction function f(X, lambda) evaluated at the face's quadrature point (the face centre) */
int orc_add_neumann_function(orc_problem* p, int n_faces, const int32_t* face_elem, const int32_t* face_local,
                             orc_point_fn f, void* user);
/* Manipulator-style point loads: after the Dirichlet treatment, R[dof] += lambda * value. */
int orc_add_point_loads(orc_problem* p, int n, const int32_t* dofs, const double* values);
/* When set, the tangent moduli are recomputed for every (i,j) node pair of every Gauss point,
 * as the reference does (nonlinearelastic.hh:318 called from :395).  Results are identical. */
int orc_set_faithful_moduli(orc_problem* p, int on);

int orc_get_alpha(const orc_problem* p, double* alpha);
int orc_set_alpha(orc_problem* p, const double* alpha);

/* element level (calculateVector / calculateMatrix / calculateScalar) */
int orc_element_vector(orc_problem* p, int e, const double* u, double lambda, double* out24);
int orc_element_matrix(orc_problem* p, int e, const double* u, double lambda, double* out576_colmajor);
int orc_element_energy(orc_problem* p, int e, const double* u, double lambda, double* energy);
/* calculateAt (nonlinearelastic.hh:237-271): type 0 PK2, 1 Kirchhoff, 2 Cauchy stress of element e at local xi,
 * Voigt [11,22,33,23,13,12] without shear factors; EAS elements (enhancedassumedstrains.hh:127-188) use the stored
 * alpha: GL adds M(xi) alpha to the strain (F compatible), H / HT enhance the displacement gradient */
int orc_calculate_at(orc_problem* p, int e, const double* u, int type, const double* xi, double* out6);
int orc_update_state(orc_problem* p, const double* u, double lambda, const double* correction);

/* assembler */
int orc_assemble_vector(orc_problem* p, const double* u, double lambda, int dbc, double* out);
/* returns nnz; pass NULL arrays to query sizes.  CSC: col_ptr (ncols+1), row_idx (nnz), values (nnz) */
int64_t orc_pattern_nnz(orc_problem* p, int dbc);
int orc_assemble_matrix_csc(orc_problem* p, const double* u, double lambda, int dbc, int64_t* col_ptr,
                            int32_t* row_idx, double* values);
int orc_reduced_size(orc_problem* p);
/* constraintsBelow (assembler/interface.hh:50-62): out[i] = number of constrained dofs with index < i (n values) */
int orc_constraints_below(const orc_problem* p, int32_t* out);
/* Jacobi-preconditioned CG (the reference's si_ConjugateGradient) on a symmetric CSC matrix: x = A^{-1} b to
 * ||r|| <= rtol ||b|| or max_iter iterations (ORC_ERR_NOT_CONVERGED); iterations returns the count. */
int orc_cg_jacobi_csc(int n, const int64_t* col_ptr, const int32_t* row_idx, const double* values, const double* b,
                      double* x, double rtol, int max_iter, int* iterations);

/* Newton-Raphson (newtonraphson.hh:193-257) under LoadControl (loadcontrol.inl:17-52).
 * tol_mode 0: absolute ||R|| <= tol (reference default); 1: ||R|| <= tol * ||R at step start||.
 * u (in/out, n dofs), lambda0 in *lambda (in/out).
 * iterations[steps+1], res_norms[steps+1]: per solve (index 0 = initial equilibrium solve).
 * Returns ORC_OK, or ORC_ERR_NOT_CONVERGED with the number of completed solves in *n_solves. */
int orc_load_control(orc_problem* p, int load_steps, double t_begin, double t_end, double tol, int tol_mode,
                     int max_iter, int solver, double cg_rtol, double* u, double* lambda, int32_t* iterations,
                     double* res_norms, int* n_solves, int* total_iterations);

/* Threads of the oracle's CG (default 1; matrix-vector products and vector updates split into fixed row ranges,
 * partial sums added in range order, so results depend only on the count).  Assembly stays serial. */
int orc_set_threads(int n);
/* One load step of LoadControl (loadcontrol.inl:54-57) with Newton-Raphson (newtonraphson.hh:193-257): lambda +=
 * dlambda, Newton from u to ||R|| <= tol ||R at the step start|| (tol_mode 1) or ||R|| <= tol (0), Full Dirichlet
 * handling, no inhomogeneous Dirichlet values.  stats[6]: Newton iterations, linear-solver (CG) iterations, seconds
 * in residual assembly, in tangent assembly, in linear solves, final ||R||. */
int orc_load_step(orc_problem* p, double dlambda, double tol, int tol_mode, int max_iter, int solver, double cg_rtol,
                  double* u, double* lambda, double* stats);

/* Path following (pathfollowing.inl:25-73) with Newton-Raphson and a scalar subsidiary function
 * (newtonraphsonwithscalarsubsidiaryfunction.hh:207-316).  kind: ORC_PF_* (pathfollowingfunctions.hh);
 * controlled: DisplacementControl's dof indices; target_iterations > 0 selects AdaptiveStepSizing::IterationBased
 * (0 = NoOp).  Full Dirichlet handling; inhomogeneous Dirichlet values (orc_set_dirichlet_values) only with the
 * arc length.  iterations / res_norms / lambdas: steps + 1 entries (the solve at load step -1 first); psi: the arc
 * length's scaling factor after the run. */
enum { ORC_PF_ARC_LENGTH = 0, ORC_PF_LOAD_CONTROL = 1, ORC_PF_DISPLACEMENT_CONTROL = 2 };
int orc_path_following(orc_problem* p, int kind, int steps, double step_size, int n_controlled,
                       const int32_t* controlled, int target_iterations, double tol, int max_iter, int solver,
                       double cg_rtol, double* u, double* lambda, int32_t* iterations, double* res_norms,
                       double* lambdas, double* psi, int* n_solves, int* total_iterations);
/* The same routine on the two-dof operator of tests/src/testpathfollowing.cpp:26-40 (idbc = 1: only w is free and
 * u = 0.1 lambda is prescribed, :80-94); pins the routine against that test's golden values.  d_steps: (u, w)
 * after each of the steps + 1 solves. */
int orc_path_following_toy(int kind, int idbc, int steps, double step_size, int target_iterations, double tol,
                           int max_iter, double* d2, double* lambda, int32_t* iterations, double* lambdas,
                           double* d_steps, int* n_solves);

#ifdef __cplusplus
}
#endif
#endif
