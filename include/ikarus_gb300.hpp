// ikarus_gb300.hpp -- header-only C++ facade over the C ABI (ikarus_gb300.h) with the reference's names.
//
// namespace Ikarus::GB300 mirrors the part of ikarus-project/ikarus v0.4.9 this library replaces:
//   FiniteElements            ~ std::vector<FE> of nonLinearElastic(NeoHooke) [+ eas<ES>(n)] [+ Neumann load]
//   FERequirements            ~ FERequirements<displacement, loadfactor>      (ferequirements.hh:222-407)
//   SparseFlatAssembler       ~ SparseFlatAssembler + AssemblerManipulator    (simpleassemblers.hh:108-177)
//   LinearSolver              ~ LinearSolver(SolverTypeTag)                    (linearsolver.hh:49-233)
//   NewtonRaphson             ~ NewtonRaphson with NRSettings / observers      (newtonraphson.hh:27-303)
//   LoadControl               ~ LoadControl via ControlRoutineFactory::create  (loadcontrol.hh:29-113)
//   PathFollowing             ~ PathFollowing with NewtonRaphsonWithSubsidiaryFunction, ArcLength /
//                               LoadControlSubsidiaryFunction / DisplacementControl, AdaptiveStepSizing
//                               (pathfollowing.hh:148-236, pathfollowingfunctions.hh, adaptivestepsizing.hh)
// Errors are thrown where the reference throws (NotImplemented, InvalidStateException) and as
// Ikarus::GB300::Error otherwise; det C <= 0 throws NonPositiveDetC instead of aborting.
#pragma once
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ikarus_gb300.h"

namespace Ikarus::GB300 {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
struct NotImplemented : Error {
  using Error::Error;
};
struct InvalidStateException : Error {
  using Error::Error;
};
struct NonPositiveDetC : Error {
  using Error::Error;
};

inline void check(int code, const char* what) {
  if (code == IKR_OK) return;
  char buf[512];
  ikr_last_error(buf, sizeof(buf));
  const std::string msg = std::string(what) + ": " + buf;
  if (code == IKR_ERR_NOT_IMPLEMENTED) throw NotImplemented(code, msg);
  if (code == IKR_ERR_INVALID_STATE) throw InvalidStateException(code, msg);
  if (code == IKR_ERR_NONPOSITIVE_DETC) throw NonPositiveDetC(code, msg);
  throw Error(code, msg);
}

enum class DBCOption : int32_t { Raw = IKR_DBC_RAW, Reduced = IKR_DBC_REDUCED, Full = IKR_DBC_FULL };
enum class VectorAffordance : int32_t { noAffordance = 0, forces = IKR_VEC_FORCES };
enum class MatrixAffordance : int32_t { noAffordance = 0, stiffness = IKR_MAT_STIFFNESS };
enum class ScalarAffordance : int32_t { noAffordance = 0, mechanicalPotentialEnergy = 1 };
enum class EAS : int32_t { none = 0, GreenLagrangeStrain = 1, DisplacementGradient = 2, DisplacementGradientTransposed = 3 };
// the reference's 19 tags with their values (linearsolver.hh:28-31), then the device solvers of this library; what
// each runs on the device is listed in ikarus_gb300.h
enum class SolverTypeTag : int32_t {
  none = IKR_SOLVER_NONE,
  si_ConjugateGradient = IKR_SOLVER_SI_CONJUGATE_GRADIENT,
  si_LeastSquaresConjugateGradient = IKR_SOLVER_SI_LEAST_SQUARES_CONJUGATE_GRADIENT,
  si_BiCGSTAB = IKR_SOLVER_SI_BICGSTAB,
  sd_SimplicialLLT = IKR_SOLVER_SD_SIMPLICIAL_LLT,
  sd_SimplicialLDLT = IKR_SOLVER_SD_SIMPLICIAL_LDLT,
  sd_SparseLU = IKR_SOLVER_SD_SPARSE_LU,
  sd_SparseQR = IKR_SOLVER_SD_SPARSE_QR,
  sd_CholmodSupernodalLLT = IKR_SOLVER_SD_CHOLMOD_SUPERNODAL_LLT,
  sd_UmfPackLU = IKR_SOLVER_SD_UMFPACK_LU,
  sd_SuperLU = IKR_SOLVER_SD_SUPER_LU,
  d_PartialPivLU = IKR_SOLVER_D_PARTIAL_PIV_LU,
  d_FullPivLU = IKR_SOLVER_D_FULL_PIV_LU,
  d_HouseholderQR = IKR_SOLVER_D_HOUSEHOLDER_QR,
  d_ColPivHouseholderQR = IKR_SOLVER_D_COL_PIV_HOUSEHOLDER_QR,
  d_FullPivHouseholderQR = IKR_SOLVER_D_FULL_PIV_HOUSEHOLDER_QR,
  d_CompleteOrthogonalDecomposition = IKR_SOLVER_D_COMPLETE_ORTHOGONAL_DECOMPOSITION,
  d_LLT = IKR_SOLVER_D_LLT,
  d_LDLT = IKR_SOLVER_D_LDLT,
  gpu_PCG_BlockJacobi = IKR_SOLVER_GPU_PCG_BLOCK_JACOBI,
  gpu_PCG_Batched = IKR_SOLVER_GPU_PCG_BATCHED
};
enum class Precision : int32_t { fp64 = IKR_PRECISION_FP64, fp32 = IKR_PRECISION_FP32 };
// material law of the elements (NeoHooke / StVenantKirchhoff with lambda, mu; BlatzKo with mu only)
enum class Material : int32_t {
  NeoHooke = IKR_MATERIAL_NEOHOOKE,
  StVenantKirchhoff = IKR_MATERIAL_SVK,
  BlatzKo = IKR_MATERIAL_BLATZKO
};
enum class NonLinearSolverMessages : int32_t { INIT = 0, ITERATION_STARTED, ITERATION_ENDED, RESIDUALNORM_UPDATED,
                                               CORRECTIONNORM_UPDATED, CORRECTION_UPDATED, SOLUTION_CHANGED,
                                               FINISHED_SUCESSFULLY };
enum class ControlMessages : int32_t { CONTROL_STARTED = 0, CONTROL_ENDED, STEP_STARTED, STEP_ENDED, SOLUTION_CHANGED };

struct LamesFirstParameterAndShearModulus {
  double lambda, mu;
};
// physicshelper.hh:81-85, 123-127, 276-280
inline LamesFirstParameterAndShearModulus toLamesFirstParameterAndShearModulus(double emodul, double nu) {
  return {emodul * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), emodul / (2.0 * (1.0 + nu))};
}

class FiniteElements {
 public:
  FiniteElements(const std::vector<double>& coords, const std::vector<int32_t>& conn,
                 LamesFirstParameterAndShearModulus mat, EAS eas = EAS::none, int n_eas = 0)
      : n_nodes_((int32_t)(coords.size() / 3)), n_elems_((int32_t)(conn.size() / 8)), n_eas_(n_eas) {
    check(ikr_fes_create(&h_, n_nodes_, coords.data(), n_elems_, conn.data(), mat.lambda, mat.mu, (int32_t)eas, n_eas),
          "FiniteElements");
  }
  ~FiniteElements() { ikr_fes_destroy(h_); }
  FiniteElements(const FiniteElements&) = delete;
  FiniteElements& operator=(const FiniteElements&) = delete;
  void addNeumannBoundaryLoad(const std::vector<int32_t>& face_elem, const std::vector<int32_t>& face_local,
                              const std::vector<double>& traction) {
    check(ikr_fes_add_neumann(h_, (int32_t)face_elem.size(), face_elem.data(), face_local.data(), traction.data()),
          "neumannBoundaryLoad");
  }
  void setMaterial(Material m) { check(ikr_fes_set_material(h_, (int32_t)m), "material"); }
  int32_t size() const { return n_elems_; }
  int32_t dofs() const { return 3 * n_nodes_; }
  int32_t numberOfInternalVariables() const { return n_eas_; }
  ikr_fes handle() const { return h_; }

 private:
  ikr_fes h_ = nullptr;
  int32_t n_nodes_, n_elems_, n_eas_;
};

class FERequirements {
 public:
  explicit FERequirements(const FiniteElements& fes, double load_factor = 0.0) : n_(fes.dofs()) {
    check(ikr_req_create(&h_, fes.handle()), "FERequirements");
    insertParameter(load_factor);
  }
  ~FERequirements() { ikr_req_destroy(h_); }
  FERequirements(const FERequirements&) = delete;
  FERequirements& operator=(const FERequirements&) = delete;
  void insertGlobalSolution(const std::vector<double>& u) {
    check(ikr_req_insert_global_solution(h_, u.data()), "insertGlobalSolution");
  }
  std::vector<double> globalSolution() const {
    std::vector<double> u(n_);
    check(ikr_req_global_solution(h_, u.data()), "globalSolution");
    return u;
  }
  void insertParameter(double lf) { check(ikr_req_insert_parameter(h_, lf), "insertParameter"); }
  double parameter() const {
    double v = 0;
    check(ikr_req_parameter(h_, &v), "parameter");
    return v;
  }
  ikr_req handle() const { return h_; }

 private:
  ikr_req h_ = nullptr;
  int32_t n_;
};

// calculateVector / calculateMatrix over an element range (mixin.hh:126-152); matrices column-major
inline std::vector<double> calculateVector(const FiniteElements& fes, const FERequirements& req,
                                           VectorAffordance aff, int32_t e0, int32_t e1) {
  std::vector<double> out(24 * (size_t)(e1 - e0));
  check(ikr_fe_calculate_vector(fes.handle(), req.handle(), (int32_t)aff, e0, e1, out.data()), "calculateVector");
  return out;
}
inline std::vector<double> calculateMatrix(const FiniteElements& fes, const FERequirements& req,
                                           MatrixAffordance aff, int32_t e0, int32_t e1) {
  std::vector<double> out(576 * (size_t)(e1 - e0));
  check(ikr_fe_calculate_matrix(fes.handle(), req.handle(), (int32_t)aff, e0, e1, out.data()), "calculateMatrix");
  return out;
}

class SparseFlatAssembler {
 public:
  SparseFlatAssembler(const FiniteElements& fes, const std::vector<uint8_t>& fixed, Precision p = Precision::fp64)
      : n_(fes.dofs()) {
    check(ikr_assembler_create(&h_, fes.handle(), fixed.data(), (int32_t)p), "SparseFlatAssembler");
  }
  ~SparseFlatAssembler() { ikr_assembler_destroy(h_); }
  SparseFlatAssembler(const SparseFlatAssembler&) = delete;
  SparseFlatAssembler& operator=(const SparseFlatAssembler&) = delete;
  void bind(const FERequirements& req, DBCOption dbc = DBCOption::Full) {
    check(ikr_assembler_bind(h_, req.handle(), (int32_t)dbc), "bind");
    dbc_ = dbc;
  }
  // AssemblerManipulator hook vec[dof] += lambda * value
  void bindPointLoads(const std::vector<int32_t>& dofs, const std::vector<double>& values) {
    check(ikr_assembler_add_point_loads(h_, (int32_t)dofs.size(), dofs.data(), values.data()), "point loads");
  }
  DBCOption dBCOption() const { return dbc_; }
  int32_t size() const { return n_; }
  int32_t reducedSize() const {
    int32_t s = 0;
    check(ikr_assembler_reduced_size(h_, &s), "reducedSize");
    return s;
  }
  std::vector<double> vector(const FERequirements& req, VectorAffordance aff, DBCOption dbc) {
    std::vector<double> out(dbc == DBCOption::Reduced ? reducedSize() : n_);
    check(ikr_assembler_vector(h_, req.handle(), (int32_t)aff, (int32_t)dbc, out.data()), "vector");
    return out;
  }
  struct CSC {
    int32_t n;
    std::vector<int64_t> colPtr;
    std::vector<int32_t> rowIdx;
    std::vector<double> values;
  };
  // assembles on the device; export=true also copies the scalar column-major matrix to the host
  CSC matrix(const FERequirements& req, MatrixAffordance aff, DBCOption dbc, bool exportToHost = true) {
    check(ikr_assembler_matrix(h_, req.handle(), (int32_t)aff, (int32_t)dbc), "matrix");
    CSC m{dbc == DBCOption::Reduced ? reducedSize() : n_, {}, {}, {}};
    if (!exportToHost) return m;
    int64_t nnz = 0;
    check(ikr_assembler_matrix_nnz(h_, (int32_t)dbc, &nnz), "nnz");
    m.colPtr.resize(m.n + 1);
    m.rowIdx.resize(nnz);
    m.values.resize(nnz);
    check(ikr_assembler_export_csc(h_, (int32_t)dbc, m.colPtr.data(), m.rowIdx.data(), m.values.data()), "export");
    return m;
  }
  ikr_asm handle() const { return h_; }

 private:
  ikr_asm h_ = nullptr;
  int32_t n_;
  DBCOption dbc_ = DBCOption::Full;
};

class LinearSolver {
 public:
  explicit LinearSolver(SolverTypeTag tag = SolverTypeTag::gpu_PCG_BlockJacobi) {
    check(ikr_linear_solver_create(&h_, (int32_t)tag), "LinearSolver");
  }
  ~LinearSolver() { ikr_linear_solver_destroy(h_); }
  LinearSolver(const LinearSolver&) = delete;
  LinearSolver& operator=(const LinearSolver&) = delete;
  void setTolerance(double rtol, int32_t maxIter = 100000) {
    check(ikr_linear_solver_set_tolerance(h_, rtol, maxIter), "setTolerance");
  }
  void analyzePattern(SparseFlatAssembler& a) { check(ikr_linear_solver_analyze_pattern(h_, a.handle()), "analyze"); }
  void factorize(SparseFlatAssembler& a) { check(ikr_linear_solver_factorize(h_, a.handle()), "factorize"); }
  void compute(SparseFlatAssembler& a) {
    analyzePattern(a);
    factorize(a);
  }
  void solve(SparseFlatAssembler& a, std::vector<double>& x, const std::vector<double>& b) {
    x.resize(b.size());
    check(ikr_linear_solver_solve(h_, a.handle(), x.data(), b.data()), "solve");
  }
  // no reference counterpart: coarse correction of the block-Jacobi CG with nSlabs slab aggregates (0 = off)
  void setCoarseSpace(int32_t nSlabs) { check(ikr_linear_solver_set_coarse_space(h_, nSlabs), "setCoarseSpace"); }
  ikr_ls handle() const { return h_; }

 private:
  ikr_ls h_ = nullptr;
};

struct NRSettings {  // newtonraphson.hh:27-32
  double tol = 1e-8;
  int maxIter = 20;
  int minIter = 0;
};

struct NonLinearSolverInformation {  // solverinfos.hh:20-32
  bool success = false;
  double residualNorm = 0, correctionNorm = 0;
  int iterations = -1;
  int64_t linearIterations = 0;
  explicit operator bool() const { return success; }
};

struct NewtonRaphsonConfig {
  NRSettings parameters{};
  ikr_nr_settings extended{};  // this library's additions (relative test, forcing, refinement)
  NewtonRaphsonConfig() { ikr_nr_settings_default(&extended); }
};

class NewtonRaphson {
 public:
  using Observer = std::function<void(NonLinearSolverMessages, const ikr_nr_state&)>;
  NewtonRaphson(SparseFlatAssembler& a, LinearSolver& ls, NewtonRaphsonConfig cfg = {}) {
    ikr_nr_settings st = cfg.extended;
    st.tol = cfg.parameters.tol;
    st.max_iter = cfg.parameters.maxIter;
    st.min_iter = cfg.parameters.minIter;
    check(ikr_newton_create(&h_, a.handle(), ls.handle(), &st), "NewtonRaphson");
  }
  ~NewtonRaphson() { ikr_newton_destroy(h_); }
  NewtonRaphson(const NewtonRaphson&) = delete;
  NewtonRaphson& operator=(const NewtonRaphson&) = delete;
  void subscribe(Observer f) {
    observers_.push_back(std::make_unique<Observer>(std::move(f)));
    check(ikr_newton_subscribe(h_, &NewtonRaphson::tramp, observers_.back().get()), "subscribe");
  }
  [[nodiscard]] NonLinearSolverInformation solve(FERequirements& req, double stepSize = 0.0) {
    ikr_nr_info i{};
    check(ikr_newton_solve(h_, req.handle(), stepSize, &i), "NewtonRaphson::solve");
    return {i.success != 0, i.residual_norm, i.correction_norm, i.iterations, i.linear_iterations};
  }
  ikr_nr handle() const { return h_; }

 private:
  static void tramp(int32_t m, const ikr_nr_state* s, void* u) {
    (*static_cast<Observer*>(u))(static_cast<NonLinearSolverMessages>(m), *s);
  }
  ikr_nr h_ = nullptr;
  std::vector<std::unique_ptr<Observer>> observers_;
};

struct ControlInformation {  // controlinfos.hh:22-32
  bool success = false;
  std::vector<NonLinearSolverInformation> solverInfos;
  int totalIterations = 0;
  std::string name = "Load Control";
};

class LoadControl {
 public:
  using Observer = std::function<void(ControlMessages, const ikr_control_state&)>;
  LoadControl(NewtonRaphson& nr, int loadSteps, double tbegin, double tend) : steps_(loadSteps) {
    check(ikr_load_control_create(&h_, nr.handle(), loadSteps, tbegin, tend), "LoadControl");
  }
  ~LoadControl() { ikr_load_control_destroy(h_); }
  LoadControl(const LoadControl&) = delete;
  LoadControl& operator=(const LoadControl&) = delete;
  void subscribe(Observer f) {
    observers_.push_back(std::make_unique<Observer>(std::move(f)));
    check(ikr_load_control_subscribe(h_, &LoadControl::tramp, observers_.back().get()), "subscribe");
  }
  [[nodiscard]] ControlInformation run(FERequirements& req) {
    std::vector<ikr_nr_info> infos(steps_ + 1);
    ikr_control_info ci{};
    check(ikr_load_control_run(h_, req.handle(), &ci, infos.data(), (int32_t)infos.size()), "LoadControl::run");
    ControlInformation out;
    out.success = ci.success != 0;
    out.totalIterations = ci.total_iterations;
    for (int i = 0; i < ci.n_solver_infos && i < (int)infos.size(); ++i)
      out.solverInfos.push_back({infos[i].success != 0, infos[i].residual_norm, infos[i].correction_norm,
                                 infos[i].iterations, infos[i].linear_iterations});
    return out;
  }

 private:
  static void tramp(int32_t m, const ikr_control_state* s, void* u) {
    (*static_cast<Observer*>(u))(static_cast<ControlMessages>(m), *s);
  }
  ikr_lc h_ = nullptr;
  int steps_;
  std::vector<std::unique_ptr<Observer>> observers_;
};

// Subsidiary functions of PathFollowing (pathfollowingfunctions.hh:88-368)
struct ArcLength {
  static constexpr int32_t kind = IKR_PF_ARC_LENGTH;
  std::vector<int32_t> controlledIndices{};
};
struct LoadControlSubsidiaryFunction {
  static constexpr int32_t kind = IKR_PF_LOAD_CONTROL;
  std::vector<int32_t> controlledIndices{};
};
struct DisplacementControl {
  static constexpr int32_t kind = IKR_PF_DISPLACEMENT_CONTROL;
  explicit DisplacementControl(std::vector<int32_t> idx) : controlledIndices(std::move(idx)) {}
  std::vector<int32_t> controlledIndices;
};
// AdaptiveStepSizing (adaptivestepsizing.hh:14-57)
namespace AdaptiveStepSizing {
struct NoOp {
  static constexpr int32_t kind = 0;
  int targetIterations() const { return 0; }
};
struct IterationBased {
  static constexpr int32_t kind = 1;
  int targetIterations() const { return target_; }
  void setTargetIterations(int t) {
    if (t == 0) throw InvalidStateException(IKR_ERR_INVALID_STATE, "TargetIterations should not be equal to 0.");
    target_ = t;
  }

 private:
  int target_ = 0;
};
}  // namespace AdaptiveStepSizing

// PathFollowing(nr, steps, stepSize, pathFollowingType, adaptiveStepSizing) (pathfollowing.hh:185-194) with
// NewtonRaphsonWithSubsidiaryFunction; the NewtonRaphson object supplies assembler, linear solver and tolerances
class PathFollowing {
 public:
  using Observer = std::function<void(ControlMessages, const ikr_control_state&)>;
  template <typename PF = ArcLength, typename ASS = AdaptiveStepSizing::NoOp>
  PathFollowing(NewtonRaphson& nr, int steps, double stepSize, const PF& pft = {}, const ASS& ass = {})
      : steps_(steps) {
    check(ikr_path_following_create(&h_, nr.handle(), steps, stepSize, PF::kind,
                                    (int32_t)pft.controlledIndices.size(),
                                    pft.controlledIndices.empty() ? nullptr : pft.controlledIndices.data()),
          "PathFollowing");
    if (ASS::kind == 1) check(ikr_path_following_set_adaptive_step_sizing(h_, 1, ass.targetIterations()), "steps");
  }
  ~PathFollowing() { ikr_path_following_destroy(h_); }
  PathFollowing(const PathFollowing&) = delete;
  PathFollowing& operator=(const PathFollowing&) = delete;
  void subscribe(Observer f) {
    observers_.push_back(std::make_unique<Observer>(std::move(f)));
    check(ikr_path_following_subscribe(h_, &PathFollowing::tramp, observers_.back().get()), "subscribe");
  }
  [[nodiscard]] ControlInformation run(FERequirements& req) {
    std::vector<ikr_nr_info> infos(steps_ + 1);
    ikr_control_info ci{};
    check(ikr_path_following_run(h_, req.handle(), &ci, infos.data(), (int32_t)infos.size()), "PathFollowing::run");
    ControlInformation out;
    out.success = ci.success != 0;
    out.totalIterations = ci.total_iterations;
    for (int i = 0; i < ci.n_solver_infos && i < (int)infos.size(); ++i)
      out.solverInfos.push_back({infos[i].success != 0, infos[i].residual_norm, infos[i].correction_norm,
                                 infos[i].iterations, infos[i].linear_iterations});
    return out;
  }

 private:
  static void tramp(int32_t m, const ikr_control_state* s, void* u) {
    (*static_cast<Observer*>(u))(static_cast<ControlMessages>(m), *s);
  }
  ikr_pf h_ = nullptr;
  int steps_;
  std::vector<std::unique_ptr<Observer>> observers_;
};

}  // namespace Ikarus::GB300
