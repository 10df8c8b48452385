// Path following on the device: PathFollowing::run (pathfollowing.inl:25-73) driving Newton-Raphson with a scalar
// subsidiary function (newtonraphsonwithscalarsubsidiaryfunction.hh:207-316).  Every Newton iteration solves the
// bordered system through two solves with the same tangent, K dR = -R and K dL = Fext0 - F_idbc, and combines them
// with the subsidiary function's derivatives:
//   dlambda = (-f - dfdDD . dR) / (dfdDD . dL + dfdDlambda),   dD = dR + dlambda dL.
// Subsidiary functions (pathfollowingfunctions.hh): ArcLength (:88-203), LoadControlSubsidiaryFunction (:217-281),
// DisplacementControl (:295-368); step-size adaptation AdaptiveStepSizing::IterationBased
// (adaptivestepsizing.hh:36-57).  Vectors stay on the device; only the scalars of the bordering (dot products)
// come back to the host.
#include <string>

#include "host_internal.h"

using namespace ikr_host;

struct ikr_pf_s {
  ikr_nr nr = nullptr;
  int steps = 1;
  double step_size0 = 0;
  int kind = IKR_PF_ARC_LENGTH;
  std::vector<int32_t> controlled;
  int adaptive = 0, target_iterations = 0;
  std::vector<ControlObserver> obs;
  std::vector<std::unique_ptr<ListenerBase>> listeners;
  std::string name;  // PathFollowing::name (pathfollowing.hh:175)
  // ArcLength's private state (pathfollowingfunctions.hh:200-202)
  double psi = 0;
  bool computed = false;
  // SubsidiaryArgs (pathfollowingfunctions.hh:30-41); DD and the controlled-dof mask live on the device
  double step_size = 0, Dlambda = 0, f = 0, dfdDlambda = 0;
  double dfdDD_scale = 0;  // dfdDD = dfdDD_scale * DD (arc length) or * (mask . DD) (displacement control)
  int current_step = 0;
  DBuf<double> DD, DDc, mask, fext0, dR, dL, b2, u_save, part, out;
  // warm start of the load column: its right-hand side Fext0 (- F_idbc) changes little along the path, so the
  // previous dL is the initial guess of the next solve
  bool warm = true, dl_valid = false;
  DBuf<double> dl_res, dl_corr;
  int64_t dl_skipped = 0;
  // initial prediction of the last run: refinement sweeps, final relative FP64 residual, CG iterations
  int pred_sweeps = 0;
  double pred_rel = 0.0;
  int64_t pred_cg = 0;
};

namespace {

// syncParameterAndGlobalSolution's change of u when lambda grows by dlambda, squared (idbcIncrement, common.hh:38-51)
double idbc_delta_sq(ikr_pf pf, ikr_asm a, ikr_req r, double dlambda) {
  if (!a->has_idbc) return 0.0;
  ikr_fes f = a->fes;
  pf->part.alloc(1024);
  pf->out.alloc(1);
  ikr::launch_idbc_delta_sq(r->u.p, a->idbc_rate.p, r->lambda + dlambda, a->n, pf->part.p, pf->out.p, f->stream);
  count(2);
  double h = 0;
  CK(cudaMemcpyAsync(&h, pf->out.p, sizeof(double), cudaMemcpyDeviceToHost, f->stream));
  CK(cudaStreamSynchronize(f->stream));
  return h;
}

// dfdDD . v
double dfdDD_dot(ikr_pf pf, ikr_fes f, const double* v, int64_t n) {
  if (pf->dfdDD_scale == 0.0) return 0.0;
  const double* d = pf->kind == IKR_PF_DISPLACEMENT_CONTROL ? pf->DDc.p : pf->DD.p;
  return pf->dfdDD_scale * device_dot(f, d, v, n, pf->part, pf->out);
}

// the subsidiary function and its derivatives at the current state (operator() of the three kinds)
void subsidiary(ikr_pf pf, ikr_asm a, ikr_req r) {
  ikr_fes f = a->fes;
  const int64_t n = a->n;
  if (pf->kind == IKR_PF_ARC_LENGTH) {  // pathfollowingfunctions.hh:102-115
    const double d2 = idbc_delta_sq(pf, a, r, pf->Dlambda);
    const double dd2 = device_dot(f, pf->DD.p, pf->DD.p, n, pf->part, pf->out);
    const double root = std::sqrt(dd2 + d2 + pf->psi * pf->psi * pf->Dlambda * pf->Dlambda);
    pf->f = root - pf->step_size;
    if (!pf->computed) {
      pf->dfdDD_scale = 0.0;
      pf->dfdDlambda = 0.0;
    } else {
      pf->dfdDD_scale = 1.0 / root;
      const double dhat02 = d2 / (pf->Dlambda * pf->Dlambda);  // Dhat0 = idbcDelta / Dlambda
      pf->dfdDlambda = ((dhat02 + pf->psi * pf->psi) * pf->Dlambda) / root;
    }
  } else if (pf->kind == IKR_PF_LOAD_CONTROL) {  // :230-236
    pf->f = pf->Dlambda - pf->step_size;
    pf->dfdDD_scale = 0.0;
    pf->dfdDlambda = 1.0;
  } else {  // :316-324
    ikr::launch_mul64(pf->DDc.p, pf->DD.p, pf->mask.p, n, f->stream);
    count(1);
    const double nrm = std::sqrt(device_dot(f, pf->DDc.p, pf->DDc.p, n, pf->part, pf->out));
    pf->f = nrm - pf->step_size;
    pf->dfdDlambda = 0.0;
    pf->dfdDD_scale = 1.0 / nrm;
  }
}

// F_idbc = K_raw du_D/dlambda on the free dofs (obtainForcesDueToIDBC, functionhelper.hh:170-184) into a->idbc_force
void idbc_force(ikr_asm a, ikr_req r) {
  ikr_fes f = a->fes;
  assemble_matrix(a, r, IKR_DBC_RAW);
  a->idbc_force.alloc(a->n);
  ikr::launch_spmv64(a->bsr(), a->fp32, a->idbc_rate.p, a->idbc_force.p, f->stream);
  count(1);
}

// NewtonRaphsonWithSubsidiaryFunction::solve (newtonraphsonwithscalarsubsidiaryfunction.hh:207-316)
void pf_solve(ikr_pf pf, ikr_req r, ikr_nr_info* info) {
  ikr_nr nr = pf->nr;
  ikr_asm a = nr->asm_;
  ikr_fes f = a->fes;
  const ikr_nr_settings& st = nr->st;
  const int64_t n = a->n;
  cudaStream_t s = f->stream;
  ikr_nr_info inf{};
  inf.success = 1;
  inf.residual_norm = INFINITY;
  inf.correction_norm = INFINITY;
  inf.iterations = -1;
  ikr_nr_state state{r, INFINITY, INFINITY, 0, r->lambda};
  auto notify = [&](int msg) {
    state.residual_norm = inf.residual_norm;
    state.correction_norm = inf.correction_norm;
    state.iterations = inf.iterations < 0 ? 0 : inf.iterations;
    state.load_factor = r->lambda;
    for (auto& o : nr->obs) o.cb(msg, &state, o.user);
  };
  notify(IKR_NLS_INIT);
  nr->corr.alloc(n);
  nr->rhs.alloc(n);
  pf->fext0.alloc(n);
  pf->dR.alloc(n);
  pf->dL.alloc(n);
  pf->b2.alloc(n);
  pf->u_save.alloc(n);
  // Fext0 = -R(u = 0, lambda = 1): the load is lambda Fext0 (:225-232)
  CK(cudaMemcpyAsync(pf->u_save.p, r->u.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  const double lam_save = r->lambda;
  auto restore = [&]() {
    CK(cudaMemcpyAsync(r->u.p, pf->u_save.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    r->lambda = lam_save;
    r->version++;
  };
  CK(cudaMemsetAsync(r->u.p, 0, sizeof(double) * n, s));
  r->lambda = 1.0;
  r->version++;
  try {
    assemble_vector(a, r, IKR_DBC_FULL);
  } catch (...) {
    restore();  // the caller's state is left as it was
    throw;
  }
  ikr::launch_scale64(pf->fext0.p, a->R.p, -1.0, n, s);
  count(1);
  restore();
  assemble_vector(a, r, IKR_DBC_FULL);
  subsidiary(pf, a, r);
  double rnorm = device_norm(f, a->R.p, n, nr->nrm_part, nr->nrm_out);  // :244, without f
  inf.residual_norm = rnorm;
  const double thr = st.tol_mode == 1 ? st.tol * rnorm : st.tol;
  if (!a->nb) a->build_pattern();
  nr->ls->setup(a);
  int iter = 0;
  double rprev = rnorm;
  int64_t lin = 0;
  while (rnorm > thr && iter < st.max_iter) {  // :254
    notify(IKR_NLS_ITERATION_STARTED);
    // second column Fext0 - idbcForce(req) (:260-263)
    if (a->has_idbc) {
      idbc_force(a, r);
      CK(cudaMemcpyAsync(pf->b2.p, pf->fext0.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      ikr::launch_idbc_force(pf->b2.p, a->idbc_force.p, a->node_fixed.p, -1.0, n, s);
      count(1);
    }
    assemble_matrix(a, r, IKR_DBC_FULL);
    nr->ls->factorize(a);
    double eta = st.linear_rtol;
    if (st.forcing == 1) {  // Eisenstat-Walker as in the load-control Newton solve
      double ew = iter == 0 ? st.linear_rtol : 0.9 * (rnorm / rprev) * (rnorm / rprev);
      ew = std::min(ew, st.linear_rtol);
      const double need_eta = 0.5 * thr / std::max(rnorm, 1e-300);
      eta = std::min(std::max(std::max(ew, need_eta), st.linear_rtol_min), st.linear_rtol);
    }
    ikr::launch_scale64(nr->rhs.p, a->R.p, -1.0, n, s);
    count(1);
    // both columns with the same tangent (one matrix stream per CG iteration for the two when the solver
    // runs a persistent kind).  The load column starts from the previous dL: the CG solves for the change c with
    // K c = b2 - K dL_prev to the same accuracy relative to b2 (no solve when dL_prev already meets it).
    const double* b2 = a->has_idbc ? pf->b2.p : pf->fext0.p;
    if (pf->warm && pf->dl_valid) {
      pf->dl_res.alloc(n);
      pf->dl_corr.alloc(n);
      ikr::launch_residual64(a->bsr(), a->fp32, pf->dL.p, b2, pf->dl_res.p, s);
      count(1);
      const double nb2 = device_norm(f, b2, n, nr->nrm_part, nr->nrm_out);
      const double nres = device_norm(f, pf->dl_res.p, n, nr->nrm_part, nr->nrm_out);
      if (nres <= eta * nb2) {
        lin += nr->ls->solve(a, nr->rhs.p, pf->dR.p, eta, st.linear_max_iter, st.refinements);
        ++pf->dl_skipped;
      } else {
        lin += nr->ls->solve2(a, nr->rhs.p, pf->dl_res.p, pf->dR.p, pf->dl_corr.p, eta, st.linear_max_iter,
                              st.refinements, eta * nb2 / nres);
        ikr::launch_axpy64(pf->dL.p, pf->dl_corr.p, 1.0, n, s);
        count(1);
      }
    } else {
      lin += nr->ls->solve2(a, nr->rhs.p, b2, pf->dR.p, pf->dL.p, eta, st.linear_max_iter, st.refinements);
    }
    pf->dl_valid = true;
    const double dlam = (-pf->f - dfdDD_dot(pf, f, pf->dR.p, n)) /
                        (dfdDD_dot(pf, f, pf->dL.p, n) + pf->dfdDlambda);  // :275-276
    CK(cudaMemcpyAsync(nr->corr.p, pf->dR.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    ikr::launch_axpy64(nr->corr.p, pf->dL.p, dlam, n, s);
    count(1);
    const double dd2 = device_dot(f, nr->corr.p, nr->corr.p, n, nr->nrm_part, nr->nrm_out);
    inf.correction_norm = std::sqrt(dd2 + dlam * dlam);  // :291
    notify(IKR_NLS_CORRECTION_UPDATED);
    if (nr->fe_state) update_state(f, r, nr->corr.p);
    ikr::launch_axpy64(r->u.p, nr->corr.p, 1.0, n, s);
    ikr::launch_axpy64(pf->DD.p, nr->corr.p, 1.0, n, s);
    count(2);
    r->lambda += dlam;
    pf->Dlambda += dlam;
    if (a->has_idbc) idbc_sync(a, r);
    r->version++;
    assemble_vector(a, r, IKR_DBC_FULL);
    subsidiary(pf, a, r);
    const double rx = device_norm(f, a->R.p, n, nr->nrm_part, nr->nrm_out);
    rprev = rnorm;
    rnorm = std::sqrt(rx * rx + pf->f * pf->f);  // :298
    inf.residual_norm = rnorm;
    notify(IKR_NLS_SOLUTION_CHANGED);
    notify(IKR_NLS_CORRECTIONNORM_UPDATED);
    notify(IKR_NLS_RESIDUALNORM_UPDATED);
    ++iter;
    inf.iterations = iter;
    notify(IKR_NLS_ITERATION_ENDED);
    if (!std::isfinite(rnorm)) break;
  }
  if (iter == st.max_iter || !std::isfinite(rnorm)) inf.success = 0;
  inf.iterations = iter;
  inf.linear_iterations = lin;
  if (inf.success) notify(IKR_NLS_FINISHED_SUCESSFULLY);
  if (info) *info = inf;
}

// initialPrediction of the three kinds (pathfollowingfunctions.hh:132-174, :249-255, :330-336)
void initial_prediction(ikr_pf pf, ikr_req r) {
  ikr_nr nr = pf->nr;
  ikr_asm a = nr->asm_;
  ikr_fes f = a->fes;
  const ikr_nr_settings& st = nr->st;
  const int64_t n = a->n;
  cudaStream_t s = f->stream;
  if (pf->kind == IKR_PF_LOAD_CONTROL) {
    pf->Dlambda = pf->step_size;
    r->lambda = pf->Dlambda;
  } else if (pf->kind == IKR_PF_DISPLACEMENT_CONTROL) {
    // DD(controlled) = stepSize (the other entries keep their value); u = DD
    ikr::launch_mul64(pf->DDc.p, pf->DD.p, pf->mask.p, n, s);
    ikr::launch_axpy64(pf->DD.p, pf->DDc.p, -1.0, n, s);
    ikr::launch_axpy64(pf->DD.p, pf->mask.p, pf->step_size, n, s);
    CK(cudaMemcpyAsync(r->u.p, pf->DD.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    count(3);
    r->version++;
  } else {
    const double dlambda = 1.0;
    const double dhat02 = idbc_delta_sq(pf, a, r, dlambda) / (dlambda * dlambda);
    r->lambda = dlambda;
    r->version++;
    assemble_vector(a, r, IKR_DBC_FULL);
    // With an FP32 tangent the solve below is refined against the FP64 tangent: psi, and with it where every
    // arc-length step lands on the path, then agrees with the FP64 form (an FP32 solve alone is off by up to
    // cond(K) eps_32).  The FP64 tangent (and the FP64 K_raw of the prescribed values) are assembled into the
    // assembler's FP64 value array with the same kernels.
    const bool mixed = a->fp32;
    ikr::Bsr k64{};
    if (mixed) {
      a->val64.alloc(9 * (size_t)a->npad);
      a->fp32 = false;
      try {
        if (a->has_idbc) {
          idbc_force(a, r);
          ikr::launch_idbc_force(a->R.p, a->idbc_force.p, a->node_fixed.p, 1.0, n, s);
          count(1);
        }
        assemble_matrix(a, r, IKR_DBC_FULL);
      } catch (...) {
        a->fp32 = true;
        throw;
      }
      k64 = a->bsr();
      a->fp32 = true;
    } else if (a->has_idbc) {  // R += idbcForceFunction(req)
      idbc_force(a, r);
      ikr::launch_idbc_force(a->R.p, a->idbc_force.p, a->node_fixed.p, 1.0, n, s);
      count(1);
    }
    assemble_matrix(a, r, IKR_DBC_FULL);
    nr->ls->factorize(a);
    nr->rhs.alloc(n);
    ikr::launch_scale64(nr->rhs.p, a->R.p, -1.0, n, s);
    count(1);
    // the reference factorises a direct solver here; the CG runs to the tightest tolerance configured
    const double eta = st.forcing == 1 ? st.linear_rtol_min : st.linear_rtol;
    pf->pred_cg = nr->ls->solve(a, nr->rhs.p, pf->DD.p, eta, st.linear_max_iter, st.refinements);
    pf->pred_sweeps = 0;
    pf->pred_rel = 0.0;
    if (mixed) {  // iterative refinement: r = b - K64 DD in FP64, correction by the FP32 CG
      // A sweep cannot reduce the residual by more than about cond(K) eps_32 (the FP32 tangent's own error),
      // so the correction's CG tolerance follows the reduction the previous sweep achieved.
      constexpr double kTarget = 1e-10;
      constexpr int kSweeps = 20;
      pf->dl_res.alloc(n);
      pf->dl_corr.alloc(n);
      const double nb = device_norm(f, nr->rhs.p, n, nr->nrm_part, nr->nrm_out);
      double inner = 1e-2, prev = -1.0;
      for (int k = 0;; ++k) {
        ikr::launch_residual64(k64, false, pf->DD.p, nr->rhs.p, pf->dl_res.p, s);
        count(1);
        const double nres = device_norm(f, pf->dl_res.p, n, nr->nrm_part, nr->nrm_out);
        pf->pred_rel = nb > 0.0 ? nres / nb : 0.0;
        if (!(nres > kTarget * nb) || k == kSweeps) break;
        if (prev > 0.0) inner = std::min(0.25, std::max(1e-3, 0.25 * nres / prev));
        prev = nres;
        pf->pred_cg += nr->ls->solve(a, pf->dl_res.p, pf->dl_corr.p, inner, st.linear_max_iter, 0);
        ikr::launch_axpy64(pf->DD.p, pf->dl_corr.p, 1.0, n, s);
        count(1);
        pf->pred_sweeps = k + 1;
      }
    }
    const double dd2 = device_dot(f, pf->DD.p, pf->DD.p, n, pf->part, pf->out);
    pf->psi = std::sqrt(dd2 + dhat02);
    const double sc = std::sqrt(dd2 + dhat02 + pf->psi * pf->psi * dlambda * dlambda);
    ikr::launch_scale64(pf->DD.p, pf->DD.p, pf->step_size / sc, n, s);
    count(1);
    pf->Dlambda = pf->step_size / sc;
    const double idbc2 = dhat02 * pf->Dlambda * pf->Dlambda;  // ||idbcDelta * Dlambda / dlambda||^2
    ikr::launch_axpy64(r->u.p, pf->DD.p, 1.0, n, s);
    count(1);
    r->lambda = pf->Dlambda;
    if (a->has_idbc) idbc_sync(a, r);
    r->version++;
    const double ddn2 = device_dot(f, pf->DD.p, pf->DD.p, n, pf->part, pf->out);
    pf->psi = std::sqrt((idbc2 + ddn2) / (pf->Dlambda * pf->Dlambda));
  }
  pf->computed = true;
}

// intermediatePrediction of the three kinds (:188-195, :269-274, :339-344)
void intermediate_prediction(ikr_pf pf, ikr_req r) {
  ikr_asm a = pf->nr->asm_;
  need(pf->computed, IKR_ERR_INVALID_STATE, "initialPrediction has to be called before intermediatePrediction.");
  if (pf->kind == IKR_PF_LOAD_CONTROL) {
    r->lambda += pf->Dlambda;
    return;
  }
  ikr::launch_axpy64(r->u.p, pf->DD.p, 1.0, a->n, a->fes->stream);
  count(1);
  r->version++;
  if (pf->kind == IKR_PF_DISPLACEMENT_CONTROL) return;
  r->lambda += pf->Dlambda;
  if (a->has_idbc) idbc_sync(a, r);
}

}  // namespace

extern "C" {

int ikr_path_following_create(ikr_pf* out, ikr_nr nr, int32_t steps, double step_size, int32_t kind,
                              int32_t n_controlled, const int32_t* controlled) {
  return guarded([&] {
    need(out && nr, IKR_ERR_ARG, "null argument");
    need(steps > 0, IKR_ERR_INVALID_STATE, "Number of steps should be greater than zero.");  // pathfollowing.hh:192
    need(kind >= IKR_PF_ARC_LENGTH && kind <= IKR_PF_DISPLACEMENT_CONTROL, IKR_ERR_ARG, "unknown path-following kind");
    auto pf = std::make_unique<ikr_pf_s>();
    pf->nr = nr;
    pf->steps = steps;
    pf->step_size0 = step_size;
    pf->kind = kind;
    if (kind == IKR_PF_DISPLACEMENT_CONTROL) {
      ikr_asm a = nr->asm_;
      need(n_controlled > 0 && controlled, IKR_ERR_ARG, "displacement control needs controlled dofs");
      std::vector<uint8_t> seen(a->n, 0);
      for (int k = 0; k < n_controlled; ++k) {
        const int32_t d = controlled[k];
        need(d >= 0 && d < a->n, IKR_ERR_ARG, "controlled dof out of range");
        need(!a->fixed_h[d], IKR_ERR_ARG, "controlled dof is constrained");
        need(!seen[d], IKR_ERR_ARG, "controlled dof repeated");
        seen[d] = 1;
      }
      pf->controlled.assign(controlled, controlled + n_controlled);
    }
    nr->fe_state = true;  // the elements' state update follows the solver, as in the control-routine factory
    *out = pf.release();
  });
}
int ikr_path_following_destroy(ikr_pf pf) {
  return guarded([&] { delete pf; });
}
int ikr_path_following_set_adaptive_step_sizing(ikr_pf pf, int32_t kind, int32_t target_iterations) {
  return guarded([&] {
    need(pf, IKR_ERR_ARG, "null argument");
    need(kind == 0 || kind == 1, IKR_ERR_ARG, "unknown step-size adaptation");
    if (kind == 1)  // IterationBased::setTargetIterations (adaptivestepsizing.hh:51-55)
      need(target_iterations != 0, IKR_ERR_INVALID_STATE, "TargetIterations should not be equal to 0.");
    pf->adaptive = kind;
    pf->target_iterations = kind == 1 ? target_iterations : 0;
  });
}
int ikr_path_following_subscribe(ikr_pf pf, ikr_control_observer cb, void* user) {
  return guarded([&] {
    need(pf && cb, IKR_ERR_ARG, "null argument");
    pf->obs.push_back({cb, user});
  });
}
int ikr_path_following_subscribe_logger(ikr_pf pf, ikr_log_sink sink, void* user) {
  return guarded([&] {
    need(pf, IKR_ERR_ARG, "null argument");
    ControlObserver o{};
    pf->listeners.push_back(make_control_logger(sink, user, &o));
    pf->obs.push_back(o);
  });
}
int ikr_path_following_subsidiary_args(ikr_pf pf, double* out6) {
  return guarded([&] {
    need(pf && out6, IKR_ERR_ARG, "null argument");
    out6[0] = pf->step_size;
    out6[1] = pf->Dlambda;
    out6[2] = pf->f;
    out6[3] = pf->dfdDlambda;
    out6[4] = pf->psi;
    out6[5] = pf->current_step;
  });
}
int ikr_path_following_stats(ikr_pf pf, double* out4) {
  return guarded([&] {
    need(pf && out4, IKR_ERR_ARG, "null argument");
    out4[0] = pf->pred_sweeps;
    out4[1] = pf->pred_rel;
    out4[2] = (double)pf->pred_cg;
    out4[3] = (double)pf->dl_skipped;
  });
}
int ikr_path_following_set_warm_start(ikr_pf pf, int32_t on) {
  return guarded([&] {
    need(pf, IKR_ERR_ARG, "null argument");
    pf->warm = on != 0;
  });
}
int ikr_path_following_increment(ikr_pf pf, double* dd) {
  return guarded([&] {
    need(pf && dd, IKR_ERR_ARG, "null argument");
    ikr_asm a = pf->nr->asm_;
    if (!pf->DD.p) {
      std::fill(dd, dd + a->n, 0.0);
      return;
    }
    CK(cudaMemcpyAsync(dd, pf->DD.p, sizeof(double) * a->n, cudaMemcpyDeviceToHost, a->fes->stream));
    CK(cudaStreamSynchronize(a->fes->stream));
  });
}

int ikr_path_following_run(ikr_pf pf, ikr_req r, ikr_control_info* info, ikr_nr_info* infos, int32_t capacity) {
  return guarded([&] {
    need(pf && r, IKR_ERR_ARG, "null argument");
    ikr_nr nr = pf->nr;
    ikr_asm a = nr->asm_;
    ikr_fes f = a->fes;
    need(r->fes == f, IKR_ERR_ARG, "requirement of another element set");
    need(f->n_inst == 0 || nr->ls->tag != IKR_SOLVER_GPU_PCG_BATCHED, IKR_ERR_NOT_IMPLEMENTED,
         "path following of batched instances");
    need(!a->idbc_value, IKR_ERR_NOT_IMPLEMENTED,
         "path following with Dirichlet values given as a function (use ikr_assembler_set_dirichlet_values)");
    // the load-control and displacement-control subsidiary functions do not handle inhomogeneous Dirichlet values
    // (checkHasNoValidIDBCForceFunction, pathfollowingfunctions.hh:22-26)
    need(!a->has_idbc || pf->kind == IKR_PF_ARC_LENGTH, IKR_ERR_NOT_IMPLEMENTED,
         "The given path following function is not implemented to handle inhomogeneous Dirichlet BCs.");
    const int64_t n = a->n;
    cudaStream_t s = f->stream;
    // SubsidiaryArgs::setZero (pathfollowingfunctions.hh:58-68) and ArcLength's fresh state
    pf->DD.alloc(n);
    pf->DDc.alloc(n);
    CK(cudaMemsetAsync(pf->DD.p, 0, sizeof(double) * n, s));
    pf->Dlambda = pf->f = pf->dfdDlambda = pf->dfdDD_scale = 0.0;
    pf->current_step = 0;
    pf->psi = 0.0;
    pf->computed = false;
    pf->dl_valid = false;
    pf->dl_skipped = 0;
    if (pf->kind == IKR_PF_DISPLACEMENT_CONTROL) {
      std::vector<double> m(n, 0.0);
      for (int32_t d : pf->controlled) m[d] = 1.0;
      pf->mask.alloc(n);
      CK(cudaMemcpyAsync(pf->mask.p, m.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));
    }
    ikr_control_info ci{};
    static const char* kNames[] = {"Arc length", "Load Control", "Displacement Control"};  // pathfollowingfunctions.hh
    pf->name = std::string("Path following with ") + kNames[pf->kind];
    ikr_control_state cs{r, -1, 0.0, r->lambda, 0, pf->name.c_str()};
    auto notify = [&](int msg) {
      cs.load_factor = r->lambda;
      for (auto& o : pf->obs) o.cb(msg, &cs, o.user);
    };
    ikr_nr_info ni{};
    auto record = [&]() {  // updateAndNotifyControlInfo (pathfollowing.hh:229-235)
      if (infos && ci.n_solver_infos < capacity) infos[ci.n_solver_infos] = ni;
      ci.n_solver_infos++;
      ci.total_iterations += ni.iterations;
      ci.total_linear_iterations += ni.linear_iterations;
      cs.total_iterations = ci.total_iterations;
      notify(IKR_CONTROL_SOLUTION_CHANGED);
      notify(IKR_STEP_ENDED);
    };
    notify(IKR_CONTROL_STARTED);
    pf->step_size = pf->step_size0;
    cs.load_step = -1;
    notify(IKR_STEP_STARTED);
    nr->inst_failed.clear();
    pf_solve(pf, r, &ni);
    record();
    if (ni.success) {
      cs.load_step = 0;
      cs.step_size = pf->step_size0;
      notify(IKR_STEP_STARTED);
      initial_prediction(pf, r);
      pf_solve(pf, r, &ni);
      record();
      bool ok = ni.success != 0;
      for (int ls = 1; ok && ls < pf->steps; ++ls) {
        pf->current_step = ls;
        cs.load_step = ls;
        // AdaptiveStepSizing::IterationBased (adaptivestepsizing.hh:36-47)
        if (pf->adaptive == 1 && pf->current_step != 0 && ni.iterations > pf->target_iterations)
          pf->step_size = std::sqrt((double)pf->target_iterations / ni.iterations) * pf->step_size;
        intermediate_prediction(pf, r);
        cs.step_size = pf->step_size;
        notify(IKR_STEP_STARTED);
        pf_solve(pf, r, &ni);
        record();
        ok = ni.success != 0;
      }
      if (ok) {
        notify(IKR_CONTROL_ENDED);
        ci.success = 1;
      }
    }
    if (info) *info = ci;
  });
}

}  // extern "C"
