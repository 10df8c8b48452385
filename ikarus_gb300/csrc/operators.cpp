// The reference's operator and listener objects around the assembler and the solvers:
//   * assembler.scalar (simpleassemblers.inl scalarImpl): sum of the element energies in element order;
//   * DifferentiableFunctionFactory::op (utils/differentiablefunctionfactory.hh:24-51): energy -> forces -> tangent
//     or forces -> tangent over the assembler, evaluated through the assembler's own device assembly;
//   * NewtonRaphson::residual() / jacobian() / updateFunction() (newtonraphson.hh:260-287);
//   * NonLinearSolverLogger (utils/listener/nonlinearsolverlogger.hh:22-95) and ControlLogger
//     (controllogger.hh:22-66, controllogger.cpp), printing the reference's lines.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "host_internal.h"

using namespace ikr_host;

struct ikr_nlo_s {
  ikr_asm a = nullptr;
  int32_t saff = 0, vaff = 0, maff = 0, dbc = IKR_DBC_FULL;
};

namespace {

// a C-ABI call made from inside another: its failure becomes this call's failure with the same status and message
void forward(int code) {
  if (code == IKR_OK) return;
  char buf[512];
  ikr_last_error(buf, sizeof(buf));
  throw IkrError(code, buf);
}

class LineSink {
 public:
  LineSink(ikr_log_sink sink, void* user) : sink_(sink), user_(user) {}
  void operator()(const char* fmt, ...) const {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (sink_) sink_(buf, user_);
    else std::printf("[info] %s\n", buf);
  }

 private:
  ikr_log_sink sink_;
  void* user_;
};

// NonLinearSolverLogger for a domain that is not a plain vector (FERequirements): iteration, ||R||, ||dx||, lambda
class NonLinearSolverLogger : public ListenerBase {
 public:
  NonLinearSolverLogger(ikr_log_sink sink, void* user) : log_(sink, user) {}
  static void update(int32_t msg, const ikr_nr_state* st, void* self) {
    static_cast<NonLinearSolverLogger*>(self)->on(msg, st);
  }

 private:
  void on(int32_t msg, const ikr_nr_state* st) {
    switch (msg) {
      case IKR_NLS_INIT:
        iters_ = 1;
        r_norm_ = d_norm_ = 0.0;
        log_("Non-linear solver started:");
        log_("%-11s %-20s %-20s %-20s", "Ite", "normR", "normD", "lambda");
        log_("-------------------------------------------------------------------------------");
        break;
      case IKR_NLS_ITERATION_ENDED:
        log_(" %-10d %-20.2e %-20.2e %-20.2e", iters_, r_norm_, d_norm_, lambda_);
        ++iters_;
        break;
      case IKR_NLS_RESIDUALNORM_UPDATED: r_norm_ = st->residual_norm; break;
      case IKR_NLS_SOLUTION_CHANGED: lambda_ = st->load_factor; break;
      case IKR_NLS_CORRECTIONNORM_UPDATED: d_norm_ = st->correction_norm; break;
      case IKR_NLS_FINISHED_SUCESSFULLY: log_("Number of iterations: %d", st->iterations); break;
      default: break;
    }
  }
  LineSink log_;
  int iters_ = 0;
  double r_norm_ = 0.0, d_norm_ = 0.0, lambda_ = 0.0;
};

class ControlLogger : public ListenerBase {
 public:
  ControlLogger(ikr_log_sink sink, void* user) : log_(sink, user) {}
  static void update(int32_t msg, const ikr_control_state* st, void* self) {
    static_cast<ControlLogger*>(self)->on(msg, st);
  }

 private:
  void on(int32_t msg, const ikr_control_state* st) {
    static const char* kRule = "===============================================================================";
    switch (msg) {
      case IKR_STEP_ENDED: log_("%s", kRule); break;
      case IKR_CONTROL_STARTED:
        start_ = std::chrono::high_resolution_clock::now();
        log_("%s", kRule);
        log_("Started %s", st->name ? st->name : "");
        log_("%s", kRule);
        break;
      case IKR_STEP_STARTED:
        log_("Load step: %4d %49s %.2e", st->load_step, "Step size = ", st->step_size);
        log_("-------------------------------------------------------------------------------");
        break;
      case IKR_CONTROL_ENDED: {
        const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(
            std::chrono::high_resolution_clock::now() - start_);
        log_("End of %s", st->name ? st->name : "");
        log_("Total number of iterations: %3d", st->total_iterations);
        log_("Elapsed time: %lld ms", (long long)ms.count());
        break;
      }
      default: break;
    }
  }
  LineSink log_;
  std::chrono::time_point<std::chrono::high_resolution_clock> start_{};
};

}  // namespace

namespace ikr_host {
std::unique_ptr<ListenerBase> make_control_logger(ikr_log_sink sink, void* user, ControlObserver* obs) {
  auto l = std::make_unique<ControlLogger>(sink, user);
  *obs = ControlObserver{&ControlLogger::update, l.get()};
  return l;
}
}  // namespace ikr_host

extern "C" {

int ikr_assembler_scalar(ikr_asm a, ikr_req r, int32_t aff, double* out) {
  return guarded([&] {
    need(a && r && r->fes == a->fes && out, IKR_ERR_ARG, "invalid arguments");
    const int ne = a->fes->ne;
    std::vector<double> e(ne);
    forward(ikr_fe_calculate_scalar(a->fes, r, aff, 0, ne, e.data()));
    double s = 0.0;
    for (double v : e) s += v;  // element order, as the reference's assembler loop
    *out = s;
  });
}

int ikr_nonlinear_operator_create(ikr_nlo* out, ikr_asm a, int32_t saff, int32_t vaff, int32_t maff, int32_t dbc) {
  return guarded([&] {
    need(out && a, IKR_ERR_ARG, "null argument");
    need(dbc >= IKR_DBC_RAW && dbc <= IKR_DBC_FULL, IKR_ERR_ARG, "invalid DBCOption");
    need(vaff == IKR_VEC_FORCES && maff == IKR_MAT_STIFFNESS, IKR_ERR_NOT_IMPLEMENTED,
         "the affordance collection must hold forces and stiffness (AffordanceCollections::elastoStatics)");
    need(saff == IKR_SCALAR_NO_AFFORDANCE || saff == IKR_SCALAR_MECHANICAL_POTENTIAL_ENERGY, IKR_ERR_NOT_IMPLEMENTED,
         "ScalarAffordance not implemented");
    auto f = std::make_unique<ikr_nlo_s>();
    f->a = a;
    f->saff = saff;
    f->vaff = vaff;
    f->maff = maff;
    f->dbc = dbc;
    *out = f.release();
  });
}

int ikr_nonlinear_operator_destroy(ikr_nlo f) {
  return guarded([&] { delete f; });
}

int ikr_nonlinear_operator_evaluate(ikr_nlo f, int32_t order, ikr_req r, double* out, int32_t* kind) {
  return guarded([&] {
    need(f && r, IKR_ERR_ARG, "null argument");
    const bool energy = f->saff != IKR_SCALAR_NO_AFFORDANCE;
    need(order >= 0 && order <= (energy ? 2 : 1), IKR_ERR_ARG, "derivative order beyond the operator's");
    const int k = energy ? order : order + 1;  // 0 scalar, 1 vector, 2 matrix
    if (kind) *kind = k;
    if (k == 0) {
      double v = 0.0;
      forward(ikr_assembler_scalar(f->a, r, f->saff, &v));
      if (out) *out = v;
    } else if (k == 1) {
      forward(ikr_assembler_vector(f->a, r, f->vaff, f->dbc, out));
    } else {
      forward(ikr_assembler_matrix(f->a, r, f->maff, f->dbc));
    }
  });
}

int ikr_newton_residual(ikr_nr nr, ikr_req r, double* out) {
  return guarded([&] {
    need(nr && r, IKR_ERR_ARG, "null argument");
    forward(ikr_assembler_vector(nr->asm_, r, IKR_VEC_FORCES, IKR_DBC_FULL, out));
  });
}

int ikr_newton_jacobian(ikr_nr nr, ikr_req r) {
  return guarded([&] {
    need(nr && r, IKR_ERR_ARG, "null argument");
    forward(ikr_assembler_matrix(nr->asm_, r, IKR_MAT_STIFFNESS, IKR_DBC_FULL));
  });
}

int ikr_newton_update(ikr_nr nr, ikr_req r, const double* dx) {
  return guarded([&] {
    need(nr && r && dx && r->fes == nr->asm_->fes, IKR_ERR_ARG, "invalid arguments");
    ikr_asm a = nr->asm_;
    const int64_t n = a->n;
    DBuf<double> d;
    d.upload(dx, n, a->fes->stream);
    ikr::launch_axpy64(r->u.p, d.p, 1.0, n, a->fes->stream);
    count(1);
    if (a->has_idbc) idbc_sync(a, r);
    r->version++;
    CK(cudaStreamSynchronize(a->fes->stream));
  });
}

int ikr_newton_graph_iterations(ikr_nr nr, int64_t* n) {
  return guarded([&] {
    need(nr && n, IKR_ERR_ARG, "null argument");
    *n = nr->graph_iterations;
  });
}

int ikr_newton_subscribe_logger(ikr_nr nr, ikr_log_sink sink, void* user) {
  return guarded([&] {
    need(nr, IKR_ERR_ARG, "null argument");
    auto l = std::make_unique<NonLinearSolverLogger>(sink, user);
    nr->obs.push_back({&NonLinearSolverLogger::update, l.get()});
    nr->listeners.push_back(std::move(l));
  });
}

int ikr_load_control_subscribe_logger(ikr_lc lc, ikr_log_sink sink, void* user) {
  return guarded([&] {
    need(lc, IKR_ERR_ARG, "null argument");
    ControlObserver o{};
    lc->listeners.push_back(make_control_logger(sink, user, &o));
    lc->obs.push_back(o);
  });
}

}  // extern "C"
