// Host side of the batched instances (independent problems of one element set, solver tag 101): the Newton-Raphson
// over the instances, the planner of the batched CG's launches and the precision escalation of a batched load control.
// Every instance runs its own Newton iteration and relative convergence test; one assembly and one sequence of
// batched CG launches serve all instances still in the solve.
#include <exception>
#include <thread>

#include "host_internal.h"

namespace ikr_host {

// The planner itself, on given co-resident capacities (caps[v]: CTAs of variant v, cluster_cap: 16-CTA clusters),
// rows and widest slice per running instance; kept free of device calls so that it is tested on the host.
BatchChoice choose_batch_plan(const std::vector<int>& rows, const std::vector<int>& width, bool fp32, int forced,
                              const int (&caps)[6], int cluster_cap) {
  const int n = (int)rows.size();
  BatchChoice out;
  out.ctas.assign(n, 1);
  // FP32: one instance per 16-CTA cluster (vectors and sums in distributed shared memory) while the running
  // instances fit one cluster each and the device holds all their clusters at once
  if (fp32 && (forced == -1 || forced == 4)) {
    // chosen by the planner only for instances of at most 512 rows: its iteration grows with the rows per CTA (the
    // distributed-shared-memory gathers of 27 blocks per thread), measured 8.4 us at 297 rows against 9.2 us for
    // eight threads per row, but 15.2 against 9.2 us at 2 673 rows
    const int max_rows = forced == 4 ? ikr::batched_cluster_rows() : std::min(512, ikr::batched_cluster_rows());
    bool fits = n <= cluster_cap;
    for (int k = 0; k < n && fits; ++k) fits = rows[k] <= max_rows && width[k] <= ikr::batched_cluster_width();
    if (fits) {
      out.variant = 4;
      out.ctas.assign(n, 16);
      return out;
    }
  }
  std::vector<int> cand;
  if (forced >= 0 && forced != 4) cand.push_back(forced);
  else if (forced == -1) cand = fp32 ? std::vector<int>{3, 2, 1} : std::vector<int>{5, 3, 2, 1};
  std::vector<int> c(n, 1);
  for (int v : cand) {
    if (v == 0) break;
    const int rpc = ikr::batched_pcg_rows_per_cta(v), maxw = ikr::batched_pcg_max_width(v);
    bool fits = true;
    int64_t tot = 0;
    // sixteen threads per row pays (FP64) while groups stay small; beyond 64 CTAs the wider group barrier costs more
    // than the spread FP64 work saves (measured on one 2 673-row instance: 23.3 against 20.5 us per iteration)
    const int max_group = v == 5 ? 64 : 256;
    for (int k = 0; k < n && fits; ++k) {
      const int ck = std::max(1, (rows[k] + rpc - 1) / rpc);
      fits = ck <= max_group && width[k] <= maxw;
      c[k] = ck;
      tot += ck;
    }
    if (fits && tot <= caps[v]) {
      out.variant = v;
      out.ctas = c;
      out.cooperative = std::any_of(c.begin(), c.end(), [](int x) { return x > 1; });
      return out;
    }
  }
  // rows looped per thread: C_i ~ rows over the smallest rows-per-CTA q (>= 64 rows per CTA) whose groups fit;
  // with more instances than resident CTAs every group is one CTA (an ordinary launch; no CTA waits on another)
  const int cap = caps[0];
  auto sizes_for = [&](int64_t q, std::vector<int>& o) {
    int64_t t = 0;
    for (int k = 0; k < n; ++k) {
      int64_t ck = (rows[k] + q - 1) / q;
      ck = std::min<int64_t>(ck, std::max(1, rows[k] / 64));
      ck = std::max<int64_t>(1, std::min<int64_t>(ck, 32));
      o[k] = (int)ck;
      t += ck;
    }
    return t;
  };
  if (n < cap) {
    int64_t lo = 1, hi = *std::max_element(rows.begin(), rows.end()) + 1;
    std::vector<int> tmp(n);
    while (lo < hi) {  // smallest rows-per-CTA q whose groups fit the resident CTAs
      const int64_t mid = (lo + hi) / 2;
      if (sizes_for(mid, tmp) <= cap) hi = mid;
      else lo = mid + 1;
    }
    sizes_for(lo, out.ctas);
  }
  out.cooperative = std::any_of(out.ctas.begin(), out.ctas.end(), [](int x) { return x > 1; });
  return out;
}

// CTA groups of one batched CG launch over the instances in `run` (choose_batch_plan on the device's co-resident
// capacities, a share of them while another solver's batched CG runs concurrently); largest instances first.
static void plan_batch_launch(ikr_nr nr, ikr_fes f, ikr_asm a, bool fp32, const std::vector<int>& run) {
  auto& P = nr->plan;
  const int sms = num_sms();
  const int nr_ = (int)run.size();
  std::vector<int> rows(nr_), width(nr_, 0), order(nr_);
  for (int k = 0; k < nr_; ++k) {
    const int r0 = f->inst_off_h[run[k]], r1 = f->inst_off_h[run[k] + 1];
    rows[k] = r1 - r0, order[k] = k;
    for (int sl = r0 >> 5; r1 > r0 && sl <= (r1 - 1) >> 5; ++sl)
      width[k] = std::max(width[k], a->slice_off_h[sl + 1] - a->slice_off_h[sl]);
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return rows[x] > rows[y]; });
  auto share = [&](int cap) { return std::max(1, (int)(cap * P.share)); };
  int caps[6];
  for (int v = 0; v < 6; ++v) caps[v] = v == 4 ? 0 : share(ikr::batched_pcg_capacity(fp32, v, sms));
  const BatchChoice ch =
      choose_batch_plan(rows, width, fp32, P.variant, caps, fp32 ? share(ikr::batched_cluster_capacity()) : 0);
  std::vector<int32_t> ci, cf, cs;
  if (ch.variant == 4) {  // one cluster per instance: the kernel takes the instance of each cluster
    for (int k : order) ci.push_back(run[k]);
  } else {
    for (int k : order) {
      const int first = (int)ci.size();
      for (int m = 0; m < ch.ctas[k]; ++m) ci.push_back(run[k]), cf.push_back(first), cs.push_back(ch.ctas[k]);
    }
  }
  cudaStream_t s = f->stream;
  P.n_cta = (int)ci.size();
  P.cur_variant = ch.variant;
  P.cooperative = ch.cooperative;
  // the arrays keep their allocation across launches (a plan has at most max(instances, resident CTAs) entries)
  size_t cap = (size_t)f->n_inst;
  for (int v = 0; v < 6; ++v)
    if (v != 4) cap = std::max(cap, (size_t)ikr::batched_pcg_capacity(fp32, v, sms));
  for (auto* b : {&P.cta_inst, &P.cta_first, &P.cta_size})
    if (b->n < cap) b->alloc(cap);
  if (P.part.n < 4 * cap) P.part.alloc(4 * cap);
  CK(cudaMemcpyAsync(P.cta_inst.p, ci.data(), sizeof(int32_t) * ci.size(), cudaMemcpyHostToDevice, s));
  if (!cf.empty()) {
    CK(cudaMemcpyAsync(P.cta_first.p, cf.data(), sizeof(int32_t) * cf.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(P.cta_size.p, cs.data(), sizeof(int32_t) * cs.size(), cudaMemcpyHostToDevice, s));
  }
}

// The batched CG of one Newton iteration: the instances with act set start their PCG on -R; the solve runs as a
// sequence of launches of 128, 256, ... (at most 4096) iterations, each re-planned over the instances still
// running, so that the hard instances that outlast the others get more CTAs and one row per thread.  Instances not
// in the solve get a zero correction.  cgit: CG iterations per instance (0 for those not in the solve).
static void batched_cg(ikr_nr nr, ikr_fes f, ikr_asm a, const std::vector<uint8_t>& act, std::vector<int32_t>& cgit) {
  const int ni = f->n_inst;
  cudaStream_t s = f->stream;
  auto& P = nr->plan;
  ikr::PcgWork& w = nr->ls->w;
  const ikr_nr_settings& st = nr->st;
  CK(cudaMemsetAsync(nr->corr.p, 0, sizeof(double) * a->n, s));
  std::vector<int> run;
  for (int i = 0; i < ni; ++i)
    if (act[i]) run.push_back(i);
  std::fill(cgit.begin(), cgit.end(), 0);
  if (run.empty()) return;
  P.st.alloc(4 * (size_t)ni);
  P.flag.alloc(ni);
  P.counters.alloc(ni);
  std::vector<int32_t> flag(ni), its(ni);
  int chunk = std::max(1, P.first_chunk);
  bool first = true;
  while (!run.empty()) {
    plan_batch_launch(nr, f, a, a->fp32, run);
    if (P.cur_variant == 4)
      CK(ikr::launch_batched_pcg_cluster(a->bsr(), w.minv, nr->rhs.p, nr->corr.p, P.n_cta, f->inst_off.p,
                                         P.cta_inst.p, w.x, w.r, w.z, w.p0, w.p1, nr->inst_rtol.p, st.linear_max_iter,
                                         chunk, first ? 1 : 0, P.st.p, nr->inst_cg_iters.p, P.flag.p,
                                         nr->inst_cg_res.p, s));
    else
      CK(ikr::launch_batched_pcg(a->bsr(), a->fp32, P.cur_variant, w.minv, nr->rhs.p, nr->corr.p, P.n_cta,
                                 f->inst_off.p, P.cta_inst.p, P.cta_first.p, P.cta_size.p, w.x, w.r, w.z, w.p0, w.p1,
                                 w.q, nr->inst_rtol.p, st.linear_max_iter, chunk, first ? 1 : 0, P.st.p,
                                 nr->inst_cg_iters.p, P.flag.p, nr->inst_cg_res.p, P.part.p, P.counters.p, ni,
                                 P.cooperative, s));
    count(1);
    ++P.launches;
    ++P.launches_by_variant[P.cur_variant];
    first = false;
    chunk = std::min(2 * chunk, std::max(chunk, 4096));
    P.flag.download(flag.data(), ni, s);
    CK(cudaStreamSynchronize(s));
    std::vector<int> next;
    for (int i : run) {
      if (flag[i] < 0) fail(IKR_ERR_TIMEOUT, "a bounded wait in the batched CG gave up (instance %d)", i);
      if (flag[i] == 0) next.push_back(i);
    }
    run.swap(next);
  }
  nr->inst_cg_iters.download(its.data(), ni, s);
  CK(cudaStreamSynchronize(s));
  for (int i = 0; i < ni; ++i) cgit[i] = act[i] ? its[i] : 0;
}

// Instances whose elements invert (det C <= 0, or a non-finite state) are taken out of the solve: their element status goes to a
// per-instance flag, they get no further corrections, count as failed (converged = -1 in the instance info)
// and do not stop the other instances.  The failures persist until reset_instance_failures.
void nr_solve_batched(ikr_nr nr, ikr_req r, ikr_nr_info* info) {
  ikr_asm a = nr->asm_;
  ikr_fes f = a->fes;
  cudaStream_t s = f->stream;
  const ikr_nr_settings& st = nr->st;
  const int ni = f->n_inst;
  const int64_t n = a->n;
  if ((int)nr->inst_failed.size() != ni) nr->inst_failed.assign(ni, 0);
  for (int i = 0; i < ni && i < (int)nr->inst_excluded.size(); ++i) {
    if (nr->inst_excluded[i]) nr->inst_failed[i] = 3;  // kept out by the caller
    else if (nr->inst_failed[i] == 3) nr->inst_failed[i] = 0;  // no longer kept out
  }
  struct StatusScope {  // per-instance element status for the duration of the solve
    ikr_fes f;
    explicit StatusScope(ikr_fes ff) : f(ff) { f->inst_status_on = true; }
    ~StatusScope() { f->inst_status_on = false; }
  } scope(f);
  std::vector<int> ist(ni);
  auto collect_failures = [&]() {
    f->inst_status.download(ist.data(), ni, s);
    CK(cudaStreamSynchronize(s));
    bool any_bad = false;
    for (int i = 0; i < ni; ++i)
      if (ist[i]) {
        any_bad = true;
        if (ist[i] & ~(ikr::kStatusNonPositiveDetC | ikr::kStatusNonFinite))
          fail(IKR_ERR_ARG, "device status %d in instance %d", ist[i], i);
        nr->inst_failed[i] = 1;
      }
    if (any_bad) CK(cudaMemsetAsync(f->inst_status.p, 0, sizeof(int) * ni, s));
  };
  nr->corr.alloc(n);
  nr->rhs.alloc(n);
  nr->inst_norm.alloc(ni);
  nr->inst_rtol.alloc(ni);
  nr->inst_cg_iters.alloc(ni);
  nr->inst_cg_res.alloc(ni);
  std::vector<double> rn(ni), r0(ni), rprev(ni), thr(ni), eta(ni);
  std::vector<uint8_t> act(ni), careful(ni, 0);
  std::vector<int32_t> cgit(ni);
  nr->inst_iters.assign(ni, 0);
  nr->inst_lin.assign(ni, 0);
  nr->inst_conv.assign(ni, 0);
  // the observers see the largest residual norm over the instances still in the solve and the batch's Newton
  // iteration count (newtonraphson.hh:193-257 notifies per iteration; here one iteration serves every instance)
  ikr_nr_state state{r, INFINITY, INFINITY, 0, r->lambda};
  auto notify = [&](int msg, int it) {
    double m = 0.0;
    for (int i = 0; i < ni; ++i)
      if (!nr->inst_failed[i] && std::isfinite(rn[i])) m = std::max(m, rn[i]);
    state.residual_norm = m;
    state.iterations = it;
    state.load_factor = r->lambda;
    for (auto& o : nr->obs) o.cb(msg, &state, o.user);
  };
  auto norms = [&]() {
    ikr::launch_instance_norms(a->R.p, ni, f->inst_off.p, nr->inst_norm.p, s);
    count(1);
    nr->inst_norm.download(rn.data(), ni, s);
    CK(cudaStreamSynchronize(s));
  };
  assemble_vector(a, r, IKR_DBC_FULL);
  collect_failures();
  norms();
  r0 = rn;
  for (int i = 0; i < ni; ++i) {
    thr[i] = st.tol_mode == 1 ? st.tol * r0[i] : st.tol;
    act[i] = rn[i] > thr[i] && !nr->inst_failed[i];
  }
  notify(IKR_NLS_INIT, 0);
  if (!a->nb) a->build_pattern();
  nr->ls->setup(a);
  int iter = 0;
  int64_t lin = 0;
  auto any = [&] { return std::any_of(act.begin(), act.end(), [](uint8_t v) { return v != 0; }); };
  while ((any() && iter < st.max_iter) || iter < st.min_iter) {
    notify(IKR_NLS_ITERATION_STARTED, iter);
    assemble_matrix(a, r, IKR_DBC_FULL);
    collect_failures();
    for (int i = 0; i < ni; ++i)
      if (nr->inst_failed[i]) act[i] = 0;
    nr->ls->factorize(a);
    for (int i = 0; i < ni; ++i) {
      double e = st.linear_rtol;
      if (st.forcing == 1 && nr->inst_iters[i] > 0) {
        e = std::min(st.linear_rtol, 0.9 * (rn[i] / rprev[i]) * (rn[i] / rprev[i]));
        e = std::max(e, 0.5 * thr[i] / std::max(rn[i], 1e-300));
        e = std::min(std::max(e, st.linear_rtol_min), st.linear_rtol);
      }
      eta[i] = careful[i] ? std::min(e, st.linear_rtol_min) : e;
    }
    nr->inst_rtol.upload(eta.data(), ni, s);
    ikr::launch_scale64(nr->rhs.p, a->R.p, -1.0, n, s);
    count(1);
    batched_cg(nr, f, a, act, cgit);
    if (nr->take_out_unsolved) {  // the CG ran out of iterations above its tolerance: no usable direction
      std::vector<double> relres(ni);
      nr->inst_cg_res.download(relres.data(), ni, s);
      CK(cudaStreamSynchronize(s));
      for (int i = 0; i < ni; ++i)
        if (act[i] && cgit[i] >= st.linear_max_iter && !(relres[i] <= eta[i])) nr->inst_failed[i] = 4;
    }
    std::vector<uint8_t> failed_before(nr->inst_failed);
    if (st.max_backtracks > 0) {
      nr->u_old.alloc(n);
      CK(cudaMemcpyAsync(nr->u_old.p, r->u.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    }
    ikr::launch_axpy64(r->u.p, nr->corr.p, 1.0, n, s);
    count(1);
    r->version++;
    for (int i = 0; i < ni; ++i) rprev[i] = rn[i];
    assemble_vector(a, r, IKR_DBC_FULL);
    collect_failures();
    // instances whose corrected state inverts an element go back and take half their step, up to
    // max_backtracks times; the others keep their full step
    std::vector<double> step(ni, 1.0);
    for (int bt = 0; bt < st.max_backtracks; ++bt) {
      bool any_new = false;
      for (int i = 0; i < ni; ++i)
        if (nr->inst_failed[i] && !failed_before[i] && act[i]) {
          nr->inst_failed[i] = 0;
          step[i] *= 0.5;
          any_new = true;
          ++nr->backtracks;
        }
      if (!any_new) break;
      nr->inst_step.upload(step.data(), ni, s);
      ikr::launch_instance_step(r->u.p, nr->u_old.p, nr->corr.p, ni, f->inst_off.p, nr->inst_step.p, s);
      count(1);
      r->version++;
      assemble_vector(a, r, IKR_DBC_FULL);
      collect_failures();
    }
    // an instance that still inverts after the halvings goes back, once per solve, to the state before this
    // correction and takes its next corrections with the tightest linear tolerance (an inexact direction, not the
    // load step, is the usual cause in the FP32 form); inverting again takes it out
    if (st.max_backtracks > 0) {
      bool any_retry = false;
      for (int i = 0; i < ni; ++i)
        if (nr->inst_failed[i] && !failed_before[i] && act[i] && !careful[i]) {
          nr->inst_failed[i] = 0;
          careful[i] = 1;
          step[i] = 0.0;
          any_retry = true;
          ++nr->backtracks;
        }
      if (any_retry) {
        nr->inst_step.upload(step.data(), ni, s);
        ikr::launch_instance_step(r->u.p, nr->u_old.p, nr->corr.p, ni, f->inst_off.p, nr->inst_step.p, s);
        count(1);
        r->version++;
        assemble_vector(a, r, IKR_DBC_FULL);
        collect_failures();
      }
    }
    notify(IKR_NLS_SOLUTION_CHANGED, iter);
    norms();
    for (int i = 0; i < ni; ++i) {
      lin += cgit[i];
      nr->inst_lin[i] += cgit[i];
      if (act[i]) nr->inst_iters[i]++;
      act[i] = rn[i] > thr[i] && std::isfinite(rn[i]) && !nr->inst_failed[i];
    }
    ++iter;
    notify(IKR_NLS_RESIDUALNORM_UPDATED, iter);
    notify(IKR_NLS_ITERATION_ENDED, iter);
  }
  // an instance still above its tolerance after max_iter is taken out as well (status -2), so that one
  // instance's failure does not end the others' load path; the solve succeeds when every instance not taken out
  // converged
  bool ok = true;
  for (int i = 0; i < ni; ++i) {
    if (nr->inst_failed[i]) {
      const int fl = nr->inst_failed[i];
      nr->inst_conv[i] = fl == 3 ? -3 : (fl == 2 ? -2 : (fl == 4 ? -4 : -1));
    } else if (rn[i] <= thr[i]) {
      nr->inst_conv[i] = 1;
    } else {
      nr->inst_conv[i] = -2;
      nr->inst_failed[i] = 2;
    }
  }
  for (int i = 0; i < ni; ++i) ok = ok && nr->inst_conv[i] != 0;
  nr->inst_res = rn;
  ikr_nr_info inf{};
  inf.success = ok ? 1 : 0;
  inf.residual_norm = *std::max_element(rn.begin(), rn.end());
  inf.correction_norm = 0.0;
  inf.iterations = iter;
  inf.linear_iterations = lin;
  if (ok) notify(IKR_NLS_FINISHED_SUCESSFULLY, iter);
  if (info) *info = inf;
}

// precision escalation of batched load steps (ikr_load_control_set_escalation)
void escalation_begin(ikr_lc lc, ikr_req r) {
  ikr_fes f = r->fes;
  const int ni = f->n_inst;
  lc->escalated.assign(ni, 0);
  lc->esc_conv.assign(ni, 0);
  lc->esc_nr->inst_failed.assign(ni, 0);
  lc->esc_nr->inst_excluded.assign(ni, 1);
  ikr_req e = lc->esc_req;
  CK(cudaStreamSynchronize(f->stream));
  CK(cudaMemcpyAsync(e->u.p, r->u.p, sizeof(double) * r->u.n, cudaMemcpyDeviceToDevice, e->fes->stream));
  CK(cudaStreamSynchronize(e->fes->stream));
  e->lambda = r->lambda;
  e->version++;
}

static void copy_instance(ikr_fes f, double* dst, const double* src, int i, cudaStream_t s) {
  const int64_t o = 3LL * f->inst_off_h[i], n = 3LL * (f->inst_off_h[i + 1] - f->inst_off_h[i]);
  CK(cudaMemcpyAsync(dst + o, src + o, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
}

// one step of the escalation solver over the instances in `sel` (the others kept out) at load factor lambda
static ikr_nr_info escalation_solve(ikr_lc lc, double lambda, double step, const std::vector<uint8_t>& sel) {
  ikr_nr en = lc->esc_nr;
  ikr_req e = lc->esc_req;
  const int ni = (int)sel.size();
  for (int i = 0; i < ni; ++i) en->inst_excluded[i] = sel[i] ? 0 : 1;
  e->lambda = lambda;
  e->version++;
  ikr_nr_info ei{};
  nr_solve(en, e, step, &ei);
  for (int i = 0; i < ni; ++i)
    if (sel[i]) lc->esc_conv[i] = en->inst_conv[i];
  return ei;
}

// A load step with escalation.  The run's solver does the step for the instances it holds; the instances it takes
// out in this step start again from the state at the step's start in the escalation solver, which solves them
// together with the instances escalated in earlier steps -- or, with esc_concurrent, the earlier ones on a second
// host thread and stream while the run's solver works and the fresh ones after it.  Every escalated instance's
// displacement is copied back.
void escalated_step(ikr_lc lc, ikr_req r, double step, double ref, ikr_nr_info& ni) {
  ikr_fes f = r->fes;
  ikr_req e = lc->esc_req;
  const int n_inst = f->n_inst;
  const std::vector<uint8_t> old = lc->escalated;
  const bool any_old = std::any_of(old.begin(), old.end(), [](uint8_t v) { return v != 0; });
  const double lambda = r->lambda;
  ikr_nr_info e1{}, e2{};
  const bool overlap = any_old && lc->esc_concurrent;
  if (overlap) {
    std::exception_ptr err;
    lc->nr->plan.share = 0.5;
    lc->esc_nr->plan.share = 0.5;
    std::thread worker([&] {
      try {
        e1 = escalation_solve(lc, lambda, step, old);
      } catch (...) {
        err = std::current_exception();
      }
    });
    struct Join {  // the worker is joined however the run's solve ends
      std::thread& t;
      ikr_lc lc;
      ~Join() {
        if (t.joinable()) t.join();
        lc->nr->plan.share = 1.0;
        lc->esc_nr->plan.share = 1.0;
      }
    } join{worker, lc};
    nr_solve(lc->nr, r, step, &ni, ref);
    worker.join();
    if (err) std::rethrow_exception(err);
  } else {
    nr_solve(lc->nr, r, step, &ni, ref);
  }
  CK(cudaStreamSynchronize(f->stream));
  // one after the other, the step's escalation solve takes the earlier and the fresh instances together (one Newton
  // loop whose length is the slowest instance's); overlapped, the earlier ones are done and the fresh ones follow
  std::vector<uint8_t> sel = overlap ? std::vector<uint8_t>(n_inst, 0) : old;
  for (int i = 0; i < n_inst; ++i) {
    const int c = lc->nr->inst_conv[i];
    if (!lc->escalated[i] && (c == -1 || c == -2 || c == -4)) {
      copy_instance(f, e->u.p, lc->u_start.p, i, e->fes->stream);
      lc->escalated[i] = 1;
      sel[i] = 1;
    }
  }
  const bool any_sel = std::any_of(sel.begin(), sel.end(), [](uint8_t v) { return v != 0; });
  if (any_sel) e2 = escalation_solve(lc, lambda, step, sel);
  bool any = false;
  for (int i = 0; i < n_inst; ++i)
    if (lc->escalated[i]) copy_instance(f, r->u.p, e->u.p, i, e->fes->stream), any = true;
  CK(cudaStreamSynchronize(e->fes->stream));
  if (!any) return;
  r->version++;
  // the step succeeds when every instance is converged in one of the two solvers or taken out by the escalation
  // solver too; Newton and CG iterations of both solvers add up
  bool ok = true;
  for (int i = 0; i < n_inst; ++i) ok = ok && (lc->escalated[i] ? lc->esc_conv[i] != 0 : lc->nr->inst_conv[i] != 0);
  ni.success = ok ? 1 : 0;
  ni.iterations += e1.iterations + e2.iterations;
  ni.linear_iterations += e1.linear_iterations + e2.linear_iterations;
  ni.residual_norm = std::max({ni.residual_norm, overlap ? e1.residual_norm : 0.0, any_sel ? e2.residual_norm : 0.0});
}

}  // namespace ikr_host

extern "C" {

int ikr_batched_plan_preview(int32_t n, const int32_t* rows, const int32_t* widths, int32_t fp32, int32_t variant,
                             const int32_t* caps6, int32_t cluster_cap, int32_t* out_variant, int32_t* out_ctas) {
  return guarded([&] {
    need(n > 0 && rows && widths && caps6 && out_variant && out_ctas && variant >= -1 && variant <= 5, IKR_ERR_ARG,
         "invalid argument");
    std::vector<int> r(rows, rows + n), w(widths, widths + n);
    int caps[6];
    for (int v = 0; v < 6; ++v) caps[v] = caps6[v];
    const ikr_host::BatchChoice ch = ikr_host::choose_batch_plan(r, w, fp32 != 0, variant, caps, cluster_cap);
    *out_variant = ch.variant;
    for (int k = 0; k < n; ++k) out_ctas[k] = ch.ctas[k];
  });
}
}  // extern "C"
