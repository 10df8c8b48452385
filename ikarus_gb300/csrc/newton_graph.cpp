// A Newton iteration as one CUDA graph launch.
//
// Launched one by one, an iteration of the mixed form is about 25 launches with five host round trips (status after
// the tangent, the CG scalars, the correction norm, status after the residual, the residual norm).  Captured once,
// the same launches -- tangent assembly (one launch per colour class, the row kernel or element blocks + gather,
// manipulator entries), block-Jacobi inverse, right-hand side, CG init, the persistent cooperative CG, the
// correction, its norm, u += correction, residual assembly, its norm -- and the copies of the norms, the CG scalars
// and the element status into pinned host memory run as one graph launch followed by one synchronisation.  The
// values that change between iterations are read by the kernels from device scalars the graph fills from pinned host
// memory at its start: the CG tolerance (Eisenstat-Walker forcing) and the load factor.  Everything else the launches
// take (buffers, kernel choices, grid sizes) is part of the capture's key; a change recaptures.  Results are
// bit-identical to the launch-by-launch iteration (same kernels, same order, same reductions).
#include <vector>

#include "host_internal.h"

namespace ikr_host {

bool step_graph_eligible(ikr_nr nr, ikr_req r) {
  ikr_asm a = nr->asm_;
  ikr_ls ls = nr->ls;
  ikr_fes f = a->fes;
  const ikr_nr_settings& st = nr->st;
  if (!st.step_graphs || (nr->step_graph && nr->step_graph->unsupported)) return false;
  return r->fes == f && f->na == 0 && f->n_inst == 0 && !a->has_idbc && !a->dual64 && st.refinements <= 0 &&
         st.max_backtracks <= 0 && ls->tag != IKR_SOLVER_GPU_PCG_BATCHED && ls->factorized && ls->asm_ == a &&
         ls->tuned_for == a && ls->persistent() && !ls->w.coarse && ls->outer_m == 0 && !ls->direct && !ls->profile &&
         f->epb_r > 0 && (a->fp32 ? f->epb_k32 : f->epb_k64) > 0 && (!a->fp32 || a->tan_path > 0) && a->nb > 0 &&
         !f->trac_dirty;
}

namespace {

std::vector<const void*> graph_key(ikr_nr nr, ikr_req r) {
  ikr_asm a = nr->asm_;
  ikr_ls ls = nr->ls;
  ikr_fes f = a->fes;
  const ikr::PcgWork& w = ls->w;
  auto v = [](int64_t x) { return reinterpret_cast<const void*>(x); };
  return {a, r, r->u.p, a->R.p, a->values(), nr->corr.p, nr->rhs.p, w.x, w.r, w.z, w.p0, w.p1, w.q, w.minv, w.scal,
          w.part_a, w.part_b, v(w.spmv_kind), v(w.keep_g), v(w.grid), v(w.barrier_polls), v(f->epb_r),
          v(a->fp32 ? f->epb_k32 : f->epb_k64), v(a->tan_path), a->me_idx.p, v((int64_t)a->me_idx.n), a->pl_dof.p,
          v((int64_t)a->pl_dof.n), f->trac.p, f->trac_idx.p, f->args().ext, v(nr->st.linear_max_iter),
          v(ls->point_jacobi), a->eblk.p};
}

bool capture(ikr_nr nr, ikr_req r, NewtonStepGraph& G) {
  ikr_asm a = nr->asm_;
  ikr_ls ls = nr->ls;
  ikr_fes f = a->fes;
  cudaStream_t s = f->stream;
  const int64_t n = a->n;
  if (G.exec) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  const int64_t launches0 = g_launches.load();
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  bool ok = false;
  try {
    CK(cudaMemcpyAsync(G.dev.p, G.host, 2 * sizeof(double), cudaMemcpyHostToDevice, s));  // rtol, lambda
    CK(cudaMemsetAsync(f->status.p, 0, sizeof(int), s));
    f->capture_lambda = G.dev.p + 1;
    assemble_matrix(a, r, IKR_DBC_FULL, false);
    ikr::launch_block_jacobi(a->bsr(), ls->fp32, ls->w.minv, ls->point_jacobi, s);
    ikr::launch_scale64(nr->rhs.p, a->R.p, -1.0, n, s);
    ls->w.rtol_dev = G.dev.p;
    ikr::launch_pcg_init(a->bsr(), ls->w, nr->rhs.p, 0.0, nr->st.linear_max_iter, s);
    ls->w.rtol_dev = nullptr;
    CK(ikr::launch_pcg_persistent(a->bsr(), ls->w, ls->w.spmv_kind - ls->first_persistent_kind(), s));
    ikr::launch_pcg_result(ls->w, nr->corr.p, 1.0, s);
    ikr::launch_norm2(nr->corr.p, n, G.part.p, G.dev.p + 2, s);
    ikr::launch_axpy64(r->u.p, nr->corr.p, 1.0, n, s);
    assemble_vector(a, r, IKR_DBC_FULL, false);
    ikr::launch_norm2(a->R.p, n, G.part.p + 1024, G.dev.p + 3, s);
    count(10);
    CK(cudaMemcpyAsync(G.host + 2, G.dev.p + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(G.host + 4, ls->w.scal, ikr::kNScal * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(G.host + 4 + ikr::kNScal, f->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    ok = true;
  } catch (const IkrError&) {
    ok = false;
  }
  f->capture_lambda = nullptr;
  ls->w.rtol_dev = nullptr;
  err = cudaStreamEndCapture(s, &g);
  G.launches = g_launches.load() - launches0;
  g_launches.fetch_sub(G.launches);  // nothing ran yet; counted per graph launch
  if (ok && err == cudaSuccess) err = cudaGraphInstantiate(&G.exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (!ok || err != cudaSuccess) {
    cudaGetLastError();  // a capture the driver refuses leaves the iterations launch by launch
    if (G.exec) cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
    G.unsupported = true;
    return false;
  }
  return true;
}

}  // namespace

int64_t step_graph_iteration(ikr_nr nr, ikr_req r, double rtol, double* corr_norm, double* res_norm) {
  ikr_asm a = nr->asm_;
  ikr_ls ls = nr->ls;
  ikr_fes f = a->fes;
  cudaStream_t s = f->stream;
  if (!nr->step_graph) nr->step_graph = std::make_unique<NewtonStepGraph>();
  NewtonStepGraph& G = *nr->step_graph;
  if (!G.host) CK(cudaMallocHost(&G.host, sizeof(double) * (5 + ikr::kNScal)));
  G.dev.alloc(4);
  G.part.alloc(2048);
  nr->corr.alloc(a->n);
  nr->rhs.alloc(a->n);
  f->refresh_function_loads(r->lambda);  // host-evaluated loads at this load factor (before the launch)
  std::vector<const void*> key = graph_key(nr, r);
  if (!G.exec || key != G.key) {
    if (!capture(nr, r, G)) return -1;
    G.key = key;
  }
  G.host[0] = rtol;
  G.host[1] = r->lambda;
  CK(cudaGraphLaunch(G.exec, s));
  count(G.launches);
  CK(cudaStreamSynchronize(s));
  ++nr->graph_iterations;
  r->version++;
  const double* sc = G.host + 4;
  int status = 0;
  std::memcpy(&status, G.host + 4 + ikr::kNScal, sizeof(int));
  ls->last_iters = (int)sc[ikr::kIters];
  ls->last_rel = sc[ikr::kBB] > 0 ? std::sqrt(sc[ikr::kRR] / sc[ikr::kBB]) : 0.0;
  if (status) f->check_status();  // the status word is still set on the device: report it as launch by launch
  if (sc[ikr::kDone] == 6.0) fail(IKR_ERR_TIMEOUT, "a bounded wait in the persistent CG gave up");
  if (sc[ikr::kDone] == 3.0)
    fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp zero or not finite) after %d iterations", ls->last_iters);
  *corr_norm = G.host[2];
  *res_norm = G.host[3];
  return ls->last_iters;
}

}  // namespace ikr_host
