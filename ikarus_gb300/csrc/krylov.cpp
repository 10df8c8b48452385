// FP64 outer Krylov solve of the mixed form: flexible GMRES on the FP64 tangent, right-preconditioned by the FP32
// block-Jacobi CG on its FP32 rounding.
//
// Why: the mixed form's FP32 tangent differs from the FP64 one by its rounding, and a correction computed with it
// is off by about cond(K) eps_32 relative.  Where that exceeds one -- the nearly incompressible block with
// nu = 0.4999 -- neither an inexact Newton step with the FP32 tangent nor classical iterative refinement (whose
// sweeps contract by the same factor) converges.  Here the FP32 CG is only the preconditioner of a Krylov method
// whose operator is the FP64 tangent: each Arnoldi step applies the FP32 CG once (to a loose relative tolerance)
// and the FP64 product once, and the outer residual b - K64 x is minimised in FP64 over all directions found so
// far (Saad, "A flexible inner-outer preconditioned GMRES algorithm", SIAM J. Sci. Comput. 14 (1993); the
// mixed-precision use follows Carson & Higham's GMRES-based iterative refinement, SIAM J. Sci. Comput. 40
// (2018)).  The correction then solves the FP64 Newton system to the requested relative tolerance, whatever the
// FP32 tangent's error, as long as the FP32 CG is a useful preconditioner.
//
// Layout: V (m + 1 vectors) and Z (m vectors) dof-major FP64; the Hessenberg matrix, Givens rotations and the
// small triangular solve live on the host (m <= 64).  Orthogonalisation is classical Gram-Schmidt applied twice
// (two fixed-order multi-dot / multi-axpy passes), so a solve is bit-identical run to run.
#include <cmath>
#include <vector>

#include "host_internal.h"

namespace ikr_host {

int64_t fgmres_solve(ikr_ls ls, ikr_asm a, const double* b, double* x, double eta) {
  ikr_fes f = a->fes;
  cudaStream_t s = f->stream;
  const int64_t n = a->n;
  const int m = ls->outer_m;
  need(m > 0 && m <= ikr::kKrylovMaxBasis - 1, IKR_ERR_ARG, "FP64 outer solve: restart length out of range");
  need(a->fp32 && a->val64.p && a->k64_stamp == a->k_stamp && a->k_stamp > 0, IKR_ERR_INVALID_STATE,
       "the FP64 outer solve needs the FP64 twin of the last assembled tangent (assemble after enabling it)");
  ikr::Bsr A64 = a->bsr();
  A64.val = a->val64.p;
  ls->gm_V.alloc((size_t)(m + 1) * n);
  ls->gm_Z.alloc((size_t)m * n);
  ls->gm_w.alloc(n);
  ls->gm_r.alloc(n);
  ls->gm_h.alloc(2 * ikr::kKrylovMaxBasis);
  ls->gm_c.alloc(ikr::kKrylovMaxBasis);
  ls->gm_part.alloc((size_t)(m + 1) * ikr::multi_dot_blocks(n));
  double* V = ls->gm_V.p;
  double* Z = ls->gm_Z.p;
  double* w = ls->gm_w.p;
  double* r = ls->gm_r.p;
  double* h1 = ls->gm_h.p;
  double* h2 = ls->gm_h.p + ikr::kKrylovMaxBasis;
  auto norm = [&](const double* v) { return device_norm(f, v, n, ls->gm_npart, ls->gm_nout); };

  CK(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
  CK(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  const double bnorm = norm(r);
  ls->last_outer = 0;
  ls->last_cycles = 0;
  ls->last_rel = 0.0;
  ls->last_iters = 0;
  if (bnorm == 0.0) return 0;
  const double target = eta * bnorm;
  double beta = bnorm;
  int64_t inner = 0;
  int outer = 0, cycles = 0;
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hc(m + 2), hh(2 * ikr::kKrylovMaxBasis), y(m);
  while (beta > target && outer < ls->outer_max_iter) {
    ++cycles;
    ikr::launch_scale64(V, r, 1.0 / beta, n, s);
    count(1);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;  // Arnoldi steps of this cycle
    while (k < m && outer < ls->outer_max_iter) {
      double* vk = V + (size_t)k * n;
      double* zk = Z + (size_t)k * n;
      inner += ls->solve_device(a, vk, zk, ls->inner_rtol, ls->inner_max_iter);  // z_k ~ K32^-1 v_k (FP32 CG)
      ikr::launch_spmv64(A64, false, zk, w, s);                                 // w = K64 z_k
      // classical Gram-Schmidt, twice
      ikr::launch_multi_dot(V, n, k + 1, w, n, ls->gm_part.p, h1, s);
      ikr::launch_multi_axpy(w, V, n, k + 1, h1, -1.0, n, s);
      ikr::launch_multi_dot(V, n, k + 1, w, n, ls->gm_part.p, h2, s);
      ikr::launch_multi_axpy(w, V, n, k + 1, h2, -1.0, n, s);
      count(7);
      CK(cudaMemcpyAsync(hh.data(), ls->gm_h.p, sizeof(double) * 2 * ikr::kKrylovMaxBasis, cudaMemcpyDeviceToHost,
                         s));
      const double hn = norm(w);  // synchronises the stream (hh is then on the host)
      for (int i = 0; i <= k; ++i) hc[i] = hh[i] + hh[ikr::kKrylovMaxBasis + i];
      hc[k + 1] = hn;
      ++outer;
      if (hn > 0.0) {
        ikr::launch_scale64(V + (size_t)(k + 1) * n, w, 1.0 / hn, n, s);
        count(1);
      }
      // previous rotations, then the new one that zeroes hc[k + 1]
      for (int i = 0; i < k; ++i) {
        const double t = cs[i] * hc[i] + sn[i] * hc[i + 1];
        hc[i + 1] = -sn[i] * hc[i] + cs[i] * hc[i + 1];
        hc[i] = t;
      }
      const double rho = std::hypot(hc[k], hc[k + 1]);
      need(rho > 0.0 && std::isfinite(rho), IKR_ERR_CG_BREAKDOWN, "FP64 outer solve: singular Hessenberg column");
      cs[k] = hc[k] / rho;
      sn[k] = hc[k + 1] / rho;
      hc[k] = rho;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      for (int i = 0; i <= k; ++i) H[(size_t)i * m + k] = hc[i];
      ++k;
      if (std::fabs(g[k]) <= target || hn == 0.0) break;
    }
    // y = H(1:k, 1:k)^-1 g(1:k), x += Z y
    for (int i = k - 1; i >= 0; --i) {
      double t = g[i];
      for (int j = i + 1; j < k; ++j) t -= H[(size_t)i * m + j] * y[j];
      y[i] = t / H[(size_t)i * m + i];
    }
    CK(cudaMemcpyAsync(ls->gm_c.p, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    ikr::launch_multi_axpy(x, Z, n, k, ls->gm_c.p, 1.0, n, s);
    // the true FP64 residual decides (and restarts from it)
    ikr::launch_residual64(A64, false, x, b, r, s);
    count(2);
    beta = norm(r);
    need(std::isfinite(beta), IKR_ERR_CG_BREAKDOWN, "FP64 outer solve: residual not finite");
  }
  ls->last_outer = outer;
  ls->last_cycles = cycles;
  ls->last_rel = beta / bnorm;
  ls->last_iters = (int)inner;
  return inner;
}

}  // namespace ikr_host
