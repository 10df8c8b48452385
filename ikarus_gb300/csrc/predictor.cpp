// Learned Newton predictor for LoadControl: a POD basis of displacement increments plus a small MLP
// (BF16 weights, FP32 accumulation) trained on the GPU with the kernels of mlp.cu.  No counterpart in the
// reference, whose LoadControl predictor only increments the load factor (loadcontrol.inl:54-57).
//
// Features of load step k: the path's load parameters, the new load factor and the POD coordinates of the two
// previous converged increments; target: the change of the increment's POD coordinates from step k-1 to k (the
// increment itself on a path's first step).  Prediction = u + du_{k-1} + Phi * MLP(...); it is kept only if its
// FP64 residual is smaller than that of the previous-increment prediction u + du_{k-1} (its fallback), and the
// Newton test of the step stays relative to the residual of the unpredicted state.
#include <cstring>
#include <random>

#include "host_internal.h"

// ---- small dense linear algebra on the host (l <= a few hundred) -------------------------------------------
namespace {

// A = R^T R (upper R, row-major l x l); false if not positive definite
bool cholesky_upper(std::vector<double> A, int l, std::vector<double>& R) {
  R.assign((size_t)l * l, 0.0);
  for (int j = 0; j < l; ++j) {
    double s = A[(size_t)j * l + j];
    for (int k = 0; k < j; ++k) s -= R[(size_t)k * l + j] * R[(size_t)k * l + j];
    if (!(s > 0.0)) return false;
    const double d = std::sqrt(s);
    R[(size_t)j * l + j] = d;
    for (int i = j + 1; i < l; ++i) {
      double t = A[(size_t)j * l + i];
      for (int k = 0; k < j; ++k) t -= R[(size_t)k * l + j] * R[(size_t)k * l + i];
      R[(size_t)j * l + i] = t / d;
    }
  }
  return true;
}
// (R^{-1})^T for upper triangular R (row-major)
std::vector<double> inv_upper_transposed(const std::vector<double>& R, int l) {
  std::vector<double> X((size_t)l * l, 0.0);  // X = R^{-1}, upper
  for (int j = 0; j < l; ++j) {
    X[(size_t)j * l + j] = 1.0 / R[(size_t)j * l + j];
    for (int i = j - 1; i >= 0; --i) {
      double s = 0.0;
      for (int k = i + 1; k <= j; ++k) s += R[(size_t)i * l + k] * X[(size_t)k * l + j];
      X[(size_t)i * l + j] = -s / R[(size_t)i * l + i];
    }
  }
  std::vector<double> T((size_t)l * l);
  for (int i = 0; i < l; ++i)
    for (int j = 0; j < l; ++j) T[(size_t)i * l + j] = X[(size_t)j * l + i];
  return T;
}
// cyclic Jacobi eigen-decomposition of a symmetric matrix: A = V diag(w) V^T, eigenpairs sorted descending
void jacobi_eigen(std::vector<double> A, int l, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)l * l, 0.0);
  for (int i = 0; i < l; ++i) V[(size_t)i * l + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < l; ++p)
      for (int q = p + 1; q < l; ++q) off += A[(size_t)p * l + q] * A[(size_t)p * l + q];
    if (off < 1e-30) break;
    for (int p = 0; p < l; ++p)
      for (int q = p + 1; q < l; ++q) {
        const double apq = A[(size_t)p * l + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double app = A[(size_t)p * l + p], aqq = A[(size_t)q * l + q];
        const double th = 0.5 * (aqq - app) / apq;
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < l; ++k) {
          const double akp = A[(size_t)k * l + p], akq = A[(size_t)k * l + q];
          A[(size_t)k * l + p] = c * akp - s * akq;
          A[(size_t)k * l + q] = s * akp + c * akq;
        }
        for (int k = 0; k < l; ++k) {
          const double apk = A[(size_t)p * l + k], aqk = A[(size_t)q * l + k];
          A[(size_t)p * l + k] = c * apk - s * aqk;
          A[(size_t)q * l + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < l; ++k) {
          const double vkp = V[(size_t)k * l + p], vkq = V[(size_t)k * l + q];
          V[(size_t)k * l + p] = c * vkp - s * vkq;
          V[(size_t)k * l + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(l);
  for (int i = 0; i < l; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int a, int b) { return A[(size_t)a * l + a] > A[(size_t)b * l + b]; });
  std::vector<double> V2((size_t)l * l);
  w.resize(l);
  for (int j = 0; j < l; ++j) {
    w[j] = A[(size_t)ord[j] * l + ord[j]];
    for (int i = 0; i < l; ++i) V2[(size_t)i * l + j] = V[(size_t)i * l + ord[j]];
  }
  V.swap(V2);
}

std::vector<float> to_f32(const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); }

}  // namespace

// ---- multilayer perceptron ------------------------------------------------------------------------------------
namespace ikr_host {

struct Mlp {
  int n_in = 0, width = 0, depth = 0, n_out = 0;
  std::vector<int> dims;                  // n_in, width (x depth), n_out
  std::vector<int64_t> w_off, b_off, wb_off;
  int64_t n_params = 0, n_wb = 0;
  DBuf<float> p, g, m, v;                 // FP32 master parameters, gradients, Adam moments
  DBuf<uint16_t> wb;                      // BF16 copies of the weight matrices
  DBuf<int64_t> bf_index;                 // parameter -> BF16 slot (or -1 for biases)
  DBuf<float> act, dact, xb, tb, part;    // activations, their gradients, batch buffers, loss partials
  DBuf<int32_t> idx;
  int cap_batch = 0;
  int adam_step = 0;

  int layers() const { return (int)dims.size() - 1; }

  void init(int nin, int w, int d, int nout, uint64_t seed, cudaStream_t s) {
    n_in = nin, width = w, depth = d, n_out = nout;
    dims.clear();
    dims.push_back(nin);
    for (int i = 0; i < d; ++i) dims.push_back(w);
    dims.push_back(nout);
    w_off.clear(), b_off.clear(), wb_off.clear();
    n_params = n_wb = 0;
    for (int l = 0; l < layers(); ++l) {
      w_off.push_back(n_params);
      wb_off.push_back(n_wb);
      n_params += (int64_t)dims[l + 1] * dims[l];
      n_wb += (int64_t)dims[l + 1] * dims[l];
      b_off.push_back(n_params);
      n_params += dims[l + 1];
    }
    std::vector<float> h(n_params, 0.f);
    std::vector<int64_t> bi(n_params, -1);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < layers(); ++l) {  // Glorot-uniform weights, zero biases
      const double a = std::sqrt(6.0 / (dims[l] + dims[l + 1]));
      std::uniform_real_distribution<double> U(-a, a);
      for (int64_t k = 0; k < (int64_t)dims[l + 1] * dims[l]; ++k) {
        h[w_off[l] + k] = (float)U(rng);
        bi[w_off[l] + k] = wb_off[l] + k;
      }
    }
    p.upload(h.data(), h.size(), s);
    bf_index.upload(bi.data(), bi.size(), s);
    g.alloc(n_params), m.alloc(n_params), v.alloc(n_params);
    CK(cudaMemsetAsync(m.p, 0, sizeof(float) * n_params, s));
    CK(cudaMemsetAsync(v.p, 0, sizeof(float) * n_params, s));
    wb.alloc(n_wb);
    ikr::launch_to_bf16(p.p, wb.p, bf_index.p, n_params, s);
    count(1);
    adam_step = 0;
  }

  void set_params(const float* h, cudaStream_t s) {
    p.upload(h, n_params, s);
    ikr::launch_to_bf16(p.p, wb.p, bf_index.p, n_params, s);
    count(1);
  }

  // activation layout: for layer l, Z_l and Y_l (B x dims[l+1]) consecutively
  int64_t act_size(int B) const {
    int64_t t = 0;
    for (int l = 0; l < layers(); ++l) t += 2LL * B * dims[l + 1];
    return t;
  }
  float* Z(int l, int B) {
    int64_t o = 0;
    for (int i = 0; i < l; ++i) o += 2LL * B * dims[i + 1];
    return act.p + o;
  }
  float* Y(int l, int B) { return Z(l, B) + (int64_t)B * dims[l + 1]; }
  float* dZ(int l, int B) { return dact.p + (Z(l, B) - act.p); }
  float* dY(int l, int B) { return dact.p + (Y(l, B) - act.p); }

  void ensure(int B) {
    if (B <= cap_batch) return;
    cap_batch = B;
    act.alloc(act_size(B));
    dact.alloc(act_size(B));
    xb.alloc((size_t)B * n_in);
    tb.alloc((size_t)B * n_out);
    part.alloc(((size_t)B * n_out + 255) / 256 + 1);
  }
  const uint16_t* W(int l) const { return wb.p + wb_off[l]; }

  // X: B x n_in on the device; output in Y(last)
  float* forward(const float* X, int B, cudaStream_t s) {
    ensure(B);
    const float* in = X;
    for (int l = 0; l < layers(); ++l) {
      const int din = dims[l], dout = dims[l + 1];
      ikr::launch_gemm(B, dout, din, in, false, false, din, W(l), true, true, din, Z(l, B), dout, 1.f, 0.f, s);
      ikr::launch_bias_act(Z(l, B), Y(l, B), p.p + b_off[l], B, dout, l + 1 < layers(), s);
      count(2);
      in = Y(l, B);
    }
    return Y(layers() - 1, B);
  }

  // MSE loss against T (B x n_out) and gradients of all parameters into g (straight-through BF16 weights)
  double loss_grad(const float* X, const float* T, int B, cudaStream_t s) {
    float* out = forward(X, B, s);
    const int L = layers();
    const int64_t n = (int64_t)B * n_out;
    const int nb = ikr::launch_mse(out, T, dY(L - 1, B), n, 1.f / (float)n, part.p, s);
    count(1);
    for (int l = L - 1; l >= 0; --l) {
      const int din = dims[l], dout = dims[l + 1];
      float* dz = dZ(l, B);
      CK(cudaMemcpyAsync(dz, dY(l, B), sizeof(float) * (size_t)B * dout, cudaMemcpyDeviceToDevice, s));
      if (l + 1 < L) {
        ikr::launch_gelu_backward(dz, Z(l, B), (int64_t)B * dout, s);
        count(1);
      }
      const float* xin = l == 0 ? X : Y(l - 1, B);
      // dW = dZ^T X  (dout x din),  db = column sums of dZ,  dX = dZ W
      ikr::launch_gemm(dout, din, B, dz, false, true, dout, xin, false, false, din, g.p + w_off[l], din, 1.f, 0.f, s);
      ikr::launch_colsum(dz, g.p + b_off[l], B, dout, s);
      count(2);
      if (l > 0) {
        ikr::launch_gemm(B, din, dout, dz, false, false, dout, W(l), true, false, din, dY(l - 1, B), din, 1.f, 0.f, s);
        count(1);
      }
    }
    std::vector<float> hp(nb);
    CK(cudaMemcpyAsync(hp.data(), part.p, sizeof(float) * nb, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    double loss = 0.0;
    for (float x : hp) loss += x;
    return loss;
  }

  // Adam over mini-batches of (X, T) rows held on the device; returns the mean loss of the last epoch
  double train(const float* X, const float* T, int n, int epochs, int batch, float lr, uint64_t seed, cudaStream_t s) {
    batch = std::max(1, std::min(batch, n));
    ensure(batch);
    std::mt19937_64 rng(seed);
    std::vector<int32_t> perm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    idx.alloc(n);
    double last = 0.0;
    for (int ep = 0; ep < epochs; ++ep) {
      std::shuffle(perm.begin(), perm.end(), rng);
      idx.upload(perm.data(), perm.size(), s);
      double tot = 0.0;
      int nbatch = 0;
      for (int b0 = 0; b0 + batch <= n; b0 += batch) {
        ikr::launch_gather_rows(X, idx.p + b0, xb.p, batch, n_in, s);
        ikr::launch_gather_rows(T, idx.p + b0, tb.p, batch, n_out, s);
        count(2);
        tot += loss_grad(xb.p, tb.p, batch, s);
        ++nbatch;
        ++adam_step;
        ikr::launch_adam(p.p, g.p, m.p, v.p, wb.p, bf_index.p, n_params, lr, 0.9f, 0.999f, 1e-8f, adam_step, s);
        count(1);
      }
      last = nbatch ? tot / nbatch : 0.0;
    }
    return last;
  }
};

}  // namespace ikr_host

struct ikr_mlp_s {
  cudaStream_t stream = nullptr;
  ikr_host::Mlp net;
  ~ikr_mlp_s() {
    if (stream) cudaStreamDestroy(stream);
  }
};

struct SnapMeta {
  int path, step;
  double lambda;
};

struct ikr_pred_s {
  ikr_fes fes = nullptr;
  int n = 0, n_par = 0, k = 0, width = 0, depth = 0;
  uint64_t seed = 0;
  int64_t cap = 0, n_snap = 0;
  ikr_host::DBuf<float> snaps;  // column j (an FP32 increment of n dofs) at snaps + j * n
  std::vector<SnapMeta> meta;
  std::vector<std::vector<double>> theta;  // per path
  ikr_host::DBuf<float> phi;               // k x n row-major (= n x k column-major)
  std::vector<double> sv;
  ikr_host::Mlp net;
  std::vector<float> xmean, xstd, ymean, ystd;
  bool trained = false;
  ikr_host::DBuf<float> c1, c2, cpred, xin, dvec;
  int n_in() const { return n_par + 1 + 2 * k; }
};

namespace ikr_host {
namespace {

// c (k) = Phi^T d (n)
void project(ikr_pred p, const float* d, float* c, cudaStream_t s) {
  ikr::launch_gemm(p->k, 1, p->n, p->phi.p, false, false, p->n, d, false, false, 1, c, 1, 1.f, 0.f, s);
  count(1);
}

// features of one step: [theta, lambda, c_prev1, c_prev2] standardised
std::vector<float> features(ikr_pred p, const std::vector<double>& th, double lambda, const float* c1h,
                            const float* c2h) {
  std::vector<float> x(p->n_in());
  int o = 0;
  for (int i = 0; i < p->n_par; ++i) x[o++] = (float)th[i];
  x[o++] = (float)lambda;
  for (int i = 0; i < p->k; ++i) x[o++] = c1h ? c1h[i] : 0.f;
  for (int i = 0; i < p->k; ++i) x[o++] = c2h ? c2h[i] : 0.f;
  return x;
}

// randomized range finder + Rayleigh-Ritz on the snapshot matrix S (n x m): Phi = leading k left singular vectors
void pod_build(ikr_pred p, cudaStream_t s) {
  const int64_t n = p->n;
  const int m = (int)p->n_snap;
  const int k = std::min(p->k, m);
  const int l = std::min(k + 16, m);
  DBuf<float> omega, Yt, Zt, Qt, Bm, tmp;
  DBuf<double> G;
  omega.alloc((size_t)m * l);
  ikr::launch_randn(omega.p, (int64_t)m * l, p->seed ^ 0x5DEECE66Dull, s);
  Yt.alloc((size_t)l * n);
  Zt.alloc((size_t)l * m);
  // Yt (l x n) = Omega^T St;  St = S viewed row-major m x n
  ikr::launch_gemm(l, (int)n, m, omega.p, false, true, l, p->snaps.p, false, false, (int)n, Yt.p, (int)n, 1.f, 0.f, s);
  for (int it = 0; it < 2; ++it) {  // two power iterations: Zt = Yt St^T, Yt = Zt St
    ikr::launch_gemm(l, m, (int)n, Yt.p, false, false, (int)n, p->snaps.p, false, true, (int)n, Zt.p, m, 1.f, 0.f, s);
    ikr::launch_gemm(l, (int)n, m, Zt.p, false, false, m, p->snaps.p, false, false, (int)n, Yt.p, (int)n, 1.f, 0.f, s);
  }
  count(5);
  // CholeskyQR2: Q^T = R^{-T} Y^T
  G.alloc((size_t)l * l);
  Qt.alloc((size_t)l * n);
  tmp.alloc((size_t)l * l);
  std::vector<double> Gh((size_t)l * l), R;
  float* cur = Yt.p;
  float* nxt = Qt.p;
  for (int pass = 0; pass < 2; ++pass) {
    ikr::launch_gram64(cur, n, l, G.p, s);
    count(1);
    G.download(Gh.data(), Gh.size(), s);
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < l; ++i) Gh[(size_t)i * l + i] *= 1.0 + 1e-10;  // guards exact rank deficiency
    if (!cholesky_upper(Gh, l, R)) fail(IKR_ERR_SINGULAR, "POD: snapshot range is rank deficient");
    const std::vector<float> RiT = to_f32(inv_upper_transposed(R, l));
    tmp.upload(RiT.data(), RiT.size(), s);
    ikr::launch_gemm(l, (int)n, l, tmp.p, false, false, l, cur, false, false, (int)n, nxt, (int)n, 1.f, 0.f, s);
    count(1);
    std::swap(cur, nxt);
  }
  // B = Q^T S (l x m); eigen-decomposition of B B^T gives the left singular vectors in the Q basis
  Bm.alloc((size_t)l * m);
  ikr::launch_gemm(l, m, (int)n, cur, false, false, (int)n, p->snaps.p, false, true, (int)n, Bm.p, m, 1.f, 0.f, s);
  ikr::launch_gram64(Bm.p, m, l, G.p, s);  // rows of Bm as columns of length m
  count(2);
  G.download(Gh.data(), Gh.size(), s);
  CK(cudaStreamSynchronize(s));
  std::vector<double> w, V;
  jacobi_eigen(Gh, l, w, V);
  p->sv.resize(l);
  for (int i = 0; i < l; ++i) p->sv[i] = std::sqrt(std::max(w[i], 0.0));
  // Phi^T (k x n) = U_k^T Q^T
  std::vector<float> Ut((size_t)k * l);
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < l; ++j) Ut[(size_t)i * l + j] = (float)V[(size_t)j * l + i];
  tmp.upload(Ut.data(), Ut.size(), s);
  p->phi.alloc((size_t)p->k * n);
  CK(cudaMemsetAsync(p->phi.p, 0, sizeof(float) * p->phi.n, s));
  ikr::launch_gemm(k, (int)n, l, tmp.p, false, false, l, cur, false, false, (int)n, p->phi.p, (int)n, 1.f, 0.f, s);
  count(1);
  CK(cudaStreamSynchronize(s));
}

}  // namespace

void predictor_begin(ikr_lc lc, ikr_req r) {
  lc->hist = 0;
  lc->phist.clear();
  if (lc->pred_kind == 0 && !lc->record) return;
  const int64_t n = 3LL * r->fes->nn;
  lc->u_step0.alloc(n);
  lc->u_try.alloc(n);
  lc->du1.alloc(n);
  lc->du2.alloc(n);
}

// Candidates of a load step (u0 = converged state of the previous step at the new load factor):
//   previous increment  u0 + du1 (the "previous-step" predictor; needs one recorded increment)
//   learned             u0 + du1 + Phi c (kind 2: the network predicts the POD coordinates c of the change of
//                       the increment; on the first step, without du1, it predicts the increment itself)
// A candidate whose residual assembly meets det C <= 0 is discarded.  Kind 1 keeps the previous increment;
// kind 2 keeps the learned candidate only when its FP64 residual norm is below that of its fallback (the
// previous increment, or the unpredicted state on the first step), unless the gate is off.
double predictor_apply(ikr_lc lc, ikr_req r, int step) {
  ikr_fes f = r->fes;
  cudaStream_t s = f->stream;
  const int64_t n = 3LL * f->nn;
  if (lc->pred_kind == 0 && !lc->record) return 0.0;
  CK(cudaMemcpyAsync(lc->u_step0.p, r->u.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  if (lc->pred_kind == 0) return 0.0;
  ikr_asm a = lc->nr->asm_;
  assemble_vector(a, r, IKR_DBC_FULL);
  const double r_plain = device_norm(f, a->R.p, n, lc->pred_part, lc->pred_out);
  ikr_lc_s::PredRecord rec{(double)step, r_plain, -1.0, -1.0, 0.0, -1.0};
  // FP64 residual norm at u0 + d (+ du1); +inf when an element inverts
  auto residual_at = [&](const float* d, bool plus_du1) -> double {
    ikr::launch_base_plus_scaled(r->u.p, lc->u_step0.p, d, 1.0, n, s);
    if (plus_du1) ikr::launch_add_f32(r->u.p, lc->du1.p, n, s);
    count(plus_du1 ? 2 : 1);
    r->version++;
    try {
      assemble_vector(a, r, IKR_DBC_FULL);
    } catch (const IkrError& e) {
      if (e.code != IKR_ERR_NONPOSITIVE_DETC) throw;
      return INFINITY;
    }
    return device_norm(f, a->R.p, n, lc->pred_part, lc->pred_out);
  };
  const bool has_prev = lc->hist >= 1;
  if (has_prev) rec.r_fallback = residual_at(lc->du1.p, false);
  const float* dl = nullptr;
  if (lc->pred_kind == 2 && lc->pred && lc->pred->trained) {
    ikr_pred p = lc->pred;
    p->c1.alloc(p->k), p->c2.alloc(p->k), p->cpred.alloc(p->k), p->dvec.alloc(n);
    std::vector<float> c1h(p->k, 0.f), c2h(p->k, 0.f);
    if (lc->hist >= 1) {
      project(p, lc->du1.p, p->c1.p, s);
      p->c1.download(c1h.data(), p->k, s);
    }
    if (lc->hist >= 2) {
      project(p, lc->du2.p, p->c2.p, s);
      p->c2.download(c2h.data(), p->k, s);
    }
    CK(cudaStreamSynchronize(s));
    std::vector<float> x = features(p, lc->theta, r->lambda, lc->hist >= 1 ? c1h.data() : nullptr,
                                    lc->hist >= 2 ? c2h.data() : nullptr);
    for (size_t i = 0; i < x.size(); ++i) x[i] = (x[i] - p->xmean[i]) / p->xstd[i];
    p->xin.upload(x.data(), x.size(), s);
    float* y = p->net.forward(p->xin.p, 1, s);
    std::vector<float> yh(p->k);
    CK(cudaMemcpyAsync(yh.data(), y, sizeof(float) * p->k, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int i = 0; i < p->k; ++i) yh[i] = yh[i] * p->ystd[i] + p->ymean[i];
    p->cpred.upload(yh.data(), yh.size(), s);
    // d (1 x n) = c^T Phi^T
    ikr::launch_gemm(1, (int)n, p->k, p->cpred.p, false, false, p->k, p->phi.p, false, false, (int)n, p->dvec.p,
                     (int)n, 1.f, 0.f, s);
    count(1);
    dl = p->dvec.p;
    rec.r_learned = residual_at(dl, has_prev);
  }
  // second-order extrapolation of the path, u0 + du1 + (du1 - du2) (kind 3, from the third step on)
  const bool quad = lc->pred_kind == 3 && lc->hist >= 2;
  if (quad) {
    ikr::launch_base_plus_scaled(r->u.p, lc->u_step0.p, lc->du1.p, 2.0, n, s);
    ikr::launch_add_scaled_f32(r->u.p, lc->du2.p, -1.0, n, s);
    count(2);
    r->version++;
    try {
      assemble_vector(a, r, IKR_DBC_FULL);
      rec.spare = device_norm(f, a->R.p, n, lc->pred_part, lc->pred_out);
    } catch (const IkrError& e) {
      if (e.code != IKR_ERR_NONPOSITIVE_DETC) throw;
      rec.spare = INFINITY;
    }
  }
  const double r_fb = has_prev ? rec.r_fallback : r_plain;
  int keep = 0;  // 0 unpredicted, 1 previous increment, 2 learned, 3 second-order extrapolation
  if (has_prev && std::isfinite(rec.r_fallback)) keep = 1;
  if (dl && std::isfinite(rec.r_learned) && (!lc->gated || rec.r_learned < r_fb)) keep = 2;
  if (quad && std::isfinite(rec.spare) && (!lc->gated || rec.spare < r_fb)) keep = 3;
  // leave u at the kept state (the last one evaluated may be another)
  const int last = quad ? 3 : (dl ? 2 : (has_prev ? 1 : 0));
  if (keep != last) {
    if (keep == 0) {
      CK(cudaMemcpyAsync(r->u.p, lc->u_step0.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    } else if (keep == 1) {
      ikr::launch_base_plus_scaled(r->u.p, lc->u_step0.p, lc->du1.p, 1.0, n, s);
      count(1);
    }
    r->version++;
  }
  rec.kept = keep;
  if (lc->pred_kind == 2 || lc->pred_kind == 3) {
    if (keep == lc->pred_kind) lc->accepted++;
    else lc->rejected++;
  } else {
    if (keep == 1) lc->accepted++;
    else lc->rejected++;
  }
  lc->phist.push_back(rec);
  return r_plain;
}

void predictor_end_step(ikr_lc lc, ikr_req r, int step) {
  if (lc->pred_kind == 0 && !lc->record) return;
  ikr_fes f = r->fes;
  cudaStream_t s = f->stream;
  const int64_t n = 3LL * f->nn;
  std::swap(lc->du1.p, lc->du2.p);  // du2 <- previous du1
  ikr::launch_diff_to_f32(r->u.p, lc->u_step0.p, lc->du1.p, n, s);
  count(1);
  lc->hist = std::min(lc->hist + 1, 2);
  if (lc->record && lc->pred) {
    ikr_pred p = lc->pred;
    if (p->n_snap >= p->cap) fail(IKR_ERR_ARG, "predictor snapshot capacity (%lld) exhausted", (long long)p->cap);
    CK(cudaMemcpyAsync(p->snaps.p + p->n_snap * n, lc->du1.p, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
    p->meta.push_back({lc->path_id, step, r->lambda});
    p->n_snap++;
  }
}

}  // namespace ikr_host

using namespace ikr_host;

extern "C" {

// ---- MLP handle (gradient checks and stand-alone training) ----------------------------------------------------
int ikr_mlp_create(ikr_mlp* out, int32_t n_in, int32_t width, int32_t depth, int32_t n_out, uint64_t seed) {
  return guarded([&] {
    need(out && n_in > 0 && width > 0 && depth >= 0 && n_out > 0, IKR_ERR_ARG, "invalid network shape");
    auto m = std::make_unique<ikr_mlp_s>();
    CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    m->net.init(n_in, width, depth, n_out, seed, m->stream);
    CK(cudaStreamSynchronize(m->stream));
    *out = m.release();
  });
}
int ikr_mlp_destroy(ikr_mlp m) {
  return guarded([&] { delete m; });
}
int ikr_mlp_num_params(ikr_mlp m, int64_t* n) {
  return guarded([&] {
    need(m && n, IKR_ERR_ARG, "null argument");
    *n = m->net.n_params;
  });
}
int ikr_mlp_get_params(ikr_mlp m, float* out) {
  return guarded([&] {
    need(m && out, IKR_ERR_ARG, "null argument");
    m->net.p.download(out, m->net.n_params, m->stream);
    CK(cudaStreamSynchronize(m->stream));
  });
}
int ikr_mlp_set_params(ikr_mlp m, const float* in) {
  return guarded([&] {
    need(m && in, IKR_ERR_ARG, "null argument");
    m->net.set_params(in, m->stream);
    CK(cudaStreamSynchronize(m->stream));
  });
}
int ikr_mlp_forward(ikr_mlp m, int32_t batch, const float* x, float* y) {
  return guarded([&] {
    need(m && x && y && batch > 0, IKR_ERR_ARG, "invalid arguments");
    DBuf<float> dx;
    dx.upload(x, (size_t)batch * m->net.n_in, m->stream);
    float* out = m->net.forward(dx.p, batch, m->stream);
    CK(cudaMemcpyAsync(y, out, sizeof(float) * (size_t)batch * m->net.n_out, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
  });
}
int ikr_mlp_loss_grad(ikr_mlp m, int32_t batch, const float* x, const float* t, float* loss, float* grad) {
  return guarded([&] {
    need(m && x && t && batch > 0, IKR_ERR_ARG, "invalid arguments");
    DBuf<float> dx, dt;
    dx.upload(x, (size_t)batch * m->net.n_in, m->stream);
    dt.upload(t, (size_t)batch * m->net.n_out, m->stream);
    const double l = m->net.loss_grad(dx.p, dt.p, batch, m->stream);
    if (loss) *loss = (float)l;
    if (grad) m->net.g.download(grad, m->net.n_params, m->stream);
    CK(cudaStreamSynchronize(m->stream));
  });
}
int ikr_mlp_train(ikr_mlp m, int32_t n, const float* X, const float* T, int32_t epochs, int32_t batch, float lr,
                  uint64_t seed, float* final_loss) {
  return guarded([&] {
    need(m && X && T && n > 0 && epochs >= 0, IKR_ERR_ARG, "invalid arguments");
    DBuf<float> dX, dT;
    dX.upload(X, (size_t)n * m->net.n_in, m->stream);
    dT.upload(T, (size_t)n * m->net.n_out, m->stream);
    const double l = m->net.train(dX.p, dT.p, n, epochs, batch, lr, seed, m->stream);
    if (final_loss) *final_loss = (float)l;
    CK(cudaStreamSynchronize(m->stream));
  });
}

// ---- predictor --------------------------------------------------------------------------------------------------
int ikr_predictor_create(ikr_pred* out, ikr_fes fes, int32_t n_params, int32_t n_modes, int32_t width, int32_t depth,
                         int64_t capacity, uint64_t seed) {
  return guarded([&] {
    need(out && fes && n_params >= 0 && n_modes > 0 && width > 0 && depth >= 0 && capacity > 0, IKR_ERR_ARG,
         "invalid predictor arguments");
    auto p = std::make_unique<ikr_pred_s>();
    p->fes = fes;
    p->n = 3 * fes->nn;
    p->n_par = n_params;
    p->k = n_modes;
    p->width = width;
    p->depth = depth;
    p->seed = seed;
    p->cap = capacity;
    p->snaps.alloc((size_t)capacity * p->n);
    *out = p.release();
  });
}
int ikr_predictor_destroy(ikr_pred p) {
  return guarded([&] { delete p; });
}
int ikr_predictor_num_snapshots(ikr_pred p, int64_t* n) {
  return guarded([&] {
    need(p && n, IKR_ERR_ARG, "null argument");
    *n = p->n_snap;
  });
}
int ikr_predictor_fit(ikr_pred p, int32_t epochs, int32_t batch, float lr, float* final_loss, double* pod_energy) {
  return guarded([&] {
    need(p, IKR_ERR_ARG, "null argument");
    need(p->n_snap >= 4, IKR_ERR_INVALID_STATE, "too few recorded increments to train the predictor");
    cudaStream_t s = p->fes->stream;
    pod_build(p, s);
    const int m = (int)p->n_snap, k = p->k, nin = p->n_in();
    // POD coordinates of every snapshot: C (k x m) = Phi^T S
    DBuf<float> C;
    C.alloc((size_t)k * m);
    ikr::launch_gemm(k, m, p->n, p->phi.p, false, false, p->n, p->snaps.p, false, true, p->n, C.p, m, 1.f, 0.f, s);
    count(1);
    std::vector<float> Ch((size_t)k * m);
    C.download(Ch.data(), Ch.size(), s);
    CK(cudaStreamSynchronize(s));
    // samples: features from the same path's previous two increments; targets the change of the increment
    std::vector<float> X((size_t)m * nin), T((size_t)m * k);
    std::vector<float> col1(k), col2(k);
    for (int j = 0; j < m; ++j) {
      const SnapMeta& mt = p->meta[j];
      const bool h1 = j >= 1 && p->meta[j - 1].path == mt.path && mt.step >= 1;
      const bool h2 = j >= 2 && p->meta[j - 2].path == mt.path && mt.step >= 2;
      for (int i = 0; i < k; ++i) {
        col1[i] = h1 ? Ch[(size_t)i * m + j - 1] : 0.f;
        col2[i] = h2 ? Ch[(size_t)i * m + j - 2] : 0.f;
        // target: the change of the increment's POD coordinates (the increment itself on a path's first step)
        T[(size_t)j * k + i] = Ch[(size_t)i * m + j] - col1[i];
      }
      const std::vector<float> x = features(p, p->theta[mt.path], mt.lambda, col1.data(), col2.data());
      std::copy(x.begin(), x.end(), X.begin() + (size_t)j * nin);
    }
    auto stats = [&](const std::vector<float>& A, int cols, std::vector<float>& mean, std::vector<float>& sd) {
      mean.assign(cols, 0.f);
      sd.assign(cols, 1.f);
      for (int c = 0; c < cols; ++c) {
        double s1 = 0, s2 = 0;
        for (int j = 0; j < m; ++j) s1 += A[(size_t)j * cols + c];
        const double mu = s1 / m;
        for (int j = 0; j < m; ++j) s2 += (A[(size_t)j * cols + c] - mu) * (A[(size_t)j * cols + c] - mu);
        mean[c] = (float)mu;
        const double sdv = std::sqrt(s2 / m);
        sd[c] = sdv > 1e-12 ? (float)sdv : 1.f;
      }
    };
    stats(X, nin, p->xmean, p->xstd);
    stats(T, k, p->ymean, p->ystd);
    for (int j = 0; j < m; ++j) {
      for (int c = 0; c < nin; ++c) X[(size_t)j * nin + c] = (X[(size_t)j * nin + c] - p->xmean[c]) / p->xstd[c];
      for (int c = 0; c < k; ++c) T[(size_t)j * k + c] = (T[(size_t)j * k + c] - p->ymean[c]) / p->ystd[c];
    }
    p->net.init(nin, p->width, p->depth, k, p->seed, s);
    DBuf<float> dX, dT;
    dX.upload(X.data(), X.size(), s);
    dT.upload(T.data(), T.size(), s);
    const double loss = p->net.train(dX.p, dT.p, m, epochs, batch, lr, p->seed + 1, s);
    CK(cudaStreamSynchronize(s));
    p->trained = true;
    if (final_loss) *final_loss = (float)loss;
    if (pod_energy) {
      double tot = 0, top = 0;
      for (size_t i = 0; i < p->sv.size(); ++i) {
        tot += p->sv[i] * p->sv[i];
        if ((int)i < k) top += p->sv[i] * p->sv[i];
      }
      *pod_energy = tot > 0 ? top / tot : 0.0;
    }
  });
}

int ikr_load_control_set_predictor(ikr_lc lc, int32_t kind, ikr_pred p, const double* params, int32_t record) {
  return guarded([&] {
    need(lc && kind >= 0 && kind <= 3, IKR_ERR_ARG, "invalid predictor kind");
    need(kind != 2 || p, IKR_ERR_ARG, "the learned predictor needs a predictor object");
    need(!record || p, IKR_ERR_ARG, "recording needs a predictor object");
    lc->pred_kind = kind;
    lc->pred = p;
    lc->record = record != 0;
    lc->accepted = lc->rejected = 0;
    if (p) {
      lc->theta.assign(params ? params : nullptr, params ? params + p->n_par : nullptr);
      if (!params) lc->theta.assign(p->n_par, 0.0);
      if (lc->record) {
        lc->path_id = (int)p->theta.size();
        p->theta.push_back(lc->theta);
      }
    }
  });
}
int ikr_load_control_set_predictor_gate(ikr_lc lc, int32_t gated) {
  return guarded([&] {
    need(lc, IKR_ERR_ARG, "null argument");
    lc->gated = gated != 0;
  });
}
int ikr_load_control_predictor_history(ikr_lc lc, int32_t capacity, double* out, int32_t* n) {
  return guarded([&] {
    need(lc && n && capacity >= 0 && (capacity == 0 || out), IKR_ERR_ARG, "invalid arguments");
    *n = (int32_t)lc->phist.size();
    const int m = std::min<int>(capacity, (int)lc->phist.size());
    for (int i = 0; i < m; ++i) {
      const auto& h = lc->phist[i];
      const double v[6] = {h.step, h.r_plain, h.r_fallback, h.r_learned, h.kept, 0.0};
      std::copy(v, v + 6, out + 6 * i);
    }
  });
}
int ikr_load_control_predictor_stats(ikr_lc lc, int32_t* accepted, int32_t* rejected) {
  return guarded([&] {
    need(lc, IKR_ERR_ARG, "null argument");
    if (accepted) *accepted = lc->accepted;
    if (rejected) *rejected = lc->rejected;
  });
}

}  // extern "C"
