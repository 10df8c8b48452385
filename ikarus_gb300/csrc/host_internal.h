// Internals of the host layer shared by host.cpp (finite elements, assembler, solver, Newton, LoadControl)
// and predictor.cpp (learned Newton predictor).  One CUDA stream per finite-element set; every object built on
// that set (requirements, assembler, solver, Newton, LoadControl, predictor) issues its work on it.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ikarus_gb300.h"
#include "kernels.h"

namespace ikr_host {

extern thread_local std::string g_last_error;
extern std::atomic<int64_t> g_launches;

struct IkrError : std::runtime_error {
  int code;
  IkrError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw IkrError(code, buf);
}

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) fail(IKR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}
#define CK(x) cuda_check((x), #x)

inline void count(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

template <typename F>
int guarded(F&& f) {
  try {
    f();
    return IKR_OK;
  } catch (const IkrError& e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return IKR_ERR_ARG;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return IKR_ERR_ARG;
  }
}

// device buffer
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    CK(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void download(T* h, size_t count, cudaStream_t s) const {
    if (count) CK(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
};

inline int num_sms() {
  static int sms = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 152;
    return v > 0 ? v : 152;
  }();
  return sms;
}

}  // namespace ikr_host
using namespace ikr_host;

// ------------------------------------------------------------------------------------------------------------
struct ikr_fes_s {
  int nn = 0, ne = 0, na = 0, eas = 0;
  int material = IKR_MATERIAL_NEOHOOKE;
  ikr::HyperParams hyper;  // the functions of IKR_MATERIAL_HYPERELASTIC
  // elements per block of the displacement element kernel, chosen by timing at the first assembly of each kind
  // (0 = not chosen yet): residual, FP64 tangent, FP32 tangent
  int epb_r = 0, epb_k64 = 0, epb_k32 = 0;
  double lam = 0, mu = 0;
  cudaStream_t stream = nullptr;
  std::vector<int32_t> conn_h;  // row-major n_elems x 8
  DBuf<double> X;
  DBuf<int32_t> conn;  // corner-major
  DBuf<double> alpha;  // n_alpha x n_elems
  DBuf<double> eas_geo;
  DBuf<double> eas_y, eas_Y;
  uint64_t eas_cache_key = 0;  // (req id, solution version, alpha version) hash of the cached D^{-1}R~, D^{-1}L
  uint64_t alpha_version = 1;
  // colours
  std::vector<int32_t> colour_ptr;
  DBuf<int32_t> colour_elems;
  // Neumann faces
  std::vector<std::vector<std::pair<int, std::array<double, 3>>>> faces;
  DBuf<int32_t> trac_idx;
  DBuf<double> trac;
  bool trac_dirty = false;
  // loads given as functions f(X, lambda), evaluated on the host whenever the load factor changes: volume loads
  // at the Gauss points, Neumann faces at their quadrature point; their sum per element in ext (24 per element)
  struct FaceFnSet {
    ikr_point_fn f;
    void* user;
    std::vector<int32_t> slot_elem, face_ptr, face_local;  // faces grouped by element (traction kernel layout)
    std::vector<double> points;                            // quadrature point of every face, grouped order
  };
  std::vector<std::pair<ikr_point_fn, void*>> vol_fns;
  std::vector<FaceFnSet> face_fns;
  std::vector<double> X_h;    // coordinates (host copy)
  std::vector<double> xgp_h;  // Gauss-point positions (host, computed once on the device)
  DBuf<double> ext;
  bool ext_dirty = false;
  double ext_lambda = 0.0;
  // while a Newton iteration is captured as a graph: the device scalar its residual launches read the load factor from
  const double* capture_lambda = nullptr;
  DBuf<int> status;
  DBuf<double> scratch_out;  // element-level outputs
  DBuf<double> lam_e, mu_e;  // per-element Lame parameters (empty: lam / mu everywhere)
  // independent instances: disjoint contiguous node ranges [inst_off[i], inst_off[i+1])
  int n_inst = 0;
  std::vector<int32_t> inst_off_h;
  DBuf<int32_t> inst_off, inst_order;
  // per-instance element status, used instead of `status` while a batched Newton solve runs (an instance
  // whose elements invert is taken out of that solve instead of failing all instances)
  DBuf<int32_t> elem_inst;
  DBuf<int> inst_status;
  bool inst_status_on = false;

  ~ikr_fes_s() {
    if (stream) cudaStreamDestroy(stream);
  }

  ikr::ElemArgs args() const {
    ikr::ElemArgs a;
    a.n_nodes = nn;
    a.n_elems = ne;
    a.X = X.p;
    a.conn = conn.p;
    a.lam = lam;
    a.mu = mu;
    a.material = material;
    a.hyper = hyper;
    a.eas_kind = na > 0 ? eas : 0;
    a.n_alpha = na;
    a.alpha = alpha.p;
    a.eas_geo = eas_geo.p;
    a.eas_y = eas_y.p;
    a.eas_Y = eas_Y.p;
    a.trac_idx = trac_idx.n ? trac_idx.p : nullptr;
    a.trac = trac.p;
    a.ext = (vol_fns.empty() && face_fns.empty()) ? nullptr : ext.p;
    a.status = status.p;
    a.lam_e = lam_e.n ? lam_e.p : nullptr;
    a.mu_e = mu_e.n ? mu_e.p : nullptr;
    if (inst_status_on) {
      a.elem_inst = elem_inst.p;
      a.inst_status = inst_status.p;
    }
    return a;
  }

  void refresh_tractions() {
    if (!trac_dirty) return;
    std::vector<int32_t> idx(ne, -1), slot_elem, face_ptr{0}, face_local;
    std::vector<double> t;
    for (int e = 0; e < ne; ++e) {
      if (faces[e].empty()) continue;
      idx[e] = (int32_t)slot_elem.size();
      slot_elem.push_back(e);
      for (auto& f : faces[e]) {
        face_local.push_back(f.first);
        t.insert(t.end(), f.second.begin(), f.second.end());
      }
      face_ptr.push_back((int32_t)face_local.size());
    }
    trac_idx.upload(idx.data(), idx.size(), stream);
    DBuf<int32_t> d_se, d_fp, d_fl;
    DBuf<double> d_t;
    d_se.upload(slot_elem.data(), slot_elem.size(), stream);
    d_fp.upload(face_ptr.data(), face_ptr.size(), stream);
    d_fl.upload(face_local.data(), face_local.size(), stream);
    d_t.upload(t.data(), t.size(), stream);
    trac.alloc(std::max<size_t>(1, 24 * slot_elem.size()));
    ikr::launch_traction_loads(X.p, conn.p, ne, (int)slot_elem.size(), d_se.p, d_fp.p, d_fl.p, d_t.p, trac.p, stream);
    count(1);
    CK(cudaStreamSynchronize(stream));
    trac_dirty = false;
  }

  // the function-defined loads at load factor lambda (re-evaluated only when lambda or the loads changed)
  void refresh_function_loads(double lambda) {
    if (vol_fns.empty() && face_fns.empty()) return;
    if (!ext_dirty && ext.p && lambda == ext_lambda) return;
    ext.alloc(24 * (size_t)ne);
    CK(cudaMemsetAsync(ext.p, 0, sizeof(double) * 24 * (size_t)ne, stream));
    if (!vol_fns.empty()) {
      if (xgp_h.empty()) {
        DBuf<double> d;
        d.alloc(24 * (size_t)ne);
        ikr::launch_gauss_points(X.p, conn.p, ne, d.p, stream);
        count(1);
        xgp_h.resize(24 * (size_t)ne);
        d.download(xgp_h.data(), xgp_h.size(), stream);
        CK(cudaStreamSynchronize(stream));
      }
      std::vector<double> b(24 * (size_t)ne);
      DBuf<double> db;
      for (auto& vf : vol_fns) {
        vf.first(8 * ne, xgp_h.data(), lambda, b.data(), vf.second);
        db.upload(b.data(), b.size(), stream);
        ikr::launch_volume_loads(X.p, conn.p, ne, db.p, ext.p, stream);
        count(1);
        CK(cudaStreamSynchronize(stream));
      }
    }
    for (auto& fs : face_fns) {
      const int nf = (int)fs.face_local.size(), ns = (int)fs.slot_elem.size();
      std::vector<double> t(3 * (size_t)nf);
      fs.f(nf, fs.points.data(), lambda, t.data(), fs.user);
      DBuf<int32_t> d_se, d_fp, d_fl;
      DBuf<double> d_t, vals;
      d_se.upload(fs.slot_elem.data(), ns, stream);
      d_fp.upload(fs.face_ptr.data(), fs.face_ptr.size(), stream);
      d_fl.upload(fs.face_local.data(), nf, stream);
      d_t.upload(t.data(), t.size(), stream);
      vals.alloc(24 * (size_t)ns);
      ikr::launch_traction_loads(X.p, conn.p, ne, ns, d_se.p, d_fp.p, d_fl.p, d_t.p, vals.p, stream);
      ikr::launch_add_slot_loads(d_se.p, ns, vals.p, ext.p, stream);
      count(2);
      CK(cudaStreamSynchronize(stream));
    }
    ext_lambda = lambda;
    ext_dirty = false;
  }

  void check_status() {
    int h = 0;
    CK(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (h) {
      CK(cudaMemsetAsync(status.p, 0, sizeof(int), stream));
      if (h & ikr::kStatusNonPositiveDetC)
        fail(IKR_ERR_NONPOSITIVE_DETC, "Determinant of right Cauchy Green tensor C must be greater than zero");
      if (h & ikr::kStatusSingularD) fail(IKR_ERR_SINGULAR, "EAS matrix D is singular");
      if (h & ikr::kStatusPatternOverflow) fail(IKR_ERR_ARG, "a node couples with more than 128 nodes");
      if (h & ikr::kStatusMaterialDomain)
        fail(IKR_ERR_INVALID_STATE, "The material parameter Jm should be greater than (W1 - 3)");
      fail(IKR_ERR_ARG, "device status %d", h);
    }
  }

  void launch_elements(const ikr::ElemArgs& a, int mode, bool fp32, const int32_t* list, int n, int base) {
    if (na > 0) ikr::launch_eas_element(a, mode, fp32, list, n, base, stream);
    else ikr::launch_disp_element(a, mode, fp32, list, n, base, stream);
    count(1);
  }
  // one launch per colour class: deterministic scatter without atomics
  void launch_coloured(const ikr::ElemArgs& a, int mode, bool fp32) {
    for (size_t c = 0; c + 1 < colour_ptr.size(); ++c) {
      const int n = colour_ptr[c + 1] - colour_ptr[c];
      launch_elements(a, mode, fp32, colour_elems.p + colour_ptr[c], n, 0);
    }
  }
};

struct ikr_req_s {
  ikr_fes fes = nullptr;
  DBuf<double> u;
  double lambda = 0.0;
  uint64_t id = 0;
  uint64_t version = 1;
};

struct ikr_asm_s {
  ikr_fes fes = nullptr;
  int n = 0, nred = 0;
  bool fp32 = false;
  std::vector<uint8_t> fixed_h;
  std::vector<int32_t> cb_h;
  DBuf<uint8_t> node_fixed;
  // inhomogeneous Dirichlet values u_D(lambda) = lambda * idbc_rate on constrained dofs (empty: none); with a value
  // function (idbc_value), u_D(lambda) = idbc_value(X_node, lambda) at every node, evaluated on the host for each new
  // load factor into idbc_vals, and idbc_rate its lambda-derivative at 1 (the IDBC forces)
  DBuf<double> idbc_rate, idbc_force, idbc_vals;
  bool has_idbc = false;
  ikr_point_fn idbc_value = nullptr;
  void* idbc_user = nullptr;
  double idbc_vals_lambda = 0.0;
  bool idbc_vals_valid = false;
  // pattern
  int64_t nb = 0, npad = 0;
  int nslices = 0;
  DBuf<int32_t> ne_ptr, ne_elems;  // elements of every node, ascending (row-tangent kernel)
  // FP32 tangent kernel: 0 = not chosen yet, 1 = coloured element kernel, 2 = row kernel, 3 = element blocks +
  // gather; req = forced choice
  int tan_path = 0, tan_req = 0;
  // element blocks + gather: the FP32 blocks of every element, the inverse element-to-block map, the slice of every
  // block column group
  DBuf<float> eblk;
  DBuf<int32_t> inv_ptr, inv_idx, gslice;
  void build_gather_map() {
    if (inv_idx.p) return;
    ikr_fes f = fes;
    cudaStream_t s = f->stream;
    if (64LL * f->ne * ikr::kElemBlockCount * 2 >= (1LL << 31))
      fail(IKR_ERR_NOT_IMPLEMENTED, "element-block tangent: too many elements for 32-bit block codes");
    DBuf<int32_t> cnt, cursor;
    cnt.alloc(npad);
    cursor.alloc(npad);
    CK(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * npad, s));
    CK(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * npad, s));
    ikr::launch_tangent_inverse_count(slot.p, f->ne, cnt.p, s);
    inv_ptr.alloc(npad + 1);
    ikr::launch_exclusive_scan(cnt.p, inv_ptr.p, (int)npad, s);
    inv_idx.alloc(64LL * f->ne);
    ikr::launch_tangent_inverse_fill(slot.p, f->ne, inv_ptr.p, cursor.p, inv_idx.p, npad, s);
    count(4);
    std::vector<int32_t> gs(npad / 32);
    for (int sl = 0; sl < nslices; ++sl)
      for (int g = slice_off_h[sl]; g < slice_off_h[sl + 1]; ++g) gs[g] = sl;
    gslice.upload(gs.data(), gs.size(), s);
    eblk.alloc((size_t)f->ne * ikr::kElemBlockCount * 9);
    CK(cudaStreamSynchronize(s));
  }
  DBuf<int32_t> row_ptr, col, diag, slot, slice_off, col_sell;
  std::vector<int32_t> row_ptr_h, col_h, slice_off_h;
  DBuf<double> val64;
  DBuf<float> val32;
  int matrix_dbc = -1;  // option of the last assembled matrix
  // FP32 tangent with an FP64 twin: when dual64 is set (a linear solver with the FP64 outer Krylov solve asks for
  // it), the tangent is assembled in FP64 into val64 and val32 is its FP32 rounding.  k_stamp counts matrix
  // assemblies, k64_stamp is the assembly whose FP64 twin val64 holds.
  bool dual64 = false;
  uint64_t k_stamp = 0, k64_stamp = 0;
  // vector
  DBuf<double> R;
  int vector_dbc = -1;
  DBuf<int32_t> pl_dof;
  DBuf<double> pl_val;
  std::map<int32_t, double> pl_h;
  // manipulator matrix entries K(row, col) += value after every matrix assembly: (row, col) -> value, and their
  // value indices in the sliced-ELL storage
  std::map<std::pair<int32_t, int32_t>, double> me_h;
  DBuf<int64_t> me_idx;
  DBuf<double> me_val;
  DBuf<double> norm_part, norm_out;
  ikr_req bound_req = nullptr;
  int bound_dbc = IKR_DBC_FULL;

  ikr::Bsr bsr() const {
    ikr::Bsr b;
    b.n_rows = fes->nn;
    b.n_blocks = nb;
    b.row_ptr = row_ptr.p;
    b.col = col.p;
    b.n_slices = nslices;
    b.n_padded = npad;
    b.slice_off = slice_off.p;
    b.col_sell = col_sell.p;
    b.diag = diag.p;
    b.val = fp32 ? (const void*)val32.p : (const void*)val64.p;
    return b;
  }
  void* values() { return fp32 ? (void*)val32.p : (void*)val64.p; }

  void build_pattern() {
    ikr_fes f = fes;
    cudaStream_t s = f->stream;
    DBuf<int32_t> cnt, cursor, rcnt;
    cnt.alloc(f->nn);
    ne_ptr.alloc(f->nn + 1);
    cursor.alloc(f->nn);
    ne_elems.alloc(8LL * f->ne);
    ikr::launch_node_elem_count(f->conn.p, f->ne, f->nn, cnt.p, s);
    ikr::launch_exclusive_scan(cnt.p, ne_ptr.p, f->nn, s);
    ikr::launch_node_elem_fill(f->conn.p, f->ne, ne_ptr.p, cursor.p, ne_elems.p, f->nn, s);
    rcnt.alloc(f->nn);
    ikr::launch_row_build(f->conn.p, f->ne, f->nn, ne_ptr.p, ne_elems.p, nullptr, rcnt.p, false, f->status.p, s);
    row_ptr.alloc(f->nn + 1);
    ikr::launch_exclusive_scan(rcnt.p, row_ptr.p, f->nn, s);
    count(7);
    int32_t total = 0;
    CK(cudaMemcpyAsync(&total, row_ptr.p + f->nn, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    f->check_status();
    nb = total;
    col.alloc(nb);
    ikr::launch_row_build(f->conn.p, f->ne, f->nn, ne_ptr.p, ne_elems.p, row_ptr.p, col.p, true, f->status.p, s);
    // sliced-ELL storage: widest row of every slice of 32 rows, scanned into block-column offsets
    nslices = (f->nn + 31) / 32;
    DBuf<int32_t> slen;
    slen.alloc(nslices);
    slice_off.alloc(nslices + 1);
    ikr::launch_slice_lengths(row_ptr.p, f->nn, slen.p, s);
    ikr::launch_exclusive_scan(slen.p, slice_off.p, nslices, s);
    int32_t width = 0;
    CK(cudaMemcpyAsync(&width, slice_off.p + nslices, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    npad = 32LL * width;
    col_sell.alloc(npad);
    ikr::launch_sell_fill(row_ptr.p, col.p, slice_off.p, f->nn, col_sell.p, s);
    slot.alloc(64LL * f->ne);
    diag.alloc(f->nn);
    ikr::launch_slot_map(f->conn.p, f->ne, row_ptr.p, col.p, slice_off.p, slot.p, diag.p, f->nn, s);
    count(6);
    row_ptr_h.resize(f->nn + 1);
    col_h.resize(nb);
    slice_off_h.resize(nslices + 1);
    row_ptr.download(row_ptr_h.data(), row_ptr_h.size(), s);
    col.download(col_h.data(), col_h.size(), s);
    slice_off.download(slice_off_h.data(), slice_off_h.size(), s);
    CK(cudaStreamSynchronize(s));
    f->check_status();
    if (fp32) val32.alloc(9 * npad);
    else val64.alloc(9 * npad);
  }
  // block id of CSR entry k (the (k - row_ptr[r])-th block of row r)
  int64_t block_id(int r, int64_t k) const { return (slice_off_h[r >> 5] + (k - row_ptr_h[r])) * 32LL + (r & 31); }
};

namespace ikr_host {
// FP64 outer Krylov solve of an FP32 tangent with an FP64 twin (krylov.cpp): x = K64^{-1} b to ||b - K64 x|| <=
// eta ||b|| by flexible GMRES, right-preconditioned by the FP32 block-Jacobi CG on K32; returns inner CG iterations
int64_t fgmres_solve(ikr_ls ls, ikr_asm a, const double* b, double* x, double eta);
}  // namespace ikr_host

struct ikr_ls_s {
  int tag = IKR_SOLVER_GPU_PCG_BLOCK_JACOBI;
  // what the reference tag runs (include/ikarus_gb300.h): point-Jacobi CG (Eigen's iterative solvers), a
  // direct-accuracy FP64 solve (sparse direct tags), nothing on a sparse tangent (dense tags)
  bool point_jacobi = false, direct = false, dense = false;
  double rtol = 1e-10;
  int max_iter = 100000;
  ikr_asm asm_ = nullptr;
  bool fp32 = false;
  ikr::PcgWork w;
  DBuf<double> dx, dp, dq, dmv, pa, pb, scal;
  DBuf<float> fx, fp, fq, fmv;
  DBuf<double> dz, dr, dp1, dzb, dw0, dw1, pc;  // dzb / fzb, dw / fw: one-reduction CG (second z, w = M^-1 q)
  DBuf<float> fz, fr, fp1, fzb, fw0, fw1;
  double* scal_h = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t tev[2] = {nullptr, nullptr};  // timing events of the SpMV tuner
  // SpMV kernel choice (kernels.h PcgWork::spmv_kind / keep_g): requested kind and L2 keep fraction, -1 =
  // chosen by the tuner at the first factorize on an assembler
  int spmv_req = -1;
  double keep_req = -1.0;
  ikr_asm tuned_for = nullptr;
  double keep_frac = 0.0;
  double tuned_us = 0.0;
  // CG iterations are launched as CUDA graphs of chunk_len iterations.  In profiling mode two graphs
  // alternate, each with its own event-record nodes around every SpMV, so the SpMV device time of the
  // chunk that just finished can be read while the next one runs.
  // Without graphs (use_graphs = false) the same kernels are launched one by one, which profilers that
  // cannot follow kernels inside graphs need.
  cudaGraphExec_t chunk[2] = {nullptr, nullptr};
  int chunk_len = 16;
  bool use_graphs = true;
  bool profile = false;
  std::vector<cudaEvent_t> pev[2];
  double prof_ms = 0.0;
  int64_t prof_n = 0;
  int last_iters = 0;
  double last_rel = 0.0;
  bool factorized = false;
  DBuf<double> b64, x64, r64, c64;  // refinement work
  // second right-hand side of solve2 (its own CG vectors and scalars; matrix, preconditioner, grid and L2
  // policy are w's) and the partials of the two-RHS persistent kernel (4 and 8 per CTA)
  bool multi_rhs = true;
  ikr::PcgWork w2;
  // Coarse correction of the CG (coarse.cu), off by default: coarse_req > 0 slab aggregates of equal node
  // count along the mesh's longest extent, six rigid-body modes each; rebuilt (A_c and its inverse) at every
  // factorize.  Two-kernel CG forms only (the tuner then skips the persistent ones).
  int coarse_req = 0;
  // A_c is rebuilt at every coarse_refresh-th factorize (1: every one); an older A_c = P^T K_old P is still SPD,
  // so the CG stays exact with it and only its iteration count can grow
  int coarse_refresh = 1;
  struct CoarseSet {
    int since_rebuild = 0;  // factorizations that reused the current A_c
    ikr_asm built_for = nullptr;
    int n_slabs = 0, reach = 0, n_colours = 0, dropped = 0;
    ikr::Coarse C;
    DBuf<float> y4;
    DBuf<int32_t> nodes, chunk_off, agg_chunk, agg_colour;
    std::vector<int32_t> agg_chunk_h;
    DBuf<double> rpart, gpart, V, W, ainv64, e64, cpart;
    DBuf<float> ainv32, e32;
    std::vector<double> gpart_h, ac, inv, fac;
    std::vector<float> inv32;
  } co;
  DBuf<double> dx2, dr2, dz2, dp2, dp12, pa2, pb2, pbi2, scal2;
  DBuf<float> fx2, fr2, fz2, fp2, fp12;
  // FP64 outer Krylov solve (krylov.cpp), off while outer_m = 0: restart length, tolerance and iteration cap of
  // the inner FP32 CG, cap on outer iterations; Arnoldi basis V, directions Z and small device work
  int outer_m = 0;
  double inner_rtol = 1e-2;
  int inner_max_iter = 2000;
  int outer_max_iter = 2000;
  int last_outer = 0, last_cycles = 0;
  DBuf<double> gm_V, gm_Z, gm_w, gm_r, gm_h, gm_part, gm_c, gm_npart, gm_nout;

  ~ikr_ls_s() {
    drop_graphs();
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : tev)
      if (e) cudaEventDestroy(e);
    for (auto& v : pev)
      for (auto e : v) cudaEventDestroy(e);
    if (scal_h) cudaFreeHost(scal_h);
  }

  void drop_graphs() {
    for (auto& g : chunk)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }

  void set_profile(bool on) {
    if (on != profile) drop_graphs();
    profile = on;
    prof_ms = 0.0;
    prof_n = 0;
  }

  void setup(ikr_asm a) {
    a->dual64 = outer_m > 0 && a->fp32;  // the FP64 outer solve needs the FP64 twin of every later assembly
    if (asm_ == a && w.n_rows == a->fes->nn && fp32 == a->fp32 && w.grid) return;
    drop_graphs();
    asm_ = a;
    fp32 = a->fp32;
    const int nr = a->fes->nn;
    const size_t n = 4 * (size_t)nr;  // CG vectors are node-padded (x, y, z, 0)
    w = ikr::PcgWork{};
    w.n_rows = nr;
    w.fp32 = fp32;
    w.sms = num_sms();
    w.grid = 4 * w.sms;
    tuned_for = nullptr;
    if (fp32) {
      fx.alloc(n), fr.alloc(n), fz.alloc(n), fp.alloc(n), fp1.alloc(n), fq.alloc(n), fmv.alloc(9 * (size_t)nr);
      fzb.alloc(n), fw0.alloc(n), fw1.alloc(n);
      w.x = fx.p, w.r = fr.p, w.z = fz.p, w.p0 = fp.p, w.p1 = fp1.p, w.q = fq.p, w.minv = fmv.p;
      w.z2 = fzb.p, w.w0 = fw0.p, w.w1 = fw1.p;
    } else {
      dx.alloc(n), dr.alloc(n), dz.alloc(n), dp.alloc(n), dp1.alloc(n), dq.alloc(n), dmv.alloc(9 * (size_t)nr);
      dzb.alloc(n), dw0.alloc(n), dw1.alloc(n);
      w.x = dx.p, w.r = dr.p, w.z = dz.p, w.p0 = dp.p, w.p1 = dp1.p, w.q = dq.p, w.minv = dmv.p;
      w.z2 = dzb.p, w.w0 = dw0.p, w.w1 = dw1.p;
    }
    pc.alloc(16 * (size_t)w.grid);
    w.part_c = pc.p;
    pa.alloc(2 * (size_t)w.grid);  // two-kernel CG: 1 per block; persistent CG: 2 per CTA (parity)
    pb.alloc(4 * (size_t)w.grid);  // two-kernel CG: 2 per block; persistent CG: 4 per CTA
    scal.alloc(ikr::kNScal);
    w.part_a = pa.p;
    w.part_b = pb.p;
    w.scal = scal.p;
    if (!scal_h) CK(cudaMallocHost(&scal_h, sizeof(double) * 2 * ikr::kNScal));
    for (auto& e : ev)
      if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto& e : tev)
      if (!e) CK(cudaEventCreate(&e));
    b64.alloc(3 * (size_t)nr), x64.alloc(3 * (size_t)nr), r64.alloc(3 * (size_t)nr), c64.alloc(3 * (size_t)nr);
  }

  void set_launch(bool graphs, int len) {
    if (graphs != use_graphs || len != chunk_len) drop_graphs();
    if (len != chunk_len)
      for (auto& v : pev) {
        for (auto e : v) cudaEventDestroy(e);
        v.clear();
      }
    use_graphs = graphs;
    chunk_len = len;
  }

  // the kernels of one chunk; with profiling, cudaEventRecordExternal makes the records event-record nodes
  // when captured (a plain record during capture would only become an internal dependency)
  void issue_chunk(int gi, cudaStream_t s) {
    const ikr::Bsr A = asm_->bsr();
    const unsigned flags = use_graphs ? cudaEventRecordExternal : cudaEventRecordDefault;
    for (int k = 0; k < chunk_len; ++k) {
      if (profile) CK(cudaEventRecordWithFlags(pev[gi][2 * k], s, flags));
      ikr::launch_pcg_spmv(A, w, k & 1, s);
      if (profile) CK(cudaEventRecordWithFlags(pev[gi][2 * k + 1], s, flags));
      ikr::launch_pcg_update(A, w, k & 1, s);
      if (w.coarse) ikr::launch_coarse_correction(co.C, w, false, s);
    }
  }

  void build_chunk(cudaStream_t s) {
    const int ng = profile ? 2 : 1;
    for (int gi = 0; gi < ng; ++gi) {
      if (profile && pev[gi].empty()) {
        pev[gi].resize(2 * chunk_len);
        for (auto& e : pev[gi]) CK(cudaEventCreate(&e));
      }
      if (!use_graphs || chunk[gi]) continue;
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      issue_chunk(gi, s);
      CK(cudaStreamEndCapture(s, &g));
      CK(cudaGraphInstantiate(&chunk[gi], g, 0));
      cudaGraphDestroy(g);
    }
  }
  void launch_chunk(int gi, cudaStream_t s) {
    if (use_graphs) CK(cudaGraphLaunch(chunk[gi], s));
    else issue_chunk(gi, s);
    count((w.coarse ? 4 : 2) * chunk_len);
  }
  // SpMV device time of the first `working` iterations of a finished profiled chunk
  void read_profile(int gi, int working) {
    for (int k = 0; k < working && k < chunk_len; ++k) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, pev[gi][2 * k], pev[gi][2 * k + 1]));
      prof_ms += ms;
      ++prof_n;
    }
  }

  void factorize(ikr_asm a) {
    if (tag == IKR_SOLVER_NONE) fail(IKR_ERR_INVALID_STATE, "SolverTypeTag::none has no linear solver");
    if (dense) fail(IKR_ERR_NOT_IMPLEMENTED, "This solver does not support solving with sparse matrices.");
    if (direct && a->fp32 && outer_m == 0)
      fail(IKR_ERR_NOT_IMPLEMENTED, "a direct-accuracy solve of an FP32 tangent needs the FP64 outer solve");
    setup(a);
    ikr::launch_block_jacobi(a->bsr(), fp32, w.minv, point_jacobi, a->fes->stream);
    count(1);
    factorized = true;
    w.coarse = 0;
    if (coarse_req > 0) coarse_operator(a);  // before the tuner: the fused kinds are timed with it
    if (tag != IKR_SOLVER_GPU_PCG_BATCHED && tuned_for != a) tune(a);
    if (coarse_req > 0) {
      if (persistent())
        fail(IKR_ERR_ARG, "the coarse correction runs with the two-kernel CG kinds or the fused coarse kinds only");
      w.coarse = 1;
    } else if (coarse_fused()) {
      fail(IKR_ERR_ARG, "the fused coarse CG kinds need a coarse space (set_coarse_space)");
    }
  }

  // ---- coarse correction: aggregates, A_c = P^T K P and its inverse (coarse.cu has the device side) ----

  // slab aggregates and the per-node mode data, once per assembler and slab count
  void coarse_layout(ikr_asm a) {
    ikr_fes f = a->fes;
    if (f->n_inst != 0) fail(IKR_ERR_NOT_IMPLEMENTED, "coarse correction of element sets with independent instances");
    if (a->matrix_dbc != IKR_DBC_FULL) fail(IKR_ERR_NOT_IMPLEMENTED, "coarse correction needs a Full-DBC tangent");
    drop_graphs();
    cudaStream_t s = f->stream;
    const int nn = f->nn;
    const int S = std::min(coarse_req, nn);
    std::vector<double> X(3 * (size_t)nn);
    f->X.download(X.data(), X.size(), s);
    CK(cudaStreamSynchronize(s));
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < nn; ++i)
      for (int c = 0; c < 3; ++c) lo[c] = std::min(lo[c], X[3 * i + c]), hi[c] = std::max(hi[c], X[3 * i + c]);
    int ax = 0;
    for (int c = 1; c < 3; ++c)
      if (hi[c] - lo[c] > hi[ax] - lo[ax]) ax = c;
    // nodes in order of their coordinate along the longest axis, cut into S runs of equal count; each run
    // sorted by node id (monotone gathers)
    std::vector<int32_t> order(nn);
    for (int i = 0; i < nn; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int32_t i, int32_t j) { return X[3 * i + ax] < X[3 * j + ax]; });
    std::vector<int32_t> agg(nn), agg_off(S + 1);
    for (int k = 0; k <= S; ++k) agg_off[k] = (int32_t)((int64_t)k * nn / S);
    for (int a_ = 0; a_ < S; ++a_) {
      std::sort(order.begin() + agg_off[a_], order.begin() + agg_off[a_ + 1]);
      for (int k = agg_off[a_]; k < agg_off[a_ + 1]; ++k) agg[order[k]] = a_;
    }
    // centroids, offsets, free-dof masks
    std::vector<double> cen(3 * (size_t)S, 0.0);
    for (int i = 0; i < nn; ++i)
      for (int c = 0; c < 3; ++c) cen[3 * agg[i] + c] += X[3 * i + c];
    for (int a_ = 0; a_ < S; ++a_)
      for (int c = 0; c < 3; ++c) cen[3 * a_ + c] /= (double)(agg_off[a_ + 1] - agg_off[a_]);
    std::vector<float> y4(4 * (size_t)nn);
    for (int i = 0; i < nn; ++i) {
      int mask = 0;
      for (int c = 0; c < 3; ++c) {
        y4[4 * i + c] = (float)(X[3 * i + c] - cen[3 * agg[i] + c]);
        if (!a->fixed_h[3 * (size_t)i + c]) mask |= 1 << c;
      }
      const int32_t bits = agg[i] | (mask << 24);
      std::memcpy(&y4[4 * i + 3], &bits, sizeof(bits));
    }
    // reach: the largest aggregate distance of two coupled nodes; colours of a distance-2 colouring of the
    // aggregate chain (any 2 reach + 1 consecutive aggregates differ)
    int reach = 0;
    for (int i = 0; i < nn; ++i)
      for (int k = a->row_ptr_h[i]; k < a->row_ptr_h[i + 1]; ++k) reach = std::max(reach, std::abs(agg[i] - agg[a->col_h[k]]));
    if (reach > 3)
      fail(IKR_ERR_ARG, "coarse correction: slabs thinner than the elements couple %d slabs apart; use fewer slabs",
           reach);
    const int ncol = std::min(2 * reach + 1, S);
    std::vector<int32_t> colour(S);
    for (int a_ = 0; a_ < S; ++a_) colour[a_] = a_ % ncol;
    // chunks of at most 2048 nodes per aggregate: one 1024-thread CTA of the restrict kernel each, one CTA per SM
    // (its registers), so about as many chunks as SMs keep the launch in one wave
    constexpr int kChunk = 2048;
    std::vector<int32_t> chunk_off{0};
    co.agg_chunk_h.assign(1, 0);
    for (int a_ = 0; a_ < S; ++a_) {
      for (int k = agg_off[a_]; k < agg_off[a_ + 1]; k += kChunk) chunk_off.push_back(std::min(k + kChunk, agg_off[a_ + 1]));
      co.agg_chunk_h.push_back((int32_t)chunk_off.size() - 1);
    }
    const int nchunks = (int)chunk_off.size() - 1;
    co.y4.upload(y4.data(), y4.size(), s);
    co.nodes.upload(order.data(), order.size(), s);
    co.chunk_off.upload(chunk_off.data(), chunk_off.size(), s);
    co.agg_chunk.upload(co.agg_chunk_h.data(), co.agg_chunk_h.size(), s);
    co.agg_colour.upload(colour.data(), colour.size(), s);
    co.rpart.alloc(6 * (size_t)nchunks);
    const size_t nc = 6 * (size_t)S;
    if (fp32) co.ainv32.alloc(nc * nc), co.e32.alloc(nc);
    else co.ainv64.alloc(nc * nc), co.e64.alloc(nc);
    ikr::Coarse& C = co.C;
    C.n_rows = nn, C.n_agg = S, C.n_c = (int)nc, C.n_chunks = nchunks;
    C.y4 = reinterpret_cast<const float4*>(co.y4.p);
    C.nodes = co.nodes.p, C.chunk_off = co.chunk_off.p, C.agg_chunk = co.agg_chunk.p, C.agg_colour = co.agg_colour.p;
    C.rpart = co.rpart.p;
    C.ainv = fp32 ? (const void*)co.ainv32.p : (const void*)co.ainv64.p;
    C.e = fp32 ? (void*)co.e32.p : (void*)co.e64.p;
    CK(cudaStreamSynchronize(s));  // host vectors above go out of scope
    co.built_for = a, co.n_slabs = S, co.reach = reach, co.n_colours = ncol;
  }

  // A_c = P^T K P from probe products (one SpMV per colour and mode), then its inverse
  void coarse_operator(ikr_asm a) {
    if (co.built_for != a || co.n_slabs != std::min(coarse_req, a->fes->nn) ||
        (fp32 ? (const void*)co.ainv32.p : (const void*)co.ainv64.p) != co.C.ainv) {
      coarse_layout(a);
      co.since_rebuild = 0;
    } else if (co.since_rebuild + 1 < coarse_refresh) {
      ++co.since_rebuild;  // keep A_c of an earlier tangent of this assembler
      return;
    }
    co.since_rebuild = 0;
    cudaStream_t s = a->fes->stream;
    const ikr::Bsr A = a->bsr();
    const int S = co.n_slabs, nc = 6 * S, nch = co.C.n_chunks, ncol = co.n_colours;
    co.cpart.alloc(2 * (size_t)(nc + 2) * w.grid);  // partials of the fused coarse CG (parity, CTA, coarse dof)
    w.coarse_part = co.cpart.p;
    w.coarse_part_ctas = w.grid;
    const int64_t n3 = 3LL * a->fes->nn;
    co.V.alloc(6 * (size_t)n3), co.W.alloc(6 * (size_t)n3);
    co.gpart.alloc(36 * (size_t)nch * ncol);
    for (int c = 0; c < ncol; ++c) {
      ikr::launch_coarse_probe(co.C, c, co.V.p, s);
      for (int m = 0; m < 6; ++m) ikr::launch_spmv64(A, fp32, co.V.p + m * n3, co.W.p + m * n3, s);
      ikr::launch_coarse_galerkin(co.C, co.W.p, co.gpart.p + 36LL * nch * c, s);
      count(8);
    }
    co.gpart_h.resize(co.gpart.n);
    co.gpart.download(co.gpart_h.data(), co.gpart.n, s);
    CK(cudaStreamSynchronize(s));
    // the blocks: row aggregate b, column aggregate = the one aggregate of colour c within reach of b
    co.ac.assign((size_t)nc * nc, 0.0);
    for (int c = 0; c < ncol; ++c)
      for (int b = 0; b < S; ++b) {
        int col_agg = -1;
        for (int d = -co.reach; d <= co.reach; ++d)
          if (b + d >= 0 && b + d < S && (b + d) % ncol == c) col_agg = b + d;
        if (col_agg < 0) continue;
        double blk[36] = {};
        for (int k = co.agg_chunk_h[b]; k < co.agg_chunk_h[b + 1]; ++k)
          for (int q = 0; q < 36; ++q) blk[q] += co.gpart_h[36 * ((size_t)nch * c + k) + q];
        for (int r = 0; r < 6; ++r)
          for (int m = 0; m < 6; ++m) co.ac[(size_t)(6 * b + r) * nc + 6 * col_agg + m] = blk[6 * r + m];
      }
    for (int i = 0; i < nc; ++i)
      for (int j = 0; j < i; ++j) {
        const double v = 0.5 * (co.ac[(size_t)i * nc + j] + co.ac[(size_t)j * nc + i]);
        co.ac[(size_t)i * nc + j] = co.ac[(size_t)j * nc + i] = v;
      }
    co.dropped = band_spd_inverse(co.ac, nc, 6 * (co.reach + 1) - 1, co.fac, co.inv);
    if (fp32) {
      co.inv32.assign(co.inv.begin(), co.inv.end());
      co.ainv32.upload(co.inv32.data(), co.inv32.size(), s);
    } else {
      co.ainv64.upload(co.inv.data(), co.inv.size(), s);
    }
    CK(cudaStreamSynchronize(s));
  }

  // Inverse of the symmetric matrix A (n x n, zero outside half bandwidth bw) by a band Cholesky factorisation
  // A = L L^T.  A pivot at or below 1e-9 of its diagonal entry marks a mode that depends on the earlier ones (or
  // has no free dof): its column of L is the unit vector and its row and column of the inverse are zero, so the
  // returned matrix is symmetric positive semi-definite.  Returns the number of such modes.
  static int band_spd_inverse(const std::vector<double>& A, int n, int bw, std::vector<double>& L,
                              std::vector<double>& inv) {
    L.assign((size_t)n * n, 0.0);
    std::vector<char> drop(n, 0);
    int dropped = 0;
    for (int j = 0; j < n; ++j) {
      const int k0 = std::max(0, j - bw);
      double d = A[(size_t)j * n + j];
      for (int k = k0; k < j; ++k) d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
      if (!(A[(size_t)j * n + j] > 0.0) || !(d > 1e-9 * A[(size_t)j * n + j])) {
        drop[j] = 1, ++dropped;
        for (int k = k0; k < j; ++k) L[(size_t)j * n + k] = 0.0;  // the mode leaves the factorisation
        L[(size_t)j * n + j] = 1.0;
        continue;
      }
      const double ljj = std::sqrt(d);
      L[(size_t)j * n + j] = ljj;
      for (int i = j + 1; i <= std::min(n - 1, j + bw); ++i) {
        double v = A[(size_t)i * n + j];
        for (int k = std::max(0, i - bw); k < j; ++k) v -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
        L[(size_t)i * n + j] = v / ljj;
      }
    }
    inv.assign((size_t)n * n, 0.0);
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i) {
      if (drop[i]) continue;
      // L y = e_i (y_k = 0 for k < i), then L^T x = y
      for (int k = 0; k < n; ++k) y[k] = 0.0;
      for (int k = i; k < n; ++k) {
        double v = (k == i) ? 1.0 : 0.0;
        for (int l = std::max(i, k - bw); l < k; ++l) v -= L[(size_t)k * n + l] * y[l];
        y[k] = v / L[(size_t)k * n + k];
      }
      for (int k = n - 1; k >= 0; --k) {
        double v = y[k];
        for (int l = k + 1; l <= std::min(n - 1, k + bw); ++l) v -= L[(size_t)l * n + k] * y[l];
        y[k] = v / L[(size_t)k * n + k];
      }
      for (int k = 0; k < n; ++k) inv[(size_t)k * n + i] = drop[k] ? 0.0 : y[k];
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) {
        const double v = 0.5 * (inv[(size_t)i * n + j] + inv[(size_t)j * n + i]);
        inv[(size_t)i * n + j] = inv[(size_t)j * n + i] = v;
      }
    return dropped;
  }

  void set_kernel(int kind, double keep) {
    spmv_req = kind;
    keep_req = keep;
    tuned_for = nullptr;
    drop_graphs();
  }

  // SpMV kernel and L2 keep fraction: the requested ones, or the fastest of timed CG iterations (right-hand
  // side of ones, tolerance 0) on the assembled tangent.  The kinds are timed with an L2 keep share of 0.45, then
  // the keep fractions in increasing order with the fastest kind.
  void tune(ikr_asm a) {
    drop_graphs();
    w.coarse = 0;  // kinds are timed as plain block-Jacobi iterations
    const ikr::Bsr A = a->bsr();
    const int64_t total_g = A.n_padded / 32;
    auto apply = [&](int kind, double keep) {
      w.spmv_kind = kind;
      keep_frac = kind > 0 ? keep : 0.0;
      w.keep_g = (int64_t)(keep_frac * (double)total_g);
    };
    tuned_for = a;
    tuned_us = 0.0;
    if (spmv_req >= 0 && keep_req >= 0.0) {
      apply(spmv_req, keep_req);
      return;
    }
    cudaStream_t s = a->fes->stream;
    ikr::launch_fill64(b64.p, 1.0, 3LL * A.n_rows, s);
    ikr::launch_pcg_init(A, w, b64.p, 0.0, 1 << 30, s);
    count(3);
    int parity = 0;
    // each candidate: the least of 3 timed runs (the kinds differ by a few per cent)
    auto time_it = [&](int kind, double keep) {
      apply(kind, keep);
      constexpr int kWarm = 2, kTimed = 16;
      double best_us = 1e300;
      for (int rep = 0; rep < 3; ++rep) {
        for (int i = 0; i < kWarm; ++i, parity ^= 1)
          ikr::launch_pcg_spmv(A, w, parity, s), ikr::launch_pcg_update(A, w, parity, s);
        CK(cudaEventRecord(tev[0], s));
        for (int i = 0; i < kTimed; ++i, parity ^= 1)
          ikr::launch_pcg_spmv(A, w, parity, s), ikr::launch_pcg_update(A, w, parity, s);
        CK(cudaEventRecord(tev[1], s));
        CK(cudaEventSynchronize(tev[1]));
        count(2 * (kWarm + kTimed));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, tev[0], tev[1]));
        best_us = std::min(best_us, 1e3 * ms / kTimed);
      }
      return best_us;
    };
    // persistent kinds: a solve of kTimed iterations after one untimed solve, per iteration (long enough that the
    // launch overhead and run-to-run noise stay below the few per cent that separate the variants)
    auto time_persistent = [&](int kind, double keep) {
      apply(kind, keep);
      constexpr int kTimed = 160;
      double us = 1e300;
      for (int rep = 0; rep < 4; ++rep) {  // the first run warms up; the least of the other three counts
        ikr::launch_pcg_init(A, w, b64.p, 0.0, kTimed, s);
        CK(cudaEventRecord(tev[0], s));
        CK(ikr::launch_pcg_persistent(A, w, kind - first_persistent_kind(), s));
        CK(cudaEventRecord(tev[1], s));
        CK(cudaEventSynchronize(tev[1]));
        count(3);
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, tev[0], tev[1]));
        if (rep > 0) us = std::min(us, 1e3 * ms / kTimed);
      }
      return us;
    };
    // fused coarse kinds: as the persistent kinds, with the coarse part (init leaves r.D^-1 r for it)
    auto time_coarse = [&](int kind, double keep) {
      apply(kind, keep);
      constexpr int kTimed = 160;
      double us = 1e300;
      w.coarse = 1;
      for (int rep = 0; rep < 4; ++rep) {
        ikr::launch_pcg_init(A, w, b64.p, 0.0, kTimed, s);
        CK(cudaEventRecord(tev[0], s));
        CK(ikr::launch_pcg_coarse(A, w, co.C, kind - first_coarse_kind(), s));
        CK(cudaEventRecord(tev[1], s));
        CK(cudaEventSynchronize(tev[1]));
        count(3);
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, tev[0], tev[1]));
        if (rep > 0) us = std::min(us, 1e3 * ms / kTimed);
      }
      w.coarse = 0;
      return us;
    };
    auto time_kind = [&](int kind, double keep) {
      if (kind >= first_coarse_kind()) return time_coarse(kind, keep);
      return kind >= first_persistent_kind() ? time_persistent(kind, keep) : time_it(kind, keep);
    };
    int best_kind = spmv_req >= 0 ? spmv_req : 0;
    double best = 1e300;
    if (spmv_req < 0) {
      // the kinds are compared with a mid L2 keep share (the share changes their ranking), kind 0 has none
      constexpr double kProbeKeep = 0.45;
      for (int k = 0; k <= ikr::spmv_staged_variants(); ++k) {
        const double us = time_it(k, k > 0 ? kProbeKeep : 0.0);
        if (us < best) best = us, best_kind = k;
      }
      for (int v = 0; v < ikr::pcg_persistent_variants() && coarse_req == 0; ++v) {
        if (!ikr::pcg_persistent_eligible(A, w, v)) continue;
        const double us = time_persistent(first_persistent_kind() + v, kProbeKeep);
        if (us < best) best = us, best_kind = first_persistent_kind() + v;
      }
      // with a coarse space the fused kinds are preferred whenever one fits: they replace the two-kernel form's
      // two extra kernels per iteration (its timed iterations above exclude the coarse part)
      if (coarse_req > 0) {
        double best_c = 1e300;
        for (int v = 0; v < ikr::pcg_coarse_variants(); ++v) {
          if (!ikr::pcg_coarse_eligible(A, w, co.C, v)) continue;
          const double us = time_coarse(first_coarse_kind() + v, kProbeKeep);
          if (us < best_c) best_c = us, best_kind = first_coarse_kind() + v;
        }
        if (best_c < 1e300) best = best_c;
      }
      // the two-kernel CG state was advanced by the persistent trials' inits: restart it for the keep trials
      ikr::launch_pcg_init(A, w, b64.p, 0.0, 1 << 30, s);
      count(2);
    } else if (best_kind >= first_coarse_kind()) {
      if (coarse_req <= 0) fail(IKR_ERR_ARG, "the fused coarse CG kinds need a coarse space (set_coarse_space)");
      if (!ikr::pcg_coarse_eligible(A, w, co.C, best_kind - first_coarse_kind()))
        fail(IKR_ERR_ARG, "the fused coarse CG variant does not fit this system");
    } else if (best_kind >= first_persistent_kind() && coarse_req > 0) {
      fail(IKR_ERR_ARG, "the coarse correction runs with the two-kernel CG kinds (0 .. %d) or the fused coarse kinds",
           first_persistent_kind() - 1);
    } else if (best_kind >= first_persistent_kind() && !ikr::pcg_persistent_eligible(A, w, best_kind - first_persistent_kind())) {
      fail(IKR_ERR_ARG, "the persistent CG variant does not fit this system (too many slices per warp)");
    }
    double best_keep = keep_req >= 0.0 ? keep_req : 0.0;
    if (keep_req < 0.0 && best_kind > 0) {
      best = time_kind(best_kind, 0.0);
      for (double f : {0.3, 0.45, 0.6, 0.75}) {
        const double us = time_kind(best_kind, f);
        if (us < best) best = us, best_keep = f;
      }
    } else if (best >= 1e300) {
      best = time_kind(best_kind, best_keep);
    }
    apply(best_kind, best_keep);
    tuned_us = best;
    double* sc = scal_h;
    CK(cudaMemcpyAsync(sc, scal.p, sizeof(double) * ikr::kNScal, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (sc[ikr::kDone] == 6.0) fail(IKR_ERR_TIMEOUT, "a bounded wait in the staged SpMV gave up while tuning");
  }

  static int first_persistent_kind() { return 1 + ikr::spmv_staged_variants(); }
  static int first_coarse_kind() { return first_persistent_kind() + ikr::pcg_persistent_variants(); }
  bool persistent() const { return w.spmv_kind >= first_persistent_kind() && w.spmv_kind < first_coarse_kind(); }
  bool coarse_fused() const { return w.spmv_kind >= first_coarse_kind(); }

  // the whole CG with the coarse correction in one cooperative launch: init, fused kernel, one read of the scalars
  int solve_coarse_fused(ikr_asm a, const double* b, double* x, double rt, int maxit) {
    cudaStream_t s = a->fes->stream;
    const ikr::Bsr A = a->bsr();
    ikr::launch_pcg_init(A, w, b, rt, maxit, s);
    count(2);
    if (profile) CK(cudaEventRecord(tev[0], s));
    CK(ikr::launch_pcg_coarse(A, w, co.C, w.spmv_kind - first_coarse_kind(), s));
    count(1);
    if (profile) CK(cudaEventRecord(tev[1], s));
    CK(cudaMemcpyAsync(scal_h, scal.p, sizeof(double) * ikr::kNScal, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const double done = scal_h[ikr::kDone];
    last_iters = (int)scal_h[ikr::kIters];
    last_rel = scal_h[ikr::kBB] > 0 ? std::sqrt(scal_h[ikr::kRR] / scal_h[ikr::kBB]) : 0.0;
    if (profile) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, tev[0], tev[1]));
      prof_ms += ms;
      prof_n += last_iters;
    }
    ikr::launch_pcg_result(w, x, 1.0, s);
    count(1);
    if (done == 6.0) fail(IKR_ERR_TIMEOUT, "a bounded wait in the fused coarse CG gave up");
    if (done == 3.0) fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp zero or not finite) after %d iterations", last_iters);
    return last_iters;
  }

  // the whole CG in one cooperative launch: init, persistent kernel, one read of the scalars
  int solve_persistent(ikr_asm a, const double* b, double* x, double rt, int maxit) {
    cudaStream_t s = a->fes->stream;
    const ikr::Bsr A = a->bsr();
    ikr::launch_pcg_init(A, w, b, rt, maxit, s);
    count(2);
    if (profile) CK(cudaEventRecord(tev[0], s));
    CK(ikr::launch_pcg_persistent(A, w, w.spmv_kind - first_persistent_kind(), s));
    count(1);
    w.withhold_first_arrival = 0;  // the test switch acts on one launch
    if (profile) CK(cudaEventRecord(tev[1], s));
    CK(cudaMemcpyAsync(scal_h, scal.p, sizeof(double) * ikr::kNScal, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const double done = scal_h[ikr::kDone];
    last_iters = (int)scal_h[ikr::kIters];
    last_rel = scal_h[ikr::kBB] > 0 ? std::sqrt(scal_h[ikr::kRR] / scal_h[ikr::kBB]) : 0.0;
    if (profile) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, tev[0], tev[1]));
      prof_ms += ms;
      prof_n += last_iters;
    }
    ikr::launch_pcg_result(w, x, 1.0, s);
    count(1);
    if (done == 6.0) fail(IKR_ERR_TIMEOUT, "a bounded wait in the persistent CG gave up");
    if (done == 3.0) fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp zero or not finite) after %d iterations", last_iters);
    return last_iters;
  }

  // x = K^{-1} b on the device (FP64 in / out); returns CG iterations
  int solve_device(ikr_asm a, const double* b, double* x, double rt, int maxit) {
    if (!factorized || asm_ != a) fail(IKR_ERR_INVALID_STATE, "linear solver not factorized for this assembler");
    if (persistent()) return solve_persistent(a, b, x, rt, maxit);
    if (coarse_fused()) return solve_coarse_fused(a, b, x, rt, maxit);
    cudaStream_t s = a->fes->stream;
    const ikr::Bsr A = a->bsr();
    build_chunk(s);
    ikr::launch_pcg_init(A, w, b, rt, maxit, s);
    count(2);
    if (w.coarse) {
      ikr::launch_coarse_correction(co.C, w, true, s);
      count(2);
    }
    // Chunks of CG iterations are launched one ahead of the host check: once the device flags
    // convergence the chunk in flight returns at entry, so polling never stalls the GPU.
    constexpr int NS = ikr::kNScal;
    auto gi = [&](int k) { return profile ? (k & 1) : 0; };
    auto iters_in = [&](int slot) { return (int)scal_h[NS * slot + ikr::kIters]; };
    int k = 0, prev_iters = 0;
    launch_chunk(gi(0), s);
    CK(cudaMemcpyAsync(scal_h, scal.p, sizeof(double) * NS, cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(ev[0], s));
    for (;;) {
      ++k;
      launch_chunk(gi(k), s);
      CK(cudaMemcpyAsync(scal_h + NS * (k & 1), scal.p, sizeof(double) * NS, cudaMemcpyDeviceToHost, s));
      CK(cudaEventRecord(ev[k & 1], s));
      CK(cudaEventSynchronize(ev[(k - 1) & 1]));
      if (profile) {
        const int it = iters_in((k - 1) & 1);
        read_profile((k - 1) & 1, it - prev_iters);
        prev_iters = it;
      }
      if (scal_h[NS * ((k - 1) & 1) + ikr::kDone] != 0.0) break;
    }
    CK(cudaStreamSynchronize(s));
    const double* sc = scal_h + NS * (k & 1);  // state after the last (no-op) chunk
    const double done = sc[ikr::kDone];
    last_iters = (int)sc[ikr::kIters];
    last_rel = sc[ikr::kBB] > 0 ? std::sqrt(sc[ikr::kRR] / sc[ikr::kBB]) : 0.0;
    ikr::launch_pcg_result(w, x, 1.0, s);
    count(1);
    if (done == 6.0) fail(IKR_ERR_TIMEOUT, "a bounded wait in the staged SpMV gave up");
    if (done == 3.0) fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp zero or not finite) after %d iterations", last_iters);
    return last_iters;
  }

  // the second right-hand side's work (same sizes as w)
  void setup2() {
    if (w2.scal && w2.n_rows == w.n_rows && w2.fp32 == w.fp32 && w2.grid == w.grid) return;
    w2 = w;
    const size_t n = 4 * (size_t)w.n_rows;
    if (fp32) {
      fx2.alloc(n), fr2.alloc(n), fz2.alloc(n), fp2.alloc(n), fp12.alloc(n);
      w2.x = fx2.p, w2.r = fr2.p, w2.z = fz2.p, w2.p0 = fp2.p, w2.p1 = fp12.p;
    } else {
      dx2.alloc(n), dr2.alloc(n), dz2.alloc(n), dp2.alloc(n), dp12.alloc(n);
      w2.x = dx2.p, w2.r = dr2.p, w2.z = dz2.p, w2.p0 = dp2.p, w2.p1 = dp12.p;
    }
    w2.q = nullptr;
    pbi2.alloc(4 * (size_t)w.grid);
    scal2.alloc(ikr::kNScal);
    w2.part_a = nullptr;
    w2.part_b = pbi2.p;  // written by the init kernel only
    w2.scal = scal2.p;
    pa2.alloc(4 * (size_t)w.grid);
    pb2.alloc(8 * (size_t)w.grid);
  }

  // x0 = K^{-1} b0 and x1 = K^{-1} b1 with the same tangent.  With a persistent CG kind both run in one
  // cooperative launch that streams the matrix once per iteration for the two; otherwise (or with refinement
  // sweeps, or when disabled) one solve after the other.  Returns the CG iterations of both right-hand sides.
  int64_t solve2(ikr_asm a, const double* b0, const double* b1, double* x0, double* x1, double rt, int maxit,
                 int refinements, double rt1 = -1.0) {
    if (rt1 < 0.0) rt1 = rt;
    if (direct) rt = std::min(rt, rtol), rt1 = std::min(rt1, rtol);
    if (!factorized || asm_ != a) fail(IKR_ERR_INVALID_STATE, "linear solver not factorized for this assembler");
    const ikr::Bsr A = a->bsr();
    // FP64 CG iterations are bound by GB300's FP64 pipe, not by the matrix stream: two right-hand sides cost
    // twice the time in one launch as well, so only the FP32 tangent runs them together (and only without the
    // FP64 outer solve, whose operator is the FP64 tangent)
    bool two = multi_rhs && fp32 && persistent() && refinements <= 0 && outer_m == 0;
    if (two) {
      setup2();
      w2.minv = w.minv, w2.keep_g = w.keep_g, w2.spmv_kind = w.spmv_kind;
      two = ikr::pcg_persistent2_eligible(A, w, w2, w.spmv_kind - first_persistent_kind());
    }
    if (!two) {
      const int64_t i0 = solve(a, b0, x0, rt, maxit, refinements);
      const int64_t i1 = solve(a, b1, x1, rt1, maxit, refinements);
      last_iters = (int)(i0 + i1);
      return i0 + i1;
    }
    cudaStream_t s = a->fes->stream;
    ikr::launch_pcg_init(A, w, b0, rt, maxit, s);
    ikr::launch_pcg_init(A, w2, b1, rt1, maxit, s);
    count(4);
    if (profile) CK(cudaEventRecord(tev[0], s));
    CK(ikr::launch_pcg_persistent2(A, w, w2, w.spmv_kind - first_persistent_kind(), pa2.p, pb2.p, s));
    count(1);
    if (profile) CK(cudaEventRecord(tev[1], s));
    CK(cudaMemcpyAsync(scal_h, scal.p, sizeof(double) * ikr::kNScal, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(scal_h + ikr::kNScal, scal2.p, sizeof(double) * ikr::kNScal, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    ikr::launch_pcg_result(w, x0, 1.0, s);
    ikr::launch_pcg_result(w2, x1, 1.0, s);
    count(2);
    const double* s0 = scal_h;
    const double* s1 = scal_h + ikr::kNScal;
    const int it0 = (int)s0[ikr::kIters], it1 = (int)s1[ikr::kIters];
    if (profile) {  // one matrix stream per iteration of the longer solve
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, tev[0], tev[1]));
      prof_ms += ms;
      prof_n += std::max(it0, it1);
    }
    last_iters = it0 + it1;
    last_rel = s0[ikr::kBB] > 0 ? std::sqrt(s0[ikr::kRR] / s0[ikr::kBB]) : 0.0;
    for (const double* sc : {s0, s1}) {
      if (sc[ikr::kDone] == 6.0) fail(IKR_ERR_TIMEOUT, "a bounded wait in the persistent CG gave up");
      if (sc[ikr::kDone] == 3.0)
        fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp zero or not finite) after %d iterations", (int)sc[ikr::kIters]);
    }
    return last_iters;
  }

  // x = K^{-1} b with optional FP64 iterative refinement around the (possibly FP32) CG; with the FP64 outer
  // Krylov solve on (outer_m > 0) an FP32 tangent is solved against its FP64 twin instead
  int64_t solve(ikr_asm a, const double* b, double* x, double rt, int maxit, int refinements) {
    if (direct) rt = std::min(rt, rtol);  // a direct solver's accuracy, whatever the Newton's linear tolerance
    if (outer_m > 0 && a->fp32) return fgmres_solve(this, a, b, x, rt);
    int64_t its = solve_device(a, b, x, rt, maxit);
    if (refinements <= 0) return its;
    cudaStream_t s = a->fes->stream;
    const int64_t n = 3LL * a->fes->nn;
    for (int k = 0; k < refinements; ++k) {
      ikr::launch_residual64(a->bsr(), fp32, x, b, r64.p, s);  // r = b - K x in FP64 accumulation
      its += solve_device(a, r64.p, c64.p, rt, maxit);
      ikr::launch_axpy64(x, c64.p, 1.0, n, s);
      count(2);
    }
    return its;
  }
};

// listeners owned by the broadcaster they are subscribed to (operators.cpp: the reference's loggers)
struct ListenerBase {
  virtual ~ListenerBase() = default;
};

struct Observer {
  ikr_nr_observer cb;
  void* user;
};
struct ControlObserver {
  ikr_control_observer cb;
  void* user;
};

// One Newton iteration captured as a CUDA graph (newton_graph.cpp): tangent assembly, block-Jacobi inverse, the
// persistent CG, update, residual assembly and both norms; the host writes the CG tolerance and the load factor into
// `host` before a launch and reads the norms, the CG scalars and the element status from it after.
struct NewtonStepGraph {
  cudaGraphExec_t exec = nullptr;
  std::vector<const void*> key;  // what the captured launches depend on; a change recaptures
  int64_t launches = 0;          // kernel launches per graph launch
  bool unsupported = false;      // the capture failed (then the iterations run launch by launch)
  double* host = nullptr;        // pinned: [0] rtol, [1] lambda, [2] |corr|, [3] |R|, [4 ..] CG scalars, then status
  DBuf<double> dev;              // [0] rtol, [1] lambda, [2] |corr|, [3] |R|
  DBuf<double> part;             // partial sums of the two norms
  ~NewtonStepGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (host) cudaFreeHost(host);
  }
};

struct ikr_nr_s {
  ikr_asm asm_ = nullptr;
  ikr_ls ls = nullptr;
  ikr_nr_settings st{};
  std::unique_ptr<NewtonStepGraph> step_graph;
  int64_t graph_iterations = 0;  // Newton iterations run as graph launches since creation
  std::vector<Observer> obs;
  std::vector<std::unique_ptr<ListenerBase>> listeners;
  bool fe_state = false;
  DBuf<double> corr, rhs;
  DBuf<double> nrm_part, nrm_out;
  // per-instance state of the last solve (element sets with instances)
  std::vector<int32_t> inst_iters;
  std::vector<int64_t> inst_lin;  // CG iterations per instance over the solve
  std::vector<double> inst_res;
  std::vector<int8_t> inst_conv;     // 1 converged, 0 not, -1 taken out after an element inversion
  std::vector<uint8_t> inst_failed;  // taken out since the last reset (LoadControl::run, newton_solve): 1 inverted,
                                     // 2 above tolerance after max_iter, 3 kept out by the caller, 4 CG unsolved
  bool take_out_unsolved = false;    // batched: a CG still above its tolerance after linear_max_iter takes the
                                     // instance out (status -4)
  std::vector<uint8_t> inst_excluded;  // instances the caller keeps out of every solve (ikr_newton_exclude_instances)
  DBuf<double> u_old, alpha_old, inst_step;  // backtracking: state before the correction, per-instance steps
  int64_t backtracks = 0;                    // corrections halved since creation
  DBuf<double> inst_norm, inst_rtol;
  DBuf<int32_t> inst_cg_iters;
  DBuf<double> inst_cg_res;
  // CTA groups of the batched CG (kernels.h launch_batched_pcg), re-planned before every launch over the running instances
  struct BatchPlan {
    int n_cta = 0;
    int cur_variant = 0;         // kernels.h launch_batched_pcg variant of the current plan (4: clusters)
    bool cooperative = false;
    DBuf<int32_t> cta_inst, cta_first, cta_size;
    DBuf<double> part;
    DBuf<unsigned int> counters;
    DBuf<double> st;             // rz, r.r, b.b, beta per instance between the launches of one solve
    DBuf<int32_t> flag;          // per instance: 0 running, 1 finished, 2 breakdown, -1 a wait gave up
    int64_t launches = 0;        // batched CG launches since creation
    int64_t launches_by_variant[6] = {0, 0, 0, 0, 0, 0};
    int variant = -1;            // -1: the planner's choice; 0..4 that variant where it fits, else the row loop
    double share = 1.0;          // share of the device's co-resident CTAs a plan may use (0.5 while another
                                 // solver's batched CG runs concurrently)
    int first_chunk = 128;       // iterations of a solve's first launch (doubling for the next ones, at most 4096)
  } plan;
};

struct ikr_lc_s {
  ikr_nr nr = nullptr;
  int steps = 1;
  double t0 = 0, t1 = 1;
  // batched solves: precision escalation (ikr_load_control_set_escalation).  An instance the solver takes out in a
  // load step is solved again from the state at the start of that step by esc_nr on esc_req (an FP64 twin of the
  // element set) and stays there for the rest of the run; its displacement is copied back into the run's requirement
  // at every step end.
  ikr_nr esc_nr = nullptr;
  ikr_req esc_req = nullptr;
  std::vector<uint8_t> escalated;
  std::vector<int8_t> esc_conv;  // status of each escalated instance in esc_nr (instance_info codes)
  bool esc_concurrent = false;   // instances escalated in earlier steps are solved on a second host thread and
                                 // stream while the run's solver does the step (each planner then uses half of the
                                 // co-resident CTAs, so both cooperative launches fit the device at once)
  DBuf<double> u_start;
  std::vector<ControlObserver> obs;
  std::vector<std::unique_ptr<ListenerBase>> listeners;
  // Newton predictor of each load step (the reference only increments the load factor,
  // loadcontrol.inl:54-57): 0 = none, 1 = previous increment, 2 = learned, which falls back to the previous
  // increment when its FP64 residual is not smaller (predictor.cpp).  `record` appends each converged
  // increment to the predictor's training snapshots.
  int pred_kind = 0;
  ikr_pred pred = nullptr;
  std::vector<double> theta;  // load parameters of the current path (learned predictor features)
  bool record = false;
  int path_id = 0;
  int accepted = 0, rejected = 0;
  bool gated = true;  // the learned candidate must beat its fallback's FP64 residual norm
  DBuf<double> u_step0, u_try, pred_part, pred_out;
  DBuf<float> du1, du2;  // last two converged increments (FP32)
  int hist = 0;          // how many increments are in du1 / du2
  // per load step of the last run: FP64 residual norms of the unpredicted state, of the previous-increment
  // candidate and of the learned candidate (-1 when not evaluated, inf when an element inverted), and the
  // state kept (0 unpredicted, 1 previous increment, 2 learned)
  struct PredRecord {
    double step, r_plain, r_fallback, r_learned, kept, spare;
  };
  std::vector<PredRecord> phist;
};

// ------------------------------------------------------------------------------------------------------------
namespace ikr_host {
// load-control predictor hooks (predictor.cpp)
void predictor_begin(ikr_lc lc, ikr_req r);
// after lambda += dlambda: tries the configured prediction, keeps it only if its residual is smaller, and returns
// the residual norm of the unpredicted state (the reference norm of the relative Newton test), 0 without predictor
double predictor_apply(ikr_lc lc, ikr_req r, int step);
void predictor_end_step(ikr_lc lc, ikr_req r, int step);
void need(bool c, int code, const char* msg);
double device_norm(ikr_fes f, const double* x, int64_t n, DBuf<double>& part, DBuf<double>& out);
double device_dot(ikr_fes f, const double* x, const double* y, int64_t n, DBuf<double>& part, DBuf<double>& out);
// sync = false: capture-safe (the kernels were tuned before; no status read, no host callback)
void assemble_vector(ikr_asm a, ikr_req r, int dbc, bool sync = true);
void assemble_matrix(ikr_asm a, ikr_req r, int dbc, bool sync = true);
void update_state(ikr_fes f, ikr_req r, const double* corr_dev);
// syncParameterAndGlobalSolution: u = lambda * rate where that value is nonzero
void idbc_sync(ikr_asm a, ikr_req r);
// Newton iterations as CUDA graphs (newton_graph.cpp): whether this solve's configuration allows it, and one
// iteration (tangent at u, solve to rtol, u += correction, residual at u); returns the CG iterations, -1 when the
// capture was refused (the iteration then runs launch by launch)
bool step_graph_eligible(ikr_nr nr, ikr_req r);
int64_t step_graph_iteration(ikr_nr nr, ikr_req r, double rtol, double* corr_norm, double* res_norm);
// ControlLogger (operators.cpp): a listener and the control observer that feeds it
std::unique_ptr<ListenerBase> make_control_logger(ikr_log_sink sink, void* user, ControlObserver* obs);
// Newton-Raphson solve (newtonraphson.hh:193-257); ref_norm > 0 replaces the initial residual norm as the
// reference of the relative convergence test
void nr_solve(ikr_nr nr, ikr_req r, double step_size, ikr_nr_info* info, double ref_norm = 0.0);
// batched_host.cpp: the batched Newton, the batched CG's planner and the precision escalation of a load control
struct BatchChoice {
  int variant = 0;
  bool cooperative = false;
  std::vector<int> ctas;  // CTAs per instance (in the input order); 16 per instance for the cluster variant
};
BatchChoice choose_batch_plan(const std::vector<int>& rows, const std::vector<int>& width, bool fp32, int forced,
                              const int (&caps)[6], int cluster_cap);
void nr_solve_batched(ikr_nr nr, ikr_req r, ikr_nr_info* info);
void escalation_begin(ikr_lc lc, ikr_req r);
void escalated_step(ikr_lc lc, ikr_req r, double step, double ref, ikr_nr_info& ni);
}  // namespace ikr_host
