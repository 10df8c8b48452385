// Host layer of the GB300-native Newton-Raphson / LoadControl path: the C ABI of include/ikarus_gb300.h.
// One CUDA stream per finite-element set; every object built on that set (requirements, assembler,
// solver, Newton, LoadControl) issues its work on it.  Kernels live in element.cu, sparse.cu, solver.cu.
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

namespace {

thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};

struct IkrError : std::runtime_error {
  int code;
  IkrError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw IkrError(code, buf);
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) fail(IKR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}
#define CK(x) cuda_check((x), #x)

void count(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

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

int num_sms() {
  static int sms = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 152;
    return v > 0 ? v : 152;
  }();
  return sms;
}

}  // namespace

// ------------------------------------------------------------------------------------------------------------
struct ikr_fes_s {
  int nn = 0, ne = 0, na = 0, eas = 0;
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
  DBuf<int> status;
  DBuf<double> scratch_out;  // element-level outputs

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
    a.eas_kind = na > 0 ? eas : 0;
    a.n_alpha = na;
    a.alpha = alpha.p;
    a.eas_geo = eas_geo.p;
    a.eas_y = eas_y.p;
    a.eas_Y = eas_Y.p;
    a.trac_idx = trac_idx.n ? trac_idx.p : nullptr;
    a.trac = trac.p;
    a.status = status.p;
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
  // pattern
  int64_t nb = 0;
  DBuf<int32_t> row_ptr, col, diag, slot;
  std::vector<int32_t> row_ptr_h, col_h;
  DBuf<double> val64;
  DBuf<float> val32;
  int matrix_dbc = -1;  // option of the last assembled matrix
  // vector
  DBuf<double> R;
  int vector_dbc = -1;
  DBuf<int32_t> pl_dof;
  DBuf<double> pl_val;
  std::map<int32_t, double> pl_h;
  DBuf<double> norm_part, norm_out;
  ikr_req bound_req = nullptr;
  int bound_dbc = IKR_DBC_FULL;

  ikr::Bsr bsr() const {
    ikr::Bsr b;
    b.n_rows = fes->nn;
    b.n_blocks = nb;
    b.row_ptr = row_ptr.p;
    b.col = col.p;
    b.diag = diag.p;
    b.val = fp32 ? (const void*)val32.p : (const void*)val64.p;
    return b;
  }
  void* values() { return fp32 ? (void*)val32.p : (void*)val64.p; }

  void build_pattern() {
    ikr_fes f = fes;
    cudaStream_t s = f->stream;
    DBuf<int32_t> cnt, ne_ptr, cursor, ne_elems, rcnt;
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
    slot.alloc(64LL * f->ne);
    diag.alloc(f->nn);
    ikr::launch_slot_map(f->conn.p, f->ne, row_ptr.p, col.p, slot.p, diag.p, f->nn, s);
    count(3);
    row_ptr_h.resize(f->nn + 1);
    col_h.resize(nb);
    row_ptr.download(row_ptr_h.data(), row_ptr_h.size(), s);
    col.download(col_h.data(), col_h.size(), s);
    CK(cudaStreamSynchronize(s));
    f->check_status();
    if (fp32) val32.alloc(9 * nb);
    else val64.alloc(9 * nb);
  }
};

struct ikr_ls_s {
  int tag = IKR_SOLVER_GPU_PCG_BLOCK_JACOBI;
  double rtol = 1e-10;
  int max_iter = 100000;
  ikr_asm asm_ = nullptr;
  bool fp32 = false;
  ikr::PcgWork w;
  DBuf<double> dx, dp, dq, dmv, pa, pb, scal;
  DBuf<float> fx, fp, fq, fmv;
  DBuf<double> dz, dr, dp1;
  DBuf<float> fz, fr, fp1;
  double* scal_h = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // CG iterations are launched as CUDA graphs of chunk_len iterations.  In profiling mode two graphs
  // alternate, each with its own event-record nodes around every SpMV, so the SpMV device time of the
  // chunk that just finished can be read while the next one runs.
  cudaGraphExec_t chunk[2] = {nullptr, nullptr};
  int chunk_len = 16;
  bool profile = false;
  std::vector<cudaEvent_t> pev[2];
  double prof_ms = 0.0;
  int64_t prof_n = 0;
  int last_iters = 0;
  double last_rel = 0.0;
  bool factorized = false;
  DBuf<double> b64, x64, r64, c64;  // refinement work

  ~ikr_ls_s() {
    drop_graphs();
    for (auto& e : ev)
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
    if (asm_ == a && w.n_rows == a->fes->nn && fp32 == a->fp32 && w.grid) return;
    drop_graphs();
    asm_ = a;
    fp32 = a->fp32;
    const int nr = a->fes->nn;
    const size_t n = 3 * (size_t)nr;
    w = ikr::PcgWork{};
    w.n_rows = nr;
    w.fp32 = fp32;
    w.grid = 4 * num_sms();
    if (fp32) {
      fx.alloc(n), fr.alloc(n), fz.alloc(n), fp.alloc(n), fp1.alloc(n), fq.alloc(n), fmv.alloc(9 * (size_t)nr);
      w.x = fx.p, w.r = fr.p, w.z = fz.p, w.p0 = fp.p, w.p1 = fp1.p, w.q = fq.p, w.minv = fmv.p;
    } else {
      dx.alloc(n), dr.alloc(n), dz.alloc(n), dp.alloc(n), dp1.alloc(n), dq.alloc(n), dmv.alloc(9 * (size_t)nr);
      w.x = dx.p, w.r = dr.p, w.z = dz.p, w.p0 = dp.p, w.p1 = dp1.p, w.q = dq.p, w.minv = dmv.p;
    }
    pa.alloc(w.grid);
    pb.alloc(2 * (size_t)w.grid);
    scal.alloc(ikr::kNScal);
    w.part_a = pa.p;
    w.part_b = pb.p;
    w.scal = scal.p;
    if (!scal_h) CK(cudaMallocHost(&scal_h, sizeof(double) * 2 * ikr::kNScal));
    for (auto& e : ev)
      if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b64.alloc(n), x64.alloc(n), r64.alloc(n), c64.alloc(n);
  }

  void build_chunk(cudaStream_t s) {
    const int ng = profile ? 2 : 1;
    const ikr::Bsr A = asm_->bsr();
    for (int gi = 0; gi < ng; ++gi) {
      if (chunk[gi]) continue;
      if (profile && pev[gi].empty()) {
        pev[gi].resize(2 * chunk_len);
        for (auto& e : pev[gi]) CK(cudaEventCreate(&e));
      }
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < chunk_len; ++k) {
        // cudaEventRecordExternal turns the records into event-record nodes of the graph (a plain record
        // during capture would only become an internal dependency)
        if (profile) CK(cudaEventRecordWithFlags(pev[gi][2 * k], s, cudaEventRecordExternal));
        ikr::launch_pcg_spmv(A, w, k & 1, s);
        if (profile) CK(cudaEventRecordWithFlags(pev[gi][2 * k + 1], s, cudaEventRecordExternal));
        ikr::launch_pcg_update(A, w, k & 1, s);
      }
      CK(cudaStreamEndCapture(s, &g));
      CK(cudaGraphInstantiate(&chunk[gi], g, 0));
      cudaGraphDestroy(g);
    }
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
    setup(a);
    ikr::launch_block_jacobi(a->bsr(), fp32, w.minv, tag == IKR_SOLVER_SI_CONJUGATE_GRADIENT, a->fes->stream);
    count(1);
    factorized = true;
  }

  // x = K^{-1} b on the device (FP64 in / out); returns CG iterations
  int solve_device(ikr_asm a, const double* b, double* x, double rt, int maxit) {
    if (!factorized || asm_ != a) fail(IKR_ERR_INVALID_STATE, "linear solver not factorized for this assembler");
    cudaStream_t s = a->fes->stream;
    const ikr::Bsr A = a->bsr();
    build_chunk(s);
    ikr::launch_pcg_init(A, w, b, rt, maxit, s);
    count(2);
    // Chunks of CG iterations are launched one ahead of the host check: once the device flags
    // convergence the chunk in flight returns at entry, so polling never stalls the GPU.
    constexpr int NS = ikr::kNScal;
    auto graph = [&](int k) { return chunk[profile ? (k & 1) : 0]; };
    auto iters_in = [&](int slot) {
      return (int)std::max(scal_h[NS * slot + ikr::kIters], scal_h[NS * slot + ikr::kIters + 1]);
    };
    int k = 0, prev_iters = 0;
    CK(cudaGraphLaunch(graph(0), s));
    count(2 * chunk_len);
    CK(cudaMemcpyAsync(scal_h, scal.p, sizeof(double) * NS, cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(ev[0], s));
    for (;;) {
      ++k;
      CK(cudaGraphLaunch(graph(k), s));
      count(2 * chunk_len);
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
    last_iters = (int)std::max(sc[ikr::kIters], sc[ikr::kIters + 1]);
    last_rel = sc[ikr::kBB] > 0 ? std::sqrt(sc[ikr::kRR] / sc[ikr::kBB]) : 0.0;
    ikr::launch_pcg_result(w, x, 1.0, s);
    count(1);
    if (done == 3.0) fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp <= 0) after %d iterations", last_iters);
    return last_iters;
  }

  // x = K^{-1} b with optional FP64 iterative refinement around the (possibly FP32) CG
  int64_t solve(ikr_asm a, const double* b, double* x, double rt, int maxit, int refinements) {
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

struct Observer {
  ikr_nr_observer cb;
  void* user;
};
struct ControlObserver {
  ikr_control_observer cb;
  void* user;
};

struct ikr_nr_s {
  ikr_asm asm_ = nullptr;
  ikr_ls ls = nullptr;
  ikr_nr_settings st{};
  std::vector<Observer> obs;
  bool fe_state = false;
  DBuf<double> corr, rhs;
  DBuf<double> nrm_part, nrm_out;
};

struct ikr_lc_s {
  ikr_nr nr = nullptr;
  int steps = 1;
  double t0 = 0, t1 = 1;
  std::vector<ControlObserver> obs;
};

// ------------------------------------------------------------------------------------------------------------
namespace {

std::atomic<uint64_t> g_req_ids{1};

void greedy_colouring(ikr_fes f) {
  // element -> colour, smallest colour not used by an element sharing a node, elements in index order
  std::vector<int32_t> ptr(f->nn + 1, 0), elems;
  for (int e = 0; e < f->ne; ++e)
    for (int v = 0; v < 8; ++v) ptr[f->conn_h[8 * e + v] + 1]++;
  for (int i = 0; i < f->nn; ++i) ptr[i + 1] += ptr[i];
  elems.resize(ptr[f->nn]);
  std::vector<int32_t> cur(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < f->ne; ++e)
    for (int v = 0; v < 8; ++v) elems[cur[f->conn_h[8 * e + v]]++] = e;
  std::vector<int32_t> colour(f->ne, -1);
  int ncol = 0;
  std::vector<uint8_t> used;
  for (int e = 0; e < f->ne; ++e) {
    used.assign(ncol + 1, 0);
    for (int v = 0; v < 8; ++v) {
      const int n = f->conn_h[8 * e + v];
      for (int k = ptr[n]; k < ptr[n + 1]; ++k) {
        const int o = elems[k];
        if (colour[o] >= 0) used[colour[o]] = 1;
      }
    }
    int c = 0;
    while (c < ncol && used[c]) ++c;
    colour[e] = c;
    ncol = std::max(ncol, c + 1);
  }
  f->colour_ptr.assign(ncol + 1, 0);
  for (int e = 0; e < f->ne; ++e) f->colour_ptr[colour[e] + 1]++;
  for (int c = 0; c < ncol; ++c) f->colour_ptr[c + 1] += f->colour_ptr[c];
  std::vector<int32_t> list(f->ne), pos(f->colour_ptr.begin(), f->colour_ptr.end() - 1);
  for (int e = 0; e < f->ne; ++e) list[pos[colour[e]]++] = e;
  f->colour_elems.upload(list.data(), list.size(), f->stream);
}

double device_norm(ikr_fes f, const double* x, int64_t n, DBuf<double>& part, DBuf<double>& out) {
  part.alloc(1024);
  out.alloc(1);
  ikr::launch_norm2(x, n, part.p, out.p, f->stream);
  count(2);
  double h = 0;
  CK(cudaMemcpyAsync(&h, out.p, sizeof(double), cudaMemcpyDeviceToHost, f->stream));
  CK(cudaStreamSynchronize(f->stream));
  return h;
}

void need(bool c, int code, const char* msg) {
  if (!c) fail(code, "%s", msg);
}

// EAS condensation cache key: valid while the same requirement, solution and alpha are in place
uint64_t cache_key(ikr_req r, ikr_fes f) { return (r->id * 0x9E3779B97F4A7C15ull) ^ (r->version << 20) ^ f->alpha_version; }

void assemble_vector(ikr_asm a, ikr_req r, int dbc) {
  ikr_fes f = a->fes;
  f->refresh_tractions();
  a->R.alloc(a->n);
  CK(cudaMemsetAsync(a->R.p, 0, sizeof(double) * a->n, f->stream));
  ikr::ElemArgs args = f->args();
  args.u = r->u.p;
  args.load_factor = r->lambda;
  args.node_fixed = (dbc == IKR_DBC_RAW) ? nullptr : a->node_fixed.p;
  args.R = a->R.p;
  f->launch_coloured(args, ikr::kWantR, false);
  ikr::launch_vector_finish(a->R.p, nullptr, f->nn, a->pl_dof.p, a->pl_val.p, (int)a->pl_dof.n, r->lambda, f->stream);
  if (a->pl_dof.n) count(1);
  a->vector_dbc = dbc;
  if (f->na > 0) f->eas_cache_key = cache_key(r, f);
  f->check_status();
}

void assemble_matrix(ikr_asm a, ikr_req r, int dbc) {
  ikr_fes f = a->fes;
  if (!a->nb) a->build_pattern();
  const uint8_t* nf = (dbc == IKR_DBC_RAW) ? nullptr : a->node_fixed.p;
  ikr::launch_bsr_reset(a->values(), a->fp32, a->nb, a->diag.p, nf, f->nn, f->stream);
  count(nf ? 1 : 0);
  ikr::ElemArgs args = f->args();
  args.u = r->u.p;
  args.load_factor = r->lambda;
  args.node_fixed = nf;
  args.Kval = a->values();
  args.slot = a->slot.p;
  f->launch_coloured(args, ikr::kWantK, a->fp32);
  a->matrix_dbc = dbc;
  f->check_status();
}

void ensure_eas_cache(ikr_fes f, ikr_req r) {
  if (f->na == 0) return;
  if (f->eas_cache_key == cache_key(r, f)) return;
  // recompute D^{-1} R~ and D^{-1} L at the current state through an element-level residual pass
  DBuf<double> tmp;
  tmp.alloc(24 * (size_t)f->ne);
  ikr::ElemArgs args = f->args();
  args.u = r->u.p;
  args.load_factor = r->lambda;
  args.elem_vec = tmp.p;
  f->launch_elements(args, ikr::kWantR | ikr::kElemOut, false, nullptr, f->ne, 0);
  CK(cudaStreamSynchronize(f->stream));
  f->check_status();
  f->eas_cache_key = cache_key(r, f);
}

void update_state(ikr_fes f, ikr_req r, const double* corr_dev) {
  if (f->na == 0) return;
  ensure_eas_cache(f, r);
  ikr::ElemArgs args = f->args();
  args.u = r->u.p;
  ikr::launch_eas_update(args, f->alpha.p, corr_dev, f->stream);
  count(1);
  f->alpha_version++;
}

}  // namespace

// ------------------------------------------------------------------------------------------------------------
extern "C" {

int ikr_version(void) { return 100; }
int ikr_last_error(char* buf, int32_t len) {
  if (!buf || len <= 0) return IKR_ERR_ARG;
  std::snprintf(buf, (size_t)len, "%s", g_last_error.c_str());
  return IKR_OK;
}
int64_t ikr_kernel_launches(void) { return g_launches.load(); }

int ikr_fes_create(ikr_fes* out, int32_t n_nodes, const double* coords, int32_t n_elems, const int32_t* conn,
                   double lambda, double mu, int32_t eas_kind, int32_t n_alpha) {
  return guarded([&] {
    need(out && coords && conn && n_nodes > 0 && n_elems > 0, IKR_ERR_ARG, "invalid mesh arguments");
    need(eas_kind >= 0 && eas_kind <= 3, IKR_ERR_ARG, "invalid EAS kind");
    if (n_alpha != 0) {
      const bool ok = (eas_kind == IKR_EAS_GREEN_LAGRANGE && (n_alpha == 9 || n_alpha == 21)) ||
                      ((eas_kind == IKR_EAS_DISPLACEMENT_GRADIENT ||
                        eas_kind == IKR_EAS_DISPLACEMENT_GRADIENT_TRANSPOSED) && n_alpha == 9);
      // easvariants.hh:101-165: other parameter counts are not available for 3D
      need(ok, IKR_ERR_NOT_IMPLEMENTED,
           "The given EAS parameters are not available for enhancing the strain measure for the 3D case.");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) fail(IKR_ERR_NO_DEVICE, "no CUDA device");
    for (int64_t k = 0; k < 8LL * n_elems; ++k)
      need(conn[k] >= 0 && conn[k] < n_nodes, IKR_ERR_ARG, "connectivity references a missing node");
    auto f = std::make_unique<ikr_fes_s>();
    f->nn = n_nodes;
    f->ne = n_elems;
    f->na = n_alpha;
    f->eas = eas_kind;
    f->lam = lambda;
    f->mu = mu;
    CK(cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking));
    f->conn_h.assign(conn, conn + 8LL * n_elems);
    f->X.upload(coords, 3LL * n_nodes, f->stream);
    std::vector<int32_t> soa(8LL * n_elems);
    for (int e = 0; e < n_elems; ++e)
      for (int v = 0; v < 8; ++v) soa[(size_t)v * n_elems + e] = conn[8LL * e + v];
    f->conn.upload(soa.data(), soa.size(), f->stream);
    f->status.alloc(1);
    CK(cudaMemsetAsync(f->status.p, 0, sizeof(int), f->stream));
    if (n_alpha > 0) {
      f->alpha.alloc((size_t)n_alpha * n_elems);
      CK(cudaMemsetAsync(f->alpha.p, 0, sizeof(double) * f->alpha.n, f->stream));
      f->eas_geo.alloc((size_t)ikr::eas_geo_stride(eas_kind) * n_elems);
      f->eas_y.alloc((size_t)n_alpha * n_elems);
      f->eas_Y.alloc((size_t)n_alpha * 24 * n_elems);
      ikr::launch_eas_geometry(f->args(), f->eas_geo.p, f->stream);
      count(1);
    }
    greedy_colouring(f.get());
    CK(cudaStreamSynchronize(f->stream));
    *out = f.release();
  });
}

int ikr_fes_add_neumann(ikr_fes fes, int32_t n_faces, const int32_t* face_elem, const int32_t* face_local,
                        const double* traction) {
  return guarded([&] {
    need(fes && n_faces >= 0 && (n_faces == 0 || (face_elem && face_local && traction)), IKR_ERR_ARG,
         "invalid Neumann arguments");
    if (fes->faces.empty()) fes->faces.assign(fes->ne, {});
    for (int k = 0; k < n_faces; ++k) {
      need(face_elem[k] >= 0 && face_elem[k] < fes->ne && face_local[k] >= 0 && face_local[k] < 6, IKR_ERR_ARG,
           "invalid face");
      fes->faces[face_elem[k]].push_back({face_local[k], {traction[3 * k], traction[3 * k + 1], traction[3 * k + 2]}});
    }
    fes->trac_dirty = true;
  });
}

int ikr_fes_destroy(ikr_fes fes) {
  return guarded([&] {
    if (fes) cudaStreamSynchronize(fes->stream);
    delete fes;
  });
}
int ikr_fes_num_colours(ikr_fes fes, int32_t* n) {
  return guarded([&] {
    need(fes && n, IKR_ERR_ARG, "null argument");
    *n = (int32_t)fes->colour_ptr.size() - 1;
  });
}
int ikr_fes_get_alpha(ikr_fes fes, double* alpha) {
  return guarded([&] {
    need(fes && alpha, IKR_ERR_ARG, "null argument");
    std::vector<double> soa(fes->alpha.n);
    fes->alpha.download(soa.data(), soa.size(), fes->stream);
    CK(cudaStreamSynchronize(fes->stream));
    for (int e = 0; e < fes->ne; ++e)
      for (int p = 0; p < fes->na; ++p) alpha[(size_t)e * fes->na + p] = soa[(size_t)p * fes->ne + e];
  });
}
int ikr_fes_set_alpha(ikr_fes fes, const double* alpha) {
  return guarded([&] {
    need(fes && alpha, IKR_ERR_ARG, "null argument");
    std::vector<double> soa(fes->alpha.n);
    for (int e = 0; e < fes->ne; ++e)
      for (int p = 0; p < fes->na; ++p) soa[(size_t)p * fes->ne + e] = alpha[(size_t)e * fes->na + p];
    fes->alpha.upload(soa.data(), soa.size(), fes->stream);
    CK(cudaStreamSynchronize(fes->stream));
    fes->alpha_version++;
  });
}

static void element_level(ikr_fes fes, ikr_req req, int mode, int32_t e0, int32_t e1, double* out, int per) {
  need(fes && req && out && req->fes == fes, IKR_ERR_ARG, "invalid arguments");
  need(e0 >= 0 && e1 <= fes->ne && e0 <= e1, IKR_ERR_ARG, "element range out of bounds");
  const int n = e1 - e0;
  if (n == 0) return;
  fes->refresh_tractions();
  fes->scratch_out.alloc((size_t)per * n);
  ikr::ElemArgs a = fes->args();
  a.u = req->u.p;
  a.load_factor = req->lambda;
  a.elem_vec = fes->scratch_out.p;
  a.elem_mat = fes->scratch_out.p;
  a.elem_energy = fes->scratch_out.p;
  a.eas_y = nullptr;  // element-level evaluations leave the condensation cache alone
  a.eas_Y = nullptr;
  fes->launch_elements(a, mode, false, nullptr, n, e0);
  fes->scratch_out.download(out, (size_t)per * n, fes->stream);
  CK(cudaStreamSynchronize(fes->stream));
  fes->check_status();
}

int ikr_fe_calculate_vector(ikr_fes fes, ikr_req req, int32_t aff, int32_t e0, int32_t e1, double* out) {
  return guarded([&] {
    // EAS throws NotImplemented for other affordances (enhancedassumedstrains.hh:316-317)
    need(aff == IKR_VEC_FORCES, IKR_ERR_NOT_IMPLEMENTED, "VectorAffordance not implemented");
    element_level(fes, req, ikr::kWantR | ikr::kElemOut, e0, e1, out, 24);
  });
}
int ikr_fe_calculate_matrix(ikr_fes fes, ikr_req req, int32_t aff, int32_t e0, int32_t e1, double* out) {
  return guarded([&] {
    need(aff == IKR_MAT_STIFFNESS, IKR_ERR_NOT_IMPLEMENTED, "MatrixAffordance not implemented");
    element_level(fes, req, ikr::kWantK | ikr::kElemOut, e0, e1, out, 576);
  });
}
int ikr_fe_calculate_scalar(ikr_fes fes, ikr_req req, int32_t aff, int32_t e0, int32_t e1, double* out) {
  return guarded([&] {
    need(aff == IKR_SCALAR_MECHANICAL_POTENTIAL_ENERGY, IKR_ERR_NOT_IMPLEMENTED, "ScalarAffordance not implemented");
    // enhancedassumedstrains.hh:305-309: EAS elements are not derivable from a potential
    need(fes && fes->na == 0, IKR_ERR_NOT_IMPLEMENTED,
         "EAS element do not support any scalar calculations, i.e. they are not derivable from a potential");
    element_level(fes, req, ikr::kWantEnergy | ikr::kElemOut, e0, e1, out, 1);
  });
}
int ikr_fe_update_state(ikr_fes fes, ikr_req req, const double* correction, int32_t n) {
  return guarded([&] {
    need(fes && req && correction && req->fes == fes, IKR_ERR_ARG, "invalid arguments");
    if (fes->na == 0) return;
    need(n == 3 * fes->nn, IKR_ERR_NOT_IMPLEMENTED,
         "Solution vector and correction vector should be of the same size. Check if DBCOption::Full is used.");
    DBuf<double> c;
    c.upload(correction, n, fes->stream);
    update_state(fes, req, c.p);
    CK(cudaStreamSynchronize(fes->stream));
    fes->check_status();
  });
}

int ikr_req_create(ikr_req* out, ikr_fes fes) {
  return guarded([&] {
    need(out && fes, IKR_ERR_ARG, "null argument");
    auto r = std::make_unique<ikr_req_s>();
    r->fes = fes;
    r->u.alloc(3 * (size_t)fes->nn);
    CK(cudaMemsetAsync(r->u.p, 0, sizeof(double) * r->u.n, fes->stream));
    CK(cudaStreamSynchronize(fes->stream));
    r->id = g_req_ids.fetch_add(1);
    *out = r.release();
  });
}
int ikr_req_destroy(ikr_req r) {
  return guarded([&] { delete r; });
}
int ikr_req_insert_global_solution(ikr_req r, const double* u) {
  return guarded([&] {
    need(r && u, IKR_ERR_ARG, "null argument");
    r->u.upload(u, r->u.n, r->fes->stream);
    CK(cudaStreamSynchronize(r->fes->stream));
    r->version++;
  });
}
int ikr_req_global_solution(ikr_req r, double* u) {
  return guarded([&] {
    need(r && u, IKR_ERR_ARG, "null argument");
    r->u.download(u, r->u.n, r->fes->stream);
    CK(cudaStreamSynchronize(r->fes->stream));
  });
}
int ikr_req_insert_parameter(ikr_req r, double lf) {
  return guarded([&] {
    need(r, IKR_ERR_ARG, "null argument");
    r->lambda = lf;
  });
}
int ikr_req_parameter(ikr_req r, double* lf) {
  return guarded([&] {
    need(r && lf, IKR_ERR_ARG, "null argument");
    *lf = r->lambda;
  });
}
int ikr_req_solution_device(ikr_req r, double** d) {
  return guarded([&] {
    need(r && d, IKR_ERR_ARG, "null argument");
    *d = r->u.p;
  });
}
int ikr_req_copy(ikr_req dst, ikr_req src) {
  return guarded([&] {
    need(dst && src && dst->fes == src->fes, IKR_ERR_ARG, "requirements of different element sets");
    CK(cudaMemcpyAsync(dst->u.p, src->u.p, sizeof(double) * dst->u.n, cudaMemcpyDeviceToDevice, dst->fes->stream));
    dst->lambda = src->lambda;
    dst->version++;
  });
}

int ikr_assembler_create(ikr_asm* out, ikr_fes fes, const uint8_t* fixed, int32_t precision) {
  return guarded([&] {
    need(out && fes && fixed, IKR_ERR_ARG, "null argument");
    need(precision == IKR_PRECISION_FP64 || precision == IKR_PRECISION_FP32, IKR_ERR_ARG, "invalid precision");
    auto a = std::make_unique<ikr_asm_s>();
    a->fes = fes;
    a->n = 3 * fes->nn;
    a->fp32 = precision == IKR_PRECISION_FP32;
    a->fixed_h.assign(fixed, fixed + a->n);
    a->cb_h.resize(a->n);
    int c = 0;
    std::vector<uint8_t> nodemask(fes->nn, 0);
    for (int i = 0; i < a->n; ++i) {
      a->cb_h[i] = c;
      if (fixed[i]) {
        ++c;
        nodemask[i / 3] |= (uint8_t)(1u << (i % 3));
      }
    }
    a->nred = a->n - c;
    a->node_fixed.upload(nodemask.data(), nodemask.size(), fes->stream);
    CK(cudaStreamSynchronize(fes->stream));
    *out = a.release();
  });
}
int ikr_assembler_destroy(ikr_asm a) {
  return guarded([&] { delete a; });
}
int ikr_assembler_add_point_loads(ikr_asm a, int32_t n, const int32_t* dofs, const double* values) {
  return guarded([&] {
    need(a && n >= 0 && (n == 0 || (dofs && values)), IKR_ERR_ARG, "invalid point loads");
    for (int k = 0; k < n; ++k) {
      need(dofs[k] >= 0 && dofs[k] < a->n, IKR_ERR_ARG, "point load dof out of range");
      a->pl_h[dofs[k]] += values[k];
    }
    std::vector<int32_t> d;
    std::vector<double> v;
    for (auto& kv : a->pl_h) d.push_back(kv.first), v.push_back(kv.second);
    a->pl_dof.upload(d.data(), d.size(), a->fes->stream);
    a->pl_val.upload(v.data(), v.size(), a->fes->stream);
    CK(cudaStreamSynchronize(a->fes->stream));
  });
}
int ikr_assembler_bind(ikr_asm a, ikr_req r, int32_t dbc) {
  return guarded([&] {
    need(a && r && r->fes == a->fes, IKR_ERR_ARG, "requirement of another element set");
    need(dbc >= 0 && dbc <= 2, IKR_ERR_ARG, "invalid DBCOption");
    a->bound_req = r;
    a->bound_dbc = dbc;
  });
}
int ikr_assembler_size(ikr_asm a, int32_t* s) {
  return guarded([&] {
    need(a && s, IKR_ERR_ARG, "null argument");
    *s = a->n;
  });
}
int ikr_assembler_reduced_size(ikr_asm a, int32_t* s) {
  return guarded([&] {
    need(a && s, IKR_ERR_ARG, "null argument");
    *s = a->nred;
  });
}
int ikr_assembler_constraints_below(ikr_asm a, int32_t* out) {
  return guarded([&] {
    need(a && out, IKR_ERR_ARG, "null argument");
    std::copy(a->cb_h.begin(), a->cb_h.end(), out);
  });
}
int ikr_assembler_vector(ikr_asm a, ikr_req r, int32_t aff, int32_t dbc, double* out) {
  return guarded([&] {
    need(a && r && r->fes == a->fes, IKR_ERR_ARG, "invalid arguments");
    need(aff == IKR_VEC_FORCES, IKR_ERR_NOT_IMPLEMENTED, "VectorAffordance not implemented");
    need(dbc >= 0 && dbc <= 2, IKR_ERR_ARG, "invalid DBCOption");
    assemble_vector(a, r, dbc == IKR_DBC_RAW ? IKR_DBC_RAW : IKR_DBC_FULL);
    if (!out) return;
    std::vector<double> full(a->n);
    a->R.download(full.data(), full.size(), a->fes->stream);
    CK(cudaStreamSynchronize(a->fes->stream));
    if (dbc != IKR_DBC_REDUCED) {
      std::copy(full.begin(), full.end(), out);
    } else {  // getReducedVectorImpl (simpleassemblers.inl:96-118): free dofs in order
      int k = 0;
      for (int i = 0; i < a->n; ++i)
        if (!a->fixed_h[i]) out[k++] = full[i];
    }
  });
}
int ikr_assembler_vector_norm(ikr_asm a, double* nrm) {
  return guarded([&] {
    need(a && nrm && a->R.p, IKR_ERR_INVALID_STATE, "no vector assembled");
    *nrm = device_norm(a->fes, a->R.p, a->n, a->norm_part, a->norm_out);
  });
}
int ikr_assembler_matrix(ikr_asm a, ikr_req r, int32_t aff, int32_t dbc) {
  return guarded([&] {
    need(a && r && r->fes == a->fes, IKR_ERR_ARG, "invalid arguments");
    need(aff == IKR_MAT_STIFFNESS, IKR_ERR_NOT_IMPLEMENTED, "MatrixAffordance not implemented");
    need(dbc >= 0 && dbc <= 2, IKR_ERR_ARG, "invalid DBCOption");
    // Reduced = Raw restricted to the free dofs = Full restricted to the free dofs; stored as Full
    assemble_matrix(a, r, dbc == IKR_DBC_RAW ? IKR_DBC_RAW : IKR_DBC_FULL);
    a->matrix_dbc = dbc;
  });
}

static void export_csc(ikr_asm a, int dbc, int64_t* cp, int32_t* ri, double* v, int64_t* nnz_out) {
  need(a && a->nb, IKR_ERR_INVALID_STATE, "no matrix assembled");
  const bool reduced = dbc == IKR_DBC_REDUCED;
  const int nn = a->fes->nn;
  std::vector<double> val;
  if (v) {
    val.resize(9 * (size_t)a->nb);
    if (a->fp32) {
      std::vector<float> f(val.size());
      a->val32.download(f.data(), f.size(), a->fes->stream);
      CK(cudaStreamSynchronize(a->fes->stream));
      for (size_t i = 0; i < f.size(); ++i) val[i] = f[i];
    } else {
      a->val64.download(val.data(), val.size(), a->fes->stream);
      CK(cudaStreamSynchronize(a->fes->stream));
    }
  }
  // column gc = 3J + b holds rows 3I + a for every neighbour I of J in ascending order (symmetric pattern);
  // the value K(3I+a, 3J+b) sits in block (I, J) of block row I.
  const auto& rp = a->row_ptr_h;
  const auto& cl = a->col_h;
  auto block_of = [&](int I, int J) -> int64_t {
    auto b = cl.begin() + rp[I], e = cl.begin() + rp[I + 1];
    auto it = std::lower_bound(b, e, J);
    return it - cl.begin();
  };
  int64_t nnz = 0;
  int col_out = 0;
  if (cp) cp[0] = 0;
  for (int J = 0; J < nn; ++J)
    for (int b = 0; b < 3; ++b) {
      const int gc = 3 * J + b;
      if (reduced && a->fixed_h[gc]) continue;
      for (int k = rp[J]; k < rp[J + 1]; ++k) {
        const int I = cl[k];
        for (int aa = 0; aa < 3; ++aa) {
          const int gr = 3 * I + aa;
          if (reduced && a->fixed_h[gr]) continue;
          if (ri) ri[nnz] = reduced ? gr - a->cb_h[gr] : gr;
          if (v) v[nnz] = val[9 * block_of(I, J) + 3 * aa + b];
          ++nnz;
        }
      }
      ++col_out;
      if (cp) cp[col_out] = nnz;
    }
  if (nnz_out) *nnz_out = nnz;
}

int ikr_assembler_matrix_nnz(ikr_asm a, int32_t dbc, int64_t* nnz) {
  return guarded([&] {
    need(nnz, IKR_ERR_ARG, "null argument");
    if (a && !a->nb) a->build_pattern();
    export_csc(a, dbc, nullptr, nullptr, nullptr, nnz);
  });
}
int ikr_assembler_export_csc(ikr_asm a, int32_t dbc, int64_t* cp, int32_t* ri, double* v) {
  return guarded([&] {
    need(a, IKR_ERR_ARG, "null argument");
    if (v) {
      need(a->matrix_dbc >= 0, IKR_ERR_INVALID_STATE, "no matrix assembled");
      // Raw and Full differ in the stored values; Reduced can be read from either
      need(dbc == IKR_DBC_REDUCED || (dbc == IKR_DBC_RAW) == (a->matrix_dbc == IKR_DBC_RAW), IKR_ERR_INVALID_STATE,
           "the last assembled matrix has another DBCOption");
    }
    if (!a->nb) a->build_pattern();
    export_csc(a, dbc, cp, ri, v, nullptr);
  });
}
int ikr_assembler_block_pattern(ikr_asm a, int32_t* n_rows, int64_t* n_blocks, int32_t* rp, int32_t* col) {
  return guarded([&] {
    need(a, IKR_ERR_ARG, "null argument");
    if (!a->nb) a->build_pattern();
    if (n_rows) *n_rows = a->fes->nn;
    if (n_blocks) *n_blocks = a->nb;
    if (rp) std::copy(a->row_ptr_h.begin(), a->row_ptr_h.end(), rp);
    if (col) std::copy(a->col_h.begin(), a->col_h.end(), col);
  });
}

int ikr_linear_solver_create(ikr_ls* out, int32_t tag) {
  return guarded([&] {
    need(out, IKR_ERR_ARG, "null argument");
    need(tag == IKR_SOLVER_GPU_PCG_BLOCK_JACOBI || tag == IKR_SOLVER_SI_CONJUGATE_GRADIENT, IKR_ERR_NOT_IMPLEMENTED,
         "this SolverTypeTag has no device implementation");
    auto l = std::make_unique<ikr_ls_s>();
    l->tag = tag;
    *out = l.release();
  });
}
int ikr_linear_solver_destroy(ikr_ls ls) {
  return guarded([&] { delete ls; });
}
int ikr_linear_solver_set_tolerance(ikr_ls ls, double rtol, int32_t max_iter) {
  return guarded([&] {
    need(ls && rtol >= 0 && max_iter > 0, IKR_ERR_ARG, "invalid tolerance");
    ls->rtol = rtol;
    ls->max_iter = max_iter;
  });
}
int ikr_linear_solver_analyze_pattern(ikr_ls ls, ikr_asm a) {
  return guarded([&] {
    need(ls && a, IKR_ERR_ARG, "null argument");
    if (!a->nb) a->build_pattern();
    ls->setup(a);
  });
}
int ikr_linear_solver_factorize(ikr_ls ls, ikr_asm a) {
  return guarded([&] {
    need(ls && a && a->matrix_dbc >= 0, IKR_ERR_INVALID_STATE, "no matrix assembled");
    ls->factorize(a);
  });
}
int ikr_linear_solver_solve(ikr_ls ls, ikr_asm a, double* x, const double* b) {
  return guarded([&] {
    need(ls && a && x && b, IKR_ERR_ARG, "null argument");
    DBuf<double> db, dxv;
    db.upload(b, a->n, a->fes->stream);
    dxv.alloc(a->n);
    ls->solve(a, db.p, dxv.p, ls->rtol, ls->max_iter, 0);
    dxv.download(x, a->n, a->fes->stream);
    CK(cudaStreamSynchronize(a->fes->stream));
  });
}
int ikr_linear_solver_last_info(ikr_ls ls, int32_t* it, double* rel) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    if (it) *it = ls->last_iters;
    if (rel) *rel = ls->last_rel;
  });
}

int ikr_linear_solver_profile(ikr_ls ls, int32_t on) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    ls->set_profile(on != 0);
  });
}
int ikr_linear_solver_profile_read(ikr_ls ls, double* ms, int64_t* n) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    if (ms) *ms = ls->prof_ms;
    if (n) *n = ls->prof_n;
  });
}
// Allocation-free variant of the solve: the CG work set is carved out of the library's fixed device array
// (noalloc.cu) instead of cudaMalloc'ed buffers; no graphs, events or pinned buffers either, the host polls
// the device scalars with a plain copy into a static host array after every 32 iterations.
int ikr_linear_solver_solve_noalloc(ikr_asm a, const double* b, double* x, double rtol, int32_t max_iter,
                                    int32_t* iterations) {
  return guarded([&] {
    need(a && b && x, IKR_ERR_ARG, "null argument");
    if (a->fes->nn > IKR_NOALLOC_MAX_NODES)
      fail(IKR_ERR_ARG, "allocation-free solve supports at most %d nodes (%d dofs); this system has %d nodes",
           IKR_NOALLOC_MAX_NODES, 3 * IKR_NOALLOC_MAX_NODES, a->fes->nn);
    need(rtol >= 0 && max_iter > 0, IKR_ERR_ARG, "invalid tolerance");
    need(a->matrix_dbc >= 0 && a->nb > 0, IKR_ERR_INVALID_STATE, "no matrix assembled");
    void* base = nullptr;
    CK(ikr::noalloc_scratch_address(&base));
    ikr::PcgWork w;
    ikr::noalloc_workset(base, a->fes->nn, a->fp32, std::min(4 * num_sms(), ikr::kNoAllocMaxGrid), w);
    cudaStream_t s = a->fes->stream;
    const ikr::Bsr A = a->bsr();
    ikr::launch_block_jacobi(A, a->fp32, w.minv, false, s);
    ikr::launch_pcg_init(A, w, b, rtol, max_iter, s);
    count(3);
    static thread_local double sc[ikr::kNScal];
    for (;;) {
      for (int k = 0; k < 32; ++k) ikr::launch_pcg_iteration(A, w, k & 1, s);
      count(64);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(sc, w.scal, sizeof(sc), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (sc[ikr::kDone] != 0.0) break;
    }
    ikr::launch_pcg_result(w, x, 1.0, s);
    count(1);
    CK(cudaStreamSynchronize(s));
    if (iterations) *iterations = (int32_t)std::max(sc[ikr::kIters], sc[ikr::kIters + 1]);
    if (sc[ikr::kDone] == 3.0) fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp <= 0)");
    if (sc[ikr::kDone] == 2.0) fail(IKR_ERR_NOT_CONVERGED, "CG reached max_iter = %d", max_iter);
  });
}

int ikr_fes_stream(ikr_fes fes, void** stream) {
  return guarded([&] {
    need(fes && stream, IKR_ERR_ARG, "null argument");
    *stream = (void*)fes->stream;
  });
}

int ikr_nr_settings_default(ikr_nr_settings* s) {
  return guarded([&] {
    need(s, IKR_ERR_ARG, "null argument");
    *s = ikr_nr_settings{};
    s->tol = 1e-8;
    s->max_iter = 20;
    s->min_iter = 0;
    s->tol_mode = 0;
    s->forcing = 0;
    s->linear_rtol = 1e-10;
    s->linear_rtol_min = 1e-12;
    s->linear_max_iter = 100000;
    s->refinements = 0;
  });
}
int ikr_newton_create(ikr_nr* out, ikr_asm a, ikr_ls ls, const ikr_nr_settings* st) {
  return guarded([&] {
    need(out && a && ls, IKR_ERR_ARG, "null argument");
    auto nr = std::make_unique<ikr_nr_s>();
    nr->asm_ = a;
    nr->ls = ls;
    if (st) nr->st = *st;
    else ikr_nr_settings_default(&nr->st);
    *out = nr.release();
  });
}
int ikr_newton_destroy(ikr_nr nr) {
  return guarded([&] { delete nr; });
}
int ikr_newton_subscribe(ikr_nr nr, ikr_nr_observer cb, void* user) {
  return guarded([&] {
    need(nr && cb, IKR_ERR_ARG, "null argument");
    nr->obs.push_back({cb, user});
  });
}
int ikr_newton_subscribe_fe_state(ikr_nr nr, int32_t on) {
  return guarded([&] {
    need(nr, IKR_ERR_ARG, "null argument");
    nr->fe_state = on != 0;
  });
}

static void nr_solve(ikr_nr nr, ikr_req r, double step_size, ikr_nr_info* info) {
  (void)step_size;
  ikr_asm a = nr->asm_;
  ikr_fes f = a->fes;
  need(r->fes == f, IKR_ERR_ARG, "requirement of another element set");
  const ikr_nr_settings& st = nr->st;
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
  const int64_t n = a->n;
  nr->corr.alloc(n);
  nr->rhs.alloc(n);
  assemble_vector(a, r, IKR_DBC_FULL);
  double rnorm = device_norm(f, a->R.p, n, nr->nrm_part, nr->nrm_out);
  inf.residual_norm = rnorm;
  const double thr = st.tol_mode == 1 ? st.tol * rnorm : st.tol;
  bool k_valid = false;
  if (!a->nb) a->build_pattern();
  nr->ls->setup(a);
  int iter = 0;
  double rprev = rnorm;
  int64_t lin = 0;
  while ((rnorm > thr && iter < st.max_iter) || iter < st.min_iter) {
    notify(IKR_NLS_ITERATION_STARTED);
    if (!k_valid) {
      assemble_matrix(a, r, IKR_DBC_FULL);
      k_valid = true;
    }
    nr->ls->factorize(a);
    // linear tolerance: fixed, or Eisenstat-Walker (choice 2) bounded by the accuracy this step needs
    double eta = st.linear_rtol;
    if (st.forcing == 1) {
      double ew = iter == 0 ? st.linear_rtol : 0.9 * (rnorm / rprev) * (rnorm / rprev);
      ew = std::min(ew, st.linear_rtol);
      const double need_eta = 0.5 * thr / std::max(rnorm, 1e-300);
      eta = std::max(std::max(ew, need_eta), st.linear_rtol_min);
      eta = std::min(eta, st.linear_rtol);
    }
    ikr::launch_scale64(nr->rhs.p, a->R.p, -1.0, n, f->stream);
    count(1);
    lin += nr->ls->solve(a, nr->rhs.p, nr->corr.p, eta, st.linear_max_iter, st.refinements);
    inf.correction_norm = device_norm(f, nr->corr.p, n, nr->nrm_part, nr->nrm_out);
    notify(IKR_NLS_CORRECTION_UPDATED);
    if (nr->fe_state) update_state(f, r, nr->corr.p);
    ikr::launch_axpy64(r->u.p, nr->corr.p, 1.0, n, f->stream);
    count(1);
    r->version++;
    notify(IKR_NLS_CORRECTIONNORM_UPDATED);
    notify(IKR_NLS_SOLUTION_CHANGED);
    assemble_vector(a, r, IKR_DBC_FULL);
    k_valid = false;  // the reference reassembles K here (newtonraphson.hh:243); it is built when next needed
    rprev = rnorm;
    rnorm = device_norm(f, a->R.p, n, nr->nrm_part, nr->nrm_out);
    inf.residual_norm = rnorm;
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

int ikr_newton_solve(ikr_nr nr, ikr_req r, double step_size, ikr_nr_info* info) {
  return guarded([&] {
    need(nr && r, IKR_ERR_ARG, "null argument");
    nr_solve(nr, r, step_size, info);
  });
}

int ikr_load_control_create(ikr_lc* out, ikr_nr nr, int32_t steps, double t0, double t1) {
  return guarded([&] {
    need(out && nr, IKR_ERR_ARG, "null argument");
    // loadcontrol.hh:72-77
    need(steps > 0, IKR_ERR_INVALID_STATE, "Number of load steps should be greater than zero.");
    auto lc = std::make_unique<ikr_lc_s>();
    lc->nr = nr;
    lc->steps = steps;
    lc->t0 = t0;
    lc->t1 = t1;
    nr->fe_state = true;  // ControlRoutineFactory::create subscribes the elements (controlroutinefactory.hh:43-46)
    *out = lc.release();
  });
}
int ikr_load_control_destroy(ikr_lc lc) {
  return guarded([&] { delete lc; });
}
int ikr_load_control_subscribe(ikr_lc lc, ikr_control_observer cb, void* user) {
  return guarded([&] {
    need(lc && cb, IKR_ERR_ARG, "null argument");
    lc->obs.push_back({cb, user});
  });
}
int ikr_load_control_run(ikr_lc lc, ikr_req r, ikr_control_info* info, ikr_nr_info* infos, int32_t capacity) {
  return guarded([&] {
    need(lc && r, IKR_ERR_ARG, "null argument");
    const double step = (lc->t1 - lc->t0) / lc->steps;
    ikr_control_info ci{};
    ikr_control_state cs{r, 0, 0.0, r->lambda};
    auto notify = [&](int msg) {
      cs.load_factor = r->lambda;
      for (auto& o : lc->obs) o.cb(msg, &cs, o.user);
    };
    auto record = [&](const ikr_nr_info& ni) {
      if (infos && ci.n_solver_infos < capacity) infos[ci.n_solver_infos] = ni;
      ci.n_solver_infos++;
      ci.total_iterations += ni.iterations;
      ci.total_linear_iterations += ni.linear_iterations;
      notify(IKR_CONTROL_SOLUTION_CHANGED);
      notify(IKR_STEP_ENDED);
    };
    notify(IKR_CONTROL_STARTED);
    notify(IKR_STEP_STARTED);
    ikr_nr_info ni{};
    nr_solve(lc->nr, r, 0.0, &ni);  // equilibrium check at the initial load factor (loadcontrol.inl:29-34)
    record(ni);
    if (ni.success) {
      cs.step_size = step;
      bool ok = true;
      for (int ls = 0; ls < lc->steps; ++ls) {
        cs.load_step = ls;
        notify(IKR_STEP_STARTED);
        r->lambda += step;  // LoadControl::predictor (loadcontrol.inl:54-57)
        nr_solve(lc->nr, r, step, &ni);
        record(ni);
        if (!ni.success) {
          ok = false;
          break;
        }
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
