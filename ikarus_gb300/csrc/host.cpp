// Host layer of the GB300-native Newton-Raphson / LoadControl path: the C ABI of include/ikarus_gb300.h.
// Kernels live in element.cu, element_eas.cu, sparse.cu, solver.cu; shared internals in host_internal.h.
#include "host_internal.h"
// ------------------------------------------------------------------------------------------------------------
namespace ikr_host {
thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};
}  // namespace ikr_host

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

}  // namespace

namespace ikr_host {

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

double device_dot(ikr_fes f, const double* x, const double* y, int64_t n, DBuf<double>& part, DBuf<double>& out) {
  part.alloc(1024);
  out.alloc(1);
  ikr::launch_dot(x, y, n, part.p, out.p, f->stream);
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

// Elements per block of the displacement element kernel: each of 16, 32 and 64 is timed once on a complete
// coloured pass of the given kind and the fastest is kept for the element set (the choice does not change any
// result: the summation order into each block is fixed by the colouring).  `pass` runs one pass with args.epb.
template <typename Pass>
static int choose_epb(ikr_fes f, Pass pass) {
  if (f->na > 0) return 32;  // the EAS kernel has its own launch shape
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int best = 32;
  float best_ms = 1e30f;
  for (int epb : {16, 32, 64}) {
    pass(epb);  // warm
    CK(cudaEventRecord(e0, f->stream));
    pass(epb);
    CK(cudaEventRecord(e1, f->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) best_ms = ms, best = epb;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

void assemble_vector(ikr_asm a, ikr_req r, int dbc, bool sync) {
  ikr_fes f = a->fes;
  if (!sync && !(f->epb_r > 0)) fail(IKR_ERR_INVALID_STATE, "residual kernel not tuned before capture");
  if (sync) {
    f->refresh_tractions();
    f->refresh_function_loads(r->lambda);
  }
  a->R.alloc(a->n);
  CK(cudaMemsetAsync(a->R.p, 0, sizeof(double) * a->n, f->stream));
  ikr::ElemArgs args = f->args();
  args.u = r->u.p;
  args.load_factor = r->lambda;
  args.load_factor_dev = sync ? nullptr : f->capture_lambda;
  args.node_fixed = (dbc == IKR_DBC_RAW) ? nullptr : a->node_fixed.p;
  args.R = a->R.p;
  if (!f->epb_r) {
    f->epb_r = choose_epb(f, [&](int epb) {
      CK(cudaMemsetAsync(a->R.p, 0, sizeof(double) * a->n, f->stream));
      ikr::ElemArgs t = args;
      t.epb = epb;
      f->launch_coloured(t, ikr::kWantR, false);
      f->check_status();
    });
    CK(cudaMemsetAsync(a->R.p, 0, sizeof(double) * a->n, f->stream));
  }
  args.epb = f->epb_r;
  f->launch_coloured(args, ikr::kWantR, false);
  ikr::launch_vector_finish(a->R.p, nullptr, f->nn, a->pl_dof.p, a->pl_val.p, (int)a->pl_dof.n, r->lambda, f->stream,
                            args.load_factor_dev);
  if (a->pl_dof.n) count(1);
  a->vector_dbc = dbc;
  if (f->na > 0) f->eas_cache_key = cache_key(r, f);
  if (sync) f->check_status();
}

static void assemble_matrix_into(ikr_asm a, ikr_req r, int dbc, bool sync);

// The tangent in the assembler's precision; an FP32 tangent with an FP64 twin (dual64) is assembled in FP64 and
// rounded to FP32 once, so the FP32 CG and the FP64 outer solve see the same tangent.  sync = false (stream capture):
// no tuning, no status check.
void assemble_matrix(ikr_asm a, ikr_req r, int dbc, bool sync) {
  if (a->fp32 && a->dual64) {
    if (!a->nb) a->build_pattern();
    a->val64.alloc(9 * (size_t)a->npad);
    a->fp32 = false;
    try {
      assemble_matrix_into(a, r, dbc, sync);
    } catch (...) {
      a->fp32 = true;
      throw;
    }
    a->fp32 = true;
    ikr::launch_round_values(a->val64.p, a->val32.p, 9 * a->npad, a->fes->stream);
    count(1);
    a->k64_stamp = ++a->k_stamp;
    return;
  }
  assemble_matrix_into(a, r, dbc, sync);
  ++a->k_stamp;
}

static void assemble_matrix_into(ikr_asm a, ikr_req r, int dbc, bool sync) {
  ikr_fes f = a->fes;
  if (!a->nb) a->build_pattern();
  const bool timed_path = a->fp32 && f->na == 0;  // the FP32 displacement tangent chooses its kernel by timing
  if (!sync && !((a->fp32 ? f->epb_k32 : f->epb_k64) > 0 && (!timed_path || a->tan_path > 0)))
    fail(IKR_ERR_INVALID_STATE, "tangent kernels not tuned before capture");
  const uint8_t* nf = (dbc == IKR_DBC_RAW) ? nullptr : a->node_fixed.p;
  ikr::ElemArgs args = f->args();
  args.u = r->u.p;
  args.load_factor = r->lambda;
  args.node_fixed = nf;
  args.Kval = a->values();
  args.slot = a->slot.p;
  int& epb_k = a->fp32 ? f->epb_k32 : f->epb_k64;
  if (!epb_k) {
    epb_k = choose_epb(f, [&](int epb) {
      ikr::launch_bsr_reset(a->values(), a->fp32, a->npad, a->diag.p, nf, f->nn, f->stream);
      ikr::ElemArgs t = args;
      t.epb = epb;
      f->launch_coloured(t, ikr::kWantK, a->fp32);
      f->check_status();
    });
    ikr::launch_bsr_reset(a->values(), a->fp32, a->npad, a->diag.p, nf, f->nn, f->stream);
  }
  args.epb = epb_k;
  // FP32 displacement-based tangent: the coloured element kernel, the row kernel (NeoHooke on one element set) or
  // element blocks + gather, whichever is fastest
  const bool blocks_ok = a->fp32 && f->na == 0;
  const bool row_ok = blocks_ok && f->material == 0 && f->n_inst == 0;
  auto element_blocks = [&]() {
    a->build_gather_map();
    ikr::ElemArgs t = args;
    t.blk = a->eblk.p;
    f->launch_elements(t, ikr::kWantK | ikr::kElemBlocks, true, nullptr, f->ne, 0);
    ikr::launch_tangent_gather(a->bsr(), a->gslice.p, a->inv_ptr.p, a->inv_idx.p, a->eblk.p, nf,
                               static_cast<float*>(a->values()), f->stream);
    count(1);
  };
  if (blocks_ok && a->tan_req && (a->tan_req != 2 || row_ok)) a->tan_path = a->tan_req;
  if (blocks_ok && !a->tan_path) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int path : {1, 2, 3}) {
      if (path == 2 && !row_ok) continue;
      float t = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        ikr::launch_bsr_reset(a->values(), a->fp32, a->npad, a->diag.p, nf, f->nn, f->stream);
        CK(cudaEventRecord(e0, f->stream));
        if (path == 1) f->launch_coloured(args, ikr::kWantK, true);
        else if (path == 2) ikr::launch_row_tangent(args, a->ne_ptr.p, a->ne_elems.p, f->stream);
        else element_blocks();
        CK(cudaEventRecord(e1, f->stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        t = std::min(t, ms);
      }
      f->check_status();
      if (t < best) best = t, a->tan_path = path;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ikr::launch_bsr_reset(a->values(), a->fp32, a->npad, a->diag.p, nf, f->nn, f->stream);
  }
  if (blocks_ok && a->tan_path == 3) {
    element_blocks();  // writes every entry of every slice, Dirichlet treatment included: no reset
  } else {
    // zero values, unit diagonal of the constrained dofs (Full), then the read-modify-write assembly
    ikr::launch_bsr_reset(a->values(), a->fp32, a->npad, a->diag.p, nf, f->nn, f->stream);
    count(1);
    if (row_ok && a->tan_path == 2) {
      ikr::launch_row_tangent(args, a->ne_ptr.p, a->ne_elems.p, f->stream);
      count(1);
    } else {
      f->launch_coloured(args, ikr::kWantK, a->fp32);
    }
  }
  if (a->me_idx.n) {  // AssemblerManipulator matrix hooks run after the Dirichlet treatment
    ikr::launch_add_entries(a->values(), a->fp32, a->me_idx.p, a->me_val.p, (int)a->me_idx.n, f->stream);
    count(1);
  }
  a->matrix_dbc = dbc;
  if (sync) f->check_status();
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

}  // namespace ikr_host

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
    f->X_h.assign(coords, coords + 3LL * n_nodes);
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

int ikr_fes_add_volume_load(ikr_fes fes, ikr_point_fn f, void* user) {
  return guarded([&] {
    need(fes && f, IKR_ERR_ARG, "null argument");
    fes->vol_fns.push_back({f, user});
    fes->ext_dirty = true;
  });
}
int ikr_fes_clear_volume_loads(ikr_fes fes) {
  return guarded([&] {
    need(fes, IKR_ERR_ARG, "null argument");
    fes->vol_fns.clear();
    fes->ext_dirty = true;
  });
}
int ikr_fes_add_neumann_function(ikr_fes fes, int32_t n_faces, const int32_t* face_elem, const int32_t* face_local,
                                 ikr_point_fn f, void* user) {
  return guarded([&] {
    need(fes && f && n_faces >= 0 && (n_faces == 0 || (face_elem && face_local)), IKR_ERR_ARG, "invalid arguments");
    std::vector<std::pair<int32_t, int32_t>> faces;
    for (int k = 0; k < n_faces; ++k) {
      need(face_elem[k] >= 0 && face_elem[k] < fes->ne && face_local[k] >= 0 && face_local[k] < 6, IKR_ERR_ARG,
           "face out of range");
      faces.push_back({face_elem[k], face_local[k]});
    }
    std::stable_sort(faces.begin(), faces.end(),
                     [](const auto& x, const auto& y) { return x.first < y.first; });
    ikr_fes_s::FaceFnSet fs{f, user, {}, {0}, {}, {}};
    for (size_t k = 0; k < faces.size(); ++k) {
      const int e = faces[k].first, lf = faces[k].second, d = lf / 2, side = lf % 2;
      if (fs.slot_elem.empty() || fs.slot_elem.back() != e) {
        if (!fs.slot_elem.empty()) fs.face_ptr.push_back((int32_t)k);
        fs.slot_elem.push_back(e);
      }
      fs.face_local.push_back(lf);
      // the face's quadrature point: the centre of the face, the mean of its four corners
      double c[3] = {0.0, 0.0, 0.0};
      for (int v = 0; v < 8; ++v)
        if (((v >> d) & 1) == side)
          for (int i = 0; i < 3; ++i) c[i] += 0.25 * fes->X_h[3 * (size_t)fes->conn_h[8 * (size_t)e + v] + i];
      fs.points.insert(fs.points.end(), c, c + 3);
    }
    if (!fs.slot_elem.empty()) fs.face_ptr.push_back((int32_t)faces.size());
    if (!faces.empty()) fes->face_fns.push_back(std::move(fs));
    fes->ext_dirty = true;
  });
}
int ikr_fes_clear_neumann(ikr_fes fes) {
  return guarded([&] {
    need(fes, IKR_ERR_ARG, "null argument");
    fes->faces.clear();
    fes->trac_idx.release();
    fes->trac.release();
    fes->trac_dirty = false;
    fes->face_fns.clear();
    fes->ext_dirty = true;
  });
}
int ikr_fes_set_element_materials(ikr_fes fes, const double* lambda, const double* mu) {
  return guarded([&] {
    need(fes && lambda && mu, IKR_ERR_ARG, "null argument");
    fes->lam_e.upload(lambda, fes->ne, fes->stream);
    fes->mu_e.upload(mu, fes->ne, fes->stream);
    CK(cudaStreamSynchronize(fes->stream));
  });
}
int ikr_fes_set_instances(ikr_fes fes, int32_t n_inst, const int32_t* node_off) {
  return guarded([&] {
    need(fes && n_inst > 0 && node_off, IKR_ERR_ARG, "invalid instance partition");
    need(node_off[0] == 0 && node_off[n_inst] == fes->nn, IKR_ERR_ARG, "instance offsets must cover all nodes");
    std::vector<int32_t> inst_of(fes->nn);
    for (int i = 0; i < n_inst; ++i) {
      need(node_off[i + 1] > node_off[i], IKR_ERR_ARG, "empty instance");
      for (int k = node_off[i]; k < node_off[i + 1]; ++k) inst_of[k] = i;
    }
    for (int e = 0; e < fes->ne; ++e)  // instances must be independent: no element spans two of them
      for (int v = 1; v < 8; ++v)
        need(inst_of[fes->conn_h[8 * e + v]] == inst_of[fes->conn_h[8 * e]], IKR_ERR_ARG,
             "an element connects two instances");
    std::vector<int32_t> order(n_inst);
    for (int i = 0; i < n_inst; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      return node_off[a + 1] - node_off[a] > node_off[b + 1] - node_off[b];  // largest first
    });
    std::vector<int32_t> elem_inst(fes->ne);
    for (int e = 0; e < fes->ne; ++e) elem_inst[e] = inst_of[fes->conn_h[8 * e]];
    fes->n_inst = n_inst;
    fes->inst_off_h.assign(node_off, node_off + n_inst + 1);
    fes->inst_off.upload(node_off, n_inst + 1, fes->stream);
    fes->inst_order.upload(order.data(), order.size(), fes->stream);
    fes->elem_inst.upload(elem_inst.data(), elem_inst.size(), fes->stream);
    fes->inst_status.alloc(n_inst);
    CK(cudaMemsetAsync(fes->inst_status.p, 0, sizeof(int) * n_inst, fes->stream));
    CK(cudaStreamSynchronize(fes->stream));
  });
}
int ikr_newton_instance_info(ikr_nr nr, int32_t* iterations, double* residual_norms, int32_t* converged) {
  return guarded([&] {
    need(nr, IKR_ERR_ARG, "null argument");
    const size_t ni = nr->inst_iters.size();
    for (size_t i = 0; i < ni; ++i) {
      if (iterations) iterations[i] = nr->inst_iters[i];
      if (residual_norms) residual_norms[i] = nr->inst_res[i];
      if (converged) converged[i] = nr->inst_conv[i];
    }
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
  fes->refresh_function_loads(req->lambda);
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
int ikr_fe_calculate_at(ikr_fes fes, ikr_req req, int32_t result_type, int32_t e_begin, int32_t e_end,
                        const double* local, int32_t local_per_element, double* out) {
  return guarded([&] {
    need(fes && req && req->fes == fes && local && out, IKR_ERR_ARG, "invalid arguments");
    need(result_type >= IKR_RESULT_PK2_STRESS && result_type <= IKR_RESULT_CAUCHY_STRESS, IKR_ERR_NOT_IMPLEMENTED,
         "result type not implemented");
    need(e_begin >= 0 && e_end <= fes->ne && e_begin <= e_end, IKR_ERR_ARG, "element range out of bounds");
    const int count = e_end - e_begin;
    if (count == 0) return;
    cudaStream_t s = fes->stream;
    DBuf<double> xi, o;
    xi.upload(local, local_per_element ? 3 * (size_t)count : 3, s);
    o.alloc(6 * (size_t)count);
    ikr::ElemArgs args = fes->args();
    args.u = req->u.p;
    if (fes->na > 0) ikr::launch_eas_stress_at(args, e_begin, count, xi.p, local_per_element != 0, result_type, o.p, s);
    else ikr::launch_stress_at(args, e_begin, count, xi.p, local_per_element != 0, result_type, o.p, s);
    ikr_host::count(1);
    o.download(out, 6 * (size_t)count, s);
    CK(cudaStreamSynchronize(s));
    fes->check_status();
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
int ikr_assembler_add_matrix_entries(ikr_asm a, int32_t n, const int32_t* rows, const int32_t* cols,
                                     const double* values) {
  return guarded([&] {
    need(a && n >= 0 && (n == 0 || (rows && cols && values)), IKR_ERR_ARG, "invalid matrix entries");
    if (!a->nb) a->build_pattern();
    for (int k = 0; k < n; ++k)
      need(rows[k] >= 0 && rows[k] < a->n && cols[k] >= 0 && cols[k] < a->n, IKR_ERR_ARG,
           "matrix entry index out of range");
    auto value_index = [&](int32_t r, int32_t c) -> int64_t {
      const int rn = r / 3, cn = c / 3;
      const int32_t* b = a->col_h.data() + a->row_ptr_h[rn];
      const int32_t* e = a->col_h.data() + a->row_ptr_h[rn + 1];
      const int32_t* it = std::lower_bound(b, e, cn);
      if (it == e || *it != cn) return -1;
      return ikr::block_entry(a->block_id(rn, a->row_ptr_h[rn] + (it - b)), 3 * (r % 3) + c % 3);
    };
    for (int k = 0; k < n; ++k)
      if (value_index(rows[k], cols[k]) < 0)
        fail(IKR_ERR_ARG, "matrix entry (%d, %d) is not in the sparsity pattern", rows[k], cols[k]);
    for (int k = 0; k < n; ++k) a->me_h[{rows[k], cols[k]}] += values[k];
    std::vector<int64_t> idx;
    std::vector<double> val;
    for (auto& kv : a->me_h) idx.push_back(value_index(kv.first.first, kv.first.second)), val.push_back(kv.second);
    a->me_idx.upload(idx.data(), idx.size(), a->fes->stream);
    a->me_val.upload(val.data(), val.size(), a->fes->stream);
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
    val.resize(9 * (size_t)a->npad);
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
    return a->block_id(I, it - cl.begin());
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
          if (v) v[nnz] = val[ikr::block_entry(block_of(I, J), 3 * aa + b)];
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
    need((tag >= IKR_SOLVER_NONE && tag <= IKR_SOLVER_D_LDLT) || tag == IKR_SOLVER_GPU_PCG_BLOCK_JACOBI ||
             tag == IKR_SOLVER_GPU_PCG_BATCHED,
         IKR_ERR_NOT_IMPLEMENTED, "unknown SolverTypeTag");
    need(tag != IKR_SOLVER_SD_SUPER_LU, IKR_ERR_NOT_IMPLEMENTED, "sd_SuperLU: Not implemented yet.");
    auto l = std::make_unique<ikr_ls_s>();
    l->tag = tag;
    l->point_jacobi = tag >= IKR_SOLVER_SI_CONJUGATE_GRADIENT && tag <= IKR_SOLVER_SI_BICGSTAB;
    l->direct = tag >= IKR_SOLVER_SD_SIMPLICIAL_LLT && tag <= IKR_SOLVER_SD_UMFPACK_LU;
    l->dense = tag >= IKR_SOLVER_D_PARTIAL_PIV_LU && tag <= IKR_SOLVER_D_LDLT;
    if (l->direct) l->rtol = IKR_DIRECT_SOLVE_RTOL;
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
int ikr_linear_solver_set_fp64_outer(ikr_ls ls, int32_t restart, double inner_rtol, int32_t inner_max_iter,
                                     int32_t outer_max_iter) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    need(restart >= 0 && restart < ikr::kKrylovMaxBasis, IKR_ERR_ARG, "restart length must be in [0, 63]");
    need(inner_rtol > 0 && inner_rtol < 1 && inner_max_iter > 0 && outer_max_iter > 0, IKR_ERR_ARG,
         "invalid inner tolerance or iteration limits");
    need(ls->tag != IKR_SOLVER_GPU_PCG_BATCHED && !ls->dense && ls->tag != IKR_SOLVER_NONE,
         IKR_ERR_NOT_IMPLEMENTED, "the FP64 outer solve wraps the single-system CG solvers");
    ls->outer_m = restart;
    ls->inner_rtol = inner_rtol;
    ls->inner_max_iter = inner_max_iter;
    ls->outer_max_iter = outer_max_iter;
  });
}
int ikr_linear_solver_set_wait_test(ikr_ls ls, int32_t barrier_polls, int32_t withhold_first_arrival) {
  return guarded([&] {
    need(ls && barrier_polls >= 0, IKR_ERR_ARG, "invalid arguments");
    ls->w.barrier_polls = barrier_polls;
    ls->w.withhold_first_arrival = withhold_first_arrival ? 1 : 0;
  });
}
int ikr_linear_solver_outer_info(ikr_ls ls, int32_t* outer_iterations, int32_t* cycles) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    if (outer_iterations) *outer_iterations = ls->last_outer;
    if (cycles) *cycles = ls->last_cycles;
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
int ikr_linear_solver_solve2(ikr_ls ls, ikr_asm a, double* x0, double* x1, const double* b0, const double* b1) {
  return guarded([&] {
    need(ls && a && x0 && x1 && b0 && b1, IKR_ERR_ARG, "null argument");
    cudaStream_t s = a->fes->stream;
    DBuf<double> db0, db1, dx0, dx1;
    db0.upload(b0, a->n, s);
    db1.upload(b1, a->n, s);
    dx0.alloc(a->n);
    dx1.alloc(a->n);
    ls->solve2(a, db0.p, db1.p, dx0.p, dx1.p, ls->rtol, ls->max_iter, 0);
    dx0.download(x0, a->n, s);
    dx1.download(x1, a->n, s);
    CK(cudaStreamSynchronize(s));
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
int ikr_linear_solver_set_launch(ikr_ls ls, int32_t use_graphs, int32_t chunk_len) {
  return guarded([&] {
    need(ls && chunk_len >= 1 && chunk_len <= 256, IKR_ERR_ARG, "invalid launch shape");
    ls->set_launch(use_graphs != 0, chunk_len);
  });
}
int ikr_assembler_set_dirichlet_function(ikr_asm a, ikr_point_fn value, ikr_point_fn derivative, void* user) {
  return guarded([&] {
    need(a && value && derivative, IKR_ERR_ARG, "null argument");
    need(a->fes->n_inst == 0, IKR_ERR_NOT_IMPLEMENTED, "the batched solve has no inhomogeneous Dirichlet values");
    std::vector<double> rate(a->n, 0.0);
    derivative(a->fes->nn, a->fes->X_h.data(), 1.0, rate.data(), user);
    for (double v : rate) need(std::isfinite(v), IKR_ERR_ARG, "non-finite Dirichlet derivative");
    a->idbc_rate.upload(rate.data(), a->n, a->fes->stream);
    CK(cudaStreamSynchronize(a->fes->stream));
    a->idbc_value = value;
    a->idbc_user = user;
    a->idbc_vals_valid = false;
    a->has_idbc = true;
  });
}
int ikr_assembler_set_dirichlet_values(ikr_asm a, const double* rate) {
  return guarded([&] {
    need(a, IKR_ERR_ARG, "null argument");
    a->idbc_value = nullptr;
    a->idbc_vals_valid = false;
    if (!rate) {
      a->has_idbc = false;
      a->idbc_rate.release();
      return;
    }
    for (int i = 0; i < a->n; ++i) {
      need(std::isfinite(rate[i]), IKR_ERR_ARG, "non-finite Dirichlet value");
      need(rate[i] == 0.0 || a->fixed_h[i], IKR_ERR_ARG, "a Dirichlet value on a free dof");
    }
    a->idbc_rate.upload(rate, a->n, a->fes->stream);
    CK(cudaStreamSynchronize(a->fes->stream));
    a->has_idbc = true;
  });
}
int ikr_fes_set_material(ikr_fes fes, int32_t material) {
  return guarded([&] {
    need(fes, IKR_ERR_ARG, "null argument");
    need(material == IKR_MATERIAL_NEOHOOKE || material == IKR_MATERIAL_SVK || material == IKR_MATERIAL_BLATZKO,
         IKR_ERR_NOT_IMPLEMENTED, "material not implemented");
    fes->material = material;
    fes->alpha_version++;  // cached EAS condensation data depend on the material
  });
}
static_assert(ikr::kHyperMaxTerms == IKR_HYPER_MAX_TERMS, "hyperelastic term count of the C ABI and the kernels");
int ikr_fes_set_hyperelastic(ikr_fes fes, const ikr_hyperelastic* h) {
  return guarded([&] {
    need(fes && h, IKR_ERR_ARG, "null argument");
    need(h->deviatoric >= IKR_DEV_NONE && h->deviatoric <= IKR_DEV_GENT, IKR_ERR_ARG, "unknown deviatoric function");
    need(h->volumetric >= 0 && h->volumetric <= 12, IKR_ERR_ARG, "unknown volumetric function");
    const bool terms = h->deviatoric == IKR_DEV_OGDEN_TOTAL || h->deviatoric == IKR_DEV_OGDEN_DEVIATORIC ||
                       h->deviatoric == IKR_DEV_INVARIANT_BASED;
    need(!terms || (h->n_terms >= 1 && h->n_terms <= IKR_HYPER_MAX_TERMS), IKR_ERR_ARG, "n_terms out of range");
    if (h->deviatoric == IKR_DEV_INVARIANT_BASED)
      for (int i = 0; i < h->n_terms; ++i) {
        need(h->p[i] >= 0 && h->q[i] >= 0, IKR_ERR_ARG, "negative invariant exponent");
        if (h->p[i] == 0 && h->q[i] == 0)
          fail(IKR_ERR_ARG, "The exponent q%d and the exponent p%d should not be zero at the same time.", i, i);
      }
    if (h->deviatoric == IKR_DEV_OGDEN_TOTAL || h->deviatoric == IKR_DEV_OGDEN_DEVIATORIC)
      for (int i = 0; i < h->n_terms; ++i) need(h->alpha[i] != 0.0, IKR_ERR_ARG, "Ogden exponent zero");
    need(!(h->deviatoric == IKR_DEV_ARRUDA_BOYCE || h->deviatoric == IKR_DEV_GENT) || h->param > 0.0, IKR_ERR_ARG,
         "lambdaM / Jm must be positive");
    ikr::HyperParams hp;
    hp.dev = h->deviatoric;
    hp.n = terms ? h->n_terms : 1;
    for (int i = 0; i < ikr::kHyperMaxTerms; ++i) {
      hp.mu[i] = h->mu[i];
      hp.alpha[i] = h->alpha[i];
      hp.p[i] = h->p[i];
      hp.q[i] = h->q[i];
    }
    hp.param = h->param;
    hp.vol = h->volumetric;
    hp.K = h->K;
    hp.beta = h->beta;
    fes->hyper = hp;
    fes->material = IKR_MATERIAL_HYPERELASTIC;
    fes->alpha_version++;
  });
}
int ikr_fes_kernel_info(ikr_fes fes, int32_t* epb_residual, int32_t* epb_tangent64, int32_t* epb_tangent32) {
  return guarded([&] {
    need(fes, IKR_ERR_ARG, "null argument");
    if (epb_residual) *epb_residual = fes->epb_r;
    if (epb_tangent64) *epb_tangent64 = fes->epb_k64;
    if (epb_tangent32) *epb_tangent32 = fes->epb_k32;
  });
}
int ikr_cg_kind_ranges(int32_t* out4) {
  return guarded([&] {
    need(out4, IKR_ERR_ARG, "null argument");
    out4[0] = 1;
    out4[1] = ikr_ls_s::first_persistent_kind();
    out4[2] = ikr_ls_s::first_coarse_kind();
    out4[3] = out4[2] + ikr::pcg_coarse_variants();
  });
}
int ikr_linear_solver_set_kernel(ikr_ls ls, int32_t kind, double keep) {
  return guarded([&] {
    need(ls && kind >= -1 && kind <= ikr::spmv_staged_variants() + ikr::pcg_persistent_variants() + ikr::pcg_coarse_variants() &&
             (keep == -1.0 || (keep >= 0.0 && keep < 1.0)),
         IKR_ERR_ARG, "invalid SpMV kernel choice");
    ls->set_kernel(kind, keep);
  });
}
int ikr_assembler_set_tangent_kernel(ikr_asm a, int32_t path) {
  return guarded([&] {
    need(a && path >= 0 && path <= 3, IKR_ERR_ARG,
         "tangent kernel: 0 timed choice, 1 coloured, 2 rows, 3 element blocks + gather");
    a->tan_req = path;
    a->tan_path = path;
  });
}
int ikr_assembler_tangent_kernel(ikr_asm a, int32_t* path) {
  return guarded([&] {
    need(a && path, IKR_ERR_ARG, "null argument");
    *path = a->tan_path;
  });
}
int ikr_linear_solver_set_multi_rhs(ikr_ls ls, int32_t on) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    ls->multi_rhs = on != 0;
  });
}
int ikr_linear_solver_set_coarse_space(ikr_ls ls, int32_t n_slabs) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    need(n_slabs >= 0 && 6 * n_slabs <= ikr::kCoarseMaxDofs, IKR_ERR_ARG, "coarse slabs must be in [0, 128]");
    need(n_slabs == 0 || ls->tag == IKR_SOLVER_GPU_PCG_BLOCK_JACOBI || ls->direct, IKR_ERR_NOT_IMPLEMENTED,
         "the coarse correction is a preconditioner of the block-Jacobi GPU CG");
    if (n_slabs != ls->coarse_req) {
      ls->coarse_req = n_slabs;
      ls->tuned_for = nullptr;  // the kind is chosen again (two-kernel forms only with a coarse correction)
      ls->factorized = false;
      ls->drop_graphs();
      ls->co.built_for = nullptr;
      ls->w.coarse = 0;
    }
  });
}
int ikr_linear_solver_set_coarse_refresh(ikr_ls ls, int32_t every) {
  return guarded([&] {
    need(ls && every >= 1, IKR_ERR_ARG, "the coarse operator is rebuilt every n >= 1 factorizations");
    ls->coarse_refresh = every;
  });
}
int ikr_linear_solver_coarse_info(ikr_ls ls, int32_t* out4) {
  return guarded([&] {
    need(ls && out4, IKR_ERR_ARG, "null argument");
    const bool on = ls->w.coarse != 0;
    out4[0] = on ? ls->co.n_slabs : 0;
    out4[1] = on ? 6 * ls->co.n_slabs : 0;
    out4[2] = on ? ls->co.dropped : 0;
    out4[3] = on ? ls->co.n_colours : 0;
  });
}
int ikr_linear_solver_kernel_info(ikr_ls ls, int32_t* kind, double* keep, double* us) {
  return guarded([&] {
    need(ls, IKR_ERR_ARG, "null argument");
    if (kind) *kind = ls->w.spmv_kind;
    if (keep) *keep = ls->keep_frac;
    if (us) *us = ls->tuned_us;
  });
}
// Allocation-free variant of the solve: the CG work set is carved out of the library's fixed device array
// (noalloc.cu) instead of cudaMalloc'ed buffers; no graphs, events or pinned buffers either, the host polls
// the device scalars with a plain copy into a static host array after every 32 iterations.
static_assert(ikr::kNoAllocMaxRows >= IKR_NOALLOC_MAX_NODES,
              "the fixed scratch of noalloc.cu must hold the largest system the entry point accepts");
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
    if (iterations) *iterations = (int32_t)sc[ikr::kIters];
    if (sc[ikr::kDone] == 3.0) fail(IKR_ERR_CG_BREAKDOWN, "CG breakdown (p.Kp zero or not finite)");
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
    s->max_backtracks = 0;
    s->step_graphs = 1;
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

}  // extern "C"

namespace ikr_host {
// the inhomogeneous Dirichlet values at the requirement's load factor (nonlinearsolverfactory.hh:45-52)
void idbc_sync(ikr_asm a, ikr_req r) {
  if (a->idbc_value) {  // the value function at this load factor; entries that are nonzero are imposed
    if (!a->idbc_vals_valid || a->idbc_vals_lambda != r->lambda) {
      std::vector<double> v(a->n, 0.0);
      a->idbc_value(a->fes->nn, a->fes->X_h.data(), r->lambda, v.data(), a->idbc_user);
      a->idbc_vals.upload(v.data(), v.size(), a->fes->stream);
      CK(cudaStreamSynchronize(a->fes->stream));
      a->idbc_vals_lambda = r->lambda;
      a->idbc_vals_valid = true;
    }
    ikr::launch_idbc_sync(r->u.p, a->idbc_vals.p, 1.0, 3LL * a->fes->nn, a->fes->stream);
    count(1);
    r->version++;
    return;
  }
  ikr::launch_idbc_sync(r->u.p, a->idbc_rate.p, r->lambda, 3LL * a->fes->nn, a->fes->stream);
  count(1);
  r->version++;
}

void nr_solve(ikr_nr nr, ikr_req r, double step_size, ikr_nr_info* info, double ref_norm) {
  if (nr->asm_->fes->n_inst > 0 && nr->ls->tag == IKR_SOLVER_GPU_PCG_BATCHED) {
    need(nr->asm_->fes->na == 0, IKR_ERR_NOT_IMPLEMENTED, "the batched solve supports displacement-based elements");
    need(!nr->asm_->has_idbc, IKR_ERR_NOT_IMPLEMENTED, "the batched solve has no inhomogeneous Dirichlet values");
    nr_solve_batched(nr, r, info);
    return;
  }
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
  bool k_valid = false;
  if (a->has_idbc && step_size != 0.0) {
    // rx += idbcForce(x) * stepSize (newtonraphson.hh:212-215): obtainForcesDueToIDBC (functionhelper.hh:170-184)
    // = K_raw du_D/dlambda, zero at the constrained dofs
    assemble_matrix(a, r, IKR_DBC_RAW);
    a->idbc_force.alloc(n);
    ikr::launch_spmv64(a->bsr(), a->fp32, a->idbc_rate.p, a->idbc_force.p, f->stream);
    ikr::launch_idbc_force(a->R.p, a->idbc_force.p, a->node_fixed.p, step_size, n, f->stream);
    count(2);
  }
  double rnorm = device_norm(f, a->R.p, n, nr->nrm_part, nr->nrm_out);
  inf.residual_norm = rnorm;
  const double thr = st.tol_mode == 1 ? st.tol * (ref_norm > 0.0 ? ref_norm : rnorm) : st.tol;
  if (!a->nb) a->build_pattern();
  nr->ls->setup(a);
  int iter = 0;
  double rprev = rnorm;
  int64_t lin = 0;
  while ((rnorm > thr && iter < st.max_iter) || iter < st.min_iter) {
    notify(IKR_NLS_ITERATION_STARTED);
    // linear tolerance: fixed, or Eisenstat-Walker (choice 2) bounded by the accuracy this step needs
    double eta = st.linear_rtol;
    if (st.forcing == 1) {
      double ew = iter == 0 ? st.linear_rtol : 0.9 * (rnorm / rprev) * (rnorm / rprev);
      ew = std::min(ew, st.linear_rtol);
      const double need_eta = 0.5 * thr / std::max(rnorm, 1e-300);
      eta = std::max(std::max(ew, need_eta), st.linear_rtol_min);
      eta = std::min(eta, st.linear_rtol);
    }
    if (nr->ls->direct) eta = std::min(eta, nr->ls->rtol);
    // the whole iteration as one CUDA graph launch where the configuration allows it (newton_graph.cpp)
    if (!k_valid && step_graph_eligible(nr, r)) {
      double cnorm = 0.0, rnew = 0.0;
      const int64_t its = step_graph_iteration(nr, r, eta, &cnorm, &rnew);
      if (its >= 0) {
        lin += its;
        inf.correction_norm = cnorm;
        notify(IKR_NLS_CORRECTION_UPDATED);
        notify(IKR_NLS_CORRECTIONNORM_UPDATED);
        notify(IKR_NLS_SOLUTION_CHANGED);
        rprev = rnorm;
        rnorm = rnew;
        inf.residual_norm = rnorm;
        notify(IKR_NLS_RESIDUALNORM_UPDATED);
        ++iter;
        inf.iterations = iter;
        notify(IKR_NLS_ITERATION_ENDED);
        if (!std::isfinite(rnorm)) break;
        continue;
      }
    }
    if (!k_valid) {
      assemble_matrix(a, r, IKR_DBC_FULL);
      k_valid = true;
    }
    nr->ls->factorize(a);
    ikr::launch_scale64(nr->rhs.p, a->R.p, -1.0, n, f->stream);
    count(1);
    lin += nr->ls->solve(a, nr->rhs.p, nr->corr.p, eta, st.linear_max_iter, st.refinements);
    inf.correction_norm = device_norm(f, nr->corr.p, n, nr->nrm_part, nr->nrm_out);
    notify(IKR_NLS_CORRECTION_UPDATED);
    const bool eas_state = nr->fe_state && f->na > 0;
    if (st.max_backtracks > 0) {  // keep the state the correction starts from
      nr->u_old.alloc(n);
      CK(cudaMemcpyAsync(nr->u_old.p, r->u.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, f->stream));
      if (eas_state) {
        nr->alpha_old.alloc(f->alpha.n);
        CK(cudaMemcpyAsync(nr->alpha_old.p, f->alpha.p, sizeof(double) * f->alpha.n, cudaMemcpyDeviceToDevice,
                           f->stream));
      }
    }
    for (int bt = 0;; ++bt) {
      if (nr->fe_state) update_state(f, r, nr->corr.p);
      ikr::launch_axpy64(r->u.p, nr->corr.p, 1.0, n, f->stream);
      count(1);
      if (a->has_idbc) idbc_sync(a, r);  // syncParameterAndGlobalSolution (newtonraphson.hh:235-236)
      r->version++;
      try {
        assemble_vector(a, r, IKR_DBC_FULL);
        break;
      } catch (const IkrError& e) {
        if (e.code != IKR_ERR_NONPOSITIVE_DETC || bt >= st.max_backtracks) throw;
        // the corrected state inverts an element: go back and take half the step
        CK(cudaMemcpyAsync(r->u.p, nr->u_old.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, f->stream));
        if (eas_state) {
          CK(cudaMemcpyAsync(f->alpha.p, nr->alpha_old.p, sizeof(double) * f->alpha.n, cudaMemcpyDeviceToDevice,
                             f->stream));
          f->alpha_version++;
        }
        ikr::launch_scale64(nr->corr.p, nr->corr.p, 0.5, n, f->stream);
        count(1);
        r->version++;
        inf.correction_norm *= 0.5;
        ++nr->backtracks;
      }
    }
    notify(IKR_NLS_CORRECTIONNORM_UPDATED);
    notify(IKR_NLS_SOLUTION_CHANGED);
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
}  // namespace ikr_host

extern "C" {

int ikr_newton_instance_linear_iterations(ikr_nr nr, int64_t* cg_iterations) {
  return guarded([&] {
    need(nr && cg_iterations, IKR_ERR_ARG, "null argument");
    for (size_t i = 0; i < nr->inst_lin.size(); ++i) cg_iterations[i] = nr->inst_lin[i];
  });
}
int ikr_newton_set_batched_cg(ikr_nr nr, int32_t variant, int32_t first_chunk) {
  return guarded([&] {
    need(nr && first_chunk >= 0 && variant >= -1 && variant <= 5, IKR_ERR_ARG, "invalid argument");
    nr->plan.variant = variant;
    nr->plan.first_chunk = first_chunk ? first_chunk : 128;
  });
}
int ikr_newton_batched_cg_launches(ikr_nr nr, int64_t* n) {
  return guarded([&] {
    need(nr && n, IKR_ERR_ARG, "null argument");
    *n = nr->plan.launches;
  });
}
int ikr_newton_batched_cg_variant_launches(ikr_nr nr, int64_t* by_variant6) {
  return guarded([&] {
    need(nr && by_variant6, IKR_ERR_ARG, "null argument");
    for (int v = 0; v < 6; ++v) by_variant6[v] = nr->plan.launches_by_variant[v];
  });
}
int ikr_newton_set_batched_take_out(ikr_nr nr, int32_t unsolved_linear) {
  return guarded([&] {
    need(nr, IKR_ERR_ARG, "null argument");
    nr->take_out_unsolved = unsolved_linear != 0;
  });
}
int ikr_load_control_set_escalation(ikr_lc lc, ikr_nr nr64, ikr_req req64) {
  return guarded([&] {
    need(lc, IKR_ERR_ARG, "null argument");
    need((nr64 == nullptr) == (req64 == nullptr), IKR_ERR_ARG, "give both the solver and its requirement, or neither");
    if (nr64) {
      ikr_fes f = lc->nr->asm_->fes, g = nr64->asm_->fes;
      need(f->n_inst > 0 && g->n_inst == f->n_inst && g->nn == f->nn && g->inst_off_h == f->inst_off_h, IKR_ERR_ARG,
           "the escalation solver needs an element set with the same instances");
      need(req64->fes == g, IKR_ERR_ARG, "requirement of another element set");
      need(nr64 != lc->nr, IKR_ERR_ARG, "the escalation solver must be another solver");
    }
    lc->esc_nr = nr64;
    lc->esc_req = req64;
  });
}
int ikr_load_control_set_escalation_concurrent(ikr_lc lc, int32_t on) {
  return guarded([&] {
    need(lc, IKR_ERR_ARG, "null argument");
    lc->esc_concurrent = on != 0;
  });
}
int ikr_load_control_instance_status(ikr_lc lc, int32_t n, int32_t* status) {
  return guarded([&] {
    need(lc && status, IKR_ERR_ARG, "null argument");
    const auto& conv = lc->nr->inst_conv;
    for (int i = 0; i < n; ++i) {
      const bool esc = i < (int)lc->escalated.size() && lc->escalated[i];
      status[i] = esc ? lc->esc_conv[i] : (i < (int)conv.size() ? conv[i] : 0);
    }
  });
}
int ikr_load_control_escalated(ikr_lc lc, int32_t n, uint8_t* mask) {
  return guarded([&] {
    need(lc && mask, IKR_ERR_ARG, "null argument");
    for (int i = 0; i < n; ++i) mask[i] = i < (int)lc->escalated.size() ? lc->escalated[i] : 0;
  });
}
int ikr_newton_exclude_instances(ikr_nr nr, int32_t n, const uint8_t* mask) {
  return guarded([&] {
    need(nr && n >= 0 && (n == 0 || mask), IKR_ERR_ARG, "invalid argument");
    need(n == 0 || n == nr->asm_->fes->n_inst, IKR_ERR_ARG, "one mask entry per instance");
    nr->inst_excluded.assign(mask, mask + n);
  });
}
int ikr_newton_solve(ikr_nr nr, ikr_req r, double step_size, ikr_nr_info* info) {
  return guarded([&] {
    need(nr && r, IKR_ERR_ARG, "null argument");
    nr->inst_failed.clear();
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
    ikr_control_state cs{r, -1, 0.0, r->lambda, 0, "Load Control Method"};  // loadcontrol.hh:63
    auto notify = [&](int msg) {
      cs.load_factor = r->lambda;
      for (auto& o : lc->obs) o.cb(msg, &cs, o.user);
    };
    auto record = [&](const ikr_nr_info& ni) {
      if (infos && ci.n_solver_infos < capacity) infos[ci.n_solver_infos] = ni;
      ci.n_solver_infos++;
      ci.total_iterations += ni.iterations;
      ci.total_linear_iterations += ni.linear_iterations;
      cs.total_iterations = ci.total_iterations;
      notify(IKR_CONTROL_SOLUTION_CHANGED);
      notify(IKR_STEP_ENDED);
    };
    notify(IKR_CONTROL_STARTED);
    notify(IKR_STEP_STARTED);
    ikr_nr_info ni{};
    lc->nr->inst_failed.clear();
    nr_solve(lc->nr, r, 0.0, &ni);  // equilibrium check at the initial load factor (loadcontrol.inl:29-34)
    const bool esc = lc->esc_nr && r->fes->n_inst > 0;
    if (esc) escalation_begin(lc, r);
    record(ni);
    if (ni.success) {
      cs.step_size = step;
      bool ok = true;
      predictor_begin(lc, r);
      for (int ls = 0; ls < lc->steps; ++ls) {
        cs.load_step = ls;
        notify(IKR_STEP_STARTED);
        r->lambda += step;  // LoadControl::predictor (loadcontrol.inl:54-57)
        if (esc) {
          lc->u_start.alloc(r->u.n);
          CK(cudaMemcpyAsync(lc->u_start.p, r->u.p, sizeof(double) * r->u.n, cudaMemcpyDeviceToDevice, r->fes->stream));
        }
        const double ref = predictor_apply(lc, r, ls);  // optional displacement prediction, FP64-gated
        if (esc) escalated_step(lc, r, step, ref, ni);
        else nr_solve(lc->nr, r, step, &ni, ref);
        if (ni.iterations == 0 && lc->nr->asm_->has_idbc) idbc_sync(lc->nr->asm_, r);  // loadcontrol.inl:43-44
        predictor_end_step(lc, r, ls);
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
