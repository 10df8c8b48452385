// Persistent block-Jacobi PCG: a whole CG solve in one cooperative launch (sm_103a).
//
// Same iteration as the two-kernel CG of solver.cu / spmv_staged.cu (p_new = z + beta p_old formed on the fly
// for every gathered neighbour, q = K p_new, alpha = rz / p.q, x += alpha p, r -= alpha q, z = M^{-1} r,
// beta = rz_new / rz), but every CTA stays resident for all iterations and the two global reductions of an
// iteration are grid barriers:
//   * each warp owns up to MAXS slices (32 block rows each) and keeps x, r, z, p and q of its rows in registers,
//     so the update phase touches global memory only to publish z (and p_new in the product phase), which the
//     neighbours' gathers need;
//   * the matrix is streamed with the same per-warp bulk-copy pipeline as the staged SpMV; the stream of a
//     warp's chunks is cyclic over iterations, so the copies of the next iteration's first chunks are in flight
//     while the CTA waits at the barriers;
//   * a grid barrier publishes one partial per CTA (double-buffered by iteration parity), arrives on a counter
//     and waits until every CTA has arrived; every CTA then sums all partials in CTA order, so alpha, beta and
//     the convergence decision are bit-identical in all CTAs and from run to run.
// The launch is cooperative (all CTAs co-resident).  Every wait is bounded: a grid barrier or stage wait that
// gives up sets scal[kDone] = 6, the kernel drains its copies in flight (bounded) and returns.
#include <mutex>

#include "cg_grid.cuh"

namespace ikr {

namespace {

using namespace cg;

// The block-Jacobi inverses of a CTA's rows in shared memory for the whole solve (they do not change within it), so
// that the update phase after the first grid barrier of an iteration reads them without an L2 round trip -- where
// they fit beside the staging buffers.
template <typename T, int CB, int NST, int WARPS, int MAXS>
struct MinvShared {
  static constexpr int kBytes = WARPS * MAXS * 32 * 9 * (int)sizeof(T);
  static constexpr bool kOn = PersistentCfg<T, CB, NST, WARPS>::kSmemBytes + kBytes <= 200 * 1024;
  static constexpr int kDynBytes = PersistentCfg<T, CB, NST, WARPS>::kSmemBytes + (kOn ? kBytes : 0);
};

// the right-hand sides one launch solves together: per RHS its solution, residual, preconditioned residual, the
// two search-direction buffers (alternating by iteration parity) and its scalar block
template <typename T, int NR>
struct RhsSet {
  T* x[NR];
  const T* r[NR];
  T* z[NR];
  T* p0[NR];
  T* p1[NR];
  double* scal[NR];
};

// NR right-hand sides with the same matrix: every chunk of the matrix stream is staged once and multiplied
// against each unfinished RHS, so two solves cost one matrix stream per iteration instead of two.  Each RHS
// keeps its own CG scalars, iteration count and stop decision; the grid reductions carry the NR values together.
template <typename T, int CB, int NST, int WARPS, int MAXS, int MINB, int NR>
__global__ void __launch_bounds__(WARPS * 32, MINB)
    pcg_persistent_kernel(Bsr A, const T* __restrict__ val, const T* __restrict__ minv, RhsSet<T, NR> V,
                          double* part_a, double* part_b, int64_t keep_g, WaitCtl wc) {
  using C = PersistentCfg<T, CB, NST, WARPS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[WARPS][NST];
  __shared__ double sv[2 * NR];
  __shared__ T s_alpha[NR], s_tb[NR];
  __shared__ int s_dn[NR];
  __shared__ double sfull[2 * NR * WARPS * 32];
  __shared__ bool ok_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G = gridDim.x;
  const int nw = G * WARPS;
  const int gw = blockIdx.x * WARPS + warp;
  const int n_slices = A.n_slices;
  unsigned int* bar_count = &tickets(V.scal[0])[3];
  unsigned char* wbase = smem + (size_t)warp * NST * C::kStageBytes;

  // owned slices and their block ranges
  int ns = 0;
  int s_first[MAXS], s_end[MAXS];
#pragma unroll
  for (int j = 0; j < MAXS; ++j) {
    const int sj = gw + j * nw;
    s_first[j] = 0, s_end[j] = 0;
    if (sj < n_slices) {
      s_first[j] = A.slice_off[sj];
      s_end[j] = A.slice_off[sj + 1];
      ns = j + 1;
    }
  }
  // CG state of the owned rows, per RHS.  With one RHS x, r, z, p and q of the owned rows live in registers;
  // with several (kLean) only r and q do, and x, z, p of the owned rows are re-read from the global vectors
  // (which the gathers need anyway; own-row reads hit L2) to keep the register count without spills.
  constexpr bool kLean = NR > 1;
  constexpr int XS = kLean ? 1 : MAXS;
  T xr[NR][XS][3], rr_[NR][MAXS][3], zr[NR][XS][3], pr[NR][XS][3], qr[NR][MAXS][3];
  // The CG scalars are FP64 and thread 0 alone updates them (rz, r.r, beta, the stop decision); the other threads
  // get the state code, alpha and beta in the CG's type through shared memory (GB300's FP64 pipe is narrow: 512
  // threads repeating the divisions, comparisons and conversions cost microseconds per iteration)
  double rz[NR], tol2[NR], rrs[NR], beta[NR];
  int maxit[NR], it[NR], dn[NR];  // dn: 0 running, 1 converged, 2 iteration cap, 3 breakdown (as scal[kDone])
  T tbv[NR];
  bool all_done = true;
#pragma unroll
  for (int q = 0; q < NR; ++q) {
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      const int row = 32 * (gw + j * nw) + lane;
      const bool own = j < ns && row < A.n_rows;
      V3<T> r0 = {T(0), T(0), T(0)}, z0 = {T(0), T(0), T(0)};
      if (own) r0 = load3rw(V.r[q], row), z0 = load3rw(V.z[q], row);
#pragma unroll
      for (int c = 0; c < 3; ++c) qr[q][j][c] = T(0);
      rr_[q][j][0] = r0.x, rr_[q][j][1] = r0.y, rr_[q][j][2] = r0.z;
      if constexpr (!kLean) {
#pragma unroll
        for (int c = 0; c < 3; ++c) xr[q][j][c] = pr[q][j][c] = T(0);
        zr[q][j][0] = z0.x, zr[q][j][1] = z0.y, zr[q][j][2] = z0.z;
      }
    }
    const double* sc = V.scal[q];
    rz[q] = sc[kRz];
    tol2[q] = sc[kTol2];
    maxit[q] = (int)sc[kMaxIt];
    rrs[q] = sc[kRR];
    dn[q] = (int)sc[kDone];
    it[q] = (int)sc[kIters];
    beta[q] = 0.0;
    tbv[q] = T(0);
    all_done = all_done && dn[q] != 0;
  }

  using MS = MinvShared<T, CB, NST, WARPS, MAXS>;
  T* msh = reinterpret_cast<T*>(smem + C::kSmemBytes);  // used when MS::kOn
  if constexpr (MS::kOn) {
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      const int row = 32 * (gw + j * nw) + lane;
      T* d = msh + ((size_t)(warp * MAXS + j) * 32 + lane) * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) d[k] = (j < ns && row < A.n_rows) ? __ldg(minv + 9 * (int64_t)row + k) : T(0);
    }
  }
  auto minv_of = [&](int j, int row) -> const T* {
    if constexpr (MS::kOn) return msh + ((size_t)(warp * MAXS + j) * 32 + lane) * 9;
    return minv + 9 * (int64_t)row;
  };

  if (lane == 0) {
    for (int st = 0; st < NST; ++st) mbar_init(smem_addr(&bars[warp][st]), 1);
    mbar_init_fence();
  }
  __syncwarp();

  auto issue = [&](int st, const CyclicPos& P) {
    if (lane == 0) {
      const int nb = min(CB, P.gend - P.g);
      const uint32_t vb = nb * 288 * (uint32_t)sizeof(T), cb = nb * 128;
      const uint32_t b = smem_addr(&bars[warp][st]);
      unsigned char* stage = wbase + (size_t)st * C::kStageBytes;
      const uint64_t pol = l2_policy(P.g < keep_g);
      mbar_expect_tx(b, vb + cb);
      bulk_g2s(smem_addr(stage), val + (int64_t)P.g * 288, vb, b, pol);
      bulk_g2s(smem_addr(stage + C::kValBytes), A.col_sell + (int64_t)P.g * 32, cb, b, pol);
    }
  };
  auto advance = [&](CyclicPos& P) {
    P.g += CB;
    if (P.g >= P.gend) {
      P.j = (P.j + 1 == ns) ? 0 : P.j + 1;
      // s_first / s_end are indexed with a runtime j here: pick through an unrolled select
#pragma unroll
      for (int j = 0; j < MAXS; ++j)
        if (j == P.j) P.g = s_first[j], P.gend = s_end[j];
    }
  };

  CyclicPos P{0, s_first[0], s_end[0]};
  int inflight = 0;
  if (ns > 0 && !all_done) {
    for (int st = 0; st < NST; ++st) {
      issue(st, P);
      ++inflight;
      advance(P);
    }
  }
  uint32_t phase = 0;
  int st = 0;
  bool failed = false;
  unsigned int barrier_no = 0;
  int loop = 0;  // parity of the partial buffers

  while (!all_done) {
    T tb[NR];
    const T* pold[NR];
    T* pnew[NR];
    bool act[NR];
    double pq[NR];
    T pql[NR];  // a lane's p.q in the CG's type, converted once
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      act[q] = dn[q] == 0;
      tb[q] = tbv[q];
      pold[q] = (it[q] & 1) ? V.p0[q] : V.p1[q];
      pnew[q] = (it[q] & 1) ? V.p1[q] : V.p0[q];
      pq[q] = 0.0;
      pql[q] = T(0);
    }
    // ---- product phase: q = K p_new over the owned slices, every active RHS from the same staged chunk
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      if (j < ns && !failed) {
        T acc[NR][3];
#pragma unroll
        for (int q = 0; q < NR; ++q) acc[q][0] = acc[q][1] = acc[q][2] = T(0);
        for (int g = s_first[j]; g < s_end[j]; g += CB) {
          const bool okw = __all_sync(0xffffffffu, mbar_wait_bounded(smem_addr(&bars[warp][st]), (phase >> st) & 1u));
          if (!okw) {
            failed = true;
            break;
          }
          phase ^= 1u << st;
          --inflight;
          const T* sval = reinterpret_cast<const T*>(wbase + (size_t)st * C::kStageBytes);
          const int32_t* scol = reinterpret_cast<const int32_t*>(wbase + (size_t)st * C::kStageBytes + C::kValBytes);
          const int nb = min(CB, s_end[j] - g);
          int cols[CB];
#pragma unroll
          for (int k = 0; k < CB; ++k) cols[k] = k < nb ? scol[32 * k + lane] : 0;
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            if (!act[q]) continue;
            V3<T> zc[CB], pc[CB];
#pragma unroll
            for (int k = 0; k < CB; ++k) {
              zc[k] = load3rw(V.z[q], cols[k]);
              pc[k] = load3rw(pold[q], cols[k]);
            }
#pragma unroll
            for (int k = 0; k < CB; ++k) {
              if (k < nb) {
                const T x0 = zc[k].x + tb[q] * pc[k].x, x1 = zc[k].y + tb[q] * pc[k].y,
                        x2 = zc[k].z + tb[q] * pc[k].z;
                const T* v = sval + 288 * k + lane;
                acc[q][0] += v[0] * x0 + v[32] * x1 + v[64] * x2;
                acc[q][1] += v[96] * x0 + v[128] * x1 + v[160] * x2;
                acc[q][2] += v[192] * x0 + v[224] * x1 + v[256] * x2;
              }
            }
          }
          __syncwarp();  // the stage is consumed before it is refilled
          issue(st, P);
          ++inflight;
          advance(P);
          st = (st + 1 == NST) ? 0 : st + 1;
        }
        const int row = 32 * (gw + j * nw) + lane;
#pragma unroll
        for (int q = 0; q < NR; ++q) {
          if (!act[q]) continue;
          V3<T> zo, po;
          if constexpr (kLean) {
            zo = {T(0), T(0), T(0)}, po = {T(0), T(0), T(0)};
            if (row < A.n_rows) zo = load3rw(V.z[q], row), po = load3rw(pold[q], row);
          } else {
            zo = {zr[q][j][0], zr[q][j][1], zr[q][j][2]};
            po = {pr[q][j][0], pr[q][j][1], pr[q][j][2]};
          }
          const T n0 = zo.x + tb[q] * po.x, n1 = zo.y + tb[q] * po.y, n2 = zo.z + tb[q] * po.z;
          if constexpr (!kLean) pr[q][j][0] = n0, pr[q][j][1] = n1, pr[q][j][2] = n2;
          qr[q][j][0] = acc[q][0], qr[q][j][1] = acc[q][1], qr[q][j][2] = acc[q][2];
          if (row < A.n_rows) {
            store3(pnew[q], row, n0, n1, n2);
            pql[q] += n0 * acc[q][0] + n1 * acc[q][1] + n2 * acc[q][2];
          }
        }
      }
    }
    // ---- grid reduction of p.q (all RHS together)
    const int par = loop & 1;
    failed = __syncthreads_or(failed);
    if (failed) break;
#pragma unroll
    for (int q = 0; q < NR; ++q) pq[q] = double(pql[q]);
    cta_reduce_smem<NR>(pq, sfull);
    ++barrier_no;
    if (!grid_allreduce<NR>(pq, part_a + par * NR * G, bar_count, barrier_no * (unsigned)G, sv, &ok_sh, wc)) {
      failed = true;
      break;
    }
    if (threadIdx.x == 0) {
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        T a = T(0);
        if (dn[q] == 0) {
          if (!(fabs(pq[q]) > 0.0) || !isfinite(pq[q])) dn[q] = 3;  // breakdown (negative curvature alone does not stop CG)
          else a = T(rz[q] / pq[q]);
        }
        s_alpha[q] = a;
        s_dn[q] = dn[q];
      }
    }
    __syncthreads();
    T alpha[NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      alpha[q] = s_alpha[q];
      dn[q] = s_dn[q];
      act[q] = dn[q] == 0;
    }
    // ---- update phase on the owned rows
    double red2[2 * NR];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      // a lane's rows are summed in the CG's type and converted once (FP64 additions and conversions per row would
      // load GB300's narrow FP64 pipe); the CTA and grid sums above them are FP64
      T lrz = T(0), lrr = T(0);
      if (act[q]) {
        const T a = alpha[q];
#pragma unroll
        for (int j = 0; j < MAXS; ++j) {
          const int row = 32 * (gw + j * nw) + lane;
          if (j < ns && row < A.n_rows) {
            T r1[3];
            if constexpr (kLean) {
              const V3<T> pv = load3rw(pnew[q], row);
              const V3<T> xv = load3rw(V.x[q], row);
              store3(V.x[q], row, xv.x + a * pv.x, xv.y + a * pv.y, xv.z + a * pv.z);
            } else {
#pragma unroll
              for (int c = 0; c < 3; ++c) xr[q][j][c] += a * pr[q][j][c];
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              r1[c] = rr_[q][j][c] - a * qr[q][j][c];
              rr_[q][j][c] = r1[c];
            }
            const T* m = minv_of(j, row);
            T zv[3];
#pragma unroll
            for (int b = 0; b < 3; ++b) {
              zv[b] = m[3 * b] * r1[0] + m[3 * b + 1] * r1[1] + m[3 * b + 2] * r1[2];
              if constexpr (!kLean) zr[q][j][b] = zv[b];
            }
            store3(V.z[q], row, zv[0], zv[1], zv[2]);
            T trz = T(0), trr = T(0);
#pragma unroll
            for (int b = 0; b < 3; ++b) {
              trz += r1[b] * zv[b];
              trr += r1[b] * r1[b];
            }
            lrz += trz;
            lrr += trr;
          }
        }
      }
      red2[2 * q] = double(lrz);
      red2[2 * q + 1] = double(lrr);
    }
    cta_reduce_smem<2 * NR>(red2, sfull);
    ++barrier_no;
    if (!grid_allreduce<2 * NR>(red2, part_b + par * 2 * NR * G, bar_count, barrier_no * (unsigned)G, sv, &ok_sh,
                                wc)) {
      failed = true;
      break;
    }
    if (threadIdx.x == 0) {
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        if (act[q]) {
          const double rzs = red2[2 * q];
          rrs[q] = red2[2 * q + 1];
          beta[q] = rzs / rz[q];
          rz[q] = rzs;
          if (rrs[q] <= tol2[q]) dn[q] = 1;
          else if (it[q] + 1 >= maxit[q]) dn[q] = 2;
        }
        s_tb[q] = T(beta[q]);
        s_dn[q] = dn[q];
      }
    }
    __syncthreads();
    all_done = true;
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      if (act[q]) ++it[q];
      dn[q] = s_dn[q];
      tbv[q] = s_tb[q];
      all_done = all_done && dn[q] != 0;
    }
    ++loop;
  }
  // drain the copies still in flight (the cyclic stream runs ahead of the last iteration)
  for (int k = 0; k < inflight; ++k) {
    mbar_wait_bounded(smem_addr(&bars[warp][st]), (phase >> st) & 1u);
    phase ^= 1u << st;
    st = (st + 1 == NST) ? 0 : st + 1;
  }
  // solutions of the owned rows; the final scalars from CTA 0 (identical in every CTA)
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    if constexpr (!kLean) {
#pragma unroll
      for (int j = 0; j < MAXS; ++j) {
        const int row = 32 * (gw + j * nw) + lane;
        if (j < ns && row < A.n_rows) store3(V.x[q], row, xr[q][j][0], xr[q][j][1], xr[q][j][2]);
      }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      double* sc = V.scal[q];
      sc[kIters] = (double)it[q];
      sc[kRR] = rrs[q];
      sc[kRz] = rz[q];
      sc[kBeta] = beta[q];
      sc[kDone] = failed ? kDoneDeviceTimeout : (double)dn[q];
    }
    if (failed && threadIdx.x == 0) V.scal[q][kDone] = kDoneDeviceTimeout;
  }
}

template <typename T, int CB, int NST, int WARPS, int MAXS, int MINB, int NR>
cudaError_t launch_persistent(const Bsr& A, PcgWork* const* ws, double* part_a, double* part_b, cudaStream_t s,
                              bool query_only, bool* eligible) {
  using C = PersistentCfg<T, CB, NST, WARPS>;
  constexpr int kDyn = MinvShared<T, CB, NST, WARPS, MAXS>::kDynBytes;
  auto kern = pcg_persistent_kernel<T, CB, NST, WARPS, MAXS, MINB, NR>;
  static std::mutex mu;
  static int blocks_per_sm[64] = {0};
  PcgWork& w = *ws[0];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 64) dev = 63;
  int bps;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!blocks_per_sm[dev]) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kDyn);
      int b = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, C::kThreads, kDyn);
      blocks_per_sm[dev] = b > 0 ? b : -1;
    }
    bps = blocks_per_sm[dev];
  }
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  // one wave of co-resident CTAs; the partial buffers hold 2 NR w.grid (part_a) and 4 NR w.grid (part_b) values,
  // 2 NR and 4 NR per CTA here
  int grid = bps > 0 ? w.sms * bps : 0;
  if (grid > w.grid) grid = w.grid;
  const int nw = grid * WARPS;
  *eligible = coop && grid > 0 && (int64_t)nw * MAXS >= A.n_slices;
  if (query_only || !*eligible) return cudaSuccess;
  const T* val = (const T*)A.val;
  const T* minv = (const T*)w.minv;
  RhsSet<T, NR> V;
  for (int q = 0; q < NR; ++q) {
    V.x[q] = (T*)ws[q]->x;
    V.r[q] = (const T*)ws[q]->r;
    V.z[q] = (T*)ws[q]->z;
    V.p0[q] = (T*)ws[q]->p0;
    V.p1[q] = (T*)ws[q]->p1;
    V.scal[q] = ws[q]->scal;
  }
  Bsr Acopy = A;
  int64_t keep = w.keep_g;
  WaitCtl wc{w.barrier_polls > 0 ? w.barrier_polls : kBarrierSpinLimit, w.withhold_first_arrival};
  void* args[] = {&Acopy, &val, &minv, &V, &part_a, &part_b, &keep, &wc};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(C::kThreads), args, kDyn, s);
}

template <typename T, int NR>
cudaError_t dispatch(int variant, const Bsr& A, PcgWork* const* ws, double* pa, double* pb, cudaStream_t s,
                     bool query, bool* eligible) {
  if constexpr (sizeof(T) == 4) {
    if (variant == 0) return launch_persistent<float, 8, 2, 8, 4, 1, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 1) return launch_persistent<float, 4, 3, 8, 8, 1, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 2) return launch_persistent<float, 4, 2, 8, 2, 2, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 3) return launch_persistent<float, 2, 3, 8, 2, 3, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 4) return launch_persistent<float, 4, 2, 16, 2, 1, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 5) return launch_persistent<float, 4, 2, 12, 3, 1, NR>(A, ws, pa, pb, s, query, eligible);
    return launch_persistent<float, 5, 2, 16, 2, 1, NR>(A, ws, pa, pb, s, query, eligible);
  } else {
    if (variant == 0) return launch_persistent<double, 4, 2, 8, 4, 1, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 1) return launch_persistent<double, 2, 3, 8, 4, 1, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 2) return launch_persistent<double, 2, 2, 8, 2, 2, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 3) return launch_persistent<double, 1, 3, 8, 2, 2, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 4) return launch_persistent<double, 2, 2, 16, 2, 1, NR>(A, ws, pa, pb, s, query, eligible);
    if (variant == 5) return launch_persistent<double, 2, 2, 12, 3, 1, NR>(A, ws, pa, pb, s, query, eligible);
    return launch_persistent<double, 1, 3, 16, 2, 1, NR>(A, ws, pa, pb, s, query, eligible);
  }
}


// ---- one grid reduction per iteration -------------------------------------------------------------------
// The same preconditioned CG rearranged so that an iteration needs one grid-wide reduction instead of two (the
// second reduction is what dominates the fixed cost of an iteration: two grid barriers).  Iteration k of a row
// owner, with alpha_{k-1}, beta_{k-1} from the previous reduction:
//   r_k = r_{k-1} - alpha q_{k-1},  z_k = z_{k-1} - alpha w_{k-1},  x_k = x_{k-1} + alpha p_{k-1},
//   p_k = z_k + beta p_{k-1},  q_k = K p_k,  w_k = M^{-1} q_k,
// where a gathered neighbour's p_k is formed from its stored z_{k-1}, w_{k-1} and p_{k-1} with the same two
// operations, so no barrier is needed between the vector update and the product.  z follows the recurrence
// z_k = z_{k-1} - alpha w_{k-1} (= M^{-1} r_k in exact arithmetic).  The reduction carries p.q, r.w, q.z, q.w,
// r.q, q.q, r.z and r.r of the iterate; then
//   alpha_k = rho_k / p.q,  rho_{k+1} = rho_k - alpha_k (r.w + q.z) + alpha_k^2 q.w,  beta_k = rho_{k+1} / rho_k,
//   |r_{k+1}|^2 = |r_k|^2 - 2 alpha_k r.q + alpha_k^2 q.q,
// with rho_k = r_k.z_k and |r_k|^2 computed from the vectors every iteration (no drift accumulates through the
// recurrences).  Buffers: z, p and w double-buffered by iteration parity (gathers read parity k-1 while the
// owners write parity k).  Dot products accumulate in FP64.
__device__ __forceinline__ float cg1_z(float z, float w, float a) { return z - a * w; }
__device__ __forceinline__ double cg1_z(double z, double w, double a) { return z - a * w; }
__device__ __forceinline__ float cg1_p(float z, float p, float b) { return z + b * p; }
__device__ __forceinline__ double cg1_p(double z, double p, double b) { return z + b * p; }

template <typename T, int CB, int NST, int WARPS, int MAXS, int MINB>
__global__ void __launch_bounds__(WARPS * 32, MINB)
    pcg_onered_kernel(Bsr A, const T* __restrict__ val, const T* __restrict__ minv, T* __restrict__ xg,
                      const T* __restrict__ rg, T* Z0, T* Z1, T* P0, T* P1, T* W0, T* W1, double* part,
                      double* scal, int64_t keep_g) {
  using C = PersistentCfg<T, CB, NST, WARPS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[WARPS][NST];
  __shared__ double sw[WARPS * 8];
  __shared__ double sv[8];
  __shared__ bool ok_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G = gridDim.x;
  const int nw = G * WARPS;
  const int gw = blockIdx.x * WARPS + warp;
  const int n_slices = A.n_slices;
  unsigned int* bar_count = &tickets(scal)[3];
  unsigned char* wbase = smem + (size_t)warp * NST * C::kStageBytes;

  int ns = 0;
  int s_first[MAXS], s_end[MAXS];
#pragma unroll
  for (int j = 0; j < MAXS; ++j) {
    const int sj = gw + j * nw;
    s_first[j] = 0, s_end[j] = 0;
    if (sj < n_slices) {
      s_first[j] = A.slice_off[sj];
      s_end[j] = A.slice_off[sj + 1];
      ns = j + 1;
    }
  }
  // own rows: r, z (from the init kernel: Z1 holds z_0), p = q = w = 0 in registers; x (zero from the init
  // kernel) is updated in place in global memory, which keeps the kernel within its register budget
  T rr_[MAXS][3], zr[MAXS][3], pr[MAXS][3], qr[MAXS][3], wr[MAXS][3];
#pragma unroll
  for (int j = 0; j < MAXS; ++j) {
    const int row = 32 * (gw + j * nw) + lane;
    V3<T> r0 = {T(0), T(0), T(0)}, z0 = {T(0), T(0), T(0)};
    if (j < ns && row < A.n_rows) r0 = load3rw(rg, row), z0 = load3rw(Z1, row);
    rr_[j][0] = r0.x, rr_[j][1] = r0.y, rr_[j][2] = r0.z;
    zr[j][0] = z0.x, zr[j][1] = z0.y, zr[j][2] = z0.z;
#pragma unroll
    for (int c = 0; c < 3; ++c) pr[j][c] = qr[j][c] = wr[j][c] = T(0);
  }
  const double tol2 = scal[kTol2];
  const int maxit = (int)scal[kMaxIt];
  double rrs = scal[kRR], rho = scal[kRz];
  double done = scal[kDone];
  double alpha_p = 0.0, beta_p = 0.0;

  if (lane == 0) {
    for (int st = 0; st < NST; ++st) mbar_init(smem_addr(&bars[warp][st]), 1);
    mbar_init_fence();
  }
  __syncwarp();

  auto issue = [&](int st, const CyclicPos& P) {
    if (lane == 0) {
      const int nb = min(CB, P.gend - P.g);
      const uint32_t vb = nb * 288 * (uint32_t)sizeof(T), cb = nb * 128;
      const uint32_t b = smem_addr(&bars[warp][st]);
      unsigned char* stage = wbase + (size_t)st * C::kStageBytes;
      const uint64_t pol = l2_policy(P.g < keep_g);
      mbar_expect_tx(b, vb + cb);
      bulk_g2s(smem_addr(stage), val + (int64_t)P.g * 288, vb, b, pol);
      bulk_g2s(smem_addr(stage + C::kValBytes), A.col_sell + (int64_t)P.g * 32, cb, b, pol);
    }
  };
  auto advance = [&](CyclicPos& P) {
    P.g += CB;
    if (P.g >= P.gend) {
      P.j = (P.j + 1 == ns) ? 0 : P.j + 1;
#pragma unroll
      for (int j = 0; j < MAXS; ++j)
        if (j == P.j) P.g = s_first[j], P.gend = s_end[j];
    }
  };

  CyclicPos P{0, s_first[0], s_end[0]};
  int inflight = 0;
  if (ns > 0 && done == 0.0) {
    for (int st = 0; st < NST; ++st) {
      issue(st, P);
      ++inflight;
      advance(P);
    }
  }
  uint32_t phase = 0;
  int st = 0;
  bool failed = false;
  int it = (int)scal[kIters];
  unsigned int barrier_no = 0;

  while (done == 0.0) {
    const int par = it & 1;
    const T ta = T(alpha_p), tb = T(beta_p);
    T* Zw = par ? Z1 : Z0;
    const T* Zr = par ? Z0 : Z1;
    T* Pw = par ? P1 : P0;
    const T* Pr = par ? P0 : P1;
    T* Ww = par ? W1 : W0;
    const T* Wr = par ? W0 : W1;
    double red[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // p.q, r.w, q.z, q.w, r.q, q.q, r.z, r.r
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      if (j < ns && !failed) {
        const int row = 32 * (gw + j * nw) + lane;
        const bool own = row < A.n_rows;
        // lagged update with alpha_{k-1}, beta_{k-1}, then p_k; published for the neighbours' next gathers
        if (own && it > 0) {
          const V3<T> xo = load3rw(xg, row);
          store3(xg, row, xo.x + ta * pr[j][0], xo.y + ta * pr[j][1], xo.z + ta * pr[j][2]);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          rr_[j][c] = rr_[j][c] - ta * qr[j][c];
          zr[j][c] = cg1_z(zr[j][c], wr[j][c], ta);
          pr[j][c] = cg1_p(zr[j][c], pr[j][c], tb);
        }
        if (own) {
          store3(Zw, row, zr[j][0], zr[j][1], zr[j][2]);
          store3(Pw, row, pr[j][0], pr[j][1], pr[j][2]);
        }
        T a0 = T(0), a1 = T(0), a2 = T(0);
        for (int g = s_first[j]; g < s_end[j]; g += CB) {
          const bool okw = __all_sync(0xffffffffu, mbar_wait_bounded(smem_addr(&bars[warp][st]), (phase >> st) & 1u));
          if (!okw) {
            failed = true;
            break;
          }
          phase ^= 1u << st;
          --inflight;
          const T* sval = reinterpret_cast<const T*>(wbase + (size_t)st * C::kStageBytes);
          const int32_t* scol = reinterpret_cast<const int32_t*>(wbase + (size_t)st * C::kStageBytes + C::kValBytes);
          const int nb = min(CB, s_end[j] - g);
          V3<T> zc[CB], wc[CB], pc[CB];
#pragma unroll
          for (int k = 0; k < CB; ++k) {
            const int c = k < nb ? scol[32 * k + lane] : 0;
            zc[k] = load3rw(Zr, c);
            wc[k] = load3rw(Wr, c);
            pc[k] = load3rw(Pr, c);
          }
#pragma unroll
          for (int k = 0; k < CB; ++k) {
            if (k < nb) {
              const T x0 = cg1_p(cg1_z(zc[k].x, wc[k].x, ta), pc[k].x, tb);
              const T x1 = cg1_p(cg1_z(zc[k].y, wc[k].y, ta), pc[k].y, tb);
              const T x2 = cg1_p(cg1_z(zc[k].z, wc[k].z, ta), pc[k].z, tb);
              const T* v = sval + 288 * k + lane;
              a0 += v[0] * x0 + v[32] * x1 + v[64] * x2;
              a1 += v[96] * x0 + v[128] * x1 + v[160] * x2;
              a2 += v[192] * x0 + v[224] * x1 + v[256] * x2;
            }
          }
          __syncwarp();  // the stage is consumed before it is refilled
          issue(st, P);
          ++inflight;
          advance(P);
          st = (st + 1 == NST) ? 0 : st + 1;
        }
        qr[j][0] = a0, qr[j][1] = a1, qr[j][2] = a2;
        if (own) {
          const T* m = minv + 9 * (int64_t)row;
#pragma unroll
          for (int b = 0; b < 3; ++b)
            wr[j][b] = __ldg(m + 3 * b) * a0 + __ldg(m + 3 * b + 1) * a1 + __ldg(m + 3 * b + 2) * a2;
          store3(Ww, row, wr[j][0], wr[j][1], wr[j][2]);
          const T* pj = pr[j];
          const T* qj = qr[j];
          const T* rj = rr_[j];
          const T* zj = zr[j];
          const T* wj = wr[j];
          red[0] += double(pj[0] * qj[0] + pj[1] * qj[1] + pj[2] * qj[2]);
          red[1] += double(rj[0] * wj[0] + rj[1] * wj[1] + rj[2] * wj[2]);
          red[2] += double(qj[0] * zj[0] + qj[1] * zj[1] + qj[2] * zj[2]);
          red[3] += double(qj[0] * wj[0] + qj[1] * wj[1] + qj[2] * wj[2]);
          red[4] += double(rj[0] * qj[0] + rj[1] * qj[1] + rj[2] * qj[2]);
          red[5] += double(qj[0] * qj[0] + qj[1] * qj[1] + qj[2] * qj[2]);
          red[6] += double(rj[0] * zj[0] + rj[1] * zj[1] + rj[2] * zj[2]);
          red[7] += double(rj[0] * rj[0] + rj[1] * rj[1] + rj[2] * rj[2]);
        } else {
          wr[j][0] = wr[j][1] = wr[j][2] = T(0);
        }
      }
    }
    failed = __syncthreads_or(failed);
    if (failed) break;
    cta_reduce<8>(red, sw);
    ++barrier_no;
    if (!grid_allreduce<8>(red, part + par * 8 * G, bar_count, barrier_no * (unsigned)G, sv, &ok_sh,
                           WaitCtl{kBarrierSpinLimit, 0})) {
      failed = true;
      break;
    }
    rho = red[6];
    const double pq = red[0];
    if (!(fabs(pq) > 0.0) || !isfinite(pq) || !isfinite(rho)) {  // breakdown; x_k is the result
      done = 3.0;
      break;
    }
    const double alpha = rho / pq;
    const double rho_next = rho - alpha * (red[1] + red[2]) + alpha * alpha * red[3];
    rrs = red[7] - 2.0 * alpha * red[4] + alpha * alpha * red[5];
    beta_p = rho_next / rho;
    alpha_p = alpha;
    rho = rho_next;
    ++it;
    if (rrs <= tol2) done = 1.0;
    else if (it >= maxit) done = 2.0;
  }
  if (failed) done = kDoneDeviceTimeout;
  for (int k = 0; k < inflight; ++k) {
    mbar_wait_bounded(smem_addr(&bars[warp][st]), (phase >> st) & 1u);
    phase ^= 1u << st;
    st = (st + 1 == NST) ? 0 : st + 1;
  }
  // the last step's x update (x_{k+1} = x_k + alpha_k p_k) when the iteration stopped by its test
  if (done == 1.0 || done == 2.0) {
    const T tfin = T(alpha_p);
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      const int row = 32 * (gw + j * nw) + lane;
      if (j < ns && row < A.n_rows) {
        const V3<T> xo = load3rw(xg, row);
        store3(xg, row, xo.x + tfin * pr[j][0], xo.y + tfin * pr[j][1], xo.z + tfin * pr[j][2]);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[kIters] = (double)it;
    scal[kRR] = rrs;
    scal[kRz] = rho;
    scal[kBeta] = beta_p;
    scal[kDone] = done;
  }
  if (failed && threadIdx.x == 0) scal[kDone] = kDoneDeviceTimeout;
}

template <typename T, int CB, int NST, int WARPS, int MAXS, int MINB>
cudaError_t launch_onered(const Bsr& A, PcgWork& w, cudaStream_t s, bool query_only, bool* eligible) {
  using C = PersistentCfg<T, CB, NST, WARPS>;
  auto kern = pcg_onered_kernel<T, CB, NST, WARPS, MAXS, MINB>;
  static std::mutex mu;
  static int blocks_per_sm[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 64) dev = 63;
  int bps;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!blocks_per_sm[dev]) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmemBytes);
      int b = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, C::kThreads, C::kSmemBytes);
      blocks_per_sm[dev] = b > 0 ? b : -1;
    }
    bps = blocks_per_sm[dev];
  }
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  // part_c holds 16 doubles per w.grid CTA: 8 partials per CTA, double-buffered by iteration parity
  int grid = bps > 0 ? w.sms * bps : 0;
  if (grid > w.grid) grid = w.grid;
  const int nw = grid * WARPS;
  *eligible = coop && grid > 0 && w.z2 && w.w0 && w.w1 && w.part_c && (int64_t)nw * MAXS >= A.n_slices;
  if (query_only || !*eligible) return cudaSuccess;
  // W1 = w_{-1} = 0; Z1 = z_0 and P1 = p_{-1} = 0 come from the init kernel (w.z, w.p1)
  cudaError_t e = cudaMemsetAsync(w.w1, 0, sizeof(T) * 4 * (size_t)w.n_rows, s);
  if (e != cudaSuccess) return e;
  const T* val = (const T*)A.val;
  const T* minv = (const T*)w.minv;
  T* xg = (T*)w.x;
  const T* rg = (const T*)w.r;
  T *Z0 = (T*)w.z2, *Z1 = (T*)w.z, *P0 = (T*)w.p0, *P1 = (T*)w.p1, *W0 = (T*)w.w0, *W1 = (T*)w.w1;
  double* part = w.part_c;
  double* scal = w.scal;
  int64_t keep = w.keep_g;
  Bsr Acopy = A;
  void* args[] = {&Acopy, &val, &minv, &xg, &rg, &Z0, &Z1, &P0, &P1, &W0, &W1, &part, &scal, &keep};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(C::kThreads), args, C::kSmemBytes, s);
}

template <typename T>
cudaError_t dispatch_onered(int variant, const Bsr& A, PcgWork& w, cudaStream_t s, bool query, bool* eligible) {
  if constexpr (sizeof(T) == 4) {
    if (variant == 0) return launch_onered<float, 4, 2, 8, 2, 2>(A, w, s, query, eligible);
    return launch_onered<float, 8, 2, 8, 4, 1>(A, w, s, query, eligible);
  } else {
    if (variant == 0) return launch_onered<double, 2, 2, 8, 2, 2>(A, w, s, query, eligible);
    return launch_onered<double, 4, 2, 8, 4, 1>(A, w, s, query, eligible);
  }
}
constexpr int kClassicVariants = 7;
constexpr int kOneRedVariants = 2;

}  // namespace

int pcg_persistent_variants() { return kClassicVariants + kOneRedVariants; }

bool pcg_persistent_eligible(const Bsr& A, PcgWork& w, int variant) {
  bool ok = false;
  if (variant >= kClassicVariants) {
    if (w.fp32) dispatch_onered<float>(variant - kClassicVariants, A, w, nullptr, true, &ok);
    else dispatch_onered<double>(variant - kClassicVariants, A, w, nullptr, true, &ok);
    return ok;
  }
  PcgWork* ws[1] = {&w};
  if (w.fp32) dispatch<float, 1>(variant, A, ws, w.part_a, w.part_b, nullptr, true, &ok);
  else dispatch<double, 1>(variant, A, ws, w.part_a, w.part_b, nullptr, true, &ok);
  return ok;
}

cudaError_t launch_pcg_persistent(const Bsr& A, PcgWork& w, int variant, cudaStream_t s) {
  bool ok = false;
  cudaError_t e;
  if (variant >= kClassicVariants) {
    e = w.fp32 ? dispatch_onered<float>(variant - kClassicVariants, A, w, s, false, &ok)
               : dispatch_onered<double>(variant - kClassicVariants, A, w, s, false, &ok);
  } else {
    PcgWork* ws[1] = {&w};
    e = w.fp32 ? dispatch<float, 1>(variant, A, ws, w.part_a, w.part_b, s, false, &ok)
               : dispatch<double, 1>(variant, A, ws, w.part_a, w.part_b, s, false, &ok);
  }
  if (e == cudaSuccess && !ok) return cudaErrorInvalidConfiguration;
  return e;
}

bool pcg_persistent2_eligible(const Bsr& A, PcgWork& w0, PcgWork& w1, int variant) {
  if (variant >= kClassicVariants) return false;  // the one-reduction form runs one right-hand side
  bool ok = false;
  PcgWork* ws[2] = {&w0, &w1};
  if (w0.fp32) dispatch<float, 2>(variant, A, ws, nullptr, nullptr, nullptr, true, &ok);
  else dispatch<double, 2>(variant, A, ws, nullptr, nullptr, nullptr, true, &ok);
  return ok;
}

cudaError_t launch_pcg_persistent2(const Bsr& A, PcgWork& w0, PcgWork& w1, int variant, double* part_a,
                                   double* part_b, cudaStream_t s) {
  if (variant >= kClassicVariants) return cudaErrorInvalidConfiguration;
  bool ok = false;
  PcgWork* ws[2] = {&w0, &w1};
  cudaError_t e = w0.fp32 ? dispatch<float, 2>(variant, A, ws, part_a, part_b, s, false, &ok)
                          : dispatch<double, 2>(variant, A, ws, part_a, part_b, s, false, &ok);
  if (e == cudaSuccess && !ok) return cudaErrorInvalidConfiguration;
  return e;
}

}  // namespace ikr
