// Persistent block-Jacobi PCG with the coarse correction in the same cooperative launch (sm_103a).
//
//   M^-1 r = D^-1 r + P A_c^-1 P^T r          (coarse.cu: the aggregates, P and A_c = P^T K P)
//
// The iteration of cg_persistent.cu (product phase with p_new = z + beta p_old formed for every gathered
// neighbour, grid reduction of p.q, update phase on the owned rows kept in registers) with the coarse part after
// the update phase, instead of the two extra kernels per iteration of the two-kernel form:
//   1. every row adds its six mode sums P_row^T r_row into a per-warp shared array (runs of equal aggregate over
//      the lanes of a slice are summed by a segmented warp scan, the run totals added in lane order); the CTA adds
//      its warps' arrays in warp order and publishes, with r.D^-1 r and r.r (FP64), one partial per coarse dof;
//   2. grid barrier; every CTA sums the published partials of all CTAs in CTA order (four coarse dofs per warp at
//      a time, a fixed lane split and butterfly, all loads of a group in flight together), so r_c = P^T r,
//      r.D^-1 r and r.r are bit-identical in every CTA;
//   3. e = A_c^-1 r_c (threads over rows and column segments, sixteen column loads in flight), r.z = r.D^-1 r +
//      r_c.e.  The mode sums (rows, warps, CTAs), their warp scan and this product run in the CG's type (FP32 for
//      the FP32 CG: GB300's FP64 pipe is a small fraction of its FP32 rate, and e is kept in the CG's type
//      anyway); r.D^-1 r, r.r and r_c.e are FP64;
//   4. the owned rows' z = D^-1 r + P e goes to registers and to the global z the gathers read; a third grid
//      barrier (arrive and wait) publishes it before the next product phase.
// Before the first iteration the same coarse part turns the init kernel's z = D^-1 r_0 into M^-1 r_0.  All sums
// have a fixed order: a solve is bit-identical run to run.  Every wait is bounded (grid barriers and stage waits
// give up with scal[kDone] = 6 after their poll limits).
#include <algorithm>
#include <mutex>

#include "cg_grid.cuh"

namespace ikr {

namespace {

using namespace cg;

constexpr int kGridLanes = 6;  // grid partials per lane in the coarse sums: at most 192 CTAs

// per node: offset from the aggregate centroid, aggregate id (bits 0-23) and free-dof mask (bits 24-26)
struct RowP {
  float y[3];
  int agg, mask;
};
__device__ __forceinline__ RowP row_p(const float4* __restrict__ y4, int node) {
  const float4 v = __ldg(y4 + node);
  const int bits = __float_as_int(v.w);
  return {{v.x, v.y, v.z}, bits & 0xFFFFFF, (bits >> 24) & 7};
}

// grid barrier without data: arrive, wait (bounded) until `target` arrivals; false when the wait gave up.  Every
// thread fences its own global writes before the CTA arrives (they are written by many threads of the CTA).
__device__ __forceinline__ bool grid_sync(unsigned int* count, unsigned int target, bool* ok_sh, int polls) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(count, 1u);
    bool ok = false;
    for (int i = 0; i < polls; ++i) {
      unsigned int c;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(count) : "memory");
      if (c >= target) {
        ok = true;
        break;
      }
      if (i > 64) __nanosleep(16);
    }
    *ok_sh = ok;
  }
  __syncthreads();
  __threadfence();
  return *ok_sh;
}

template <typename T, int CB, int NST, int WARPS, int MAXS>
__global__ void __launch_bounds__(WARPS * 32, 1)
    pcg_coarse_kernel(Bsr A, const T* __restrict__ val, const T* __restrict__ minv, T* x, const T* r, T* z, T* p0,
                      T* p1, double* scal, Coarse Cc, double* part_a, double* cpart, int64_t keep_g, WaitCtl wc,
                      int ainv_shared) {
  using C = PersistentCfg<T, CB, NST, WARPS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[WARPS][NST];
  __shared__ double sv[2];
  __shared__ T s_alpha, s_tb;
  __shared__ int s_state;
  __shared__ double sfull[2 * WARPS * 32];
  __shared__ bool ok_sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int G = gridDim.x;
  const int nw = G * WARPS;
  const int gw = blockIdx.x * WARPS + warp;
  const int n_slices = A.n_slices;
  const int nc = Cc.n_c, nv = nc + 2;  // r.D^-1 r and r.r, then the coarse dofs
  unsigned int* bar_count = &tickets(scal)[3];
  unsigned char* wbase = smem + (size_t)warp * NST * C::kStageBytes;
  // coarse shared arrays after the stages: per-warp mode sums (WARPS x nc), r_c (+ the two dot products), e
  // coarse shared arrays after the stages: per-warp mode sums (WARPS x n_c, also the blockDim.x partials of e),
  // the two FP64 dot products, r_c and e in the CG's type
  double* rdot = reinterpret_cast<double*>(smem + (size_t)WARPS * NST * C::kStageBytes);
  T* accw = reinterpret_cast<T*>(rdot + 2);
  T* rct = accw + max(WARPS * nc, WARPS * 32);
  T* ect = rct + nc;
  T* ainv_s = ect + nc;  // A_c^-1 in shared memory for the whole solve, where it fits (ainv_shared)
  const T* ainv = static_cast<const T*>(Cc.ainv);

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
  T xr[MAXS][3], rr_[MAXS][3], zr[MAXS][3], pr[MAXS][3], qr[MAXS][3];
  RowP yp[MAXS];
#pragma unroll
  for (int j = 0; j < MAXS; ++j) {
    const int row = 32 * (gw + j * nw) + lane;
    const bool own = j < ns && row < A.n_rows;
    V3<T> r0 = {T(0), T(0), T(0)}, z0 = {T(0), T(0), T(0)};
    yp[j] = {{0.f, 0.f, 0.f}, -1, 0};
    if (own) r0 = load3rw(r, row), z0 = load3rw(z, row), yp[j] = row_p(Cc.y4, row);
    rr_[j][0] = r0.x, rr_[j][1] = r0.y, rr_[j][2] = r0.z;
    zr[j][0] = z0.x, zr[j][1] = z0.y, zr[j][2] = z0.z;
#pragma unroll
    for (int c = 0; c < 3; ++c) xr[j][c] = pr[j][c] = qr[j][c] = T(0);
  }
  const double tol2 = scal[kTol2];
  const int maxit = (int)scal[kMaxIt];
  // FP64 scalars: rz, r.r and beta are thread 0's (the others' copies are not updated); every thread keeps the
  // stop decision, the iteration count and beta in the CG's type
  double rz = 0.0, rrs = scal[kRR], done = scal[kDone], beta = 0.0;
  T tbv = T(0);
  int it = (int)scal[kIters];

  if (ainv_shared) {
    for (int k = threadIdx.x; k < nc * nc; k += blockDim.x) ainv_s[k] = __ldg(ainv + k);
    __syncthreads();
  }
  if (lane == 0) {
    for (int st = 0; st < NST; ++st) mbar_init(smem_addr(&bars[warp][st]), 1);
    mbar_init_fence();
  }
  __syncwarp();

  bool failed = false;
  unsigned int barrier_no = 0;
  int loop = 0;

  // The coarse part of z = M^-1 r for the owned rows (zr holds D^-1 r on entry, z = M^-1 r on return, also stored
  // to the global z): returns false when a grid wait gave up.  Sets rzs (r.z), rrn (r.r).
  auto coarse_part = [&](double& rzs, double& rrn) -> bool {
    for (int i = threadIdx.x; i < WARPS * nc; i += blockDim.x) accw[i] = T(0);
    __syncthreads();
    T lrz = T(0), lrr = T(0);  // a lane's r.D^-1 r and r.r in the CG's type, converted once
    T* aw = accw + (size_t)warp * nc;
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      const int a = yp[j].agg;  // -1 for rows not owned
      // in the CG's type: GB300's FP64 pipe is a small fraction of its FP32 rate, and these run for every row
      T v[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
      if (a >= 0) {
        const T r0 = (yp[j].mask & 1) ? rr_[j][0] : T(0);
        const T r1 = (yp[j].mask & 2) ? rr_[j][1] : T(0);
        const T r2 = (yp[j].mask & 4) ? rr_[j][2] : T(0);
        const T yx = T(yp[j].y[0]), yy = T(yp[j].y[1]), yz = T(yp[j].y[2]);
        // P^T r with the columns e_k (translations) and e_k x y (rotations) of the node's 3 x 6 block
        v[0] = r0, v[1] = r1, v[2] = r2;
        v[3] = -yz * r1 + yy * r2;
        v[4] = yz * r0 - yx * r2;
        v[5] = -yy * r0 + yx * r1;
        T trz = T(0), trr = T(0);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          trz += rr_[j][b] * zr[j][b];
          trr += rr_[j][b] * rr_[j][b];
        }
        lrz += trz;
        lrr += trr;
      }
      // segmented inclusive scan over runs of equal aggregate (lane order)
      const int ap = __shfl_up_sync(0xffffffffu, a, 1), an = __shfl_down_sync(0xffffffffu, a, 1);
      const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || ap != a);
      const int seg = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int m = 0; m < 6; ++m) {
          const T t = __shfl_up_sync(0xffffffffu, v[m], d);
          if (lane - d >= seg) v[m] += t;
        }
      }
      unsigned tails = __ballot_sync(0xffffffffu, a >= 0 && (lane == 31 || an != a));
      while (tails) {  // run totals into the warp's array in lane order
        const int L = __ffs(tails) - 1;
        if (lane == L) {
#pragma unroll
          for (int m = 0; m < 6; ++m) aw[6 * a + m] += v[m];
        }
        __syncwarp();
        tails &= tails - 1;
      }
    }
    // CTA partials: r.D^-1 r and r.r in FP64 (thread 0), the mode sums (warps added in order) in the CG's type,
    // coarse-dof-major: per parity 2 G doubles, then n_c G values
    double red[2] = {double(lrz), double(lrr)};
    cta_reduce_smem<2>(red, sfull);  // warp 0 holds the sums; the __syncthreads inside orders accw
    __syncthreads();
    double* cpd = cpart + (size_t)(loop & 1) * nv * G;
    T* cpm = reinterpret_cast<T*>(cpd + 2 * (size_t)G);
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
      T sum = T(0);
      for (int w = 0; w < WARPS; ++w) sum += accw[(size_t)w * nc + c];
      cpm[(size_t)c * G + blockIdx.x] = sum;
    }
    if (threadIdx.x == 0) {
      cpd[blockIdx.x] = red[0];
      cpd[G + blockIdx.x] = red[1];
    }
    ++barrier_no;
    if (!grid_sync(bar_count, barrier_no * (unsigned)G, &ok_sh, wc.polls)) return false;
    // every CTA: the sums over all CTAs in CTA order; a warp takes four values at a time and a lane the CTAs
    // lane, lane + 32, ... (at most kGridLanes of them), all loads of a group issued together: the partials sit in
    // L2, and a chain of dependent loads would cost one L2 round trip each.  Value c < 2: the FP64 dot products;
    // the others: the mode sums in the CG's type
    for (int c0 = 4 * warp; c0 < nv; c0 += 4 * WARPS) {
      double sq[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int c = c0 + q;
        if (c < 2) {
          double t[kGridLanes];
#pragma unroll
          for (int k = 0; k < kGridLanes; ++k) {
            const int g = lane + 32 * k;
            t[k] = g < G ? __ldcg(cpd + (size_t)c * G + g) : 0.0;
          }
          double a = 0.0;
#pragma unroll
          for (int k = 0; k < kGridLanes; ++k) a += t[k];
          sq[q] = a;
        } else {
          T t[kGridLanes];
#pragma unroll
          for (int k = 0; k < kGridLanes; ++k) {
            const int g = lane + 32 * k;
            t[k] = (c < nv && g < G) ? __ldcg(cpm + (size_t)(c - 2) * G + g) : T(0);
          }
          T a = T(0);
#pragma unroll
          for (int k = 0; k < kGridLanes; ++k) a += t[k];
          sq[q] = double(warp_sum(a));
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int c = c0 + q;
        if (c < 2) {
          const double v = warp_sum(sq[q]);
          if (lane == 0) rdot[c] = v;
        } else if (lane == 0 && c < nv) {
          rct[c - 2] = T(sq[q]);
        }
      }
    }
    __syncthreads();
    rrn = rdot[1];
    // e = A_c^-1 r_c (in the CG's type, as the two-kernel form keeps it): thread t forms the part of row i = t mod
    // n_c over column segment t / n_c (A_c^-1 is symmetric: the reads of column j are coalesced along i, sixteen
    // columns' loads in flight), then the segments are added in order
    {
      const int nseg = max(1, (int)blockDim.x / nc), seg_len = (nc + nseg - 1) / nseg;
      const int t = threadIdx.x, i = t % nc, seg = t / nc;
      T sum = T(0);
      if (seg < nseg) {
        const int j1 = min(nc, (seg + 1) * seg_len);
        if (ainv_shared) {
          for (int j = seg * seg_len; j < j1; ++j) sum += ainv_s[(size_t)j * nc + i] * rct[j];
        } else {
#pragma unroll 16
          for (int j = seg * seg_len; j < j1; ++j) sum += __ldg(ainv + (size_t)j * nc + i) * rct[j];
        }
      }
      accw[t] = sum;  // the mode-sum array is free again
      __syncthreads();
      if (t < nc) {
        T ev = T(0);
        for (int g = 0; g < nseg; ++g) ev += accw[g * nc + t];
        ect[t] = ev;
      }
    }
    __syncthreads();
    if (warp == 0) {
      double sd = 0.0;
      for (int i = lane; i < nc; i += 32) sd += double(rct[i]) * double(ect[i]);
      sd = warp_sum(sd);
      if (lane == 0) sv[0] = sd;
    }
    __syncthreads();
    rzs = rdot[0] + sv[0];
    // z = D^-1 r + P e on the owned rows
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      const int a = yp[j].agg;
      if (a < 0) continue;
      const T* ea = ect + 6 * a;
      const T yx = T(yp[j].y[0]), yy = T(yp[j].y[1]), yz = T(yp[j].y[2]);
      const T e0 = ea[0], e1 = ea[1], e2 = ea[2], e3 = ea[3], e4 = ea[4], e5 = ea[5];
      T d0 = e0 + e4 * yz - e5 * yy;
      T d1 = e1 + e5 * yx - e3 * yz;
      T d2 = e2 + e3 * yy - e4 * yx;
      if (!(yp[j].mask & 1)) d0 = T(0);
      if (!(yp[j].mask & 2)) d1 = T(0);
      if (!(yp[j].mask & 4)) d2 = T(0);
      zr[j][0] += d0, zr[j][1] += d1, zr[j][2] += d2;
      store3(z, 32 * (gw + j * nw) + lane, zr[j][0], zr[j][1], zr[j][2]);
    }
    return true;
  };

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
  uint32_t phase = 0;
  int st = 0;

  if (done == 0.0) {
    // z_0 = M^-1 r_0 and r_0.z_0
    double rr0 = 0.0;
    if (!coarse_part(rz, rr0)) failed = true;
    ++barrier_no;
    if (!failed && !grid_sync(bar_count, barrier_no * (unsigned)G, &ok_sh, wc.polls)) failed = true;
    ++loop;
    if (!failed && ns > 0) {
      for (int s2 = 0; s2 < NST; ++s2) {
        issue(s2, P);
        ++inflight;
        advance(P);
      }
    }
  }

  while (done == 0.0 && !failed) {
    const T tb = tbv;
    const T* pold = (it & 1) ? p0 : p1;
    T* pnew = (it & 1) ? p1 : p0;
    T pql = T(0);  // a lane's p.q in the CG's type, converted once
    // ---- product phase: q = K p_new over the owned slices
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      if (j < ns && !failed) {
        T acc3[3] = {T(0), T(0), T(0)};
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
          V3<T> zc[CB], pc[CB];
#pragma unroll
          for (int k = 0; k < CB; ++k) {
            zc[k] = load3rw(z, cols[k]);
            pc[k] = load3rw(pold, cols[k]);
          }
#pragma unroll
          for (int k = 0; k < CB; ++k) {
            if (k < nb) {
              const T x0 = zc[k].x + tb * pc[k].x, x1 = zc[k].y + tb * pc[k].y, x2 = zc[k].z + tb * pc[k].z;
              const T* v = sval + 288 * k + lane;
              acc3[0] += v[0] * x0 + v[32] * x1 + v[64] * x2;
              acc3[1] += v[96] * x0 + v[128] * x1 + v[160] * x2;
              acc3[2] += v[192] * x0 + v[224] * x1 + v[256] * x2;
            }
          }
          __syncwarp();  // the stage is consumed before it is refilled
          issue(st, P);
          ++inflight;
          advance(P);
          st = (st + 1 == NST) ? 0 : st + 1;
        }
        const int row = 32 * (gw + j * nw) + lane;
        const T n0 = zr[j][0] + tb * pr[j][0], n1 = zr[j][1] + tb * pr[j][1], n2 = zr[j][2] + tb * pr[j][2];
        pr[j][0] = n0, pr[j][1] = n1, pr[j][2] = n2;
        qr[j][0] = acc3[0], qr[j][1] = acc3[1], qr[j][2] = acc3[2];
        if (row < A.n_rows) {
          store3(pnew, row, n0, n1, n2);
          pql += n0 * acc3[0] + n1 * acc3[1] + n2 * acc3[2];
        }
      }
    }
    // ---- grid reduction of p.q
    failed = __syncthreads_or(failed);
    if (failed) break;
    double pqa[1] = {double(pql)};
    cta_reduce_smem<1>(pqa, sfull);
    ++barrier_no;
    if (!grid_allreduce<1>(pqa, part_a + (loop & 1) * G, bar_count, barrier_no * (unsigned)G, sv, &ok_sh, wc)) {
      failed = true;
      break;
    }
    // thread 0 forms alpha (and the breakdown decision) in FP64 and hands it on in the CG's type
    if (threadIdx.x == 0) {
      const bool brk = !(fabs(pqa[0]) > 0.0) || !isfinite(pqa[0]);  // breakdown
      s_state = brk ? 3 : 0;
      s_alpha = brk ? T(0) : T(rz / pqa[0]);
    }
    __syncthreads();
    if (s_state == 3) {
      done = 3.0;
      break;
    }
    const T alpha = s_alpha;
    // ---- update phase on the owned rows: x, r, z = D^-1 r
#pragma unroll
    for (int j = 0; j < MAXS; ++j) {
      const int row = 32 * (gw + j * nw) + lane;
      if (j < ns && row < A.n_rows) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          xr[j][c] += alpha * pr[j][c];
          rr_[j][c] -= alpha * qr[j][c];
        }
        const T* m = minv + 9 * (int64_t)row;
#pragma unroll
        for (int b = 0; b < 3; ++b)
          zr[j][b] = __ldg(m + 3 * b) * rr_[j][0] + __ldg(m + 3 * b + 1) * rr_[j][1] + __ldg(m + 3 * b + 2) * rr_[j][2];
      }
    }
    // ---- coarse part, r.z, r.r (one grid barrier inside), then publish z (a second)
    double rzs = 0.0;
    if (!coarse_part(rzs, rrs)) {
      failed = true;
      break;
    }
    // thread 0 forms beta and the stop decision (FP64); the others read the decision and beta in the CG's type
    if (threadIdx.x == 0) {
      beta = rzs / rz;
      rz = rzs;
      s_state = rrs <= tol2 ? 1 : (it + 1 >= maxit ? 2 : 0);
      s_tb = T(beta);
    }
    __syncthreads();
    ++it;
    tbv = s_tb;
    ++loop;
    if (s_state != 0) {  // every CTA decides alike (the same sums)
      done = s_state;
      break;
    }
    ++barrier_no;
    if (!grid_sync(bar_count, barrier_no * (unsigned)G, &ok_sh, wc.polls)) {
      failed = true;
      break;
    }
  }
  // drain the copies still in flight
  for (int k = 0; k < inflight; ++k) {
    mbar_wait_bounded(smem_addr(&bars[warp][st]), (phase >> st) & 1u);
    phase ^= 1u << st;
    st = (st + 1 == NST) ? 0 : st + 1;
  }
#pragma unroll
  for (int j = 0; j < MAXS; ++j) {
    const int row = 32 * (gw + j * nw) + lane;
    if (j < ns && row < A.n_rows) store3(x, row, xr[j][0], xr[j][1], xr[j][2]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[kIters] = (double)it;
    scal[kRR] = rrs;
    scal[kRz] = rz;
    scal[kBeta] = beta;
    scal[kDone] = failed ? kDoneDeviceTimeout : done;
  }
  if (failed && threadIdx.x == 0) scal[kDone] = kDoneDeviceTimeout;
}

template <typename T, int CB, int NST, int WARPS, int MAXS>
cudaError_t launch_coarse_cfg(const Bsr& A, PcgWork& w, const Coarse& Cc, cudaStream_t s, bool query_only,
                              bool* eligible) {
  using C = PersistentCfg<T, CB, NST, WARPS>;
  auto kern = pcg_coarse_kernel<T, CB, NST, WARPS, MAXS>;
  // dynamic shared memory: the stages, two FP64 dot products, the per-warp mode sums (also the CTA's e partials), r_c
  // and e, and A_c^-1 itself where it fits under the budget (one CTA per SM either way)
  constexpr size_t kBudget = 216 * 1024;
  const size_t nc = (size_t)Cc.n_c;
  const size_t base = (size_t)C::kSmemBytes + 2 * sizeof(double) +
                      sizeof(T) * (std::max(WARPS * nc, (size_t)WARPS * 32) + 2 * nc);
  const int ainv_shared = base + sizeof(T) * nc * nc <= kBudget ? 1 : 0;
  const size_t smem = base + (ainv_shared ? sizeof(T) * nc * nc : 0);
  const size_t smem_max = kBudget;
  static std::mutex mu;
  static int blocks_per_sm[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 64) dev = 63;
  int bps;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!blocks_per_sm[dev]) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
      int b = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, C::kThreads, smem_max);
      blocks_per_sm[dev] = b > 0 ? b : -1;
    }
    bps = blocks_per_sm[dev];
  }
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  int grid = bps > 0 ? w.sms * bps : 0;
  if (grid > w.grid) grid = w.grid;
  *eligible = coop && grid > 0 && grid <= 32 * kGridLanes && (int64_t)grid * WARPS * MAXS >= A.n_slices && Cc.n_c > 0 &&
              Cc.n_c <= kCoarseFusedMaxDofs && w.coarse_part != nullptr && grid <= w.coarse_part_ctas &&
              smem <= smem_max;
  if (query_only || !*eligible) return cudaSuccess;
  const T* val = (const T*)A.val;
  const T* minv = (const T*)w.minv;
  T* x = (T*)w.x;
  const T* r = (const T*)w.r;
  T* z = (T*)w.z;
  T* p0 = (T*)w.p0;
  T* p1 = (T*)w.p1;
  double* scal = w.scal;
  Bsr Acopy = A;
  Coarse Ccopy = Cc;
  double* pa = w.part_a;
  double* cp = w.coarse_part;
  int64_t keep = w.keep_g;
  WaitCtl wc{w.barrier_polls > 0 ? w.barrier_polls : kBarrierSpinLimit, 0};
  int ash = ainv_shared;
  void* args[] = {&Acopy, &val, &minv, &x, &r, &z, &p0, &p1, &scal, &Ccopy, &pa, &cp, &keep, &wc, &ash};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(C::kThreads), args, smem, s);
}

cudaError_t dispatch_coarse(int variant, const Bsr& A, PcgWork& w, const Coarse& Cc, cudaStream_t s, bool query,
                            bool* eligible) {
  if (w.fp32) {
    if (variant == 0) return launch_coarse_cfg<float, 4, 2, 16, 2>(A, w, Cc, s, query, eligible);
    return launch_coarse_cfg<float, 4, 2, 16, 4>(A, w, Cc, s, query, eligible);
  }
  if (variant == 0) return launch_coarse_cfg<double, 2, 2, 16, 2>(A, w, Cc, s, query, eligible);
  return launch_coarse_cfg<double, 2, 2, 16, 4>(A, w, Cc, s, query, eligible);
}

}  // namespace

int pcg_coarse_variants() { return 2; }

bool pcg_coarse_eligible(const Bsr& A, PcgWork& w, const Coarse& Cc, int variant) {
  bool ok = false;
  dispatch_coarse(variant, A, w, Cc, nullptr, true, &ok);
  return ok;
}

cudaError_t launch_pcg_coarse(const Bsr& A, PcgWork& w, const Coarse& Cc, int variant, cudaStream_t s) {
  bool ok = false;
  const cudaError_t e = dispatch_coarse(variant, A, w, Cc, s, false, &ok);
  if (e == cudaSuccess && !ok) return cudaErrorInvalidConfiguration;
  return e;
}

}  // namespace ikr
