// Many independent instances of uneven size in one element set: per-instance CG and norms (sm_103a).
//
// The instances are disjoint contiguous node ranges of one mesh, so the tangent is block diagonal by instance.
// batched_pcg_kernel runs the block-Jacobi PCG of many instances in one launch.  Each instance gets a group of CTAs
// (the host sizes the groups so that all CTAs are co-resident); the CTAs of a group split the instance's block rows
// into contiguous chunks, one thread per row.  An iteration has two group-wide reductions (p.q, then r.z and r.r):
// every CTA sums its threads' values (FP64 additions by one warp), publishes the sum, arrives on the instance's
// barrier counter with release semantics and waits (bounded) for the group; lane b of warp 0 then loads CTA b's sum
// and the butterfly adds them, so alpha, beta and the convergence decision are identical in the group's CTAs and run
// to run.  A one-CTA group needs no global barrier.  p_new = z + beta p_old is formed on the fly for every gathered
// neighbour, which removes the barrier a separate p update would need.
//
// The solves of a Newton iteration are latency-bound: a hard instance needs thousands of iterations after the easy
// ones have converged.  So the host runs a solve as a sequence of launches of at most `chunk` iterations each and
// re-plans the groups over the instances still running before every launch: the state of every instance (its
// vectors in the work arrays, rz, r.r, b.b, beta and the iteration count in `st` / `its`) carries over, the CG is
// continued, not restarted.  Kernel variants: batched_pcg_kernel with one row per thread (REG: the row's x, r, z,
// p, q and block-Jacobi inverse in registers for the whole launch) or with a thread looping over its rows (GEN: the
// state in the work arrays); batched_pcg_smem_kernel with four, eight or sixteen threads per row and the CTA's
// matrix blocks in shared memory; and, in FP32, batched_pcg_cluster_kernel with one instance per thread-block
// cluster and its vectors in distributed shared memory.  Every wait on a global barrier is bounded; a wait that gives
// up ends the instance with flag -1.
#include <map>
#include <mutex>
#include <tuple>

#include "cg_common.cuh"
#include "cg_grid.cuh"

namespace ikr {

namespace {

using namespace cg;

constexpr int kBatchThreads = 256;
constexpr int kGroupSpinLimit = 1 << 24;

// neighbour gathers from the node-padded work vectors; L2: read around L1 (values other CTAs of the group wrote)
template <bool L2>
__device__ __forceinline__ V3<float> gather3(const float* v, int node) {
  const float4* p = reinterpret_cast<const float4*>(v) + node;
  const float4 a = L2 ? __ldcg(p) : *p;
  return {a.x, a.y, a.z};
}
template <bool L2>
__device__ __forceinline__ V3<double> gather3(const double* v, int node) {
  const double2* p = reinterpret_cast<const double2*>(v) + 2 * node;
  const double2 a = L2 ? __ldcg(p) : *p;
  const double c = L2 ? __ldcg(v + 4 * node + 2) : v[4 * node + 2];
  return {a.x, a.y, c};
}

// q = K (z + tb p_old) on block row `row`; the columns of U blocks are loaded before their vector gathers so that
// the gathers of U neighbours are in flight together (four in FP32, two in FP64, within the register budget)
template <typename T, bool L2, int U = sizeof(T) == 4 ? 4 : 2>
__device__ __forceinline__ V3<T> row_product(const Bsr& A, const T* __restrict__ val, const T* zw, const T* pold, T tb,
                                             int row) {
  const int s = row >> 5, l = row & 31;
  const int gs = __ldg(A.slice_off + s), ge = __ldg(A.slice_off + s + 1);
  T a0 = T(0), a1 = T(0), a2 = T(0);
  for (int g0 = gs; g0 < ge; g0 += U) {
    int c[U];
#pragma unroll
    for (int k = 0; k < U; ++k) c[k] = g0 + k < ge ? __ldg(A.col_sell + 32 * (g0 + k) + l) : -1;
    V3<T> zv[U], pv[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      if (c[k] >= 0) {
        zv[k] = gather3<L2>(zw, c[k]);
        pv[k] = gather3<L2>(pold, c[k]);
      } else {
        zv[k] = {T(0), T(0), T(0)};
        pv[k] = zv[k];
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      if (c[k] >= 0) {
        const T* v = val + (int64_t)(g0 + k) * 288 + l;
        const T x0 = zv[k].x + tb * pv[k].x, x1 = zv[k].y + tb * pv[k].y, x2 = zv[k].z + tb * pv[k].z;
        a0 += __ldg(v) * x0 + __ldg(v + 32) * x1 + __ldg(v + 64) * x2;
        a1 += __ldg(v + 96) * x0 + __ldg(v + 128) * x1 + __ldg(v + 160) * x2;
        a2 += __ldg(v + 192) * x0 + __ldg(v + 224) * x1 + __ldg(v + 256) * x2;
      }
    }
  }
  return {a0, a1, a2};
}

template <typename T>
__device__ __forceinline__ V3<T> jacobi(const T (&m)[9], const V3<T>& r) {
  return {m[0] * r.x + m[1] * r.y + m[2] * r.z, m[3] * r.x + m[4] * r.y + m[5] * r.z,
          m[6] * r.x + m[7] * r.y + m[8] * r.z};
}
template <typename T>
__device__ __forceinline__ void load_minv(const T* __restrict__ minv, int row, T (&m)[9]) {
#pragma unroll
  for (int k = 0; k < 9; ++k) m[k] = __ldg(minv + 9 * (int64_t)row + k);
}

// Group-wide sums of N values: the CTA sum (warp 0 adds the threads' values in order), then, for a group of several
// CTAs, thread 0 publishes it (part: 2 slots x 2 values per CTA; the reductions of an iteration alternate slots, so a
// CTA that runs ahead never overwrites a sum another CTA has still to read), arrives with release semantics and polls
// (bounded) with acquire semantics; lanes of warp 0 load the group's sums (at most 256 CTAs) in a fixed assignment
// and the butterfly adds them.
// The sums are valid in warp 0; false (in warp 0) when the wait gave up.
template <int N>
__device__ __forceinline__ bool group_sum(double (&v)[N], double* sfull, double* part, int first, int size, int slot,
                                          unsigned int* counter, unsigned int target) {
  cta_reduce_smem<N>(v, sfull);
  if (threadIdx.x >= 32 || size == 1) return true;
  const int lane = threadIdx.x;
  int ok = 1;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) part[((size_t)blockIdx.x * 2 + slot) * 2 + k] = v[k];
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(counter) : "memory");
    ok = 0;
    for (int i = 0; i < kGroupSpinLimit; ++i) {
      unsigned int c;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(counter) : "memory");
      if (c >= target) {
        ok = 1;
        break;
      }
      if (i > 32) __nanosleep(32);
    }
  }
  __syncwarp();
  ok = __shfl_sync(0xffffffffu, ok, 0);
  if (!ok) return false;
  double t[8][N];  // lane b adds the sums of CTAs b, b + 32, ..., b + 224 (groups of at most 256), loads in flight
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int k = 0; k < N; ++k)
      t[u][k] = lane + 32 * u < size ? __ldcg(part + ((size_t)(first + lane + 32 * u) * 2 + slot) * 2 + k) : 0.0;
#pragma unroll
  for (int k = 0; k < N; ++k)
    v[k] = warp_sum(((t[0][k] + t[1][k]) + (t[2][k] + t[3][k])) + ((t[4][k] + t[5][k]) + (t[6][k] + t[7][k])));
  return true;
}

// Continues (or, on the first launch of a solve, starts) the PCG of every instance the launch's CTAs serve, for at
// most `chunk` iterations.  flag per instance on return: 0 still running, 1 finished (r.r <= rtol^2 b.b or max_iter
// reached), 2 breakdown (p.q not positive and finite; the current iterate stands), -1 a wait gave up.  x_out gets
// the instance's correction when it finishes.
template <typename T, bool REG>
__global__ void __launch_bounds__(kBatchThreads, REG ? 2 : 3) batched_pcg_kernel(
    Bsr A, const T* __restrict__ val, const T* __restrict__ minv, const double* __restrict__ b,
    double* __restrict__ x_out, const int32_t* __restrict__ node_off, const int32_t* __restrict__ cta_inst,
    const int32_t* __restrict__ cta_first, const int32_t* __restrict__ cta_size, T* xw, T* rw, T* zw, T* p0, T* p1,
    T* qw, const double* __restrict__ rtol_inst, int max_iter, int chunk, int first_launch, double* st,
    int32_t* its, int32_t* flag, double* __restrict__ relres_out, double* part, unsigned int* counters) {
  __shared__ double sfull[2 * kBatchThreads];
  __shared__ T s_alpha, s_tb;
  __shared__ int s_state;
  const int inst = cta_inst[blockIdx.x];
  const int first = cta_first[blockIdx.x], size = cta_size[blockIdx.x], rank = blockIdx.x - first;
  const int r0 = node_off[inst], nr = node_off[inst + 1] - r0;
  const int ra = r0 + (int)((int64_t)nr * rank / size), rb = r0 + (int)((int64_t)nr * (rank + 1) / size);
  unsigned int* counter = counters + inst;
  unsigned int bars = 0;
  const int row = ra + (int)threadIdx.x;  // REG: the thread's row
  const bool mine = row < rb;
  V3<T> xr{}, rv{}, zr{}, pr{}, qr{};
  T mv[9];
  if (REG && mine) load_minv(minv, row, mv);
  // thread 0 owns the FP64 scalars
  double rz = 0.0, rr = 0.0, bb = 0.0, beta = 0.0, tol2 = 0.0;
  int it = 0;
  if (first_launch) {  // x = 0, r = b, z = M^-1 r, p_old = 0 (so p_new = z on the first iteration)
    T lrz = T(0);
    double lrr = 0.0;
    for (int rw_ = REG ? row : ra + (int)threadIdx.x; rw_ < rb; rw_ += REG ? rb : (int)blockDim.x) {
      const V3<T> r_{T(b[3 * rw_]), T(b[3 * rw_ + 1]), T(b[3 * rw_ + 2])};
      T m[9];
      if (REG) {
#pragma unroll
        for (int k = 0; k < 9; ++k) m[k] = mv[k];
      } else {
        load_minv(minv, rw_, m);
      }
      const V3<T> z_ = jacobi(m, r_);
      store3(zw, rw_, z_.x, z_.y, z_.z);
      store3(p1, rw_, T(0), T(0), T(0));
      if (REG) {
        rv = r_, zr = z_;
      } else {
        store3(xw, rw_, T(0), T(0), T(0));
        store3(rw, rw_, r_.x, r_.y, r_.z);
      }
      lrz += r_.x * z_.x + r_.y * z_.y + r_.z * z_.z;
      lrr += double(r_.x) * double(r_.x) + double(r_.y) * double(r_.y) + double(r_.z) * double(r_.z);
    }
    double v[2] = {double(lrz), lrr};
    const bool ok = group_sum<2>(v, sfull, part, first, size, 1, counter, (++bars) * size);
    if (threadIdx.x == 0) {
      rz = v[0], bb = v[1], rr = v[1];
      s_state = ok ? 0 : -1;
    }
  } else {
    if (threadIdx.x == 0) {
      rz = st[4 * inst], rr = st[4 * inst + 1], bb = st[4 * inst + 2], beta = st[4 * inst + 3];
      s_state = 0;
    }
    it = its[inst];
    if (REG && mine) {
      xr = load3rw(xw, row), rv = load3rw(rw, row), zr = load3rw(zw, row);
      pr = load3rw((it & 1) ? p0 : p1, row);
    }
  }
  if (threadIdx.x == 0) {
    tol2 = rtol_inst[inst] * rtol_inst[inst] * bb;
    if (s_state == 0 && !(rr > tol2)) s_state = 1;
    if (s_state == 0 && it >= max_iter) s_state = 1;
    s_tb = T(beta);
  }
  __syncthreads();
  int state = s_state;
  const bool l2 = size > 1;
  for (int k = 0; state == 0 && k < chunk; ++k) {
    const T tb = s_tb;
    const T* pold = (it & 1) ? p0 : p1;
    T* pnew = (it & 1) ? p1 : p0;
    T lpq = T(0);
    if (REG) {
      if (mine) {
        qr = l2 ? row_product<T, true>(A, val, zw, pold, tb, row) : row_product<T, false>(A, val, zw, pold, tb, row);
        pr = {zr.x + tb * pr.x, zr.y + tb * pr.y, zr.z + tb * pr.z};
        store3(pnew, row, pr.x, pr.y, pr.z);
        lpq = pr.x * qr.x + pr.y * qr.y + pr.z * qr.z;
      }
    } else {
      for (int r_ = ra + (int)threadIdx.x; r_ < rb; r_ += blockDim.x) {
        const V3<T> q_ = l2 ? row_product<T, true>(A, val, zw, pold, tb, r_)
                            : row_product<T, false>(A, val, zw, pold, tb, r_);
        const V3<T> z_ = load3rw(zw, r_), po = load3rw(pold, r_);
        const V3<T> pn{z_.x + tb * po.x, z_.y + tb * po.y, z_.z + tb * po.z};
        store3(pnew, r_, pn.x, pn.y, pn.z);
        store3(qw, r_, q_.x, q_.y, q_.z);
        lpq += pn.x * q_.x + pn.y * q_.y + pn.z * q_.z;
      }
    }
    double v1[1] = {double(lpq)};
    const bool ok1 = group_sum<1>(v1, sfull, part, first, size, 0, counter, (++bars) * size);
    if (threadIdx.x == 0) {
      if (!ok1) {
        s_state = -1;
      } else if (!(fabs(v1[0]) > 0.0) || !isfinite(v1[0])) {
        s_state = 2;  // breakdown: leave with the current iterate
      } else {
        s_alpha = T(rz / v1[0]);
      }
    }
    __syncthreads();
    state = s_state;
    if (state != 0) break;
    const T alpha = s_alpha;
    T lrz = T(0);
    double lrr = 0.0;
    if (REG) {
      if (mine) {
        xr = {xr.x + alpha * pr.x, xr.y + alpha * pr.y, xr.z + alpha * pr.z};
        rv = {rv.x - alpha * qr.x, rv.y - alpha * qr.y, rv.z - alpha * qr.z};
        zr = jacobi(mv, rv);
        store3(zw, row, zr.x, zr.y, zr.z);
        lrz = rv.x * zr.x + rv.y * zr.y + rv.z * zr.z;
        lrr = double(rv.x) * double(rv.x) + double(rv.y) * double(rv.y) + double(rv.z) * double(rv.z);
      }
    } else {
      for (int r_ = ra + (int)threadIdx.x; r_ < rb; r_ += blockDim.x) {
        const V3<T> pv = load3rw(pnew, r_), qv = load3rw(qw, r_), xv = load3rw(xw, r_), r0v = load3rw(rw, r_);
        store3(xw, r_, xv.x + alpha * pv.x, xv.y + alpha * pv.y, xv.z + alpha * pv.z);
        const V3<T> r_n{r0v.x - alpha * qv.x, r0v.y - alpha * qv.y, r0v.z - alpha * qv.z};
        store3(rw, r_, r_n.x, r_n.y, r_n.z);
        T m[9];
        load_minv(minv, r_, m);
        const V3<T> z_ = jacobi(m, r_n);
        store3(zw, r_, z_.x, z_.y, z_.z);
        lrz += r_n.x * z_.x + r_n.y * z_.y + r_n.z * z_.z;
        lrr += double(r_n.x) * double(r_n.x) + double(r_n.y) * double(r_n.y) + double(r_n.z) * double(r_n.z);
      }
    }
    double v2[2] = {double(lrz), lrr};
    const bool ok2 = group_sum<2>(v2, sfull, part, first, size, 1, counter, (++bars) * size);
    ++it;
    if (threadIdx.x == 0) {
      if (!ok2) {
        s_state = -1;
      } else {
        beta = v2[0] / rz;
        rz = v2[0];
        rr = v2[1];
        s_tb = T(beta);
        if (!(rr > tol2) || it >= max_iter) s_state = 1;
      }
    }
    __syncthreads();
    state = s_state;
  }
  if (state == -1) {  // a wait gave up: report it, leave the vectors as they are
    if (rank == 0 && threadIdx.x == 0) flag[inst] = -1;
    return;
  }
  if (REG && mine && state == 0) {  // continued by the next launch
    store3(xw, row, xr.x, xr.y, xr.z);
    store3(rw, row, rv.x, rv.y, rv.z);
  }
  if (state != 0) {  // finished: the correction of the instance's rows
    for (int r_ = ra + (int)threadIdx.x; r_ < rb; r_ += blockDim.x) {
      const V3<T> xv = REG ? xr : load3rw(xw, r_);
      x_out[3 * r_] = double(xv.x), x_out[3 * r_ + 1] = double(xv.y), x_out[3 * r_ + 2] = double(xv.z);
    }
  }
  if (rank == 0 && threadIdx.x == 0) {
    st[4 * inst] = rz, st[4 * inst + 1] = rr, st[4 * inst + 2] = bb, st[4 * inst + 3] = beta;
    its[inst] = it;
    flag[inst] = state;
    relres_out[inst] = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  }
}

// The same PCG for groups whose CTAs hold few rows: TPR threads share a row (thread j of the row takes the row's
// blocks j, j + TPR, ...; the partial products are added by shuffles), and every thread copies its blocks and their
// columns into shared memory once per launch, so an iteration reads the matrix from shared memory and issues all of a
// thread's neighbour gathers at once (one L2 round trip).  Thread 0 of a row keeps the row's x, r, z, p and
// block-Jacobi inverse in registers.  Rows per CTA: kBatchThreads / TPR.  A row's slice may have at most TPR * kU
// blocks (the host checks).
template <typename T, int TPR>
struct SmemCfg {
  static constexpr int kU = (27 + TPR - 1) / TPR;  // blocks per thread: a hex node couples to at most 27 nodes
  static constexpr int kValBytes = 9 * kU * kBatchThreads * (int)sizeof(T);
  static constexpr int kBytes = kValBytes + kU * kBatchThreads * 4;
};

template <typename T, int TPR>
__global__ void __launch_bounds__(kBatchThreads, 2) batched_pcg_smem_kernel(
    Bsr A, const T* __restrict__ val, const T* __restrict__ minv, const double* __restrict__ b,
    double* __restrict__ x_out, const int32_t* __restrict__ node_off, const int32_t* __restrict__ cta_inst,
    const int32_t* __restrict__ cta_first, const int32_t* __restrict__ cta_size, T* xw, T* rw, T* zw, T* p0, T* p1,
    T* qw, const double* __restrict__ rtol_inst, int max_iter, int chunk, int first_launch, double* st,
    int32_t* its, int32_t* flag, double* __restrict__ relres_out, double* part, unsigned int* counters) {
  using C = SmemCfg<T, TPR>;
  constexpr int kU = C::kU;
  extern __shared__ __align__(16) unsigned char dsm[];
  T* sval = reinterpret_cast<T*>(dsm);                       // [9][kU][threads]
  int32_t* scol = reinterpret_cast<int32_t*>(dsm + C::kValBytes);  // [kU][threads], -1: no block
  __shared__ double sfull[2 * kBatchThreads];
  __shared__ T s_alpha, s_tb;
  __shared__ int s_state;
  const int inst = cta_inst[blockIdx.x];
  const int first = cta_first[blockIdx.x], size = cta_size[blockIdx.x], rank = blockIdx.x - first;
  const int r0 = node_off[inst], nr = node_off[inst + 1] - r0;
  const int ra = r0 + (int)((int64_t)nr * rank / size), rb = r0 + (int)((int64_t)nr * (rank + 1) / size);
  unsigned int* counter = counters + inst;
  unsigned int bars = 0;
  const int tid = threadIdx.x, j = tid % TPR;
  const int row = ra + tid / TPR;
  const bool mine = row < rb, lead = mine && j == 0;
  // this thread's blocks of its row: slice entries j, j + TPR, ... below the slice width
  {
    const int s = mine ? row >> 5 : 0, l = row & 31;
    const int gs = mine ? __ldg(A.slice_off + s) : 0, w = mine ? __ldg(A.slice_off + s + 1) - gs : 0;
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = j + TPR * u;
      const bool has = e < w;
      scol[u * kBatchThreads + tid] = has ? __ldg(A.col_sell + 32 * (gs + e) + l) : -1;
#pragma unroll
      for (int k = 0; k < 9; ++k)
        sval[(k * kU + u) * kBatchThreads + tid] = has ? __ldg(val + (int64_t)(gs + e) * 288 + l + 32 * k) : T(0);
    }
  }
  V3<T> xr{}, rv{}, zr{}, pr{};
  T mv[9];
  if (lead) load_minv(minv, row, mv);
  double rz = 0.0, rr = 0.0, bb = 0.0, beta = 0.0, tol2 = 0.0;  // thread 0's
  int it = 0;
  if (first_launch) {
    T lrz = T(0);
    double lrr = 0.0;
    if (lead) {
      rv = {T(b[3 * row]), T(b[3 * row + 1]), T(b[3 * row + 2])};
      zr = jacobi(mv, rv);
      store3(zw, row, zr.x, zr.y, zr.z);
      store3(p1, row, T(0), T(0), T(0));
      lrz = rv.x * zr.x + rv.y * zr.y + rv.z * zr.z;
      lrr = double(rv.x) * double(rv.x) + double(rv.y) * double(rv.y) + double(rv.z) * double(rv.z);
    }
    double v[2] = {double(lrz), lrr};
    const bool ok = group_sum<2>(v, sfull, part, first, size, 1, counter, (++bars) * size);
    if (tid == 0) {
      rz = v[0], bb = v[1], rr = v[1];
      s_state = ok ? 0 : -1;
    }
  } else {
    if (tid == 0) {
      rz = st[4 * inst], rr = st[4 * inst + 1], bb = st[4 * inst + 2], beta = st[4 * inst + 3];
      s_state = 0;
    }
    it = its[inst];
    if (lead) {
      xr = load3rw(xw, row), rv = load3rw(rw, row), zr = load3rw(zw, row);
      pr = load3rw((it & 1) ? p0 : p1, row);
    }
  }
  if (tid == 0) {
    tol2 = rtol_inst[inst] * rtol_inst[inst] * bb;
    if (s_state == 0 && !(rr > tol2)) s_state = 1;
    if (s_state == 0 && it >= max_iter) s_state = 1;
    s_tb = T(beta);
  }
  __syncthreads();
  int state = s_state;
  const bool l2 = size > 1;
  for (int k = 0; state == 0 && k < chunk; ++k) {
    const T tb = s_tb;
    const T* pold = (it & 1) ? p0 : p1;
    T* pnew = (it & 1) ? p1 : p0;
    T a0 = T(0), a1 = T(0), a2 = T(0);
    {
      int c[kU];
      V3<T> zv[kU], pv[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) c[u] = scol[u * kBatchThreads + tid];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (c[u] >= 0) {
          zv[u] = l2 ? gather3<true>(zw, c[u]) : gather3<false>(zw, c[u]);
          pv[u] = l2 ? gather3<true>(pold, c[u]) : gather3<false>(pold, c[u]);
        } else {
          zv[u] = {T(0), T(0), T(0)};
          pv[u] = zv[u];
        }
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const T x0 = zv[u].x + tb * pv[u].x, x1 = zv[u].y + tb * pv[u].y, x2 = zv[u].z + tb * pv[u].z;
        const T* m = sval + u * kBatchThreads + tid;
        constexpr int P = kU * kBatchThreads;
        a0 += m[0] * x0 + m[P] * x1 + m[2 * P] * x2;
        a1 += m[3 * P] * x0 + m[4 * P] * x1 + m[5 * P] * x2;
        a2 += m[6 * P] * x0 + m[7 * P] * x1 + m[8 * P] * x2;
      }
    }
#pragma unroll
    for (int o = 1; o < TPR; o <<= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    T lpq = T(0);
    if (lead) {
      pr = {zr.x + tb * pr.x, zr.y + tb * pr.y, zr.z + tb * pr.z};
      store3(pnew, row, pr.x, pr.y, pr.z);
      lpq = pr.x * a0 + pr.y * a1 + pr.z * a2;
    }
    double v1[1] = {double(lpq)};
    const bool ok1 = group_sum<1>(v1, sfull, part, first, size, 0, counter, (++bars) * size);
    if (tid == 0) {
      if (!ok1) {
        s_state = -1;
      } else if (!(fabs(v1[0]) > 0.0) || !isfinite(v1[0])) {
        s_state = 2;
      } else {
        s_alpha = T(rz / v1[0]);
      }
    }
    __syncthreads();
    state = s_state;
    if (state != 0) break;
    const T alpha = s_alpha;
    T lrz = T(0);
    double lrr = 0.0;
    if (lead) {
      xr = {xr.x + alpha * pr.x, xr.y + alpha * pr.y, xr.z + alpha * pr.z};
      rv = {rv.x - alpha * a0, rv.y - alpha * a1, rv.z - alpha * a2};
      zr = jacobi(mv, rv);
      store3(zw, row, zr.x, zr.y, zr.z);
      lrz = rv.x * zr.x + rv.y * zr.y + rv.z * zr.z;
      lrr = double(rv.x) * double(rv.x) + double(rv.y) * double(rv.y) + double(rv.z) * double(rv.z);
    }
    double v2[2] = {double(lrz), lrr};
    const bool ok2 = group_sum<2>(v2, sfull, part, first, size, 1, counter, (++bars) * size);
    ++it;
    if (tid == 0) {
      if (!ok2) {
        s_state = -1;
      } else {
        beta = v2[0] / rz;
        rz = v2[0];
        rr = v2[1];
        s_tb = T(beta);
        if (!(rr > tol2) || it >= max_iter) s_state = 1;
      }
    }
    __syncthreads();
    state = s_state;
  }
  if (state == -1) {
    if (rank == 0 && tid == 0) flag[inst] = -1;
    return;
  }
  if (lead && state == 0) {
    store3(xw, row, xr.x, xr.y, xr.z);
    store3(rw, row, rv.x, rv.y, rv.z);
  }
  if (lead && state != 0) x_out[3 * row] = double(xr.x), x_out[3 * row + 1] = double(xr.y), x_out[3 * row + 2] = double(xr.z);
  if (rank == 0 && tid == 0) {
    st[4 * inst] = rz, st[4 * inst + 1] = rr, st[4 * inst + 2] = bb, st[4 * inst + 3] = beta;
    its[inst] = it;
    flag[inst] = state;
    relres_out[inst] = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  }
}

// FP32 PCG of one instance per thread-block cluster of kClusterCtas CTAs (rows split across the cluster, one row per
// thread).  Each CTA keeps its rows' z and the two p buffers in shared memory; neighbours owned by other CTAs are read
// from their shared memory (distributed shared memory, ld.shared::cluster), and the group sums are exchanged the
// same way, so an iteration's two reductions are hardware cluster barriers (release / acquire at cluster scope) in
// place of global atomics and polls.  The CTA's matrix blocks and the owner (CTA rank, local row) of every column
// are copied to shared memory once per launch.  Clusters never wait on each other, so no co-residency is needed.
constexpr int kClusterCtas = 16;
constexpr int kClusterThreads = 192;
constexpr int kClusterWidth = 27;  // blocks per row (a hex node couples to at most 27 nodes)
struct ClusterCfg {
  static constexpr int kValBytes = 9 * kClusterWidth * kClusterThreads * 4;
  static constexpr int kColBytes = kClusterWidth * kClusterThreads * 4;
  static constexpr int kVecOff = kValBytes + kColBytes;
  static constexpr int kBytes = kVecOff + 3 * kClusterThreads * 16;  // z, p0, p1 (float4 per row)
};

__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t map_peer(uint32_t local_addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_addr), "r"(rank));
  return r;
}
__device__ __forceinline__ float4 ld_cluster_f4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr)
               : "memory");
  return v;
}
__device__ __forceinline__ double ld_cluster_f64(uint32_t addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}

// cluster-wide sums of N values: CTA sum (warp 0), published in this CTA's shared slot, cluster barrier, lane k < 16
// of warp 0 reads CTA k's slot; valid in warp 0
template <int N>
__device__ __forceinline__ void cluster_sum(double (&v)[N], double* sfull, double* red, const uint32_t* peer, int slot) {
  cta_reduce_smem<N>(v, sfull);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) red[2 * slot + k] = v[k];
  }
  cluster_sync_all();
  if (threadIdx.x < 32) {
    const uint32_t own = (uint32_t)__cvta_generic_to_shared(red + 2 * slot);
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const double t = threadIdx.x < kClusterCtas ? ld_cluster_f64(map_peer(own + 8 * k, threadIdx.x)) : 0.0;
      v[k] = warp_sum(t);
    }
  }
}

__global__ void __launch_bounds__(kClusterThreads, 1) batched_pcg_cluster_kernel(
    Bsr A, const float* __restrict__ val, const float* __restrict__ minv, const double* __restrict__ b,
    double* __restrict__ x_out, const int32_t* __restrict__ node_off, const int32_t* __restrict__ cluster_inst,
    float* xw, float* rw, float* zw, float* p0, float* p1, const double* __restrict__ rtol_inst, int max_iter,
    int chunk, int first_launch, double* st, int32_t* its, int32_t* flag, double* __restrict__ relres_out) {
  using C = ClusterCfg;
  constexpr int T = kClusterThreads, W = kClusterWidth;
  extern __shared__ __align__(16) unsigned char dsm[];
  float* sval = reinterpret_cast<float*>(dsm);                     // [9][W][T]
  int32_t* scol = reinterpret_cast<int32_t*>(dsm + C::kValBytes);  // [W][T]: owner rank << 16 | local row, -1
  float4* zs = reinterpret_cast<float4*>(dsm + C::kVecOff);        // [T] own rows' z, then p0, p1
  __shared__ double sfull[2 * T];
  __shared__ double red[4];
  __shared__ uint32_t peer[kClusterCtas];  // shared::cluster address of every CTA's dynamic shared memory
  __shared__ float s_alpha, s_tb;
  __shared__ int s_state;
  const int rank = (int)cluster_ctarank();
  const int inst = cluster_inst[blockIdx.x / kClusterCtas];
  const int r0 = node_off[inst], nr = node_off[inst + 1] - r0;
  auto row_start = [&](int k) { return r0 + (int)((int64_t)nr * k / kClusterCtas); };
  const int ra = row_start(rank), rb = row_start(rank + 1);
  const int tid = threadIdx.x, row = ra + tid;
  const bool mine = row < rb;
  if (tid < kClusterCtas) peer[tid] = map_peer((uint32_t)__cvta_generic_to_shared(dsm), tid);
  {  // this row's blocks and the owner of each column
    const int s = mine ? row >> 5 : 0, l = row & 31;
    const int gs = mine ? __ldg(A.slice_off + s) : 0, w = mine ? __ldg(A.slice_off + s + 1) - gs : 0;
    for (int u = 0; u < W; ++u) {
      int packed = -1;
      if (u < w) {
        const int c = __ldg(A.col_sell + 32 * (gs + u) + l);
        int k = (int)((int64_t)(c - r0) * kClusterCtas / nr);
        k = max(0, min(k, kClusterCtas - 1));
        while (k < kClusterCtas - 1 && c >= row_start(k + 1)) ++k;
        while (k > 0 && c < row_start(k)) --k;
        packed = (k << 16) | (c - row_start(k));
      }
      scol[u * T + tid] = packed;
#pragma unroll
      for (int k = 0; k < 9; ++k)
        sval[(k * W + u) * T + tid] = packed >= 0 ? __ldg(val + (int64_t)(gs + u) * 288 + l + 32 * k) : 0.f;
    }
  }
  V3<float> xr{}, rv{}, zr{}, pr{};
  float mv[9];
  if (mine) load_minv(minv, row, mv);
  double rz = 0.0, rr = 0.0, bb = 0.0, beta = 0.0, tol2 = 0.0;  // thread 0's
  int it = first_launch ? 0 : its[inst];
  float lrz = 0.f;
  double lrr = 0.0;
  if (mine) {
    if (first_launch) {  // x = 0, r = b, z = M^-1 r, p_old = 0
      rv = {float(b[3 * row]), float(b[3 * row + 1]), float(b[3 * row + 2])};
      zr = jacobi(mv, rv);
      lrz = rv.x * zr.x + rv.y * zr.y + rv.z * zr.z;
      lrr = double(rv.x) * double(rv.x) + double(rv.y) * double(rv.y) + double(rv.z) * double(rv.z);
    } else {
      xr = load3rw(xw, row), rv = load3rw(rw, row), zr = load3rw(zw, row);
      pr = load3rw((it & 1) ? p0 : p1, row);
    }
    zs[tid] = make_float4(zr.x, zr.y, zr.z, 0.f);
    zs[T * (1 + ((it & 1) ? 0 : 1)) + tid] = make_float4(pr.x, pr.y, pr.z, 0.f);  // p_old of iteration it
  }
  if (first_launch) {
    double v[2] = {double(lrz), lrr};
    cluster_sum<2>(v, sfull, red, peer, 1);
    if (tid == 0) rz = v[0], bb = v[1], rr = v[1];
  } else {
    cluster_sync_all();  // every CTA's z and p are in place before the first gathers
    if (tid == 0) rz = st[4 * inst], rr = st[4 * inst + 1], bb = st[4 * inst + 2], beta = st[4 * inst + 3];
  }
  if (tid == 0) {
    tol2 = rtol_inst[inst] * rtol_inst[inst] * bb;
    s_state = (!(rr > tol2) || it >= max_iter) ? 1 : 0;
    s_tb = float(beta);
  }
  __syncthreads();
  int state = s_state;
  const uint32_t zoff = C::kVecOff;
  for (int k = 0; state == 0 && k < chunk; ++k) {
    const float tb = s_tb;
    const int po = (it & 1) ? 1 : 2, pn = (it & 1) ? 2 : 1;  // p_old / p_new slots (p0 = slot 1, p1 = slot 2)
    const uint32_t off_z = zoff, off_p = zoff + po * T * 16;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    if (mine) {
#pragma unroll
      for (int u0 = 0; u0 < W; u0 += 9) {
        float4 zv[9], pv[9];
#pragma unroll
        for (int u = 0; u < 9; ++u) {
          const int packed = scol[(u0 + u) * T + tid];
          if (packed >= 0) {
            const uint32_t base = peer[packed >> 16] + 16u * (uint32_t)(packed & 0xffff);
            zv[u] = ld_cluster_f4(base + off_z);
            pv[u] = ld_cluster_f4(base + off_p);
          } else {
            zv[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            pv[u] = zv[u];
          }
        }
#pragma unroll
        for (int u = 0; u < 9; ++u) {
          const float x0 = zv[u].x + tb * pv[u].x, x1 = zv[u].y + tb * pv[u].y, x2 = zv[u].z + tb * pv[u].z;
          const float* m = sval + (u0 + u) * T + tid;
          constexpr int P = W * T;
          a0 += m[0] * x0 + m[P] * x1 + m[2 * P] * x2;
          a1 += m[3 * P] * x0 + m[4 * P] * x1 + m[5 * P] * x2;
          a2 += m[6 * P] * x0 + m[7 * P] * x1 + m[8 * P] * x2;
        }
      }
    }
    float lpq = 0.f;
    if (mine) {
      pr = {zr.x + tb * pr.x, zr.y + tb * pr.y, zr.z + tb * pr.z};
      zs[pn * T + tid] = make_float4(pr.x, pr.y, pr.z, 0.f);
      lpq = pr.x * a0 + pr.y * a1 + pr.z * a2;
    }
    double v1[1] = {double(lpq)};
    cluster_sum<1>(v1, sfull, red, peer, 0);
    if (tid == 0) {
      if (!(fabs(v1[0]) > 0.0) || !isfinite(v1[0])) s_state = 2;
      else s_alpha = float(rz / v1[0]);
    }
    __syncthreads();
    state = s_state;
    if (state != 0) break;
    const float alpha = s_alpha;
    lrz = 0.f;
    lrr = 0.0;
    if (mine) {
      xr = {xr.x + alpha * pr.x, xr.y + alpha * pr.y, xr.z + alpha * pr.z};
      rv = {rv.x - alpha * a0, rv.y - alpha * a1, rv.z - alpha * a2};
      zr = jacobi(mv, rv);
      zs[tid] = make_float4(zr.x, zr.y, zr.z, 0.f);
      lrz = rv.x * zr.x + rv.y * zr.y + rv.z * zr.z;
      lrr = double(rv.x) * double(rv.x) + double(rv.y) * double(rv.y) + double(rv.z) * double(rv.z);
    }
    double v2[2] = {double(lrz), lrr};
    cluster_sum<2>(v2, sfull, red, peer, 1);
    ++it;
    if (tid == 0) {
      beta = v2[0] / rz;
      rz = v2[0];
      rr = v2[1];
      s_tb = float(beta);
      if (!(rr > tol2) || it >= max_iter) s_state = 1;
    }
    __syncthreads();
    state = s_state;
  }
  if (mine) {
    if (state == 0) {  // continued by the next launch: the state the other variants read
      store3(xw, row, xr.x, xr.y, xr.z);
      store3(rw, row, rv.x, rv.y, rv.z);
      store3(zw, row, zr.x, zr.y, zr.z);
      store3((it & 1) ? p0 : p1, row, pr.x, pr.y, pr.z);
    } else {
      x_out[3 * row] = double(xr.x), x_out[3 * row + 1] = double(xr.y), x_out[3 * row + 2] = double(xr.z);
    }
  }
  if (rank == 0 && tid == 0) {
    st[4 * inst] = rz, st[4 * inst + 1] = rr, st[4 * inst + 2] = bb, st[4 * inst + 3] = beta;
    its[inst] = it;
    flag[inst] = state;
    relres_out[inst] = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  }
  cluster_sync_all();  // no CTA leaves while another may still read its shared memory
}

// per-instance sum of squares over dof ranges [3 node_off[i], 3 node_off[i+1]); one block per instance
__global__ void instance_norms_kernel(const double* __restrict__ x, const int32_t* __restrict__ node_off,
                                      double* __restrict__ out) {
  __shared__ double sh[33];
  const int inst = blockIdx.x;
  double s = 0.0;
  for (int i = 3 * node_off[inst] + threadIdx.x; i < 3 * node_off[inst + 1]; i += blockDim.x) s += x[i] * x[i];
  s = block_sum_all(s, sh);
  if (threadIdx.x == 0) out[inst] = sqrt(s);
}

// u = u_old + step[i] corr on the dofs of every instance i with step[i] != 1 (one block per instance)
__global__ void instance_step_kernel(double* __restrict__ u, const double* __restrict__ u_old,
                                     const double* __restrict__ corr, const int32_t* __restrict__ node_off,
                                     const double* __restrict__ step) {
  const int inst = blockIdx.x;
  const double sc = step[inst];
  if (sc == 1.0) return;
  for (int i = 3 * node_off[inst] + threadIdx.x; i < 3 * node_off[inst + 1]; i += blockDim.x)
    u[i] = u_old[i] + sc * corr[i];
}

}  // namespace

void launch_instance_step(double* u, const double* u_old, const double* corr, int n_inst, const int32_t* node_off,
                          const double* step, cudaStream_t s) {
  instance_step_kernel<<<n_inst, 256, 0, s>>>(u, u_old, corr, node_off, step);
}

// variants: 0 rows loop (state in the work arrays), 1 one row per thread (state in registers), 2 / 3 / 5 four /
// eight / sixteen threads per row with the matrix in shared memory (4, the cluster kernel, launches separately)
static int threads_per_row(int variant) { return variant == 2 ? 4 : (variant == 3 ? 8 : (variant == 5 ? 16 : 1)); }

static const void* batched_kernel(bool fp32, int variant) {
  if (fp32) {
    switch (variant) {
      case 0: return (const void*)batched_pcg_kernel<float, false>;
      case 1: return (const void*)batched_pcg_kernel<float, true>;
      case 2: return (const void*)batched_pcg_smem_kernel<float, 4>;
      case 3: return (const void*)batched_pcg_smem_kernel<float, 8>;
      default: return (const void*)batched_pcg_smem_kernel<float, 16>;
    }
  }
  switch (variant) {
    case 0: return (const void*)batched_pcg_kernel<double, false>;
    case 1: return (const void*)batched_pcg_kernel<double, true>;
    case 2: return (const void*)batched_pcg_smem_kernel<double, 4>;
    case 3: return (const void*)batched_pcg_smem_kernel<double, 8>;
    default: return (const void*)batched_pcg_smem_kernel<double, 16>;
  }
}

static int batched_smem_bytes(bool fp32, int variant) {
  switch (threads_per_row(variant)) {
    case 4: return fp32 ? SmemCfg<float, 4>::kBytes : SmemCfg<double, 4>::kBytes;
    case 8: return fp32 ? SmemCfg<float, 8>::kBytes : SmemCfg<double, 8>::kBytes;
    case 16: return fp32 ? SmemCfg<float, 16>::kBytes : SmemCfg<double, 16>::kBytes;
    default: return 0;
  }
}

// resident CTAs per SM of every variant, queried once per device (the planner asks before every launch)
static int blocks_per_sm(bool fp32, int variant) {
  static std::mutex mu;
  static std::map<std::tuple<int, bool, int>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_tuple(dev, fp32, variant);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  const void* k = batched_kernel(fp32, variant);
  const int smem = batched_smem_bytes(fp32, variant);
  int b = 0;
  if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    b = 0;
  else if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, kBatchThreads, smem) != cudaSuccess)
    b = 0;
  cache[key] = b;
  return b;
}

int batched_pcg_capacity(bool fp32, int variant, int sms) { return blocks_per_sm(fp32, variant) * sms; }


int batched_cluster_rows() { return kClusterCtas * kClusterThreads; }
int batched_cluster_width() { return kClusterWidth; }

static cudaError_t cluster_prepare() {
  const void* k = (const void*)batched_pcg_cluster_kernel;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, ClusterCfg::kBytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
}

static int cluster_capacity_query() {
  if (cluster_prepare() != cudaSuccess) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kClusterCtas);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = ClusterCfg::kBytes;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas, at[0].val.clusterDim.y = 1, at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (const void*)batched_pcg_cluster_kernel, &cfg) != cudaSuccess) return 0;
  return n;
}

int batched_cluster_capacity() {
  static std::mutex mu;
  static std::map<int, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  return cache[dev] = cluster_capacity_query();
}

cudaError_t launch_batched_pcg_cluster(const Bsr& A, const void* minv, const double* b, double* x_out, int n_clusters,
                                       const int32_t* node_off, const int32_t* cluster_inst, void* xw, void* rw,
                                       void* zw, void* p0, void* p1, const double* rtol, int max_iter, int chunk,
                                       int first_launch, double* st, int32_t* its, int32_t* flag, double* relres,
                                       cudaStream_t s) {
  cudaError_t e = cluster_prepare();
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kClusterCtas * n_clusters);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = ClusterCfg::kBytes;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas, at[0].val.clusterDim.y = 1, at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, batched_pcg_cluster_kernel, A, (const float*)A.val, (const float*)minv, b, x_out,
                            node_off, cluster_inst, (float*)xw, (float*)rw, (float*)zw, (float*)p0, (float*)p1, rtol,
                            max_iter, chunk, first_launch, st, its, flag, relres);
}
int batched_pcg_rows_per_cta(int variant) { return kBatchThreads / threads_per_row(variant); }
int batched_pcg_max_width(int variant) {
  switch (threads_per_row(variant)) {
    case 4: return 4 * SmemCfg<float, 4>::kU;
    case 8: return 8 * SmemCfg<float, 8>::kU;
    case 16: return 16 * SmemCfg<float, 16>::kU;
    default: return 1 << 30;
  }
}

cudaError_t launch_batched_pcg(const Bsr& A, bool fp32, int variant, const void* minv, const double* b, double* x_out,
                               int n_cta, const int32_t* node_off, const int32_t* cta_inst, const int32_t* cta_first,
                               const int32_t* cta_size, void* xw, void* rw, void* zw, void* p0, void* p1, void* qw,
                               const double* rtol, int max_iter, int chunk, int first_launch, double* st, int32_t* its,
                               int32_t* flag, double* relres, double* part, unsigned int* counters, int n_inst,
                               bool cooperative, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(unsigned int) * n_inst, s);
  if (e != cudaSuccess) return e;
  Bsr Acopy = A;
  const void* val = A.val;
  void* args[] = {&Acopy, &val,  &minv, &b,  &x_out, &node_off, &cta_inst, &cta_first, &cta_size,
                  &xw,    &rw,   &zw,   &p0, &p1,    &qw,       &rtol,     &max_iter,  &chunk,
                  &first_launch, &st, &its, &flag, &relres, &part, &counters};
  const void* kern = batched_kernel(fp32, variant);
  const int smem = batched_smem_bytes(fp32, variant);
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  // a group of one CTA waits on no other CTA: without multi-CTA groups an ordinary launch will do
  if (!cooperative) return cudaLaunchKernel(kern, dim3(n_cta), dim3(kBatchThreads), args, smem, s);
  return cudaLaunchCooperativeKernel(kern, dim3(n_cta), dim3(kBatchThreads), args, smem, s);
}

void launch_instance_norms(const double* x, int n_inst, const int32_t* node_off, double* out, cudaStream_t s) {
  instance_norms_kernel<<<n_inst, 256, 0, s>>>(x, node_off, out);
}

}  // namespace ikr
