// Block-Jacobi preconditioned conjugate gradients on the sliced-ELL 3x3-block tangent (sm_103a).
//
// Replaces the reference's LinearSolver solve step (ikarus/solver/linearsolver/linearsolver.hh:178-232,
// linearsolver.cpp:17-83) inside NewtonRaphson::solve (newtonraphson.hh:221-224).
//
// CG vectors are node-padded: four values per node (x, y, z, 0), so gathering a neighbour is one 16-byte
// load (FP32) or two (FP64).  One CG iteration is two kernels on a fixed grid (a multiple of the SM count):
//   spmv:   p_new = z + beta p_old (formed on the fly for every gathered neighbour, written for the thread's
//           own row), q = K p_new (one thread per block row, sliced-ELL), partial sums of p_new . q;
//           the last block to finish sums the partials in a fixed order and sets alpha = rz / (p.q).
//   update: x += alpha p, r -= alpha q, z = M^{-1} r with the 3x3 block-Jacobi inverse, partial sums of r.z
//           and r.r; the last block sums them, counts the iteration, tests rr <= rtol^2 |b|^2 and the
//           iteration limit, and sets beta for the next iteration.
// "Last block" = the block that draws the final ticket of an atomic counter after publishing its partial
// (threadfence reduction); it sums all partials in index order, so results are bit-identical run to run.
// p_old / p_new alternate between two buffers by iteration parity.  Once converged both kernels return at
// entry, so chunks of iterations can be launched ahead (and captured in a CUDA graph) while the host polls.
#include "cg_common.cuh"

namespace ikr {

namespace {

using namespace cg;
constexpr int kThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kThreads) pcg_spmv_kernel(Bsr A, const T* __restrict__ val, const T* __restrict__ z,
                                                            const T* __restrict__ pold, T* __restrict__ pnew,
                                                            T* __restrict__ q, double* part, double* scal) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (scal[kDone] != 0.0) return;
  const T beta = T(scal[kBeta]);
  // one thread per block row; a warp is one slice, so every value / column load is a 128-byte line and the
  // blocks of a row are independent loads
  double pq = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
    const int s = row >> 5, l = row & 31;
    const int g0 = A.slice_off[s], g1 = A.slice_off[s + 1];
    T a0 = T(0), a1 = T(0), a2 = T(0);
#pragma unroll 4
    for (int g = g0; g < g1; ++g) {
      const int c = __ldg(A.col_sell + 32 * g + l);
      const T* v = val + (int64_t)g * 288 + l;
      const V3<T> zc = load3(z, c), pc = load3(pold, c);
      const T x0 = zc.x + beta * pc.x, x1 = zc.y + beta * pc.y, x2 = zc.z + beta * pc.z;
      a0 += __ldg(v) * x0 + __ldg(v + 32) * x1 + __ldg(v + 64) * x2;
      a1 += __ldg(v + 96) * x0 + __ldg(v + 128) * x1 + __ldg(v + 160) * x2;
      a2 += __ldg(v + 192) * x0 + __ldg(v + 224) * x1 + __ldg(v + 256) * x2;
    }
    const V3<T> zr = load3(z, row), pr = load3(pold, row);
    const T p0 = zr.x + beta * pr.x, p1 = zr.y + beta * pr.y, p2 = zr.z + beta * pr.z;
    store3(pnew, row, p0, p1, p2);
    store3(q, row, a0, a1, a2);
    pq += double(p0 * a0 + p1 * a1 + p2 * a2);
  }
  const double tot = block_sum_all(pq, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
  if (publish_and_check_last(&tickets(scal)[0], &last)) {
    const double pqs = sum_partials(part, gridDim.x, 1, sh);
    if (threadIdx.x == 0) {
      if (scal[kDone] == 0.0) {
        // negative curvature (an indefinite tangent away from equilibrium, which the reference's LDL^T
        // factorisation solves as well) does not stop the iteration; a zero or non-finite p.Kp does
        if (!(fabs(pqs) > 0.0) || !isfinite(pqs)) scal[kDone] = 3.0;
        else scal[kAlpha] = scal[kRz] / pqs;
      }
      tickets(scal)[0] = 0u;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) pcg_update_kernel(int n_rows, const T* __restrict__ minv,
                                                              const T* __restrict__ pnew, const T* __restrict__ q,
                                                              T* x, T* r, T* z, double* part, double* scal,
                                                              int coarse) {
  __shared__ double sh[32];
  __shared__ bool last;
  if (scal[kDone] != 0.0) return;
  const T alpha = T(scal[kAlpha]);
  T rz = T(0), rr = T(0);
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {
    const V3<T> p = load3(pnew, row), qq = load3(q, row), xx = load3rw(x, row), r0 = load3rw(r, row);
    store3(x, row, xx.x + alpha * p.x, xx.y + alpha * p.y, xx.z + alpha * p.z);
    const T r1[3] = {r0.x - alpha * qq.x, r0.y - alpha * qq.y, r0.z - alpha * qq.z};
    store3(r, row, r1[0], r1[1], r1[2]);
    const T* m = minv + 9 * (int64_t)row;
    T zv[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      zv[a] = __ldg(m + 3 * a) * r1[0] + __ldg(m + 3 * a + 1) * r1[1] + __ldg(m + 3 * a + 2) * r1[2];
      rz += r1[a] * zv[a];
      rr += r1[a] * r1[a];
    }
    store3(z, row, zv[0], zv[1], zv[2]);
  }
  const double trz = block_sum_all(double(rz), sh);
  const double trr = block_sum_all(double(rr), sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = trz;
    part[2 * blockIdx.x + 1] = trr;
  }
  if (publish_and_check_last(&tickets(scal)[1], &last)) {
    const double rzs = sum_partials(part, gridDim.x, 2, sh);
    const double rrs = sum_partials(part + 1, gridDim.x, 2, sh);
    if (threadIdx.x == 0) {
      const double it = scal[kIters] + 1.0;
      scal[kIters] = it;
      scal[kRR] = rrs;
      if (rrs <= scal[kTol2]) scal[kDone] = 1.0;
      else if (it >= scal[kMaxIt]) scal[kDone] = 2.0;
      if (coarse) {
        scal[kRzF] = rzs;  // the coarse correction adds r_c . e and sets beta
      } else {
        scal[kBeta] = rzs / scal[kRz];
        scal[kRz] = rzs;
      }
      tickets(scal)[1] = 0u;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) pcg_init_kernel(int n_rows, const T* __restrict__ minv,
                                                            const double* __restrict__ b, T* x, T* r, T* z, T* pold,
                                                            double* part, double* scal, double rtol,
                                                            const double* __restrict__ rtol_dev, int max_iter,
                                                            int coarse) {
  __shared__ double sh[32];
  __shared__ bool last;
  double rz = 0.0, rr = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {
    const T rv[3] = {T(b[3 * row]), T(b[3 * row + 1]), T(b[3 * row + 2])};
    store3(r, row, rv[0], rv[1], rv[2]);
    store3(x, row, T(0), T(0), T(0));
    store3(pold, row, T(0), T(0), T(0));
    const T* m = minv + 9 * (int64_t)row;
    T zv[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      zv[a] = m[3 * a] * rv[0] + m[3 * a + 1] * rv[1] + m[3 * a + 2] * rv[2];
      rz += double(rv[a] * zv[a]);
      rr += double(rv[a]) * double(rv[a]);
    }
    store3(z, row, zv[0], zv[1], zv[2]);
  }
  const double trz = block_sum_all(rz, sh);
  const double trr = block_sum_all(rr, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = trz;
    part[2 * blockIdx.x + 1] = trr;
  }
  if (publish_and_check_last(&tickets(scal)[2], &last)) {
    const double rzs = sum_partials(part, gridDim.x, 2, sh);
    const double rrs = sum_partials(part + 1, gridDim.x, 2, sh);
    if (threadIdx.x == 0) {
      scal[kBB] = rrs;
      const double rt = rtol_dev ? *rtol_dev : rtol;  // a captured solve reads its tolerance at run time
      scal[kTol2] = rt * rt * rrs;
      scal[coarse ? kRzF : kRz] = rzs;
      scal[kBeta] = 0.0;
      scal[kAlpha] = 0.0;
      scal[kIters] = 0.0;
      scal[kRR] = rrs;
      scal[kMaxIt] = (double)max_iter;
      scal[kDone] = (rrs <= rtol * rtol * rrs) ? 1.0 : 0.0;  // b = 0
      tickets(scal)[2] = 0u;
    }
  }
}

template <typename T>
__global__ void block_jacobi_kernel(Bsr A, const T* __restrict__ val, T* __restrict__ minv, bool point) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= A.n_rows) return;
  const T* b = val + block_entry(A.diag[row], 0);
  double m[3][3], r[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m[i][j] = double(b[32 * (3 * i + j)]);
  if (point) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) r[i][j] = (i == j && m[i][i] != 0.0) ? 1.0 / m[i][i] : 0.0;
  } else {
    inv3(m, r);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) minv[9 * (int64_t)row + 3 * i + j] = T(r[i][j]);
}

// r = b - K x (or K x) with FP64 accumulation on dof-major FP64 vectors; thread per block row
template <typename T>
__global__ void residual64_kernel(Bsr A, const T* __restrict__ val, const double* __restrict__ x,
                                  const double* __restrict__ b, double* __restrict__ out, bool subtract) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n_rows; row += gridDim.x * blockDim.x) {
    const int s = row >> 5, l = row & 31;
    double a0 = 0, a1 = 0, a2 = 0;
#pragma unroll 4
    for (int g = A.slice_off[s]; g < A.slice_off[s + 1]; ++g) {
      const int c3 = 3 * A.col_sell[32 * g + l];
      const T* v = val + (int64_t)g * 288 + l;
      const double x0 = x[c3], x1 = x[c3 + 1], x2 = x[c3 + 2];
      a0 += double(v[0]) * x0 + double(v[32]) * x1 + double(v[64]) * x2;
      a1 += double(v[96]) * x0 + double(v[128]) * x1 + double(v[160]) * x2;
      a2 += double(v[192]) * x0 + double(v[224]) * x1 + double(v[256]) * x2;
    }
    const int i = 3 * row;
    out[i] = subtract ? b[i] - a0 : a0;
    out[i + 1] = subtract ? b[i + 1] - a1 : a1;
    out[i + 2] = subtract ? b[i + 2] - a2 : a2;
  }
}

// node-padded CG vector -> dof-major FP64
template <typename T>
__global__ void result_kernel(const T* __restrict__ x, double* __restrict__ out, double scale, int n_rows) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {
    const V3<T> v = load3rw(x, row);
    out[3 * row] = scale * double(v.x);
    out[3 * row + 1] = scale * double(v.y);
    out[3 * row + 2] = scale * double(v.z);
  }
}
__global__ void axpy64_kernel(double* __restrict__ y, const double* __restrict__ x, double a, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
__global__ void scale64_kernel(double* __restrict__ y, const double* __restrict__ x, double a, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

inline int blocks_for(int64_t n, int bs) { return (int)((n + bs - 1) / bs); }
inline int grid_cap(int64_t n, int bs) {
  const int b = blocks_for(n, bs);
  return b < 1216 ? (b < 1 ? 1 : b) : 1216;  // 8 blocks per SM on 152 SMs
}

}  // namespace

void launch_block_jacobi(const Bsr& A, bool fp32, void* minv, bool point_jacobi, cudaStream_t s) {
  if (fp32)
    block_jacobi_kernel<float><<<blocks_for(A.n_rows, 128), 128, 0, s>>>(A, (const float*)A.val, (float*)minv,
                                                                           point_jacobi);
  else
    block_jacobi_kernel<double><<<blocks_for(A.n_rows, 128), 128, 0, s>>>(A, (const double*)A.val, (double*)minv,
                                                                            point_jacobi);
}

void launch_pcg_init(const Bsr& A, PcgWork& w, const double* b, double rtol, int max_iter, cudaStream_t s) {
  (void)A;
  cudaMemsetAsync(w.scal, 0, sizeof(double) * kNScal, s);  // scalars and tickets start at zero
  if (w.fp32)
    pcg_init_kernel<float><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const float*)w.minv, b, (float*)w.x, (float*)w.r,
                                                        (float*)w.z, (float*)w.p1, w.part_b, w.scal, rtol, w.rtol_dev,
                                                        max_iter, w.coarse);
  else
    pcg_init_kernel<double><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const double*)w.minv, b, (double*)w.x,
                                                         (double*)w.r, (double*)w.z, (double*)w.p1, w.part_b, w.scal,
                                                         rtol, w.rtol_dev, max_iter, w.coarse);
}

void launch_pcg_spmv(const Bsr& A, PcgWork& w, int parity, cudaStream_t s) {
  void* pnew = parity ? w.p1 : w.p0;
  void* pold = parity ? w.p0 : w.p1;
  if (w.spmv_kind > 0) {
    launch_pcg_spmv_staged(A, w, w.spmv_kind - 1, pold, pnew, s);
    return;
  }
  if (w.fp32)
    pcg_spmv_kernel<float><<<w.grid, kThreads, 0, s>>>(A, (const float*)A.val, (const float*)w.z, (const float*)pold,
                                                        (float*)pnew, (float*)w.q, w.part_a, w.scal);
  else
    pcg_spmv_kernel<double><<<w.grid, kThreads, 0, s>>>(A, (const double*)A.val, (const double*)w.z,
                                                         (const double*)pold, (double*)pnew, (double*)w.q, w.part_a,
                                                         w.scal);
}
void launch_pcg_update(const Bsr& A, PcgWork& w, int parity, cudaStream_t s) {
  (void)A;
  void* pnew = parity ? w.p1 : w.p0;
  if (w.fp32)
    pcg_update_kernel<float><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const float*)w.minv, (const float*)pnew,
                                                          (const float*)w.q, (float*)w.x, (float*)w.r, (float*)w.z,
                                                          w.part_b, w.scal, w.coarse);
  else
    pcg_update_kernel<double><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const double*)w.minv, (const double*)pnew,
                                                           (const double*)w.q, (double*)w.x, (double*)w.r,
                                                           (double*)w.z, w.part_b, w.scal, w.coarse);
}
void launch_pcg_iteration(const Bsr& A, PcgWork& w, int parity, cudaStream_t s) {
  launch_pcg_spmv(A, w, parity, s);
  launch_pcg_update(A, w, parity, s);
}

void launch_pcg_result(const PcgWork& w, double* x_out, double scale, cudaStream_t s) {
  if (w.fp32) result_kernel<float><<<grid_cap(w.n_rows, 256), 256, 0, s>>>((const float*)w.x, x_out, scale, w.n_rows);
  else result_kernel<double><<<grid_cap(w.n_rows, 256), 256, 0, s>>>((const double*)w.x, x_out, scale, w.n_rows);
}

void launch_residual64(const Bsr& A, bool fp32, const double* x, const double* b, double* r, cudaStream_t s) {
  const int g = grid_cap(A.n_rows, 256);
  if (fp32) residual64_kernel<float><<<g, 256, 0, s>>>(A, (const float*)A.val, x, b, r, true);
  else residual64_kernel<double><<<g, 256, 0, s>>>(A, (const double*)A.val, x, b, r, true);
}
void launch_spmv64(const Bsr& A, bool fp32, const double* x, double* y, cudaStream_t s) {
  const int g = grid_cap(A.n_rows, 256);
  if (fp32) residual64_kernel<float><<<g, 256, 0, s>>>(A, (const float*)A.val, x, nullptr, y, false);
  else residual64_kernel<double><<<g, 256, 0, s>>>(A, (const double*)A.val, x, nullptr, y, false);
}
void launch_axpy64(double* y, const double* x, double a, int64_t n, cudaStream_t s) {
  axpy64_kernel<<<grid_cap(n, 256), 256, 0, s>>>(y, x, a, n);
}
void launch_scale64(double* y, const double* x, double a, int64_t n, cudaStream_t s) {
  scale64_kernel<<<grid_cap(n, 256), 256, 0, s>>>(y, x, a, n);
}

}  // namespace ikr
