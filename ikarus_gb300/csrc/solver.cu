// Block-Jacobi preconditioned conjugate gradients on the 3x3-block CSR tangent (sm_103a).
//
// Replaces the reference's LinearSolver solve step (ikarus/solver/linearsolver/linearsolver.hh:178-232,
// linearsolver.cpp:17-83) inside NewtonRaphson::solve (newtonraphson.hh:221-224).
//
// One CG iteration is two kernels, both on a fixed grid (a multiple of the SM count) so every reduction
// has a fixed shape and the result is bit-identical from run to run:
//   A (spmv):   sums the previous update's partials -> rz, rr; stops when rr <= rtol^2 |b|^2;
//               beta = rz / rz_old;  p_new = z + beta p_old  (formed on the fly for every gathered column,
//               written for the block's own rows);  q = K p_new;  partial sums of p_new . q.
//   B (update): sums the SpMV partials -> alpha = rz / (p.q);  x += alpha p;  r -= alpha q;  z = M^{-1} r
//               with the 3x3 block-Jacobi inverse;  partial sums of r.z and r.r.
// p_old / p_new alternate between two buffers by iteration parity, and so do the scalars rz and the
// iteration counter, so that no kernel reads a value another block of the same launch writes.
// Partial sums are accumulated per thread in the vector precision and across threads in FP64.
// Once converged, both kernels return at entry, so chunks of iterations can be launched ahead
// (and captured in a CUDA graph) and the host only polls the scalars between chunks.
#include "common.cuh"
#include "kernels.h"

namespace ikr {

namespace {

constexpr int kThreads = 256;

template <typename T>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

// deterministic redundant sum of n partials with stride st (every block computes the same value)
__device__ __forceinline__ double sum_partials(const double* __restrict__ p, int n, int st, double* sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += p[i * st];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  double r = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (threadIdx.x < 32) r = warp_sum(r);
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = r;
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) pcg_spmv_kernel(Bsr A, const T* __restrict__ val, const T* __restrict__ z,
                                                            const T* __restrict__ pold, T* __restrict__ pnew,
                                                            T* __restrict__ q, const double* __restrict__ part_b,
                                                            double* __restrict__ part_a, double* scal, int parity,
                                                            int nparts) {
  __shared__ double sh[32];
  if (scal[kDone] != 0.0) return;
  const double rz = sum_partials(part_b, nparts, 2, sh);
  const double rr = sum_partials(part_b + 1, nparts, 2, sh);
  const double iters = scal[kIters + (parity ^ 1)];
  if (rr <= scal[kTol2] || iters >= scal[kMaxIt]) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      scal[kDone] = (rr <= scal[kTol2]) ? 1.0 : 2.0;
      scal[kRR] = rr;
      scal[kIters + parity] = iters;
    }
    return;
  }
  const T beta = T(rz / scal[kRz + (parity ^ 1)]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    scal[kRz + parity] = rz;
    scal[kRR] = rr;
    scal[kIters + parity] = iters + 1.0;
  }
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  double pq = 0.0;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < A.n_rows; row += warps) {
    const int b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
    const int nv = 9 * (b1 - b0);
    const T* v = val + 9 * (int64_t)b0;
    T a0 = T(0), a1 = T(0), a2 = T(0);
    for (int idx = lane; idx < nv; idx += 32) {
      const int b = idx / 9;
      const int r9 = idx - 9 * b;
      const int ar = r9 / 3;
      const int c = r9 - 3 * ar;
      const int colv = 3 * A.col[b0 + b] + c;
      const T xv = z[colv] + beta * pold[colv];
      const T prod = v[idx] * xv;
      a0 += ar == 0 ? prod : T(0);
      a1 += ar == 1 ? prod : T(0);
      a2 += ar == 2 ? prod : T(0);
    }
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    a2 = warp_sum(a2);
    if (lane < 3) {
      const T pn = z[3 * row + lane] + beta * pold[3 * row + lane];
      const T qv = lane == 0 ? a0 : (lane == 1 ? a1 : a2);
      pnew[3 * row + lane] = pn;
      q[3 * row + lane] = qv;
      pq += double(pn * qv);
    }
  }
  const double tot = block_sum<T>(pq, sh);
  if (threadIdx.x == 0) part_a[blockIdx.x] = tot;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) pcg_update_kernel(int n_rows, const T* __restrict__ minv,
                                                              const T* __restrict__ pnew, const T* __restrict__ q,
                                                              T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                                                              const double* __restrict__ part_a,
                                                              double* __restrict__ part_b, double* scal, int parity,
                                                              int nparts) {
  __shared__ double sh[32];
  if (scal[kDone] != 0.0) return;
  const double pq = sum_partials(part_a, nparts, 1, sh);
  if (!(pq > 0.0)) {  // loss of positive definiteness or NaN
    if (blockIdx.x == 0 && threadIdx.x == 0) scal[kDone] = 3.0;
    return;
  }
  const T alpha = T(scal[kRz + parity] / pq);
  T rz = T(0), rr = T(0);
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {
    T rv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int i = 3 * row + c;
      x[i] += alpha * pnew[i];
      rv[c] = r[i] - alpha * q[i];
      r[i] = rv[c];
    }
    const T* m = minv + 9 * (int64_t)row;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const T zv = m[3 * a] * rv[0] + m[3 * a + 1] * rv[1] + m[3 * a + 2] * rv[2];
      z[3 * row + a] = zv;
      rz += rv[a] * zv;
      rr += rv[a] * rv[a];
    }
  }
  const double trz = block_sum<T>(double(rz), sh);
  const double trr = block_sum<T>(double(rr), sh);
  if (threadIdx.x == 0) {
    part_b[2 * blockIdx.x] = trz;
    part_b[2 * blockIdx.x + 1] = trr;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) pcg_init_kernel(int n_rows, const T* __restrict__ minv,
                                                            const double* __restrict__ b, T* __restrict__ x,
                                                            T* __restrict__ r, T* __restrict__ z, T* __restrict__ pold,
                                                            double* __restrict__ part_b) {
  __shared__ double sh[32];
  double rz = 0.0, rr = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {
    T rv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int i = 3 * row + c;
      rv[c] = T(b[i]);
      r[i] = rv[c];
      x[i] = T(0);
      pold[i] = T(0);
    }
    const T* m = minv + 9 * (int64_t)row;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const T zv = m[3 * a] * rv[0] + m[3 * a + 1] * rv[1] + m[3 * a + 2] * rv[2];
      z[3 * row + a] = zv;
      rz += double(rv[a] * zv);
      rr += double(rv[a]) * double(rv[a]);
    }
  }
  const double trz = block_sum<T>(rz, sh);
  const double trr = block_sum<T>(rr, sh);
  if (threadIdx.x == 0) {
    part_b[2 * blockIdx.x] = trz;
    part_b[2 * blockIdx.x + 1] = trr;
  }
}

__global__ void pcg_init_scalars_kernel(const double* __restrict__ part_b, int nparts, double* scal, double rtol,
                                        int max_iter) {
  __shared__ double sh[32];
  const double rr = sum_partials(part_b + 1, nparts, 2, sh);
  if (threadIdx.x == 0) {
    scal[kBB] = rr;
    scal[kTol2] = rtol * rtol * rr;
    scal[kRz + 0] = 1.0;
    scal[kRz + 1] = 1.0;
    scal[kDone] = 0.0;
    scal[kIters + 0] = 0.0;
    scal[kIters + 1] = 0.0;
    scal[kRR] = rr;
    scal[kMaxIt] = (double)max_iter;
  }
}

template <typename T>
__global__ void block_jacobi_kernel(Bsr A, const T* __restrict__ val, T* __restrict__ minv, bool point) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= A.n_rows) return;
  const T* b = val + 9 * (int64_t)A.diag[row];
  double m[3][3], r[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) m[i][j] = double(b[3 * i + j]);
  if (point) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) r[i][j] = (i == j && m[i][i] != 0.0) ? 1.0 / m[i][i] : 0.0;
  } else {
    inv3(m, r);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) minv[9 * (int64_t)row + 3 * i + j] = T(r[i][j]);
}

// r = b - K x with FP64 accumulation (iterative refinement / FP64 checks), warp per block row
template <typename T>
__global__ void residual64_kernel(Bsr A, const T* __restrict__ val, const double* __restrict__ x,
                                  const double* __restrict__ b, double* __restrict__ out, bool subtract) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < A.n_rows; row += warps) {
    const int b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
    const int nv = 9 * (b1 - b0);
    const T* v = val + 9 * (int64_t)b0;
    double a0 = 0, a1 = 0, a2 = 0;
    for (int idx = lane; idx < nv; idx += 32) {
      const int bb = idx / 9;
      const int r9 = idx - 9 * bb;
      const int ar = r9 / 3;
      const int c = r9 - 3 * ar;
      const double prod = double(v[idx]) * x[3 * A.col[b0 + bb] + c];
      a0 += ar == 0 ? prod : 0.0;
      a1 += ar == 1 ? prod : 0.0;
      a2 += ar == 2 ? prod : 0.0;
    }
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    a2 = warp_sum(a2);
    if (lane < 3) {
      const double kx = lane == 0 ? a0 : (lane == 1 ? a1 : a2);
      out[3 * row + lane] = subtract ? b[3 * row + lane] - kx : kx;
    }
  }
}

template <typename T>
__global__ void result_kernel(const T* __restrict__ x, double* __restrict__ out, double scale, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = scale * double(x[i]);
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
  if (w.fp32)
    pcg_init_kernel<float><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const float*)w.minv, b, (float*)w.x, (float*)w.r,
                                                        (float*)w.z, (float*)w.p1, w.part_b);
  else
    pcg_init_kernel<double><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const double*)w.minv, b, (double*)w.x,
                                                         (double*)w.r, (double*)w.z, (double*)w.p1, w.part_b);
  pcg_init_scalars_kernel<<<1, kThreads, 0, s>>>(w.part_b, w.grid, w.scal, rtol, max_iter);
}

void launch_pcg_spmv(const Bsr& A, PcgWork& w, int parity, cudaStream_t s) {
  void* pnew = parity ? w.p1 : w.p0;
  void* pold = parity ? w.p0 : w.p1;
  if (w.fp32)
    pcg_spmv_kernel<float><<<w.grid, kThreads, 0, s>>>(A, (const float*)A.val, (const float*)w.z, (const float*)pold,
                                                        (float*)pnew, (float*)w.q, w.part_b, w.part_a, w.scal, parity,
                                                        w.grid);
  else
    pcg_spmv_kernel<double><<<w.grid, kThreads, 0, s>>>(A, (const double*)A.val, (const double*)w.z,
                                                         (const double*)pold, (double*)pnew, (double*)w.q, w.part_b,
                                                         w.part_a, w.scal, parity, w.grid);
}
void launch_pcg_update(const Bsr& A, PcgWork& w, int parity, cudaStream_t s) {
  (void)A;
  void* pnew = parity ? w.p1 : w.p0;
  if (w.fp32)
    pcg_update_kernel<float><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const float*)w.minv, (const float*)pnew,
                                                          (const float*)w.q, (float*)w.x, (float*)w.r, (float*)w.z,
                                                          w.part_a, w.part_b, w.scal, parity, w.grid);
  else
    pcg_update_kernel<double><<<w.grid, kThreads, 0, s>>>(w.n_rows, (const double*)w.minv, (const double*)pnew,
                                                           (const double*)w.q, (double*)w.x, (double*)w.r,
                                                           (double*)w.z, w.part_a, w.part_b, w.scal, parity, w.grid);
}
void launch_pcg_iteration(const Bsr& A, PcgWork& w, int parity, cudaStream_t s) {
  launch_pcg_spmv(A, w, parity, s);
  launch_pcg_update(A, w, parity, s);
}

void launch_pcg_result(const PcgWork& w, double* x_out, double scale, cudaStream_t s) {
  const int64_t n = 3LL * w.n_rows;
  if (w.fp32) result_kernel<float><<<grid_cap(n, 256), 256, 0, s>>>((const float*)w.x, x_out, scale, n);
  else result_kernel<double><<<grid_cap(n, 256), 256, 0, s>>>((const double*)w.x, x_out, scale, n);
}

void launch_residual64(const Bsr& A, bool fp32, const double* x, const double* b, double* r, cudaStream_t s) {
  const int g = grid_cap(32LL * A.n_rows, 256);
  if (fp32) residual64_kernel<float><<<g, 256, 0, s>>>(A, (const float*)A.val, x, b, r, true);
  else residual64_kernel<double><<<g, 256, 0, s>>>(A, (const double*)A.val, x, b, r, true);
}
void launch_spmv64(const Bsr& A, bool fp32, const double* x, double* y, cudaStream_t s) {
  const int g = grid_cap(32LL * A.n_rows, 256);
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
