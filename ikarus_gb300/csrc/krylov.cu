// Vector kernels of the FP64 outer Krylov solve (flexible GMRES around the FP32 CG, host side in krylov.cpp):
// the Arnoldi basis V and the preconditioned directions Z are dof-major FP64 vectors of length n stored one after
// the other with leading dimension ld.
//
// All reductions have a fixed order (per-block partial sums, then one block per output summing the partials in
// block order), so a solve is bit-identical run to run.  Every kernel streams its vectors once: the products
// V^T w read each basis vector once and w from registers, the combinations read each vector once.
#include <cuda_runtime.h>

#include "kernels.h"

namespace ikr {

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 8;                     // elements of w each thread keeps in registers
constexpr int kChunk = kThreads * kPerThread;     // elements per block

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();  // red is reused by the next call
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;  // valid in thread 0
}

// part[i * nblk + block] = sum over the block's chunk of V[i] * w, i < m
__global__ void __launch_bounds__(kThreads) multi_dot_partial_kernel(const double* __restrict__ V, int64_t ld, int m,
                                                                     const double* __restrict__ w, int64_t n,
                                                                     double* __restrict__ part) {
  __shared__ double red[kThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kChunk + threadIdx.x;
  double wv[kPerThread];
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) {
    const int64_t k = base + (int64_t)j * kThreads;
    wv[j] = k < n ? w[k] : 0.0;
  }
  for (int i = 0; i < m; ++i) {
    const double* v = V + (int64_t)i * ld;
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < kPerThread; ++j) {
      const int64_t k = base + (int64_t)j * kThreads;
      if (k < n) s = fma(v[k], wv[j], s);
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[(int64_t)i * gridDim.x + blockIdx.x] = s;
  }
}

// out[i] = sum_b part[i * nblk + b] (one block per i, fixed order)
__global__ void __launch_bounds__(kThreads) sum_partials_kernel(const double* __restrict__ part, int nblk,
                                                                double* __restrict__ out) {
  __shared__ double red[kThreads / 32];
  const double* p = part + (int64_t)blockIdx.x * nblk;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblk; b += kThreads) s += p[b];
  s = block_sum(s, red);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// y += sign * sum_i c[i] V[i] (c on the device, m <= kKrylovMaxBasis)
__global__ void __launch_bounds__(kThreads) multi_axpy_kernel(double* __restrict__ y, const double* __restrict__ V,
                                                              int64_t ld, int m, const double* __restrict__ c,
                                                              double sign, int64_t n) {
  __shared__ double cs[kKrylovMaxBasis];
  for (int i = threadIdx.x; i < m; i += kThreads) cs[i] = sign * c[i];
  __syncthreads();
  for (int64_t k = (int64_t)blockIdx.x * kThreads + threadIdx.x; k < n; k += (int64_t)gridDim.x * kThreads) {
    double s = y[k];
    for (int i = 0; i < m; ++i) s = fma(cs[i], V[(int64_t)i * ld + k], s);
    y[k] = s;
  }
}

// FP32 copy of the FP64 tangent values (the mixed form's CG matrix, rounded once from the FP64 assembly)
__global__ void round_values_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    out[k] = (float)in[k];
}

int grid_for(int64_t n, int threads) {
  const int64_t g = (n + threads - 1) / threads;
  return (int)(g < 1 ? 1 : (g > 8192 ? 8192 : g));
}

}  // namespace

int multi_dot_blocks(int64_t n) { return (int)((n + kChunk - 1) / kChunk); }

void launch_multi_dot(const double* V, int64_t ld, int m, const double* w, int64_t n, double* part, double* out,
                      cudaStream_t s) {
  if (m <= 0) return;
  const int nblk = multi_dot_blocks(n);
  multi_dot_partial_kernel<<<nblk, kThreads, 0, s>>>(V, ld, m, w, n, part);
  sum_partials_kernel<<<m, kThreads, 0, s>>>(part, nblk, out);
}

void launch_multi_axpy(double* y, const double* V, int64_t ld, int m, const double* c, double sign, int64_t n,
                       cudaStream_t s) {
  if (m <= 0) return;
  multi_axpy_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(y, V, ld, m, c, sign, n);
}

void launch_round_values(const double* in, float* out, int64_t n, cudaStream_t s) {
  round_values_kernel<<<grid_for(n, 256), 256, 0, s>>>(in, out, n);
}

}  // namespace ikr
