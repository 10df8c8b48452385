// Dense-network and POD kernels of the learned Newton predictor (sm_103a).
//
// The predictor maps (load parameters, load factor, previous two displacement increments in POD coordinates)
// to the next increment's POD coordinates.  Weights are stored in BF16 (inference and training forward use
// them), master copies and all accumulation are FP32.  The matrices are small (widths of a few hundred, batches
// of a few hundred), so plain tiled CUDA-core GEMMs are the right tool; every reduction has a fixed order, so
// training is deterministic for a given seed.
#include <cuda_bf16.h>

#include <cmath>

#include "kernels.h"

namespace ikr {

namespace {

constexpr int TB = 32;  // GEMM tile

template <typename T>
__device__ __forceinline__ float to_f(T v);
template <>
__device__ __forceinline__ float to_f<float>(float v) {
  return v;
}
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

// C[M x N] = alpha * op(A) op(B) + beta * C, op(A) = A (M x K, row-major lda) or A^T (A stored K x M),
// op(B) = B (K x N, ldb) or B^T (B stored N x K).  32 x 32 tiles, 256 threads, 4 outputs per thread,
// K loop in fixed order.
template <typename TA, typename TBt, bool TRA, bool TRB>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const TA* __restrict__ A, int lda,
                                                   const TBt* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                                   float alpha, float beta) {
  __shared__ float As[TB][TB + 1];
  __shared__ float Bs[TB][TB + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // ty in 0..7
  const int row0 = blockIdx.y * TB, col0 = blockIdx.x * TB;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int k0 = 0; k0 < K; k0 += TB) {
    for (int r = ty; r < TB; r += 8) {
      // As[r][tx] = op(A)[row0 + r][k0 + tx]
      const int m = row0 + r, k = k0 + tx;
      float a = 0.f;
      if (m < M && k < K) a = TRA ? to_f(A[(size_t)k * lda + m]) : to_f(A[(size_t)m * lda + k]);
      As[r][tx] = a;
      // Bs[r][tx] = op(B)[k0 + r][col0 + tx]
      const int kb = k0 + r, n = col0 + tx;
      float b = 0.f;
      if (kb < K && n < N) b = TRB ? to_f(B[(size_t)n * ldb + kb]) : to_f(B[(size_t)kb * ldb + n]);
      Bs[r][tx] = b;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < TB; ++kk) {
      const float bv = Bs[kk][tx];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i] += As[ty + 8 * i][kk] * bv;
    }
    __syncthreads();
  }
  const int n = col0 + tx;
  if (n >= N) return;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = row0 + ty + 8 * i;
    if (m < M) {
      float* c = C + (size_t)m * ldc + n;
      *c = alpha * acc[i] + (beta != 0.f ? beta * *c : 0.f);
    }
  }
}

// Z[b][o] += bias[o]; Y = gelu(Z) (exact erf form) or Y = Z for the output layer
__global__ void bias_act_kernel(float* __restrict__ Z, float* __restrict__ Y, const float* __restrict__ bias, int B,
                                int out, bool gelu) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)B * out) return;
  const float z = Z[t] + bias[t % out];
  Z[t] = z;
  Y[t] = gelu ? 0.5f * z * (1.f + erff(z * 0.70710678118654752f)) : z;
}

// dZ = dY * gelu'(Z)
__global__ void gelu_backward_kernel(float* __restrict__ dZ, const float* __restrict__ Z, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float z = Z[t];
  const float cdf = 0.5f * (1.f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
  dZ[t] *= cdf + z * pdf;
}

// column sums (bias gradients): g[o] = sum_b dZ[b][o], fixed order
__global__ void colsum_kernel(const float* __restrict__ dZ, float* __restrict__ g, int B, int out) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= out) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += dZ[(size_t)b * out + o];
  g[o] = s;
}

// MSE loss and its gradient: dY = 2 (Y - T) / (B * out); loss partial per block (then summed on the host)
__global__ void mse_kernel(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY,
                           int64_t n, float scale, float* __restrict__ part) {
  __shared__ float sh[256];
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f;
  if (t < n) {
    const float d = Y[t] - T[t];
    dY[t] = 2.f * d * scale;
    e = d * d * scale;
  }
  sh[threadIdx.x] = e;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Adam on the FP32 master parameters; refreshes the BF16 weight copy (wmask: 1 for weights, 0 for biases)
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, __nv_bfloat16* __restrict__ wb, const int64_t* __restrict__ bf_index,
                            int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gi = g[t];
  const float mi = b1 * m[t] + (1.f - b1) * gi;
  const float vi = b2 * v[t] + (1.f - b2) * gi * gi;
  m[t] = mi;
  v[t] = vi;
  const float pi = p[t] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  p[t] = pi;
  const int64_t bi = bf_index[t];
  if (bi >= 0) wb[bi] = __float2bfloat16_rn(pi);
}

__global__ void to_bf16_kernel(const float* __restrict__ p, __nv_bfloat16* __restrict__ wb,
                               const int64_t* __restrict__ bf_index, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t bi = bf_index[t];
  if (bi >= 0) wb[bi] = __float2bfloat16_rn(p[t]);
}

// rows of a feature matrix gathered by index (mini-batch assembly)
__global__ void gather_rows_kernel(const float* __restrict__ X, const int32_t* __restrict__ idx, float* __restrict__ out,
                                   int rows, int cols) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)rows * cols) return;
  const int r = (int)(t / cols), c = (int)(t % cols);
  out[t] = X[(size_t)idx[r] * cols + c];
}

// G = Y^T Y with FP64 accumulation (Y: n x l column-major, i.e. column j at Y + j * n); one block per entry
__global__ void gram64_kernel(const float* __restrict__ Y, int64_t n, int l, double* __restrict__ G) {
  __shared__ double sh[256];
  const int i = blockIdx.x, j = blockIdx.y;
  if (j < i) return;
  const float* a = Y + (size_t)i * n;
  const float* b = Y + (size_t)j * n;
  double s = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) s += double(a[k]) * double(b[k]);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) G[i * l + j] = G[j * l + i] = sh[0];
}

// standard normal samples from a counter-based hash (Box-Muller), deterministic per (seed, index)
__device__ __forceinline__ uint32_t hash32(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return (uint32_t)x;
}
__global__ void randn_kernel(float* __restrict__ out, int64_t n, uint64_t seed) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float u1 = (hash32(seed * 0x9E3779B97F4A7C15ull + 2 * t) + 1.0f) * 2.3283064365386963e-10f;
  const float u2 = hash32(seed * 0x9E3779B97F4A7C15ull + 2 * t + 1) * 2.3283064365386963e-10f;
  out[t] = sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

// FP64 displacement increment -> FP32 snapshot column, and u += d (FP32 increment into FP64 state)
__global__ void diff_to_f32_kernel(const double* __restrict__ a, const double* __restrict__ b, float* __restrict__ out,
                                   int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] = float(a[t] - b[t]);
}
__global__ void add_f32_kernel(double* __restrict__ u, const float* __restrict__ d, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) u[t] += double(d[t]);
}
__global__ void add_scaled_f32_kernel(double* __restrict__ u, const float* __restrict__ d, double a, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    u[i] += a * double(d[i]);
}
__global__ void base_plus_scaled_kernel(double* __restrict__ u, const double* __restrict__ u0,
                                        const float* __restrict__ d, double sc, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) u[t] = u0[t] + sc * double(d[t]);
}

inline int blocks(int64_t n, int bs) { return (int)((n + bs - 1) / bs); }

template <typename TA, typename TBt, bool TRA, bool TRB>
void gemm_t(int M, int N, int K, const void* A, int lda, const void* B, int ldb, float* C, int ldc, float alpha,
            float beta, cudaStream_t s) {
  dim3 grid((N + TB - 1) / TB, (M + TB - 1) / TB);
  gemm_kernel<TA, TBt, TRA, TRB><<<grid, 256, 0, s>>>(M, N, K, (const TA*)A, lda, (const TBt*)B, ldb, C, ldc, alpha,
                                                      beta);
}

}  // namespace

void launch_gemm(int M, int N, int K, const void* A, bool a_bf16, bool trans_a, int lda, const void* B, bool b_bf16,
                 bool trans_b, int ldb, float* C, int ldc, float alpha, float beta, cudaStream_t s) {
  using bf = __nv_bfloat16;
  if (!a_bf16 && !b_bf16) {
    if (!trans_a && !trans_b) gemm_t<float, float, false, false>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, s);
    else if (!trans_a && trans_b) gemm_t<float, float, false, true>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, s);
    else if (trans_a && !trans_b) gemm_t<float, float, true, false>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, s);
    else gemm_t<float, float, true, true>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, s);
  } else if (!a_bf16 && b_bf16) {
    if (trans_b) gemm_t<float, bf, false, true>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, s);
    else gemm_t<float, bf, false, false>(M, N, K, A, lda, B, ldb, C, ldc, alpha, beta, s);
  }
}
void launch_bias_act(float* Z, float* Y, const float* bias, int B, int out, bool gelu, cudaStream_t s) {
  bias_act_kernel<<<blocks((int64_t)B * out, 256), 256, 0, s>>>(Z, Y, bias, B, out, gelu);
}
void launch_gelu_backward(float* dZ, const float* Z, int64_t n, cudaStream_t s) {
  gelu_backward_kernel<<<blocks(n, 256), 256, 0, s>>>(dZ, Z, n);
}
void launch_colsum(const float* dZ, float* g, int B, int out, cudaStream_t s) {
  colsum_kernel<<<blocks(out, 128), 128, 0, s>>>(dZ, g, B, out);
}
int launch_mse(const float* Y, const float* T, float* dY, int64_t n, float scale, float* part, cudaStream_t s) {
  const int nb = blocks(n, 256);
  mse_kernel<<<nb, 256, 0, s>>>(Y, T, dY, n, scale, part);
  return nb;
}
void launch_adam(float* p, const float* g, float* m, float* v, void* wb, const int64_t* bf_index, int64_t n, float lr,
                 float b1, float b2, float eps, int step, cudaStream_t s) {
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<blocks(n, 256), 256, 0, s>>>(p, g, m, v, (__nv_bfloat16*)wb, bf_index, n, lr, b1, b2, eps, c1, c2);
}
void launch_to_bf16(const float* p, void* wb, const int64_t* bf_index, int64_t n, cudaStream_t s) {
  to_bf16_kernel<<<blocks(n, 256), 256, 0, s>>>(p, (__nv_bfloat16*)wb, bf_index, n);
}
void launch_gather_rows(const float* X, const int32_t* idx, float* out, int rows, int cols, cudaStream_t s) {
  gather_rows_kernel<<<blocks((int64_t)rows * cols, 256), 256, 0, s>>>(X, idx, out, rows, cols);
}
void launch_gram64(const float* Y, int64_t n, int l, double* G, cudaStream_t s) {
  gram64_kernel<<<dim3(l, l), 256, 0, s>>>(Y, n, l, G);
}
void launch_randn(float* out, int64_t n, uint64_t seed, cudaStream_t s) {
  randn_kernel<<<blocks(n, 256), 256, 0, s>>>(out, n, seed);
}
void launch_diff_to_f32(const double* a, const double* b, float* out, int64_t n, cudaStream_t s) {
  diff_to_f32_kernel<<<blocks(n, 256), 256, 0, s>>>(a, b, out, n);
}
void launch_add_f32(double* u, const float* d, int64_t n, cudaStream_t s) {
  add_f32_kernel<<<blocks(n, 256), 256, 0, s>>>(u, d, n);
}
void launch_add_scaled_f32(double* u, const float* d, double a, int64_t n, cudaStream_t s) {
  add_scaled_f32_kernel<<<blocks(n, 256), 256, 0, s>>>(u, d, a, n);
}
void launch_base_plus_scaled(double* u, const double* u0, const float* d, double sc, int64_t n, cudaStream_t s) {
  base_plus_scaled_kernel<<<blocks(n, 256), 256, 0, s>>>(u, u0, d, sc, n);
}

}  // namespace ikr
