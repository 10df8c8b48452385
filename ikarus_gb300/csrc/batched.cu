// Many independent instances of uneven size in one element set: per-instance CG and norms (sm_103a).
//
// The instances are disjoint contiguous node ranges of one mesh, so the tangent is block diagonal by instance.
// batched_pcg_kernel runs the complete block-Jacobi PCG of one instance inside one CTA: the CTA's threads own
// the instance's block rows, dot products are block reductions in a fixed order, and the only synchronisation
// is __syncthreads, so the instances advance independently inside a single launch (no CTA waits on another).
// CTAs take instances largest-first (the host passes the order), which keeps the tail of the launch short.
// Instances whose Newton iteration has already converged are skipped and get a zero correction.
#include "common.cuh"
#include "kernels.h"

namespace ikr {

namespace {

constexpr int kBatchThreads = 256;

__device__ __forceinline__ double cta_sum(double v, double* sh) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (threadIdx.x < 32) r = warp_sum(r);
  if (threadIdx.x == 0) sh[32] = r;
  __syncthreads();
  r = sh[32];
  __syncthreads();
  return r;
}

// work vectors are node-padded (4 values per node) like the global CG's
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batched_pcg_kernel(
    Bsr A, const T* __restrict__ val, const T* __restrict__ minv, const double* __restrict__ b, double* __restrict__ x_out,
    const int32_t* __restrict__ node_off, const int32_t* __restrict__ order, const uint8_t* __restrict__ active,
    T* __restrict__ xw, T* __restrict__ rw, T* __restrict__ zw, T* __restrict__ pw, T* __restrict__ qw,
    const double* __restrict__ rtol_inst, int max_iter, int32_t* __restrict__ iters_out, double* __restrict__ relres_out) {
  __shared__ double sh[33];
  const int inst = order[blockIdx.x];
  const int r0 = node_off[inst], r1 = node_off[inst + 1];
  if (!active[inst]) {
    for (int i = 3 * r0 + threadIdx.x; i < 3 * r1; i += blockDim.x) x_out[i] = 0.0;
    if (threadIdx.x == 0) {
      iters_out[inst] = 0;
      relres_out[inst] = 0.0;
    }
    return;
  }
  // x = 0, r = b, z = M^{-1} r, p = z
  double rz = 0.0, bb = 0.0;
  for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
    T rv[3], zv[3];
    for (int c = 0; c < 3; ++c) rv[c] = T(b[3 * row + c]);
    const T* m = minv + 9 * (int64_t)row;
    for (int a = 0; a < 3; ++a) zv[a] = m[3 * a] * rv[0] + m[3 * a + 1] * rv[1] + m[3 * a + 2] * rv[2];
    for (int c = 0; c < 4; ++c) {
      xw[4 * row + c] = T(0);
      rw[4 * row + c] = c < 3 ? rv[c] : T(0);
      zw[4 * row + c] = c < 3 ? zv[c] : T(0);
      pw[4 * row + c] = c < 3 ? zv[c] : T(0);
    }
    for (int c = 0; c < 3; ++c) {
      rz += double(rv[c] * zv[c]);
      bb += double(rv[c]) * double(rv[c]);
    }
  }
  rz = cta_sum(rz, sh);
  bb = cta_sum(bb, sh);
  const double tol2 = rtol_inst[inst] * rtol_inst[inst] * bb;
  double rr = bb;
  int it = 0;
  while (it < max_iter && rr > tol2) {
    // q = K p on the instance's rows (neighbour rows belong to the same instance)
    double pq = 0.0;
    for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
      const int s = row >> 5, l = row & 31;
      T a0 = T(0), a1 = T(0), a2 = T(0);
      for (int g = A.slice_off[s]; g < A.slice_off[s + 1]; ++g) {
        const int c = A.col_sell[32 * g + l];
        const T* v = val + (int64_t)g * 288 + l;
        const T x0 = pw[4 * c], x1 = pw[4 * c + 1], x2 = pw[4 * c + 2];
        a0 += v[0] * x0 + v[32] * x1 + v[64] * x2;
        a1 += v[96] * x0 + v[128] * x1 + v[160] * x2;
        a2 += v[192] * x0 + v[224] * x1 + v[256] * x2;
      }
      qw[4 * row] = a0, qw[4 * row + 1] = a1, qw[4 * row + 2] = a2;
      pq += double(pw[4 * row] * a0 + pw[4 * row + 1] * a1 + pw[4 * row + 2] * a2);
    }
    pq = cta_sum(pq, sh);
    if (!(fabs(pq) > 0.0) || !isfinite(pq)) break;  // breakdown: leave with the current iterate
    const T alpha = T(rz / pq);
    double rzn = 0.0, rrn = 0.0;
    for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
      T rv[3];
      for (int c = 0; c < 3; ++c) {
        xw[4 * row + c] += alpha * pw[4 * row + c];
        rv[c] = rw[4 * row + c] - alpha * qw[4 * row + c];
        rw[4 * row + c] = rv[c];
      }
      const T* m = minv + 9 * (int64_t)row;
      for (int a = 0; a < 3; ++a) {
        const T zv = m[3 * a] * rv[0] + m[3 * a + 1] * rv[1] + m[3 * a + 2] * rv[2];
        zw[4 * row + a] = zv;
        rzn += double(rv[a] * zv);
        rrn += double(rv[a]) * double(rv[a]);
      }
    }
    rzn = cta_sum(rzn, sh);
    rr = cta_sum(rrn, sh);
    const T beta = T(rzn / rz);
    rz = rzn;
    for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x)
      for (int c = 0; c < 3; ++c) pw[4 * row + c] = zw[4 * row + c] + beta * pw[4 * row + c];
    __syncthreads();  // every p is updated before the next product reads neighbours
    ++it;
  }
  for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x)
    for (int c = 0; c < 3; ++c) x_out[3 * row + c] = double(xw[4 * row + c]);
  if (threadIdx.x == 0) {
    iters_out[inst] = it;
    relres_out[inst] = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  }
}

// per-instance sum of squares over dof ranges [3 node_off[i], 3 node_off[i+1]); one block per instance
__global__ void instance_norms_kernel(const double* __restrict__ x, const int32_t* __restrict__ node_off,
                                      double* __restrict__ out) {
  __shared__ double sh[33];
  const int inst = blockIdx.x;
  double s = 0.0;
  for (int i = 3 * node_off[inst] + threadIdx.x; i < 3 * node_off[inst + 1]; i += blockDim.x) s += x[i] * x[i];
  s = cta_sum(s, sh);
  if (threadIdx.x == 0) out[inst] = sqrt(s);
}

}  // namespace

void launch_batched_pcg(const Bsr& A, bool fp32, const void* minv, const double* b, double* x_out, int n_inst,
                        const int32_t* node_off, const int32_t* order, const uint8_t* active, void* xw, void* rw,
                        void* zw, void* pw, void* qw, const double* rtol, int max_iter, int32_t* iters,
                        double* relres, cudaStream_t s) {
  if (fp32)
    batched_pcg_kernel<float><<<n_inst, kBatchThreads, 0, s>>>(
        A, (const float*)A.val, (const float*)minv, b, x_out, node_off, order, active, (float*)xw, (float*)rw,
        (float*)zw, (float*)pw, (float*)qw, rtol, max_iter, iters, relres);
  else
    batched_pcg_kernel<double><<<n_inst, kBatchThreads, 0, s>>>(
        A, (const double*)A.val, (const double*)minv, b, x_out, node_off, order, active, (double*)xw, (double*)rw,
        (double*)zw, (double*)pw, (double*)qw, rtol, max_iter, iters, relres);
}

void launch_instance_norms(const double* x, int n_inst, const int32_t* node_off, double* out, cudaStream_t s) {
  instance_norms_kernel<<<n_inst, 256, 0, s>>>(x, node_off, out);
}

}  // namespace ikr
