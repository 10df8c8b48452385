// Many independent instances of uneven size in one element set: per-instance CG and norms (sm_103a).
//
// The instances are disjoint contiguous node ranges of one mesh, so the tangent is block diagonal by instance.
// batched_pcg_kernel runs the complete block-Jacobi PCG of every instance in one cooperative launch.  Each
// instance gets a group of CTAs sized to its node count (the host sizes the groups so that all CTAs are
// co-resident); the CTAs of a group split the instance's block rows into contiguous chunks, one thread per
// row.  An iteration has two group-wide reductions (p.q, then r.z and r.r): every CTA publishes its partial,
// arrives on the instance's barrier counter and waits for the group, then sums the group's partials in CTA
// order, so alpha, beta and the convergence decision are identical in the group's CTAs and run to run.  A
// one-CTA group needs no global barrier.  p_new = z + beta p_old is formed on the fly for every gathered
// neighbour (as in the single-system CG), which removes the barrier a separate p update would need.
// Groups never wait on each other; instances whose Newton iteration has already converged get a zero
// correction.  Every wait on a barrier is bounded; a wait that gives up marks the instance (iters = -1).
#include "cg_common.cuh"

namespace ikr {

namespace {

using namespace cg;

constexpr int kBatchThreads = 256;
constexpr int kGroupSpinLimit = 1 << 24;

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

// group-wide sums of N values per CTA: publish, arrive, wait (bounded), sum the group's partials in CTA order.
// Partials are double-buffered by `slot` (the two reductions of an iteration alternate), so a CTA that runs
// ahead never overwrites partials another CTA of the group has still to read.
template <int N>
__device__ __forceinline__ bool group_reduce(double (&v)[N], double* part, int first, int size, int slot,
                                             unsigned int* counter, unsigned int target, double* sh, bool* ok_sh) {
  double cta[N];
#pragma unroll
  for (int k = 0; k < N; ++k) cta[k] = cta_sum(v[k], sh);
  if (size == 1) {
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = cta[k];
    return true;
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) part[(size_t)(2 * blockIdx.x + slot) * 2 + k] = cta[k];
    __threadfence();
    atomicAdd(counter, 1u);
    bool ok = false;
    for (int i = 0; i < kGroupSpinLimit; ++i) {
      unsigned int c;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(counter) : "memory");
      if (c >= target) {
        ok = true;
        break;
      }
      __nanosleep(32);
    }
    *ok_sh = ok;
  }
  __syncthreads();
  __threadfence();
  const bool ok = *ok_sh;
  __syncthreads();
  if (!ok) return false;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double s = 0.0;
    for (int b = 0; b < size; ++b) s += __ldcg(part + (size_t)(2 * (first + b) + slot) * 2 + k);
    v[k] = s;
  }
  return true;
}

// q = K p_new for rows [ra, rb) with p_new = z + beta p_old formed per gathered neighbour and written for the
// own rows; returns the thread's share of p_new . q.  Neighbour values written by other CTAs of the group are
// read around L1 (L2_ONLY).
template <typename T, bool L2_ONLY>
__device__ __forceinline__ double spmv_rows(const Bsr& A, const T* __restrict__ val, const T* zw, const T* pold,
                                            T* pnew, T* qw, T tb, int ra, int rb) {
  auto ld = [](const T* p) { return L2_ONLY ? __ldcg(p) : *p; };
  double pq = 0.0;
  for (int row = ra + threadIdx.x; row < rb; row += blockDim.x) {
    const int s = row >> 5, l = row & 31;
    T a0 = T(0), a1 = T(0), a2 = T(0);
    for (int g = A.slice_off[s]; g < A.slice_off[s + 1]; ++g) {
      const int c = A.col_sell[32 * g + l];
      const T* v = val + (int64_t)g * 288 + l;
      const T x0 = ld(zw + 4 * c) + tb * ld(pold + 4 * c);
      const T x1 = ld(zw + 4 * c + 1) + tb * ld(pold + 4 * c + 1);
      const T x2 = ld(zw + 4 * c + 2) + tb * ld(pold + 4 * c + 2);
      a0 += v[0] * x0 + v[32] * x1 + v[64] * x2;
      a1 += v[96] * x0 + v[128] * x1 + v[160] * x2;
      a2 += v[192] * x0 + v[224] * x1 + v[256] * x2;
    }
    const V3<T> zr = load3rw(zw, row), pr = load3rw(pold, row);
    const T n0 = zr.x + tb * pr.x, n1 = zr.y + tb * pr.y, n2 = zr.z + tb * pr.z;
    store3(pnew, row, n0, n1, n2);
    store3(qw, row, a0, a1, a2);
    pq += double(n0 * a0 + n1 * a1 + n2 * a2);
  }
  return pq;
}

// work vectors are node-padded (4 values per node) like the global CG's
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batched_pcg_kernel(
    Bsr A, const T* __restrict__ val, const T* __restrict__ minv, const double* __restrict__ b, double* __restrict__ x_out,
    const int32_t* __restrict__ node_off, const int32_t* __restrict__ cta_inst, const int32_t* __restrict__ cta_first,
    const int32_t* __restrict__ cta_size, const uint8_t* __restrict__ active, T* xw, T* rw, T* zw, T* p0, T* p1, T* qw,
    const double* __restrict__ rtol_inst, int max_iter, int32_t* __restrict__ iters_out,
    double* __restrict__ relres_out, double* part, unsigned int* counters) {
  __shared__ double sh[33];
  __shared__ bool ok_sh;
  const int inst = cta_inst[blockIdx.x];
  const int first = cta_first[blockIdx.x], size = cta_size[blockIdx.x], rank = blockIdx.x - first;
  const int r0 = node_off[inst], r1 = node_off[inst + 1];
  // this CTA's contiguous share of the instance's rows
  const int nr = r1 - r0;
  const int ra = r0 + (int)((int64_t)nr * rank / size), rb = r0 + (int)((int64_t)nr * (rank + 1) / size);
  const bool lead = rank == 0 && threadIdx.x == 0;
  unsigned int* counter = counters + inst;
  unsigned int bars = 0;
  if (!active[inst]) {
    for (int i = 3 * ra + threadIdx.x; i < 3 * rb; i += blockDim.x) x_out[i] = 0.0;
    if (lead) {
      iters_out[inst] = 0;
      relres_out[inst] = 0.0;
    }
    return;
  }
  // x = 0, r = b, z = M^{-1} r, p_old = 0 (so p_new = z on the first iteration)
  double init[2] = {0.0, 0.0};  // r.z, r.r
  for (int row = ra + threadIdx.x; row < rb; row += blockDim.x) {
    T rv[3], zv[3];
    for (int c = 0; c < 3; ++c) rv[c] = T(b[3 * row + c]);
    const T* m = minv + 9 * (int64_t)row;
    for (int a = 0; a < 3; ++a) zv[a] = m[3 * a] * rv[0] + m[3 * a + 1] * rv[1] + m[3 * a + 2] * rv[2];
    store3(xw, row, T(0), T(0), T(0));
    store3(rw, row, rv[0], rv[1], rv[2]);
    store3(zw, row, zv[0], zv[1], zv[2]);
    store3(p1, row, T(0), T(0), T(0));
    for (int c = 0; c < 3; ++c) {
      init[0] += double(rv[c] * zv[c]);
      init[1] += double(rv[c]) * double(rv[c]);
    }
  }
  bool ok = group_reduce<2>(init, part, first, size, 0, counter, (++bars) * size, sh, &ok_sh);
  double rz = init[0];
  const double bb = init[1];
  const double tol2 = rtol_inst[inst] * rtol_inst[inst] * bb;
  double rr = bb;
  double beta = 0.0;
  int it = 0;
  while (ok && it < max_iter && rr > tol2) {
    const T tb = T(beta);
    const T* pold = (it & 1) ? p0 : p1;
    T* pnew = (it & 1) ? p1 : p0;
    // q = K p_new on this CTA's rows (neighbour rows belong to the same instance)
    double pq[1] = {0.0};
    if (size > 1) pq[0] = spmv_rows<T, true>(A, val, zw, pold, pnew, qw, tb, ra, rb);
    else pq[0] = spmv_rows<T, false>(A, val, zw, pold, pnew, qw, tb, ra, rb);
    ok = group_reduce<1>(pq, part, first, size, 1, counter, (++bars) * size, sh, &ok_sh);
    if (!ok) break;
    if (!(fabs(pq[0]) > 0.0) || !isfinite(pq[0])) break;  // breakdown: leave with the current iterate
    const T alpha = T(rz / pq[0]);
    double upd[2] = {0.0, 0.0};  // r.z, r.r of the new residual
    for (int row = ra + threadIdx.x; row < rb; row += blockDim.x) {
      const V3<T> pv = load3rw(pnew, row), qv = load3rw(qw, row), xv = load3rw(xw, row), rv0 = load3rw(rw, row);
      store3(xw, row, xv.x + alpha * pv.x, xv.y + alpha * pv.y, xv.z + alpha * pv.z);
      const T r_[3] = {rv0.x - alpha * qv.x, rv0.y - alpha * qv.y, rv0.z - alpha * qv.z};
      store3(rw, row, r_[0], r_[1], r_[2]);
      const T* m = minv + 9 * (int64_t)row;
      T zv[3];
      for (int a = 0; a < 3; ++a) zv[a] = m[3 * a] * r_[0] + m[3 * a + 1] * r_[1] + m[3 * a + 2] * r_[2];
      store3(zw, row, zv[0], zv[1], zv[2]);
      for (int a = 0; a < 3; ++a) {
        upd[0] += double(r_[a] * zv[a]);
        upd[1] += double(r_[a]) * double(r_[a]);
      }
    }
    ok = group_reduce<2>(upd, part, first, size, 0, counter, (++bars) * size, sh, &ok_sh);
    if (!ok) break;
    beta = upd[0] / rz;
    rz = upd[0];
    rr = upd[1];
    ++it;
  }
  for (int row = ra + threadIdx.x; row < rb; row += blockDim.x) {
    const V3<T> xv = load3rw(xw, row);
    x_out[3 * row] = double(xv.x), x_out[3 * row + 1] = double(xv.y), x_out[3 * row + 2] = double(xv.z);
  }
  if (lead) {
    iters_out[inst] = ok ? it : -1;
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

int batched_pcg_capacity(bool fp32, int sms) {
  int b = 0;
  if (fp32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_pcg_kernel<float>, kBatchThreads, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batched_pcg_kernel<double>, kBatchThreads, 0);
  return b * sms;
}

cudaError_t launch_batched_pcg(const Bsr& A, bool fp32, const void* minv, const double* b, double* x_out, int n_cta,
                               const int32_t* node_off, const int32_t* cta_inst, const int32_t* cta_first,
                               const int32_t* cta_size, const uint8_t* active, void* xw, void* rw, void* zw, void* p0,
                               void* p1, void* qw, const double* rtol, int max_iter, int32_t* iters, double* relres,
                               double* part, unsigned int* counters, int n_inst, bool cooperative, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(unsigned int) * n_inst, s);
  if (e != cudaSuccess) return e;
  if (!cooperative) {  // every group is one CTA: no CTA waits on another, so an ordinary launch will do
    if (fp32)
      batched_pcg_kernel<float><<<n_cta, kBatchThreads, 0, s>>>(
          A, (const float*)A.val, (const float*)minv, b, x_out, node_off, cta_inst, cta_first, cta_size, active,
          (float*)xw, (float*)rw, (float*)zw, (float*)p0, (float*)p1, (float*)qw, rtol, max_iter, iters, relres, part,
          counters);
    else
      batched_pcg_kernel<double><<<n_cta, kBatchThreads, 0, s>>>(
          A, (const double*)A.val, (const double*)minv, b, x_out, node_off, cta_inst, cta_first, cta_size, active,
          (double*)xw, (double*)rw, (double*)zw, (double*)p0, (double*)p1, (double*)qw, rtol, max_iter, iters,
          relres, part, counters);
    return cudaGetLastError();
  }
  Bsr Acopy = A;
  const void* val = A.val;
  void* args[] = {&Acopy, &val, &minv,  &b,      &x_out,    &node_off, &cta_inst, &cta_first,
                  &cta_size, &active, &xw, &rw,   &zw,       &p0,       &p1,       &qw,
                  &rtol,  &max_iter, &iters, &relres, &part, &counters};
  const void* kern = fp32 ? (const void*)batched_pcg_kernel<float> : (const void*)batched_pcg_kernel<double>;
  return cudaLaunchCooperativeKernel(kern, dim3(n_cta), dim3(kBatchThreads), args, 0, s);
}

void launch_instance_norms(const double* x, int n_inst, const int32_t* node_off, double* out, cudaStream_t s) {
  instance_norms_kernel<<<n_inst, 256, 0, s>>>(x, node_off, out);
}

}  // namespace ikr
