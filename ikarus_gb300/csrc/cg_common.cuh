// Device helpers of the CG kernels: node-padded vector access and deterministic grid reductions (sm_103a).
//
// CG vectors are node-padded: four values per node (x, y, z, 0), so gathering a neighbour is one 16-byte
// load (FP32) or two (FP64).  Grid-wide sums use the "last block" pattern: every block publishes its partial,
// draws a ticket from an atomic counter, and the block that draws the final ticket sums all partials in index
// order, so results are bit-identical run to run.
#pragma once
#include "common.cuh"
#include "kernels.h"

namespace ikr {
namespace cg {

template <typename T>
struct V3 {
  T x, y, z;
};
__device__ __forceinline__ V3<float> load3(const float* __restrict__ v, int node) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(v) + node);
  return {a.x, a.y, a.z};
}
__device__ __forceinline__ V3<double> load3(const double* __restrict__ v, int node) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(v) + 2 * node);
  return {a.x, a.y, __ldg(v + 4 * node + 2)};
}
// plain (non-__ldg) loads for vectors the kernel also writes
__device__ __forceinline__ V3<float> load3rw(const float* v, int node) {
  const float4 a = reinterpret_cast<const float4*>(v)[node];
  return {a.x, a.y, a.z};
}
__device__ __forceinline__ V3<double> load3rw(const double* v, int node) {
  const double2 a = reinterpret_cast<const double2*>(v)[2 * node];
  return {a.x, a.y, v[4 * node + 2]};
}
__device__ __forceinline__ void store3(float* v, int node, float a, float b, float c) {
  reinterpret_cast<float4*>(v)[node] = make_float4(a, b, c, 0.f);
}
__device__ __forceinline__ void store3(double* v, int node, double a, double b, double c) {
  reinterpret_cast<double2*>(v)[2 * node] = make_double2(a, b);
  reinterpret_cast<double2*>(v)[2 * node + 1] = make_double2(c, 0.0);
}

// block-wide sum, result valid in every thread
__device__ __forceinline__ double block_sum_all(double v, double* sh) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (threadIdx.x < 32) r = warp_sum(r);
  if (threadIdx.x == 0) sh[0] = r;
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

// Publishes this block's partial(s) and returns true in every thread of the block that finishes last.
__device__ __forceinline__ bool publish_and_check_last(unsigned int* ticket, bool* last_flag) {
  __threadfence();
  if (threadIdx.x == 0) *last_flag = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  const bool last = *last_flag;
  if (last) __threadfence();
  return last;
}

// fixed-order sum of n partials (stride st) by one block, read around L1
__device__ __forceinline__ double sum_partials(const double* p, int n, int st, double* sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(p + (size_t)i * st);
  return block_sum_all(s, sh);
}

__device__ __forceinline__ unsigned int* tickets(double* scal) { return reinterpret_cast<unsigned int*>(scal + kTicket); }

}  // namespace cg
}  // namespace ikr
