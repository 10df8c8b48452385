// Grid-wide primitives of the persistent CG kernels (sm_103a): CTA sums, the bounded grid barrier with a
// fixed-order all-reduce of per-CTA partials, the staging configuration and the cyclic chunk position of a warp.
#pragma once
#include "staging.cuh"

namespace ikr {
namespace cg {

constexpr int kBarrierSpinLimit = 1 << 24;  // polls (with a short sleep) before a grid barrier gives up

// CTA sums of N values: valid in thread 0 only (one __syncthreads; sw holds WARPS x N doubles)
template <int N>
__device__ __forceinline__ void cta_reduce(double (&v)[N], double* sw) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const double s = warp_sum(v[k]);
    if (lane == 0) sw[warp * N + k] = s;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double s = lane < (int)(blockDim.x >> 5) ? sw[lane * N + k] : 0.0;
      v[k] = warp_sum(s);
    }
  }
}

// CTA sums of N values with the FP64 additions done by one warp: every thread stores its values (sfull holds
// N x blockDim.x doubles), lane l of warp 0 adds those of threads l, l + 32, ... in order, then a butterfly; valid
// in warp 0.  A butterfly in every warp would cost each warp five FP64 additions per value, which on GB300's narrow
// FP64 pipe are several times this.
template <int N>
__device__ __forceinline__ void cta_reduce_smem(double (&v)[N], double* sfull) {
#pragma unroll
  for (int k = 0; k < N; ++k) sfull[k * blockDim.x + threadIdx.x] = v[k];
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      double s = 0.0;
      for (int i = threadIdx.x; i < (int)blockDim.x; i += 32) s += sfull[k * blockDim.x + i];
      v[k] = warp_sum(s);
    }
  }
}

// Grid-wide sums of N values whose CTA sums are in thread 0: thread 0 publishes them at part[cta * N + k],
// arrives on the barrier counter and waits (bounded) until `target` arrivals; then warp 0 sums all CTAs'
// partials with a fixed lane assignment and butterfly order (identical in every CTA) and every thread gets
// the sums.  Returns false when the wait gave up.
// WaitCtl: the poll limit, and (tests of the bounded wait only) CTA 0 withholding its arrival at the first barrier,
// so that every CTA's first wait runs out and the solve ends with the timeout status.
struct WaitCtl {
  int polls;
  int withhold_first;
};

template <int N>
__device__ __forceinline__ bool grid_allreduce(double (&v)[N], double* part, unsigned int* count, unsigned int target,
                                               double* sv, bool* ok_sh, WaitCtl wc) {
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) part[blockIdx.x * N + k] = v[k];
    __threadfence();
    if (!(wc.withhold_first && blockIdx.x == 0 && target == gridDim.x)) atomicAdd(count, 1u);
    bool ok = false;
    for (int i = 0; i < wc.polls; ++i) {
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
  __threadfence();  // every thread: its later plain loads observe what the other CTAs wrote before arriving
  if (!*ok_sh) return false;
  if (threadIdx.x < 32) {
    // lane l adds the partials of CTAs l, l + 32, l + 64, ... in that order; the loads of up to eight of them per
    // value are issued together (the partials sit in L2, so a dependent chain of loads would cost one L2 round trip
    // each), then the lanes' sums are combined by the butterfly
    constexpr int kU = 8;
    double s[N];
#pragma unroll
    for (int k = 0; k < N; ++k) s[k] = 0.0;
    for (int i0 = threadIdx.x; i0 < (int)gridDim.x; i0 += 32 * kU) {
      double t[kU][N];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int i = i0 + 32 * u;
#pragma unroll
        for (int k = 0; k < N; ++k) t[u][k] = i < (int)gridDim.x ? __ldcg(part + (size_t)i * N + k) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kU; ++u)
#pragma unroll
        for (int k = 0; k < N; ++k) s[k] += t[u][k];
    }
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const double v = warp_sum(s[k]);
      if (threadIdx.x == 0) sv[k] = v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = sv[k];
  return true;
}

// Quotients num[k] / den[k] formed by thread 0 and read by every thread of the CTA (the same IEEE values): an FP64
// division is a multi-instruction sequence on GB300's narrow FP64 pipe, and every thread forming it costs microseconds
// per CG iteration.  A zero or non-finite denominator gives 0.  sq holds N doubles of shared memory; the caller's
// next CTA barrier orders its reuse.
template <int N>
__device__ __forceinline__ void cta_quotients(const double (&num)[N], const double (&den)[N], double (&out)[N],
                                              double* sq) {
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) sq[k] = (den[k] != 0.0 && isfinite(den[k])) ? num[k] / den[k] : 0.0;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) out[k] = sq[k];
}

template <typename T, int CB, int NST, int WARPS>
struct PersistentCfg {
  static constexpr int kValBytes = CB * 288 * (int)sizeof(T);
  static constexpr int kColBytes = CB * 32 * 4;
  static constexpr int kStageBytes = kValBytes + kColBytes;
  static constexpr int kSmemBytes = WARPS * NST * kStageBytes;
  static constexpr int kThreads = WARPS * 32;
};

// cyclic position in a warp's chunk stream: owned slice j (slice gw + j * nw), first block g, slice end gend
struct CyclicPos {
  int j, g, gend;
};

}  // namespace cg
}  // namespace ikr
