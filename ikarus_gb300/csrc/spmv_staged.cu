// CG SpMV with bulk-copy staging of the sliced-ELL tangent into shared memory (sm_103a).
//
// Same arithmetic and outputs as the direct CG SpMV in solver.cu (p_new = z + beta p_old formed on the fly,
// q = K p_new, partial sums of p_new . q, last-block alpha), but the matrix stream is moved by the bulk-copy
// engine instead of per-thread loads: every warp owns whole slices (32 block rows) and walks their blocks in
// chunks of CB blocks.  A slice's blocks are contiguous (CB * 288 values, then CB * 32 column indices), so one
// chunk is two cp.async.bulk copies into one of the warp's NST shared-memory stages, completed on the stage's
// mbarrier.  Lane 0 keeps NST - 1 chunks in flight ahead of the chunk being multiplied, which keeps enough
// bytes outstanding per SM to run at the HBM rate with few warps; the lanes then read the stage
// bank-conflict free (lane l reads word 32 e + l of each block) and gather neighbours from L2.
// Matrix chunks are copied with an L2 policy: blocks below keep_g (slice-block index) are marked evict_last
// so that part of the matrix stays in L2 from one CG iteration to the next, the rest evict_first.
// Every wait on an mbarrier is bounded; a wait that gives up marks the CG as failed (scal[kDone] = 6), waits
// (bounded again) for the warp's copies still in flight and leaves the chunk loop.
#include <mutex>

#include "staging.cuh"

namespace ikr {

namespace {

using namespace cg;

// position in a warp's stream of chunks: slice s, first block g of the chunk, end of the slice gend
struct ChunkPos {
  int s, g, gend;
  __device__ __forceinline__ void start(const int32_t* slice_off, int s0, int n_slices) {
    s = s0;
    if (s < n_slices) g = slice_off[s], gend = slice_off[s + 1];
  }
  __device__ __forceinline__ void advance(const int32_t* slice_off, int CB, int stride, int n_slices) {
    g += CB;
    if (g >= gend) {
      s += stride;
      if (s < n_slices) g = slice_off[s], gend = slice_off[s + 1];
    }
  }
};

template <typename T, int CB, int NST, int WARPS>
struct Staged {
  static constexpr int kValBytes = CB * 288 * (int)sizeof(T);
  static constexpr int kColBytes = CB * 32 * 4;
  static constexpr int kStageBytes = kValBytes + kColBytes;
  static constexpr int kSmemBytes = WARPS * NST * kStageBytes;
  static constexpr int kThreads = WARPS * 32;
};

template <typename T, int CB, int NST, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) pcg_spmv_staged_kernel(Bsr A, const T* __restrict__ val,
                                                                     const T* __restrict__ z,
                                                                     const T* __restrict__ pold, T* __restrict__ pnew,
                                                                     T* __restrict__ q, double* part, double* scal,
                                                                     int64_t keep_g) {
  using C = Staged<T, CB, NST, WARPS>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[WARPS][NST];
  __shared__ double sh[32];
  __shared__ bool last;
  if (scal[kDone] != 0.0) return;
  const T beta = T(scal[kBeta]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* wbase = smem + (size_t)warp * NST * C::kStageBytes;
  const int nw = gridDim.x * WARPS;
  const int n_slices = A.n_slices;
  if (lane == 0) {
    for (int st = 0; st < NST; ++st) mbar_init(smem_addr(&bars[warp][st]), 1);
    mbar_init_fence();
  }
  __syncwarp();

  auto issue = [&](int st, const ChunkPos& P) {
    if (lane == 0) {
      const int nb = min(CB, P.gend - P.g);
      const uint32_t vb = nb * 288 * (uint32_t)sizeof(T), cb = nb * 128;
      const uint32_t bar = smem_addr(&bars[warp][st]);
      unsigned char* stage = wbase + (size_t)st * C::kStageBytes;
      const uint64_t pol = l2_policy(P.g < keep_g);
      mbar_expect_tx(bar, vb + cb);
      bulk_g2s(smem_addr(stage), val + (int64_t)P.g * 288, vb, bar, pol);
      bulk_g2s(smem_addr(stage + C::kValBytes), A.col_sell + (int64_t)P.g * 32, cb, bar, pol);
    }
  };

  ChunkPos P, Q;
  P.start(A.slice_off, blockIdx.x * WARPS + warp, n_slices);
  Q = P;
  int inflight = 0;
  for (int st = 0; st < NST && P.s < n_slices; ++st) {
    issue(st, P);
    ++inflight;
    P.advance(A.slice_off, CB, nw, n_slices);
  }
  uint32_t phase = 0;
  int st = 0;
  bool failed = false;
  T a0 = T(0), a1 = T(0), a2 = T(0);
  double pq = 0.0;
  while (Q.s < n_slices) {
    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(smem_addr(&bars[warp][st]), (phase >> st) & 1u));
    if (!ok) {
      failed = true;
      break;
    }
    phase ^= 1u << st;
    --inflight;
    const T* sv = reinterpret_cast<const T*>(wbase + (size_t)st * C::kStageBytes);
    const int32_t* sc = reinterpret_cast<const int32_t*>(wbase + (size_t)st * C::kStageBytes + C::kValBytes);
    const int nb = min(CB, Q.gend - Q.g);
    // all gathers of the chunk first (one L1/L2 round trip), then the products; blocks past the end of a
    // short chunk gather node 0 and are skipped
    V3<T> zc[CB], pc[CB];
#pragma unroll
    for (int k = 0; k < CB; ++k) {
      const int c = k < nb ? sc[32 * k + lane] : 0;
      zc[k] = load3(z, c);
      pc[k] = load3(pold, c);
    }
#pragma unroll
    for (int k = 0; k < CB; ++k) {
      if (k < nb) {
        const T x0 = zc[k].x + beta * pc[k].x, x1 = zc[k].y + beta * pc[k].y, x2 = zc[k].z + beta * pc[k].z;
        const T* v = sv + 288 * k + lane;
        a0 += v[0] * x0 + v[32] * x1 + v[64] * x2;
        a1 += v[96] * x0 + v[128] * x1 + v[160] * x2;
        a2 += v[192] * x0 + v[224] * x1 + v[256] * x2;
      }
    }
    __syncwarp();  // every lane is done with the stage before it is refilled
    if (P.s < n_slices) {
      issue(st, P);
      ++inflight;
      P.advance(A.slice_off, CB, nw, n_slices);
    }
    if (Q.g + CB >= Q.gend) {  // last chunk of the slice: finish the warp's 32 rows
      const int row = 32 * Q.s + lane;
      if (row < A.n_rows) {
        const V3<T> zr = load3(z, row), pr = load3(pold, row);
        const T p0 = zr.x + beta * pr.x, p1 = zr.y + beta * pr.y, p2 = zr.z + beta * pr.z;
        store3(pnew, row, p0, p1, p2);
        store3(q, row, a0, a1, a2);
        pq += double(p0 * a0 + p1 * a1 + p2 * a2);
      }
      a0 = a1 = a2 = T(0);
    }
    Q.advance(A.slice_off, CB, nw, n_slices);
    st = (st + 1 == NST) ? 0 : st + 1;
  }
  if (failed) {
    // drain: the stages still owed a copy complete in issue order after the one that timed out
    for (int k = 0; k < inflight; ++k) {
      mbar_wait_bounded(smem_addr(&bars[warp][st]), (phase >> st) & 1u);
      phase ^= 1u << st;
      st = (st + 1 == NST) ? 0 : st + 1;
    }
    if (lane == 0) scal[kDone] = kDoneDeviceTimeout;
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

template <typename T, int CB, int NST, int WARPS>
void launch_staged(const Bsr& A, PcgWork& w, const void* pold, void* pnew, cudaStream_t s) {
  using C = Staged<T, CB, NST, WARPS>;
  auto kern = pcg_spmv_staged_kernel<T, CB, NST, WARPS>;
  // per-device launch shape: attribute set and occupancy queried once per device
  static std::mutex mu;
  static int blocks_per_sm[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  int bps;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 64) dev = 63;
    if (!blocks_per_sm[dev]) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmemBytes);
      int b = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, C::kThreads, C::kSmemBytes);
      blocks_per_sm[dev] = b > 0 ? b : 1;
    }
    bps = blocks_per_sm[dev];
  }
  int grid = w.sms * bps;
  if (grid > w.grid) grid = w.grid;  // the partial buffers hold w.grid entries
  const int max_useful = (A.n_slices + WARPS - 1) / WARPS;
  if (grid > max_useful) grid = max_useful;
  if (grid < 1) grid = 1;
  kern<<<grid, C::kThreads, C::kSmemBytes, s>>>(A, (const T*)A.val, (const T*)w.z, (const T*)pold, (T*)pnew,
                                                (T*)w.q, w.part_a, w.scal, w.keep_g);
}

}  // namespace

__global__ void fill64_kernel(double* __restrict__ y, double v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = v;
}

int spmv_staged_variants() { return 4; }

void launch_fill64(double* y, double v, int64_t n, cudaStream_t s) {
  int g = (int)((n + 255) / 256);
  if (g > 1216) g = 1216;
  if (g < 1) g = 1;
  fill64_kernel<<<g, 256, 0, s>>>(y, v, n);
}

const char* spmv_staged_name(bool fp32, int v) {
  static const char* f32[] = {"staged CB8 NST2 W8", "staged CB6 NST3 W8", "staged CB4 NST4 W8", "staged CB4 NST3 W12"};
  static const char* f64[] = {"staged CB4 NST2 W8", "staged CB3 NST3 W8", "staged CB2 NST4 W8", "staged CB2 NST3 W12"};
  if (v < 0 || v >= 4) return "?";
  return fp32 ? f32[v] : f64[v];
}

void launch_pcg_spmv_staged(const Bsr& A, PcgWork& w, int variant, const void* pold, void* pnew, cudaStream_t s) {
  if (w.fp32) {
    switch (variant) {
      case 0: launch_staged<float, 8, 2, 8>(A, w, pold, pnew, s); break;
      case 1: launch_staged<float, 6, 3, 8>(A, w, pold, pnew, s); break;
      case 2: launch_staged<float, 4, 4, 8>(A, w, pold, pnew, s); break;
      default: launch_staged<float, 4, 3, 12>(A, w, pold, pnew, s); break;
    }
  } else {
    switch (variant) {
      case 0: launch_staged<double, 4, 2, 8>(A, w, pold, pnew, s); break;
      case 1: launch_staged<double, 3, 3, 8>(A, w, pold, pnew, s); break;
      case 2: launch_staged<double, 2, 4, 8>(A, w, pold, pnew, s); break;
      default: launch_staged<double, 2, 3, 12>(A, w, pold, pnew, s); break;
    }
  }
}

}  // namespace ikr
