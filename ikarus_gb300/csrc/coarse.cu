// Coarse correction of the block-Jacobi CG: an additive two-level preconditioner (sm_103a).
//
//   M^-1 r = D^-1 r + P A_c^-1 P^T r,   A_c = P^T K P
//
// D is the 3x3 block diagonal of the tangent K (the CG's block-Jacobi preconditioner).  P has six columns per
// aggregate of nodes, the rigid-body modes of that aggregate: translations e_k and rotations e_k x y about its
// centroid (y = node position - centroid), zero at constrained dofs.  With slab aggregates along a slender
// body's long axis the coarse space carries the beam-like bending and torsion modes that make block-Jacobi CG
// slow there.  M is symmetric positive definite (D^-1 SPD, P A_c^-1 P^T semi-definite), so CG stays CG.
//
// Per CG iteration, after the update kernel (which leaves z = D^-1 r and the partial r.D^-1 r in kRzF), two
// kernels:
//   restrict and solve: one CTA per chunk (up to 2048 nodes of one aggregate) writes the chunk's six sums of
//             P^T r; the CTA that finishes last sums the chunks of every aggregate in a fixed order (r_c), forms
//             e = A_c^-1 r_c with the dense inverse, r.z = r.D^-1 r + r_c.e, and beta (or the initial r.z);
//   prolong:  z += P e.
// Setup per tangent (A_c): for every colour of a distance-2 colouring of the aggregates, the six probe vectors
// sum_{a of that colour} P_{a,m} are multiplied by K (launch_spmv64) and restricted per chunk (36 sums); the
// host adds the chunks of each aggregate in a fixed order, places each block at the single aggregate of the
// colour that touches it, and inverts A_c (ikr_ls_s in host_internal.h).  All sums are fixed-order: results are
// bit-identical run to run.
#include "cg_common.cuh"

namespace ikr {

namespace {

using namespace cg;
constexpr int kThreads = 1024;       // CTA of the restrict-and-solve kernel (a chunk is up to 2048 nodes)
static_assert(kCoarseMaxDofs <= kThreads, "the coarse solve splits the coarse dofs over the threads of one CTA");
constexpr int kCoarseTicket = 4;     // ticket slot of its last-block reduction (scalar slot 14)

// node data: offset from the aggregate centroid (x, y, z) and, in the fourth lane as integer bits, the
// aggregate id (bits 0-23) and the free-dof mask (bits 24-26)
struct NodeP {
  float y[3];
  int agg;
  int mask;
};
__device__ __forceinline__ NodeP node_p(const float4* __restrict__ y4, int node) {
  const float4 v = __ldg(y4 + node);
  const int bits = __float_as_int(v.w);
  return {{v.x, v.y, v.z}, bits & 0xFFFFFF, (bits >> 24) & 7};
}

// the six mode columns of P at a node (3 x 6), masked: P[c][m]
__device__ __forceinline__ void p_cols(const NodeP& n, double P[3][6]) {
  const double yx = n.y[0], yy = n.y[1], yz = n.y[2];
  const double cols[3][6] = {{1, 0, 0, 0.0, yz, -yy}, {0, 1, 0, -yz, 0.0, yx}, {0, 0, 1, yy, -yx, 0.0}};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double on = ((n.mask >> c) & 1) ? 1.0 : 0.0;
#pragma unroll
    for (int m = 0; m < 6; ++m) P[c][m] = on * cols[c][m];
  }
}

// P^T r per chunk; the CTA that finishes last sums the chunks of every aggregate in a fixed order (r_c), forms
// e = A_c^-1 r_c with the dense inverse, r.z = r.D^-1 r + r_c.e and beta (or the initial r.z)
template <typename T>
__global__ void __launch_bounds__(kThreads) coarse_restrict_solve_kernel(Coarse C, const T* __restrict__ r,
                                                                         double* scal, int init) {
  __shared__ double sh[32];
  __shared__ double rc[kCoarseMaxDofs];
  __shared__ double red[kThreads];
  __shared__ bool last;
  if (scal[kDone] != 0.0) return;
  const int k = blockIdx.x;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int i = C.chunk_off[k] + threadIdx.x; i < C.chunk_off[k + 1]; i += blockDim.x) {
    const int node = __ldg(C.nodes + i);
    const NodeP n = node_p(C.y4, node);
    const V3<T> rv = load3(r, node);
    double P[3][6];
    p_cols(n, P);
#pragma unroll
    for (int m = 0; m < 6; ++m) s[m] += P[0][m] * double(rv.x) + P[1][m] * double(rv.y) + P[2][m] * double(rv.z);
  }
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const double t = block_sum_all(s[m], sh);
    if (threadIdx.x == 0) C.rpart[6 * k + m] = t;
  }
  if (!publish_and_check_last(&tickets(scal)[kCoarseTicket], &last)) return;
  const int nc = C.n_c;
  for (int j = threadIdx.x; j < nc; j += blockDim.x) {
    const int a = j / 6, m = j - 6 * a;
    double t = 0.0;
    for (int q = C.agg_chunk[a]; q < C.agg_chunk[a + 1]; ++q) t += __ldcg(C.rpart + 6 * q + m);
    rc[j] = t;
  }
  __syncthreads();
  // e = A_c^-1 r_c: thread t forms the part of entry i = t mod n_c over segment t / n_c of the columns (A_c^-1
  // is symmetric: column-major reads, coalesced along i; all loads of a thread independent), then the segments
  // are added in order
  const T* ainv = static_cast<const T*>(C.ainv);
  const int t = threadIdx.x, nseg = blockDim.x / nc, seg_len = (nc + nseg - 1) / nseg;
  const int i = t % nc, seg = t / nc;
  double acc = 0.0;
  if (seg < nseg) {
    const int j1 = min(nc, (seg + 1) * seg_len);
#pragma unroll 8
    for (int j = seg * seg_len; j < j1; ++j) acc += double(__ldg(ainv + (size_t)j * nc + i)) * rc[j];
  }
  red[t] = acc;
  __syncthreads();
  double qc = 0.0;
  if (t < nc) {
    double ev = 0.0;
    for (int g = 0; g < nseg; ++g) ev += red[g * nc + t];
    const T ei = T(ev);
    static_cast<T*>(C.e)[t] = ei;
    qc = rc[t] * double(ei);
  }
  qc = block_sum_all(qc, sh);
  if (threadIdx.x == 0) {
    const double rz = scal[kRzF] + qc;
    if (init) {
      scal[kRz] = rz;
      scal[kBeta] = 0.0;
    } else {
      scal[kBeta] = rz / scal[kRz];
      scal[kRz] = rz;
    }
    tickets(scal)[kCoarseTicket] = 0u;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) coarse_prolong_kernel(Coarse C, T* z, const double* __restrict__ scal) {
  __shared__ T e[kCoarseMaxDofs];
  if (scal[kDone] != 0.0) return;
  for (int j = threadIdx.x; j < C.n_c; j += blockDim.x) e[j] = static_cast<const T*>(C.e)[j];
  __syncthreads();
  for (int node = blockIdx.x * blockDim.x + threadIdx.x; node < C.n_rows; node += gridDim.x * blockDim.x) {
    const NodeP n = node_p(C.y4, node);
    const T* ea = e + 6 * n.agg;
    const T yx = T(n.y[0]), yy = T(n.y[1]), yz = T(n.y[2]);
    // t + w x y with t = e[0..2], w = e[3..5]
    T d0 = ea[0] + ea[4] * yz - ea[5] * yy;
    T d1 = ea[1] + ea[5] * yx - ea[3] * yz;
    T d2 = ea[2] + ea[3] * yy - ea[4] * yx;
    if (!(n.mask & 1)) d0 = T(0);
    if (!(n.mask & 2)) d1 = T(0);
    if (!(n.mask & 4)) d2 = T(0);
    const V3<T> zv = load3rw(z, node);
    store3(z, node, zv.x + d0, zv.y + d1, zv.z + d2);
  }
}

// probe vectors of one colour: V_m (dof-major FP64, m = 0..5, stride 3 n_rows) = P_{a,m} on the nodes of every
// aggregate a of that colour, zero elsewhere
__global__ void coarse_probe_kernel(Coarse C, int colour, double* __restrict__ V) {
  const int64_t stride = 3LL * C.n_rows;
  for (int node = blockIdx.x * blockDim.x + threadIdx.x; node < C.n_rows; node += gridDim.x * blockDim.x) {
    const NodeP n = node_p(C.y4, node);
    const bool on = __ldg(C.agg_colour + n.agg) == colour;
    double P[3][6];
    p_cols(n, P);
#pragma unroll
    for (int m = 0; m < 6; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c) V[m * stride + 3 * node + c] = on ? P[c][m] : 0.0;
  }
}

// 36 sums per chunk: part[36 k + 6 r + m] = sum over the chunk's nodes of P[:, r] . W_m
__global__ void __launch_bounds__(256) coarse_galerkin_kernel(Coarse C, const double* __restrict__ W,
                                                              double* __restrict__ part) {
  __shared__ double sh[32];
  const int64_t stride = 3LL * C.n_rows;
  const int k = blockIdx.x;
  double s[36];
#pragma unroll
  for (int q = 0; q < 36; ++q) s[q] = 0.0;
  for (int i = C.chunk_off[k] + threadIdx.x; i < C.chunk_off[k + 1]; i += blockDim.x) {
    const int node = __ldg(C.nodes + i);
    const NodeP n = node_p(C.y4, node);
    double P[3][6];
    p_cols(n, P);
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const double w0 = __ldg(W + m * stride + 3 * node), w1 = __ldg(W + m * stride + 3 * node + 1),
                   w2 = __ldg(W + m * stride + 3 * node + 2);
#pragma unroll
      for (int r = 0; r < 6; ++r) s[6 * r + m] += P[0][r] * w0 + P[1][r] * w1 + P[2][r] * w2;
    }
  }
#pragma unroll
  for (int q = 0; q < 36; ++q) {
    const double t = block_sum_all(s[q], sh);
    if (threadIdx.x == 0) part[36 * k + q] = t;
  }
}

int grid_for(int n, int bs, int cap) {
  int b = (n + bs - 1) / bs;
  return b < 1 ? 1 : (b > cap ? cap : b);
}

}  // namespace

void launch_coarse_correction(const Coarse& C, const PcgWork& w, bool init, cudaStream_t s) {
  if (w.fp32) {
    coarse_restrict_solve_kernel<float><<<C.n_chunks, kThreads, 0, s>>>(C, (const float*)w.r, w.scal, init ? 1 : 0);
    coarse_prolong_kernel<float><<<w.grid, 256, 0, s>>>(C, (float*)w.z, w.scal);
  } else {
    coarse_restrict_solve_kernel<double><<<C.n_chunks, kThreads, 0, s>>>(C, (const double*)w.r, w.scal, init ? 1 : 0);
    coarse_prolong_kernel<double><<<w.grid, 256, 0, s>>>(C, (double*)w.z, w.scal);
  }
}
void launch_coarse_probe(const Coarse& C, int colour, double* V, cudaStream_t s) {
  coarse_probe_kernel<<<grid_for(C.n_rows, 256, 1216), 256, 0, s>>>(C, colour, V);
}
void launch_coarse_galerkin(const Coarse& C, const double* W, double* part, cudaStream_t s) {
  coarse_galerkin_kernel<<<C.n_chunks, 256, 0, s>>>(C, W, part);
}

}  // namespace ikr
