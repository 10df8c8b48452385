// Device construction of the 3x3-block sparsity pattern and the per-assembly helpers (sm_103a).
//
// Reference: SparseFlatAssembler::createOccupationPattern + setFromTriplets and createLinearDOFsPerElement
// (ikarus/assembler/simpleassemblers.inl:206-265).  The scalar pattern of the reference is the set of all
// (dof_i, dof_j) pairs of every element, sorted column-major.  Because every node carries three dofs that all
// couple with the three dofs of every neighbour node, that pattern is exactly the expansion of the node-level
// pattern below into 3x3 blocks; the tests expand it and compare bit-for-bit with the oracle.
//
// Build steps (all on the device, deterministic):
//   1. node -> element incidence (counting, scan, fill, per-node sort),
//   2. per block row: the sorted unique set of nodes sharing an element with the row node,
//   3. row pointers by scan, column indices,
//   4. the element-to-block slot map (64 per element) and the diagonal block of every row.
#include "common.cuh"
#include "kernels.h"

namespace ikr {

namespace {

constexpr int kMaxRow = 128;  // nodes coupled to one node; structured hexahedral meshes need 27

__global__ void node_elem_count_kernel(const int32_t* __restrict__ conn, int ne, int32_t* cnt) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 8LL * ne) return;
  atomicAdd(&cnt[conn[t]], 1);
}

// exclusive scan with one block walking the array in tiles; out[n] = total
__global__ void scan_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, int n) {
  __shared__ int32_t buf[1024];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const int32_t v = i < n ? in[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int32_t t = threadIdx.x >= off ? buf[threadIdx.x - off] : 0;
      __syncthreads();
      buf[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < n) out[i] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

__global__ void node_elem_fill_kernel(const int32_t* __restrict__ conn, int ne, const int32_t* __restrict__ ptr,
                                      int32_t* cursor, int32_t* elems) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 8LL * ne) return;
  const int e = (int)(t % ne);
  const int n = conn[t];
  const int pos = atomicAdd(&cursor[n], 1);
  elems[ptr[n] + pos] = e;
}

__global__ void node_elem_sort_kernel(const int32_t* __restrict__ ptr, int32_t* elems, int nn) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const int b = ptr[n], e = ptr[n + 1];
  for (int i = b + 1; i < e; ++i) {  // insertion sort: a handful of entries per node
    const int32_t v = elems[i];
    int j = i - 1;
    while (j >= b && elems[j] > v) {
      elems[j + 1] = elems[j];
      --j;
    }
    elems[j + 1] = v;
  }
}

// Sorted unique neighbour set of node n.  fill = false: write the count; fill = true: write the columns.
__global__ void row_build_kernel(const int32_t* __restrict__ conn, int ne, int nn, const int32_t* __restrict__ ne_ptr,
                                 const int32_t* __restrict__ ne_elems, const int32_t* __restrict__ row_ptr,
                                 int32_t* out, bool fill, int* status) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  int32_t set[kMaxRow];
  int cnt = 0;
  bool overflow = false;
  for (int k = ne_ptr[n]; k < ne_ptr[n + 1]; ++k) {
    const int e = ne_elems[k];
    for (int v = 0; v < 8; ++v) {
      const int32_t m = conn[v * ne + e];
      int pos = cnt;
      while (pos > 0 && set[pos - 1] > m) --pos;
      if (pos > 0 && set[pos - 1] == m) continue;
      if (cnt == kMaxRow) {
        overflow = true;
        continue;
      }
      for (int j = cnt; j > pos; --j) set[j] = set[j - 1];
      set[pos] = m;
      ++cnt;
    }
  }
  if (overflow) {
    atomicOr(status, kStatusPatternOverflow);
    return;
  }
  if (!fill) {
    out[n] = cnt;
  } else {
    const int b = row_ptr[n];
    for (int j = 0; j < cnt; ++j) out[b + j] = set[j];
  }
}

__device__ __forceinline__ int find_col(const int32_t* __restrict__ col, int b, int e, int key) {
  int lo = b, hi = e;  // lower bound in [b, e)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (col[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// block id of the k-th block of row r (see Bsr in kernels.h)
__device__ __forceinline__ int32_t block_id(const int32_t* __restrict__ slice_off, int r, int k) {
  return (slice_off[r >> 5] + k) * 32 + (r & 31);
}

__global__ void slice_len_kernel(const int32_t* __restrict__ row_ptr, int nn, int32_t* slice_len) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (nn + 31) / 32) return;
  int m = 0;
  for (int r = 32 * s; r < min(nn, 32 * s + 32); ++r) m = max(m, row_ptr[r + 1] - row_ptr[r]);
  slice_len[s] = m;
}

__global__ void sell_fill_kernel(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                 const int32_t* __restrict__ slice_off, int nn, int32_t* col_sell) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (nn + 31) / 32 * 32) return;
  const int s = r >> 5;
  const int width = slice_off[s + 1] - slice_off[s];
  const int len = r < nn ? row_ptr[r + 1] - row_ptr[r] : 0;
  for (int k = 0; k < width; ++k)
    col_sell[block_id(slice_off, r, k)] = k < len ? col[row_ptr[r] + k] : (r < nn ? r : 0);
}

__global__ void slot_map_kernel(const int32_t* __restrict__ conn, int ne, const int32_t* __restrict__ row_ptr,
                                const int32_t* __restrict__ col, const int32_t* __restrict__ slice_off,
                                int32_t* slot) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 64LL * ne) return;
  const int e = (int)(t % ne);
  const int pair = (int)(t / ne);
  const int I = pair >> 3, J = pair & 7;
  const int r = conn[I * ne + e], c = conn[J * ne + e];
  slot[t] = block_id(slice_off, r, find_col(col, row_ptr[r], row_ptr[r + 1], c) - row_ptr[r]);
}

__global__ void diag_kernel(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                            const int32_t* __restrict__ slice_off, int32_t* diag, int nn) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  diag[n] = block_id(slice_off, n, find_col(col, row_ptr[n], row_ptr[n + 1], n) - row_ptr[n]);
}

// Full Dirichlet treatment of the matrix (simpleassemblers.inl:159-167): constrained rows and columns are zero
// except a unit diagonal.  The element kernels skip every constrained entry, so the reset only has to put the
// unit diagonal in place after zeroing.
template <typename T>
__global__ void unit_diag_kernel(T* val, const int32_t* __restrict__ diag, const uint8_t* __restrict__ fixed, int nn) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nn) return;
  const uint8_t m = fixed[n];
  if (!m) return;
  for (int c = 0; c < 3; ++c)
    if ((m >> c) & 1) val[block_entry(diag[n], 4 * c)] = T(1);
}

// Manipulator point loads after the Dirichlet treatment (assemblermanipulatorbuildingblocks.hh:110-115):
// R[dof] += lambda * value, one thread per distinct dof.
__global__ void point_load_kernel(double* R, const int32_t* __restrict__ dof, const double* __restrict__ val, int n,
                                  double lf, const double* __restrict__ lf_dev) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  R[dof[k]] += (lf_dev ? *lf_dev : lf) * val[k];
}

// inhomogeneous Dirichlet values: u[i] = lambda rate[i] where that value is nonzero
__global__ void idbc_sync_kernel(double* __restrict__ u, const double* __restrict__ rate, double lambda, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = lambda * rate[i];
    if (v != 0.0) u[i] = v;
  }
}
// R += step F on the free dofs (F = K_raw du_D/dlambda)
__global__ void idbc_force_kernel(double* __restrict__ R, const double* __restrict__ F,
                                  const uint8_t* __restrict__ node_fixed, double step, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!((node_fixed[i / 3] >> (i % 3)) & 1)) R[i] += step * F[i];
}

// ||sync(u, lambda_new) - u||^2: the squared change of the solution when the inhomogeneous Dirichlet values are
// re-imposed at the load factor lambda_new (entries whose prescribed value is nonzero take it)
__global__ void idbc_delta_sq_partial_kernel(const double* __restrict__ u, const double* __restrict__ rate,
                                             double lambda_new, int64_t n, double* part) {
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = lambda_new * rate[i];
    if (v != 0.0) s += (v - u[i]) * (v - u[i]);
  }
  s = warp_sum(s);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}
__global__ void mul_kernel(double* __restrict__ y, const double* __restrict__ x, const double* __restrict__ m,
                           int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i] * m[i];
}

// deterministic sum of squares: fixed grid, per-block partials, then one block sums them in order
__global__ void sumsq_partial_kernel(const double* __restrict__ x, int64_t n, double* part) {
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += x[i] * x[i];
  s = warp_sum(s);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}
__global__ void dot_partial_kernel(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                                   double* part) {
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += x[i] * y[i];
  s = warp_sum(s);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}
__global__ void sum_partials_kernel(const double* __restrict__ part, int np, double* out, bool take_sqrt) {
  __shared__ double ws[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) *out = take_sqrt ? sqrt(v) : v;
  }
}

inline int blocks_for(int64_t n, int bs) { return (int)((n + bs - 1) / bs); }

}  // namespace

constexpr int kNormGrid = 304;  // two blocks per SM on a 152-SM GB300

void launch_node_elem_count(const int32_t* conn, int n_elems, int n_nodes, int32_t* cnt, cudaStream_t s) {
  cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n_nodes, s);
  node_elem_count_kernel<<<blocks_for(8LL * n_elems, 256), 256, 0, s>>>(conn, n_elems, cnt);
}
void launch_exclusive_scan(const int32_t* in, int32_t* out, int n, cudaStream_t s) {
  scan_kernel<<<1, 1024, 0, s>>>(in, out, n);
}
void launch_node_elem_fill(const int32_t* conn, int n_elems, const int32_t* ptr, int32_t* cursor, int32_t* elems,
                           int n_nodes, cudaStream_t s) {
  cudaMemsetAsync(cursor, 0, sizeof(int32_t) * n_nodes, s);
  node_elem_fill_kernel<<<blocks_for(8LL * n_elems, 256), 256, 0, s>>>(conn, n_elems, ptr, cursor, elems);
  node_elem_sort_kernel<<<blocks_for(n_nodes, 128), 128, 0, s>>>(ptr, elems, n_nodes);
}
void launch_row_build(const int32_t* conn, int n_elems, int n_nodes, const int32_t* ne_ptr, const int32_t* ne_elems,
                      const int32_t* row_ptr, int32_t* cnt_or_col, bool fill, int* status, cudaStream_t s) {
  row_build_kernel<<<blocks_for(n_nodes, 64), 64, 0, s>>>(conn, n_elems, n_nodes, ne_ptr, ne_elems, row_ptr,
                                                           cnt_or_col, fill, status);
}
void launch_slice_lengths(const int32_t* row_ptr, int n_nodes, int32_t* slice_len, cudaStream_t s) {
  slice_len_kernel<<<blocks_for((n_nodes + 31) / 32, 128), 128, 0, s>>>(row_ptr, n_nodes, slice_len);
}
void launch_sell_fill(const int32_t* row_ptr, const int32_t* col, const int32_t* slice_off, int n_nodes,
                      int32_t* col_sell, cudaStream_t s) {
  sell_fill_kernel<<<blocks_for((n_nodes + 31) / 32 * 32LL, 128), 128, 0, s>>>(row_ptr, col, slice_off, n_nodes,
                                                                               col_sell);
}
void launch_slot_map(const int32_t* conn, int n_elems, const int32_t* row_ptr, const int32_t* col,
                     const int32_t* slice_off, int32_t* slot, int32_t* diag, int n_nodes, cudaStream_t s) {
  slot_map_kernel<<<blocks_for(64LL * n_elems, 256), 256, 0, s>>>(conn, n_elems, row_ptr, col, slice_off, slot);
  diag_kernel<<<blocks_for(n_nodes, 256), 256, 0, s>>>(row_ptr, col, slice_off, diag, n_nodes);
}
void launch_bsr_reset(void* val, bool fp32, int64_t n_padded, const int32_t* diag, const uint8_t* node_fixed,
                      int n_nodes, cudaStream_t s) {
  cudaMemsetAsync(val, 0, (size_t)n_padded * 9 * (fp32 ? 4 : 8), s);
  if (!node_fixed) return;
  if (fp32) unit_diag_kernel<float><<<blocks_for(n_nodes, 256), 256, 0, s>>>((float*)val, diag, node_fixed, n_nodes);
  else unit_diag_kernel<double><<<blocks_for(n_nodes, 256), 256, 0, s>>>((double*)val, diag, node_fixed, n_nodes);
}
// AssemblerManipulator matrix entries: val[idx[k]] += v[k] (indices unique, so no two threads touch one value)
template <typename T>
__global__ void add_entries_kernel(T* __restrict__ val, const int64_t* __restrict__ idx, const double* __restrict__ v,
                                   int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) val[idx[k]] = T(double(val[idx[k]]) + v[k]);
}
void launch_add_entries(void* val, bool fp32, const int64_t* idx, const double* v, int n, cudaStream_t s) {
  if (n <= 0) return;
  if (fp32) add_entries_kernel<float><<<blocks_for(n, 128), 128, 0, s>>>((float*)val, idx, v, n);
  else add_entries_kernel<double><<<blocks_for(n, 128), 128, 0, s>>>((double*)val, idx, v, n);
}

void launch_vector_finish(double* R, const uint8_t* node_fixed, int n_nodes, const int32_t* pl_dof,
                          const double* pl_val, int n_pl, double load_factor, cudaStream_t s,
                          const double* load_factor_dev) {
  (void)node_fixed;
  (void)n_nodes;
  if (n_pl > 0)
    point_load_kernel<<<blocks_for(n_pl, 128), 128, 0, s>>>(R, pl_dof, pl_val, n_pl, load_factor, load_factor_dev);
}
void launch_idbc_sync(double* u, const double* rate, double lambda, int64_t n, cudaStream_t s) {
  idbc_sync_kernel<<<kNormGrid, 256, 0, s>>>(u, rate, lambda, n);
}
void launch_idbc_force(double* R, const double* F, const uint8_t* node_fixed, double step, int64_t n, cudaStream_t s) {
  idbc_force_kernel<<<kNormGrid, 256, 0, s>>>(R, F, node_fixed, step, n);
}
void launch_idbc_delta_sq(const double* u, const double* rate, double lambda_new, int64_t n, double* partials,
                          double* out, cudaStream_t s) {
  idbc_delta_sq_partial_kernel<<<kNormGrid, 256, 0, s>>>(u, rate, lambda_new, n, partials);
  sum_partials_kernel<<<1, 256, 0, s>>>(partials, kNormGrid, out, false);
}
void launch_mul64(double* y, const double* x, const double* m, int64_t n, cudaStream_t s) {
  mul_kernel<<<kNormGrid, 256, 0, s>>>(y, x, m, n);
}
void launch_norm2(const double* x, int64_t n, double* partials, double* out, cudaStream_t s) {
  sumsq_partial_kernel<<<kNormGrid, 256, 0, s>>>(x, n, partials);
  sum_partials_kernel<<<1, 256, 0, s>>>(partials, kNormGrid, out, true);
}
void launch_dot(const double* x, const double* y, int64_t n, double* partials, double* out, cudaStream_t s) {
  dot_partial_kernel<<<kNormGrid, 256, 0, s>>>(x, y, n, partials);
  sum_partials_kernel<<<1, 256, 0, s>>>(partials, kNormGrid, out, false);
}

}  // namespace ikr
