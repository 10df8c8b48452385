// Kernel launch interface between the C++ host layer and the CUDA translation units.
// Plain structs of device pointers; no torch types anywhere.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ikr {

enum ElemMode : int {
  kWantR = 1,       // internal force (always FP64)
  kWantK = 2,       // tangent (FP64 or FP32 arithmetic, see KT)
  kWantEnergy = 4,  // stored energy (FP64, displacement-based only)
  kElemOut = 8,     // write element-level outputs instead of assembling
};

enum StatusBits : int {
  kStatusNonPositiveDetC = 1,  // checkPositiveOrAbort (materialhelpers.hh:119-126) on the device
  kStatusNonFinite = 2,
  kStatusSingularD = 4,        // EAS D matrix could not be factorised
  kStatusPatternOverflow = 8,  // a node couples with more nodes than the pattern builder supports
};

struct ElemArgs {
  int n_nodes = 0, n_elems = 0;
  const double* X = nullptr;     // coordinates, n_nodes x 3
  const int32_t* conn = nullptr; // corner-major: conn[v * n_elems + e]
  double lam = 0, mu = 0;        // Lame parameters of NeoHooke
  const double* u = nullptr;     // displacement, 3 * n_nodes (FP64)
  const uint8_t* node_fixed = nullptr;  // per node 3-bit Dirichlet mask; nullptr = no masking (Raw)
  // dead tractions: trac_idx[e] >= 0 indexes 24 values of sum_faces N_I t dA at load factor 1
  const int32_t* trac_idx = nullptr;
  const double* trac = nullptr;
  double load_factor = 0;
  // EAS
  int eas_kind = 0, n_alpha = 0;
  const double* alpha = nullptr;   // n_alpha x n_elems (parameter-major)
  const double* eas_geo = nullptr; // per-element centre data, see element.cu
  double* eas_y = nullptr;         // cache: D^{-1} R~ (n_alpha x n_elems)
  double* eas_Y = nullptr;         // cache: D^{-1} L  (n_alpha*24 x n_elems)
  // outputs
  double* R = nullptr;             // assembled residual (n dofs)
  void* Kval = nullptr;            // BSR values (float or double), 9 per block, row-major blocks
  const int32_t* slot = nullptr;   // 64 x n_elems: slot[(I*8+J) * n_elems + e] = BSR block of (node I, node J)
  double* elem_vec = nullptr;      // element-level: 24 per listed element
  double* elem_mat = nullptr;      // element-level: 576 per listed element, column-major
  double* elem_energy = nullptr;   // element-level: 1 per listed element
  int* status = nullptr;           // StatusBits, OR-ed
};

struct Bsr {
  int n_rows = 0;             // block rows = nodes
  int64_t n_blocks = 0;
  const int32_t* row_ptr = nullptr;
  const int32_t* col = nullptr;
  const int32_t* diag = nullptr;  // position of the diagonal block of each row
  const void* val = nullptr;      // float or double, 9 per block
};

// element.cu
void launch_disp_element(const ElemArgs& a, int mode, bool fp32_tangent, const int32_t* list, int n_list, int e_base,
                         cudaStream_t s);
void launch_eas_element(const ElemArgs& a, int mode, bool fp32_tangent, const int32_t* list, int n_list, int e_base,
                        cudaStream_t s);
void launch_eas_geometry(const ElemArgs& a, double* geo_out, cudaStream_t s);
void launch_eas_update(const ElemArgs& a, double* alpha, const double* correction, cudaStream_t s);
int eas_geo_stride(int eas_kind);
// one thread per loaded element: slot_elem[s] is the element, faces face_ptr[s]..face_ptr[s+1]-1
void launch_traction_loads(const double* X, const int32_t* conn, int n_elems, int n_slots, const int32_t* slot_elem,
                           const int32_t* face_ptr, const int32_t* face_local, const double* traction, double* trac,
                           cudaStream_t s);

// sparse.cu
void launch_node_elem_count(const int32_t* conn, int n_elems, int n_nodes, int32_t* cnt, cudaStream_t s);
void launch_exclusive_scan(const int32_t* in, int32_t* out, int n, cudaStream_t s);  // out has n+1 entries
void launch_node_elem_fill(const int32_t* conn, int n_elems, const int32_t* ptr, int32_t* cursor, int32_t* elems,
                           int n_nodes, cudaStream_t s);
void launch_row_build(const int32_t* conn, int n_elems, int n_nodes, const int32_t* ne_ptr, const int32_t* ne_elems,
                      const int32_t* row_ptr, int32_t* cnt_or_col, bool fill, int* status, cudaStream_t s);
void launch_slot_map(const int32_t* conn, int n_elems, const int32_t* row_ptr, const int32_t* col, int32_t* slot,
                     int32_t* diag, int n_nodes, cudaStream_t s);
void launch_bsr_reset(void* val, bool fp32, int64_t n_blocks, const int32_t* diag, const uint8_t* node_fixed,
                      int n_nodes, cudaStream_t s);
void launch_vector_finish(double* R, const uint8_t* node_fixed, int n_nodes, const int32_t* pl_dof,
                          const double* pl_val, int n_pl, double load_factor, cudaStream_t s);
void launch_norm2(const double* x, int64_t n, double* partials, double* out, cudaStream_t s);

// solver.cu -- block-Jacobi preconditioned CG
// device scalar slots of the CG (doubles)
enum PcgScal : int {
  kBB = 0,     // |b|^2
  kTol2 = 1,   // rtol^2 |b|^2
  kRz = 2,     // r.z by iteration parity: 2, 3
  kDone = 4,   // 0 running, 1 converged, 2 iteration limit, 3 breakdown
  kIters = 5,  // iteration count by parity: 5, 6
  kRR = 7,     // last |r|^2
  kMaxIt = 8,
  kNScal = 16
};
struct PcgWork {
  int n_rows = 0;     // block rows
  bool fp32 = false;
  void* x = nullptr;
  void* r = nullptr;
  void* z = nullptr;
  void* p0 = nullptr;
  void* p1 = nullptr;
  void* q = nullptr;
  void* minv = nullptr;        // 9 per block row
  double* part_a = nullptr;    // partials written by the SpMV kernel
  double* part_b = nullptr;    // partials written by the update kernel (2 per block: rz, rr)
  double* scal = nullptr;      // device scalars, see solver.cu
  int grid = 0;                // fixed grid (multiple of the SM count) for the partial-producing kernels
};
void launch_block_jacobi(const Bsr& A, bool fp32, void* minv, bool point_jacobi, cudaStream_t s);
void launch_pcg_init(const Bsr& A, PcgWork& w, const double* b, double rtol, int max_iter, cudaStream_t s);
void launch_pcg_iteration(const Bsr& A, PcgWork& w, int parity, cudaStream_t s);
void launch_pcg_spmv(const Bsr& A, PcgWork& w, int parity, cudaStream_t s);
void launch_pcg_update(const Bsr& A, PcgWork& w, int parity, cudaStream_t s);
void launch_pcg_result(const PcgWork& w, double* x_out, double scale, cudaStream_t s);
void launch_residual64(const Bsr& A, bool fp32, const double* x, const double* b, double* r, cudaStream_t s);

// noalloc.cu -- fixed device scratch of the allocation-free CG solve
constexpr int kNoAllocMaxRows = 32768;  // block rows (nodes) = 98304 dofs
constexpr int kNoAllocMaxGrid = 1216;   // blocks of the partial-producing CG kernels
size_t noalloc_scratch_bytes();
cudaError_t noalloc_scratch_address(void** out);  // device address on the current device (cached per device)
void noalloc_workset(void* base, int n_rows, bool fp32, int grid, PcgWork& w);
void launch_axpy64(double* y, const double* x, double a, int64_t n, cudaStream_t s);
void launch_scale64(double* y, const double* x, double a, int64_t n, cudaStream_t s);
void launch_spmv64(const Bsr& A, bool fp32, const double* x, double* y, cudaStream_t s);

}  // namespace ikr
