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
  kElemBlocks = 16, // with kWantK: write each element's 36 distinct 3x3 blocks to ElemArgs::blk (gathered afterwards)
};

enum StatusBits : int {
  kStatusNonPositiveDetC = 1,  // checkPositiveOrAbort (materialhelpers.hh:119-126) on the device
  kStatusNonFinite = 2,
  kStatusSingularD = 4,        // EAS D matrix could not be factorised
  kStatusPatternOverflow = 8,  // a node couples with more nodes than the pattern builder supports
  kStatusMaterialDomain = 16,  // a material evaluated outside its domain (Gent: Jm <= W1 - 3, gent.hh checkJm)
};

// Hyperelastic<Deviatoric<DF>, Volumetric<VF>> (materials/hyperelastic/): the deviatoric function and its
// parameters, the volumetric function VF0..VF12 and its factor K (hyperelastic.cuh evaluates them)
enum HyperDev : int {
  kDevNone = 0,
  kDevBlatzKo = 1,           // mu[0]
  kDevOgdenTotal = 2,        // mu[0..n), alpha[0..n)
  kDevOgdenDeviatoric = 3,   // mu[0..n), alpha[0..n)
  kDevInvariantBased = 4,    // mu[0..n), p[0..n), q[0..n)
  kDevArrudaBoyce = 5,       // mu[0], param = lambdaM
  kDevGent = 6,              // mu[0], param = Jm
};
constexpr int kHyperMaxTerms = 4;
struct HyperParams {
  int dev = 0, n = 0;
  double mu[kHyperMaxTerms] = {0, 0, 0, 0}, alpha[kHyperMaxTerms] = {0, 0, 0, 0};
  int p[kHyperMaxTerms] = {0, 0, 0, 0}, q[kHyperMaxTerms] = {0, 0, 0, 0};
  double param = 0;
  int vol = 0;
  double K = 0, beta = 0;
};

struct ElemArgs {
  int n_nodes = 0, n_elems = 0;
  const double* X = nullptr;     // coordinates, n_nodes x 3
  const int32_t* conn = nullptr; // corner-major: conn[v * n_elems + e]
  double lam = 0, mu = 0;        // Lame parameters
  int material = 0;              // 0 NeoHooke, 1 StVenantKirchhoff, 2 BlatzKo, 3 hyperelastic framework (hyper)
  HyperParams hyper;
  const double* lam_e = nullptr;  // per-element Lame parameters (nullptr: lam / mu for every element)
  const double* mu_e = nullptr;
  const double* u = nullptr;     // displacement, 3 * n_nodes (FP64)
  const uint8_t* node_fixed = nullptr;  // per node 3-bit Dirichlet mask; nullptr = no masking (Raw)
  // dead tractions: trac_idx[e] >= 0 indexes 24 values of sum_faces N_I t dA at load factor 1
  const int32_t* trac_idx = nullptr;
  const double* trac = nullptr;
  // loads given as functions of (X, lambda): 24 values per element, sum_q N_I b w detJ + sum_faces N_I t dA at the
  // current load factor (not scaled by it); nullptr = none
  const double* ext = nullptr;
  double load_factor = 0;
  const double* load_factor_dev = nullptr;  // when set, the load factor is read here (launches captured in a graph)
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
  int epb = 32;                    // displacement element kernel: elements per block (16, 32 or 64)
  // kElemBlocks: 36 blocks x 9 entries per element, element-major; block p = 8 d + I holds (I, I + d mod 8) for
  // d = 0..3, block 32 + I holds (I, I + 4) for I = 0..3 (tangent_block_code maps a corner pair to its block)
  void* blk = nullptr;
  // batched solves: the status of an element goes to its instance, inst_status[elem_inst[e]], instead
  const int32_t* elem_inst = nullptr;
  int* inst_status = nullptr;
};

// The tangent's 3x3 blocks are stored sliced-ELL: block rows (nodes) are grouped in slices of 32; slice s
// spans the block columns [slice_off[s], slice_off[s+1]) (its longest row), rows shorter than that are
// padded with zero blocks whose column is the row itself.  Block k of row r = 32 s + l has the id
// b = (slice_off[s] + k) * 32 + l; its column is col_sell[b] and entry e = 3i + j (row-major in the block)
// sits at val[block_entry(b, e)] = (b >> 5) * 288 + e * 32 + (b & 31), so for a fixed (k, e) the 32 rows of a
// slice are 32 consecutive values.  The sorted CSR view (row_ptr / col) describes the pattern itself.
__host__ __device__ __forceinline__ int64_t block_entry(int64_t b, int e) { return (b >> 5) * 288 + e * 32 + (b & 31); }

struct Bsr {
  int n_rows = 0;                   // block rows = nodes
  int64_t n_blocks = 0;             // blocks of the pattern (without padding)
  int n_slices = 0;
  int64_t n_padded = 0;             // 32 * slice_off[n_slices]
  const int32_t* row_ptr = nullptr; // CSR view of the pattern
  const int32_t* col = nullptr;
  const int32_t* slice_off = nullptr;
  const int32_t* col_sell = nullptr;
  const int32_t* diag = nullptr;    // block id of the diagonal block of each row
  const void* val = nullptr;        // float or double, 9 * n_padded
};

// element.cu
void launch_disp_element(const ElemArgs& a, int mode, bool fp32_tangent, const int32_t* list, int n_list, int e_base,
                         cudaStream_t s);
void launch_eas_element(const ElemArgs& a, int mode, bool fp32_tangent, const int32_t* list, int n_list, int e_base,
                        cudaStream_t s);
// element_eas_hyper.cu: the same for material 3 (the hyperelastic framework)
void launch_eas_element_hyper(const ElemArgs& a, int mode, bool fp32_tangent, const int32_t* list, int n_list,
                              int e_base, cudaStream_t s);
// the element's stored block of corner pair (I, J) for kElemBlocks, as (index p << 1) | transposed
__host__ __device__ __forceinline__ int tangent_block_code(int I, int J) {
  const int d = (J - I) & 7;
  if (d < 4) return (8 * d + I) << 1;
  if (d == 4) return I < 4 ? ((32 + I) << 1) : (((32 + J) << 1) | 1);
  return ((8 * (8 - d) + J) << 1) | 1;  // (J, I) is stored, transposed
}
constexpr int kElemBlockCount = 36;
// gathered FP32 tangent assembly (element.cu): inverse of the element-to-block map -- for every padded block id the
// element blocks that add to it, (e * 36 + p) << 1 | transposed, ascending -- and the gather that sums them, applies
// the Full Dirichlet treatment (node_fixed; unit diagonal) and writes every entry of every slice once
void launch_tangent_inverse_count(const int32_t* slot, int n_elems, int32_t* cnt, cudaStream_t s);
void launch_tangent_inverse_fill(const int32_t* slot, int n_elems, const int32_t* ptr, int32_t* cursor, int32_t* inv,
                                 int64_t n_padded, cudaStream_t s);
void launch_tangent_gather(const Bsr& A, const int32_t* gslice, const int32_t* inv_ptr, const int32_t* inv,
                           const float* blk, const uint8_t* node_fixed, float* val, cudaStream_t s);
// displacement-based NeoHooke FP32 tangent by block rows (thread per node row, no colouring; element.cu);
// ne_ptr / ne_elems: the elements of every node in ascending order
void launch_row_tangent(const ElemArgs& a, const int32_t* ne_ptr, const int32_t* ne_elems, cudaStream_t s);
void launch_eas_geometry(const ElemArgs& a, double* geo_out, cudaStream_t s);
void launch_eas_update(const ElemArgs& a, double* alpha, const double* correction, cudaStream_t s);
int eas_geo_stride(int eas_kind);
// stresses of elements [e0, e0 + count) at local points (3 per element, or 3 for all): type 0 PK2, 1 Kirchhoff,
// 2 Cauchy; 6 Voigt values per element
void launch_stress_at(const ElemArgs& a, int e0, int count, const double* xi, bool xi_per_elem, int type, double* out,
                      cudaStream_t s);
// the same for EAS elements with their stored alpha (element_eas.cu)
void launch_eas_stress_at(const ElemArgs& a, int e0, int count, const double* xi, bool xi_per_elem, int type,
                          double* out, cudaStream_t s);
// one thread per loaded element: slot_elem[s] is the element, faces face_ptr[s]..face_ptr[s+1]-1
void launch_traction_loads(const double* X, const int32_t* conn, int n_elems, int n_slots, const int32_t* slot_elem,
                           const int32_t* face_ptr, const int32_t* face_local, const double* traction, double* trac,
                           cudaStream_t s);
// global positions of the 8 Gauss points of every element, q = x + 2y + 4z (xi_d = lo for bit 0, hi for bit 1):
// xgp[(8 e + q) * 3 + c]
void launch_gauss_points(const double* X, const int32_t* conn, int n_elems, double* xgp, cudaStream_t s);
// VolumeLoad (loads/volume.hh:86-106): ext[24 e + 3 v + c] += sum_q N_v(xi_q) b[(8 e + q) * 3 + c] w_q detJ(xi_q)
void launch_volume_loads(const double* X, const int32_t* conn, int n_elems, const double* b, double* ext,
                         cudaStream_t s);
// ext[24 slot_elem[k] + i] += vals[24 k + i] (each element in at most one slot)
void launch_add_slot_loads(const int32_t* slot_elem, int n_slots, const double* vals, double* ext, cudaStream_t s);

// sparse.cu
void launch_node_elem_count(const int32_t* conn, int n_elems, int n_nodes, int32_t* cnt, cudaStream_t s);
void launch_exclusive_scan(const int32_t* in, int32_t* out, int n, cudaStream_t s);  // out has n+1 entries
void launch_node_elem_fill(const int32_t* conn, int n_elems, const int32_t* ptr, int32_t* cursor, int32_t* elems,
                           int n_nodes, cudaStream_t s);
void launch_row_build(const int32_t* conn, int n_elems, int n_nodes, const int32_t* ne_ptr, const int32_t* ne_elems,
                      const int32_t* row_ptr, int32_t* cnt_or_col, bool fill, int* status, cudaStream_t s);
// per slice of 32 rows: the longest row (slice_len has (n_nodes + 31) / 32 entries)
void launch_slice_lengths(const int32_t* row_ptr, int n_nodes, int32_t* slice_len, cudaStream_t s);
// column index of every (padded) block: the CSR columns, then the row itself for padding
void launch_sell_fill(const int32_t* row_ptr, const int32_t* col, const int32_t* slice_off, int n_nodes,
                      int32_t* col_sell, cudaStream_t s);
// element-to-block map (block ids) and the diagonal block of each row
void launch_slot_map(const int32_t* conn, int n_elems, const int32_t* row_ptr, const int32_t* col,
                     const int32_t* slice_off, int32_t* slot, int32_t* diag, int n_nodes, cudaStream_t s);
void launch_bsr_reset(void* val, bool fp32, int64_t n_padded, const int32_t* diag, const uint8_t* node_fixed,
                      int n_nodes, cudaStream_t s);
// val[idx[k]] += v[k] for n unique value indices (the assembler manipulator's matrix entries)
void launch_add_entries(void* val, bool fp32, const int64_t* idx, const double* v, int n, cudaStream_t s);
void launch_vector_finish(double* R, const uint8_t* node_fixed, int n_nodes, const int32_t* pl_dof,
                          const double* pl_val, int n_pl, double load_factor, cudaStream_t s,
                          const double* load_factor_dev = nullptr);
void launch_norm2(const double* x, int64_t n, double* partials, double* out, cudaStream_t s);
// inhomogeneous Dirichlet values: u[i] = lambda rate[i] where nonzero; R += step F on the free dofs
void launch_idbc_sync(double* u, const double* rate, double lambda, int64_t n, cudaStream_t s);
void launch_idbc_force(double* R, const double* F, const uint8_t* node_fixed, double step, int64_t n, cudaStream_t s);
// *out = sum over entries with lambda_new * rate != 0 of (lambda_new * rate - u)^2 (two launches)
void launch_idbc_delta_sq(const double* u, const double* rate, double lambda_new, int64_t n, double* partials,
                          double* out, cudaStream_t s);
void launch_mul64(double* y, const double* x, const double* m, int64_t n, cudaStream_t s);  // y = x * m
void launch_dot(const double* x, const double* y, int64_t n, double* partials, double* out, cudaStream_t s);

// solver.cu -- block-Jacobi preconditioned CG
// device scalar slots of the CG (doubles)
enum PcgScal : int {
  kBB = 0,      // |b|^2
  kTol2 = 1,    // rtol^2 |b|^2
  kRz = 2,      // r.z of the current iterate
  kDone = 4,    // 0 running, 1 converged, 2 iteration limit, 3 breakdown
  kIters = 5,   // completed iterations
  kRR = 7,      // last |r|^2
  kMaxIt = 8,
  kAlpha = 9,
  kBeta = 10,
  kRzF = 11,    // with a coarse correction: r.D^-1 r of the current iterate (coarse.cu completes r.z)
  kTicket = 12, // slots 12-14 hold six 32-bit tickets of the last-block reductions (the fifth: coarse.cu)
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
  int sms = 0;                 // SM count of the device
  int spmv_kind = 0;           // 0: direct loads (solver.cu); 1 + v: staged variant v (spmv_staged.cu);
                               // 1 + staged variants + v: persistent CG variant v (cg_persistent.cu)
  int64_t keep_g = 0;          // staged: matrix blocks [0, keep_g) are copied with an L2 evict_last policy
  // one-reduction persistent CG (variants 4 and 5 of cg_persistent.cu): a second z buffer, the two buffers of
  // w = M^-1 q and 16 partials per grid CTA
  void* z2 = nullptr;
  void* w0 = nullptr;
  void* w1 = nullptr;
  double* part_c = nullptr;
  // 1: a coarse correction (coarse.cu) follows the init and update kernels, which then leave r.D^-1 r in kRzF
  // and let it set r.z and beta
  int coarse = 0;
  // persistent CG: polls of a grid barrier before it gives up (0: the default), and a test switch with which CTA 0
  // withholds its first barrier arrival (every CTA's first wait then runs out and the solve reports the timeout)
  int barrier_polls = 0;
  int withhold_first_arrival = 0;
  // when set, the init kernel reads the relative tolerance from this device scalar instead of its argument (a solve
  // captured in a CUDA graph whose tolerance changes from launch to launch)
  const double* rtol_dev = nullptr;
  // persistent CG with the coarse correction fused in (cg_coarse.cu): 2 (n_c + 2) partials per CTA for up to
  // coarse_part_ctas CTAs
  double* coarse_part = nullptr;
  int coarse_part_ctas = 0;
};
void launch_block_jacobi(const Bsr& A, bool fp32, void* minv, bool point_jacobi, cudaStream_t s);
void launch_pcg_init(const Bsr& A, PcgWork& w, const double* b, double rtol, int max_iter, cudaStream_t s);
void launch_pcg_iteration(const Bsr& A, PcgWork& w, int parity, cudaStream_t s);
void launch_pcg_spmv(const Bsr& A, PcgWork& w, int parity, cudaStream_t s);
void launch_pcg_update(const Bsr& A, PcgWork& w, int parity, cudaStream_t s);
void launch_pcg_result(const PcgWork& w, double* x_out, double scale, cudaStream_t s);
void launch_residual64(const Bsr& A, bool fp32, const double* x, const double* b, double* r, cudaStream_t s);
// spmv_staged.cu -- the CG SpMV with bulk-copy staging of the matrix (variants differ in chunk size, pipeline
// depth and warps per CTA); same inputs, outputs and scalars as launch_pcg_spmv
int spmv_staged_variants();
const char* spmv_staged_name(bool fp32, int variant);
void launch_pcg_spmv_staged(const Bsr& A, PcgWork& w, int variant, const void* pold, void* pnew, cudaStream_t s);
void launch_fill64(double* y, double v, int64_t n, cudaStream_t s);
// cg_persistent.cu -- the whole CG solve (after launch_pcg_init) in one cooperative launch; the result in w.x
// and the scalars as after the two-kernel iterations
// coarse.cu -- coarse correction of the block-Jacobi CG (additive two-level preconditioner with the rigid-body
// modes of node aggregates); device data built by the linear solver (host_internal.h)
constexpr int kCoarseMaxDofs = 768;  // six modes per aggregate, at most 128 aggregates
struct Coarse {
  int n_rows = 0, n_agg = 0, n_c = 0, n_chunks = 0;
  const float4* y4 = nullptr;          // per node: offset from its aggregate's centroid, agg id | free mask << 24
  const int32_t* nodes = nullptr;      // node ids grouped by aggregate
  const int32_t* chunk_off = nullptr;  // nodes of chunk k: nodes[chunk_off[k] .. chunk_off[k+1])
  const int32_t* agg_chunk = nullptr;  // chunks of aggregate a: [agg_chunk[a], agg_chunk[a+1])
  const int32_t* agg_colour = nullptr; // colour of every aggregate (distance-2 colouring)
  double* rpart = nullptr;             // 6 per chunk: P^T r of the chunk
  const void* ainv = nullptr;          // A_c^-1, n_c x n_c in the CG's type
  void* e = nullptr;                   // A_c^-1 P^T r, n_c in the CG's type
};
void launch_coarse_correction(const Coarse& C, const PcgWork& w, bool init, cudaStream_t s);
// cg_coarse.cu: the persistent block-Jacobi CG with the coarse correction in the same cooperative launch (after
// launch_pcg_init with w.coarse = 1); at most kCoarseFusedMaxDofs coarse dofs (64 slabs)
constexpr int kCoarseFusedMaxDofs = 384;
int pcg_coarse_variants();
bool pcg_coarse_eligible(const Bsr& A, PcgWork& w, const Coarse& C, int variant);
cudaError_t launch_pcg_coarse(const Bsr& A, PcgWork& w, const Coarse& C, int variant, cudaStream_t s);
void launch_coarse_probe(const Coarse& C, int colour, double* V, cudaStream_t s);
void launch_coarse_galerkin(const Coarse& C, const double* W, double* part, cudaStream_t s);
int pcg_persistent_variants();
bool pcg_persistent_eligible(const Bsr& A, PcgWork& w, int variant);
cudaError_t launch_pcg_persistent(const Bsr& A, PcgWork& w, int variant, cudaStream_t s);
// the same solve for two right-hand sides with one matrix stream per iteration (w1 shares w0's matrix,
// preconditioner, grid and L2 policy); part_a / part_b hold 4 and 8 doubles per grid CTA
bool pcg_persistent2_eligible(const Bsr& A, PcgWork& w0, PcgWork& w1, int variant);
cudaError_t launch_pcg_persistent2(const Bsr& A, PcgWork& w0, PcgWork& w1, int variant, double* part_a,
                                   double* part_b, cudaStream_t s);

// batched.cu -- independent instances (disjoint contiguous node ranges) of one element set
// One launch continues (first_launch: starts) the block-Jacobi PCG of the instances its CTAs serve, for at most
// `chunk` iterations: instance i is served by the CTAs cta_first .. + cta_size - 1 listed per CTA (cta_inst,
// cta_first, cta_size; groups contiguous, at most 256 CTAs).  variant 0: a thread loops over rows with the state in
// the work arrays; 1: one row per thread (rows per CTA <= batched_pcg_rows_per_cta), the row's state in registers;
// 2 / 3 / 5: four / eight / sixteen threads per row, the CTA's matrix blocks in shared memory (rows per CTA <=
// batched_pcg_rows_per_cta, blocks per row <= batched_pcg_max_width).  xw..qw are node-padded work vectors of the
// whole set, rtol per instance; st (4 doubles), its and flag per instance carry the solve between launches (flag 0
// running, 1 finished, 2 breakdown, -1 a wait gave up); x_out gets an instance's correction when it finishes.  part
// holds 4 doubles per CTA, counters one per instance.  capacity = co-resident CTAs of the variant on the device.
int batched_pcg_capacity(bool fp32, int variant, int sms);
int batched_pcg_rows_per_cta(int variant);
int batched_pcg_max_width(int variant);
cudaError_t launch_batched_pcg(const Bsr& A, bool fp32, int variant, const void* minv, const double* b, double* x_out,
                               int n_cta, const int32_t* node_off, const int32_t* cta_inst, const int32_t* cta_first,
                               const int32_t* cta_size, void* xw, void* rw, void* zw, void* p0, void* p1, void* qw,
                               const double* rtol, int max_iter, int chunk, int first_launch, double* st, int32_t* its,
                               int32_t* flag, double* relres, double* part, unsigned int* counters, int n_inst,
                               bool cooperative, cudaStream_t s);
// FP32 only: one instance per cluster of 16 CTAs (cluster_inst per cluster), at most batched_cluster_rows() rows and
// batched_cluster_width() blocks per row; vectors and sums through distributed shared memory; same state protocol
// (st, its, flag, x_out).  capacity: clusters co-resident on the device (more run in waves; clusters never wait on
// each other).
int batched_cluster_rows();
int batched_cluster_width();
int batched_cluster_capacity();
cudaError_t launch_batched_pcg_cluster(const Bsr& A, const void* minv, const double* b, double* x_out, int n_clusters,
                                       const int32_t* node_off, const int32_t* cluster_inst, void* xw, void* rw,
                                       void* zw, void* p0, void* p1, const double* rtol, int max_iter, int chunk,
                                       int first_launch, double* st, int32_t* its, int32_t* flag, double* relres,
                                       cudaStream_t s);
void launch_instance_norms(const double* x, int n_inst, const int32_t* node_off, double* out, cudaStream_t s);
// u = u_old + step[i] corr on the dofs of instance i (instances with step 1 untouched)
void launch_instance_step(double* u, const double* u_old, const double* corr, int n_inst, const int32_t* node_off,
                          const double* step, cudaStream_t s);

// mlp.cu -- dense network (BF16 weights, FP32 accumulation) and POD helpers of the learned predictor
// C[M x N] = alpha op(A) op(B) + beta C (row-major; op = transpose when trans_*; A / B FP32 or BF16)
void launch_gemm(int M, int N, int K, const void* A, bool a_bf16, bool trans_a, int lda, const void* B, bool b_bf16,
                 bool trans_b, int ldb, float* C, int ldc, float alpha, float beta, cudaStream_t s);
void launch_bias_act(float* Z, float* Y, const float* bias, int B, int out, bool gelu, cudaStream_t s);
void launch_gelu_backward(float* dZ, const float* Z, int64_t n, cudaStream_t s);
void launch_colsum(const float* dZ, float* g, int B, int out, cudaStream_t s);
int launch_mse(const float* Y, const float* T, float* dY, int64_t n, float scale, float* part, cudaStream_t s);
void launch_adam(float* p, const float* g, float* m, float* v, void* wb, const int64_t* bf_index, int64_t n, float lr,
                 float b1, float b2, float eps, int step, cudaStream_t s);
void launch_to_bf16(const float* p, void* wb, const int64_t* bf_index, int64_t n, cudaStream_t s);
void launch_gather_rows(const float* X, const int32_t* idx, float* out, int rows, int cols, cudaStream_t s);
void launch_gram64(const float* Y, int64_t n, int l, double* G, cudaStream_t s);
void launch_randn(float* out, int64_t n, uint64_t seed, cudaStream_t s);
void launch_diff_to_f32(const double* a, const double* b, float* out, int64_t n, cudaStream_t s);
void launch_add_f32(double* u, const float* d, int64_t n, cudaStream_t s);
void launch_add_scaled_f32(double* u, const float* d, double a, int64_t n, cudaStream_t s);  // u += a d
void launch_base_plus_scaled(double* u, const double* u0, const float* d, double sc, int64_t n, cudaStream_t s);

// krylov.cu -- vector kernels of the FP64 outer Krylov solve (krylov.cpp): V holds m vectors of length n one after
// the other (leading dimension ld)
constexpr int kKrylovMaxBasis = 64;
int multi_dot_blocks(int64_t n);
// out[i] = V[i] . w for i < m; part holds m * multi_dot_blocks(n) doubles
void launch_multi_dot(const double* V, int64_t ld, int m, const double* w, int64_t n, double* part, double* out,
                      cudaStream_t s);
// y += sign * sum_{i < m} c[i] V[i], c on the device, m <= kKrylovMaxBasis
void launch_multi_axpy(double* y, const double* V, int64_t ld, int m, const double* c, double sign, int64_t n,
                       cudaStream_t s);
// out = FP32 rounding of in (n values)
void launch_round_values(const double* in, float* out, int64_t n, cudaStream_t s);

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
