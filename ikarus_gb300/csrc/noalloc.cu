// Fixed device scratch for the allocation-free CG solve (ikr_linear_solver_solve_noalloc).
//
// Some callers cannot allocate device memory once their run has started: services that size their device
// memory up front and forbid any later cudaMalloc, or hosts whose device allocations must all go through
// their own allocator.  For them the CG work vectors, the block-Jacobi inverse and the reduction slots of
// one solve live in the file-scope array below instead of cudaMalloc'ed buffers.  The array is part of the
// library image: every GPU that loads the library holds these bytes until the process exits.
//
// Host code cannot pass `g_noalloc_scratch` itself to a kernel (on the host it names a host-side shadow,
// not device memory), so the first call on each device looks up the array's device address with
// cudaGetSymbolAddress while that device is current and caches it per device.
#include <cuda_runtime.h>

#include <mutex>

#include "kernels.h"

namespace ikr {

namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }
// FP64 worst case: six node-padded CG vectors (4 values per node), the 3x3 inverse per block row, partials of
// the fixed grid, scalars
constexpr size_t kScratchBytes = 6 * align_up(sizeof(double) * 4 * kNoAllocMaxRows) +
                                 align_up(sizeof(double) * 9 * kNoAllocMaxRows) +
                                 align_up(sizeof(double) * kNoAllocMaxGrid) +
                                 align_up(sizeof(double) * 2 * kNoAllocMaxGrid) + align_up(sizeof(double) * kNScal);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

}  // namespace

size_t noalloc_scratch_bytes() { return kScratchBytes; }

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t noalloc_scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

// Carves the CG work set of n_rows block rows out of the scratch (FP32 or FP64 vectors).
void noalloc_workset(void* base, int n_rows, bool fp32, int grid, PcgWork& w) {
  unsigned char* p = static_cast<unsigned char*>(base);
  const size_t vb = align_up((fp32 ? 4 : 8) * 4 * (size_t)n_rows);
  w = PcgWork{};
  w.n_rows = n_rows;
  w.fp32 = fp32;
  w.grid = grid;
  w.x = p, p += vb;
  w.r = p, p += vb;
  w.z = p, p += vb;
  w.p0 = p, p += vb;
  w.p1 = p, p += vb;
  w.q = p, p += vb;
  w.minv = p, p += align_up((fp32 ? 4 : 8) * 9 * (size_t)n_rows);
  w.part_a = reinterpret_cast<double*>(p), p += align_up(sizeof(double) * kNoAllocMaxGrid);
  w.part_b = reinterpret_cast<double*>(p), p += align_up(sizeof(double) * 2 * kNoAllocMaxGrid);
  w.scal = reinterpret_cast<double*>(p);
}

}  // namespace ikr
