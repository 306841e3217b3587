// noalloc.cu -- the Divergence diagnostic for callers that cannot allocate
// device memory.
//
// vfs_divergence_noalloc computes the same value as vfs_poisson_divergence
// (max |div(Ucont) aj| over interior cells not next to a blanked cell) but
// needs no handle and allocates nothing.  Its scratch -- one partial maximum
// per thread block -- lives in the file-scope device array g_div_scratch
// below, which every GPU that loads this library holds until the process
// exits.  That serves callers that are not allowed to allocate at the point
// where they need the diagnostic: code that runs while a CUDA stream is being
// captured into a graph (cudaMalloc is not a stream operation and is not
// permitted during capture), and host codes that have handed all device
// memory to their own pool allocator, so that a cudaMalloc from inside their
// time-step loop would fail or fragment the pool.
//
// The size limit comes from the scratch: each block reduces at most
// kCellsPerBlock cells and the array holds kMaxBlocks partials, so a grid may
// have at most kMaxBlocks * kCellsPerBlock = 268,435,456 interior cells;
// larger grids are rejected with VFS_EINVAL before anything is launched.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "vfs_poisson.h"

namespace vfs {
void set_last_error(const std::string &msg);  // poisson.cu
}

using namespace vfs;

namespace {

constexpr int kMaxBlocks = 4096;
constexpr int kCellsPerBlock = 65536;
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

// Shared by every call on a device: one call's partials are overwritten by
// the next, so calls that overlap on the GPU (different streams, no ordering
// between them) race on this array.
static __device__ __align__(256) double g_div_scratch[kMaxBlocks];

// Device address of g_div_scratch per device, looked up once per device.
// In host code the name g_div_scratch is only a host-side stand-in; kernels
// must be given this address instead.
void *g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;


// Block b reduces interior cells [b*kCellsPerBlock, (b+1)*kCellsPerBlock)
// into scratch[b].  Every launched block writes its own slot before the
// final kernel reads it, so nothing in the scratch has to start at zero.
__global__ void __launch_bounds__(kThreads) k_div_partial_noalloc(Grid g, Box b, const double *__restrict__ nvert,
                                                                  const double *__restrict__ ucont,
                                                                  const double *__restrict__ aj, double *scratch) {
  const size_t n = b.n();
  const size_t lo = (size_t)blockIdx.x * kCellsPerBlock;
  const size_t hi = lo + kCellsPerBlock < n ? lo + kCellsPerBlock : n;
  double best = 0.;
  for (size_t c = lo + threadIdx.x; c < hi; c += kThreads) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    const double v = divergence_cell(g, nvert, ucont, aj, i, j, k);
    best = v > best ? v : best;
  }
  best = block_max(best);
  if (threadIdx.x == 0) scratch[blockIdx.x] = best;
}

__global__ void k_div_final_noalloc(const double *scratch, int nb, double *out) {
  double m = 0.;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) m = scratch[q] > m ? scratch[q] : m;
  m = block_max(m);
  if (threadIdx.x == 0) *out = m;
}

// True for memory that kernels on device `dev` may read: device memory of
// that device, or managed memory.  Device memory of another GPU is refused
// (without peer access a kernel would fault on it).
bool on_device(const void *p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

int fail(int code, const std::string &m) {
  vfs::set_last_error(m);  // reported by vfs_last_error()
  return code;
}

}  // namespace

extern "C" {

// See include/vfs_poisson.h.  The first call on a device looks up the
// scratch address (cudaGetSymbolAddress); make that first call before any
// stream capture begins.  Launches on `stream` and returns without waiting.
int vfs_divergence_noalloc(const vfs_grid_desc *gd, const double *ucont, const double *nvert, const double *aj,
                           double *maxdiv, void *stream) {
  if (!gd || !ucont || !nvert || !aj || !maxdiv) return fail(VFS_EINVAL, "null argument");
  if (gd->mx < 3 || gd->my < 3 || gd->mz < 3) return fail(VFS_EINVAL, "grid needs at least one interior cell");
  const Box b{gd->mx - 2, gd->my - 2, gd->mz - 2, 0, 0, 0};
  const size_t n = b.n();
  const size_t nb = (n + kCellsPerBlock - 1) / kCellsPerBlock;
  if (nb > (size_t)kMaxBlocks)
    return fail(VFS_EINVAL, "grid has " + std::to_string(n) + " interior cells; vfs_divergence_noalloc handles at most " +
                                std::to_string((size_t)kMaxBlocks * kCellsPerBlock));
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(VFS_ECUDA, "no current CUDA device");
  }
  if (!on_device(ucont, dev) || !on_device(nvert, dev) || !on_device(aj, dev) || !on_device(maxdiv, dev))
    return fail(VFS_EINVAL, "vfs_divergence_noalloc takes device pointers of the current device only");
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      cudaError_t e = cudaGetSymbolAddress(&g_scratch_addr[dev], g_div_scratch);
      if (e != cudaSuccess) {
        cudaGetLastError();
        g_scratch_addr[dev] = nullptr;
        return fail(VFS_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
    }
    scratch = g_scratch_addr[dev];
  }
  const Grid g{gd->mx, gd->my, gd->mz, 0, 0, 0};
  cudaStream_t st = (cudaStream_t)stream;
  k_div_partial_noalloc<<<(unsigned)nb, kThreads, 0, st>>>(g, b, nvert, ucont, aj, (double *)scratch);
  k_div_final_noalloc<<<1, 1024, 0, st>>>((const double *)scratch, (int)nb, maxdiv);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VFS_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
  return VFS_OK;
}

}  // extern "C"
