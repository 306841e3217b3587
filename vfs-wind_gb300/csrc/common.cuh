// common.cuh -- shared device helpers of the GB300 pressure-Poisson library.
//
// Two layouts are used on the device:
//   * the DA layout of the reference (Source/init.c:141-161): mx*my*mz points,
//     i fastest, index 0 and m-1 the boundary layer; used for the arrays a
//     caller hands over (coordinates, metrics, nvert, Ucont, phi, p);
//   * the interior ("box") layout nx*ny*nz (nx = mx-2), used by every solver
//     vector and operator plane so that no solver kernel touches ghost cells.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vfs {

// DA-layout grid with merged periodic flags (i_periodic || ii_periodic, ...).
struct Grid {
  int mx, my, mz;
  int px, py, pz;
  __host__ __device__ size_t n() const { return (size_t)mx * my * mz; }
  __host__ __device__ size_t at(int i, int j, int k) const {
    return ((size_t)k * my + j) * mx + i;
  }
  // Ghost remap of the reference (e.g. Source/poisson.c:1143-1161): index 0
  // and m-1 of a periodic direction stand for cells m-2 and 1.
  __host__ __device__ int remap(int i, int j, int k, int &a, int &b, int &c, int &fi, int &fj,
                                int &fk) const {
    a = i; b = j; c = k; fi = fj = fk = 0;
    if (px) { if (i == 0) { a = mx - 2; fi = 1; } else if (i == mx - 1) { a = 1; fi = 1; } }
    if (py) { if (j == 0) { b = my - 2; fj = 1; } else if (j == my - 1) { b = 1; fj = 1; } }
    if (pz) { if (k == 0) { c = mz - 2; fk = 1; } else if (k == mz - 1) { c = 1; fk = 1; } }
    return fi | fj | fk;
  }
};

// Interior box of one multigrid level.
struct Box {
  int nx, ny, nz;
  int px, py, pz;
  __host__ __device__ size_t n() const { return (size_t)nx * ny * nz; }
  __host__ __device__ size_t at(int i, int j, int k) const {
    return ((size_t)k * ny + j) * nx + i;
  }
};

// (i, j, k) of box-layout cell c, in 32-bit arithmetic (a box holds fewer
// than 2^32 cells; 64-bit integer division costs a software routine).
__device__ __forceinline__ void box_ijk(const Box &b, size_t c, int &i, int &j, int &k) {
  const uint32_t u = (uint32_t)c, nx = (uint32_t)b.nx, ny = (uint32_t)b.ny;
  const uint32_t row = u / nx, kk = row / ny;
  i = (int)(u - row * nx);
  j = (int)(row - kk * ny);
  k = (int)kk;
}

// |div(Ucont) aj| of DA cell (i, j, k), zero when the cell or one of its six
// face neighbours is blanked (nvert sum > 0.1), exactly as Divergence
// computes it (Source/main.c:956-958).  Shared by the handle's divergence
// kernel and the no-allocation entry point; both translation units are
// compiled without FMA contraction.
__device__ __forceinline__ double divergence_cell(const Grid &g, const double *__restrict__ nvert,
                                                  const double *__restrict__ ucont, const double *__restrict__ aj,
                                                  int i, int j, int k) {
#define VFS_U(a, b, c, q) ucont[g.at(a, b, c) * 3 + (q)]
#define VFS_NV(a, b, c) nvert[g.at(a, b, c)]
  double v = fabs((VFS_U(i, j, k, 0) - VFS_U(i - 1, j, k, 0) + VFS_U(i, j, k, 1) - VFS_U(i, j - 1, k, 1) +
                   VFS_U(i, j, k, 2) - VFS_U(i, j, k - 1, 2)) *
                  aj[g.at(i, j, k)]);
  if (VFS_NV(i, j, k) + VFS_NV(i, j, k + 1) + VFS_NV(i, j, k - 1) + VFS_NV(i, j + 1, k) + VFS_NV(i, j - 1, k) +
          VFS_NV(i + 1, j, k) + VFS_NV(i - 1, j, k) >
      0.1)
    v = 0.;
#undef VFS_U
#undef VFS_NV
  return v;
}

// Programmatic dependent launch (PTX griddepcontrol, sm_90 and later).  The
// V-cycle's kernels are launched with programmatic stream serialization, so
// a kernel's blocks may start while the previous kernel in the stream is
// still running its last wave.  pdl_trigger lets the next kernel start once
// every block of this one has started; pdl_wait blocks until the previous
// kernel has completed and its writes are visible.  A kernel reads only
// data that no kernel of the V-cycle writes (operator planes, line factors,
// blank flags) before pdl_wait, and writes nothing before it.  Every
// thread of such a kernel executes pdl_wait, so a kernel completes only
// after its predecessor has, and the chain stays ordered.  Launched without
// the attribute, both are no-ops.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Cells of a j-line handled by one thread of the line smoother; a line of
// ny cells uses ceil(ny / kLineChunk) threads per column.
constexpr int kLineChunk = 8;
// Threads per block the line kernels are compiled for (launch bounds): a
// block holds TI columns of ceil(ny / kLineChunk) chunks each.
constexpr int kLineMaxThreads = 384;

// Level-set context of the operator and the projection (poisson.c
// levelset branches): density and level-set field at the cells (DA layout
// of the grid in use), on = levelset, bc3/bc4/bc5 = bctype[3], [4], [5].
struct LevelSet {
  const double *rho = nullptr, *level = nullptr;
  int on = 0, bc3 = 0, bc4 = 0, bc5 = 0;
};

// Parity-split row layout of the multigrid level operators and line
// factors: within each (j, k) row the even-i cells come first, then the odd
// ones, so that the columns of one checkerboard colour ((i + k) parity) are
// contiguous and coalesce.  Vectors (x, b, r) keep the natural layout, except
// the finest FP32 level's x and right-hand side under the checkerboard
// smoother, which use this layout too (whole sectors per colour).
__host__ __device__ inline int split_pos(int i, int nx) { return (i & 1) ? ((nx + 1) >> 1) + (i >> 1) : (i >> 1); }
__host__ __device__ inline int split_cell(int p, int nx) {
  const int nh = (nx + 1) >> 1;
  return p < nh ? 2 * p : 2 * (p - nh) + 1;
}

// Stencil slot order of the reference's 19-point operator
// (Source/poisson.c:957-975): offsets (di, dj, dk) per slot.
enum { CP = 0, EP, WP, NP, SP, TP, BP, NE, SE, NW, SW, TN, BN, TS, BS, TE, BE, TW, BW, NSLOT };
__host__ __device__ inline void slot_offset(int s, int &di, int &dj, int &dk) {
  const int8_t o[NSLOT][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                              {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {1, -1, 0}, {-1, 1, 0},
                              {-1, -1, 0}, {0, 1, 1},  {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
                              {1, 0, 1},  {1, 0, -1},  {-1, 0, 1}, {-1, 0, -1}};
  di = o[s][0]; dj = o[s][1]; dk = o[s][2];
}

// Neighbour coordinates in a box: periodic wrap, otherwise clamped onto the
// cell itself (its operator coefficient is zero there by construction).
struct Nbr {
  int im, ip, jm, jp, km, kp;
  __device__ Nbr(const Box &b, int i, int j, int k) {
    im = i > 0 ? i - 1 : (b.px ? b.nx - 1 : i);
    ip = i < b.nx - 1 ? i + 1 : (b.px ? 0 : i);
    jm = j > 0 ? j - 1 : (b.py ? b.ny - 1 : j);
    jp = j < b.ny - 1 ? j + 1 : (b.py ? 0 : j);
    km = k > 0 ? k - 1 : (b.pz ? b.nz - 1 : k);
    kp = k < b.nz - 1 ? k + 1 : (b.pz ? 0 : k);
  }
};

// Linear indices of the 19 stencil points of (i,j,k) in slot order (32-bit:
// the library rejects grids whose 19 operator planes reach 2^32 entries).
// SPLIT: the vector is stored in the parity-split row layout (the finest
// FP32 level's x and right-hand side), so each column index i goes through
// split_pos.
template <bool SPLIT>
__device__ inline void stencil_index_t(const Box &b, int i, int j, int k, uint32_t idx[NSLOT]) {
  Nbr q(b, i, j, k);
  const uint32_t nx = b.nx, sl = (uint32_t)b.nx * b.ny;
  const uint32_t r0 = (uint32_t)k * sl, rm = (uint32_t)q.km * sl, rp = (uint32_t)q.kp * sl;
  const uint32_t j0 = (uint32_t)j * nx, jm = (uint32_t)q.jm * nx, jp = (uint32_t)q.jp * nx;
  const uint32_t ci = SPLIT ? split_pos(i, b.nx) : i, ce = SPLIT ? split_pos(q.ip, b.nx) : q.ip,
                 cw = SPLIT ? split_pos(q.im, b.nx) : q.im;
  idx[CP] = r0 + j0 + ci;
  idx[EP] = r0 + j0 + ce;  idx[WP] = r0 + j0 + cw;
  idx[NP] = r0 + jp + ci;  idx[SP] = r0 + jm + ci;
  idx[TP] = rp + j0 + ci;  idx[BP] = rm + j0 + ci;
  idx[NE] = r0 + jp + ce;  idx[SE] = r0 + jm + ce;
  idx[NW] = r0 + jp + cw;  idx[SW] = r0 + jm + cw;
  idx[TN] = rp + jp + ci;  idx[BN] = rm + jp + ci;
  idx[TS] = rp + jm + ci;  idx[BS] = rm + jm + ci;
  idx[TE] = rp + j0 + ce;  idx[BE] = rm + j0 + ce;
  idx[TW] = rp + j0 + cw;  idx[BW] = rm + j0 + cw;
}
__device__ inline void stencil_index(const Box &b, int i, int j, int k, uint32_t idx[NSLOT]) {
  stencil_index_t<false>(b, i, j, k, idx);
}

// ---- deterministic reductions: fixed-shape block trees ----
template <typename T>
__device__ inline T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ inline T warp_max(T v) {
  for (int o = 16; o > 0; o >>= 1) { T w = __shfl_down_sync(0xffffffffu, v, o); v = w > v ? w : v; }
  return v;
}
// Sum over the block; result valid in thread 0.  blockDim.x multiple of 32, <= 1024.
template <typename T>
__device__ inline T block_sum(T v) {
  __shared__ T sh[32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T r = 0;
  if (w == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : (T)0;
    r = warp_sum(r);
  }
  return r;
}
template <typename T>
__device__ inline T block_max(T v) {
  __shared__ T sh[32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T r = 0;
  if (w == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : (T)0;
    r = warp_max(r);
  }
  return r;
}

}  // namespace vfs
