// poisson.cu -- host side of the GB300 pressure-Poisson library: the handle,
// multigrid hierarchy set-up, the FGMRES(m) outer iteration in FP64 with an
// FP32 (or FP64) V-cycle preconditioner, CUDA-graph capture of the V-cycle,
// and the C ABI declared in include/vfs_poisson.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "kernels.cuh"
#include "vfs_poisson.h"

using namespace vfs;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (expr);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      cudaGetLastError();                                                                   \
      return fail(e_ == cudaErrorMemoryAllocation ? VFS_ENOMEM : VFS_ECUDA,                 \
                  std::string(#expr) + ": " + cudaGetErrorString(e_));                      \
    }                                                                                       \
  } while (0)

#define TRY(expr)            \
  do {                       \
    int rc_ = (expr);        \
    if (rc_ != VFS_OK) return rc_; \
  } while (0)

constexpr int kMaxLevels = 24;
constexpr int kRedBlocks = 1216;  // 8 x 152 SMs, fixed for deterministic reductions

// device helper kernels that only the host orchestration needs
__global__ void k_row_scale(size_t n, const uint8_t *rowtype, const double *aj_box, double *scale) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  scale[c] = rowtype[c] == 1 ? aj_box[c] : (rowtype[c] == 2 ? 1.0 : 0.0);
}
// one operator plane from the parity-split row layout to the natural one
__global__ void k_unsplit_plane(Box b, const float *src, float *dst) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= b.n()) return;
  const int i = (int)((uint32_t)c % (uint32_t)b.nx);
  dst[c] = src[c - i + split_pos(i, b.nx)];
}
__global__ void k_mask_box(size_t n, const uint8_t *rowtype, double *x) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n && rowtype[c] == 0) x[c] = 0.;
}
// zero x off the fluid rows: cells without a dof and identity rows (whose
// solution is 0: their right-hand side is 0)
__global__ void k_mask_fluid(size_t n, const uint8_t *rowtype, double *x) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n && rowtype[c] != 1) x[c] = 0.;
}
// ---- learned initial guess: features, training target, composition ----
// sums[0..2]: fluid sums of squares of planes 0..2, sums[3]: fluid count.
__device__ inline void block_add(double v, double *dst) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) atomicAdd(dst, v);
  }
}
// phi_{n-1}, phi_{n-2} (DA) -> extrapolation ex = 2 phi_{n-1} - phi_{n-2}
// and feature planes f0 = phi_{n-1}, f1 = phi_{n-1} - phi_{n-2}, f3 = dof;
// prev = phi_{n-1} in box layout (and in FP32), zero on the rows without an
// equation
__global__ void k_guess_prep(Grid g, Box b, const uint8_t *rt, const double *p1, const double *p2, double *ex,
                             double *prev, float *prev32, float *f0, float *f1, float *f3, double *sums) {
  // the plane sums only set the feature scales: FP32 per thread
  float s0 = 0.f, s1 = 0.f;
  int s3 = 0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < b.n(); c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    const uint8_t t = rt[c];
    const bool d = t == 1;
    const double p = t ? p1[g.at(i, j, k)] : 0.;
    const double a = d ? p : 0., q = d ? p2[g.at(i, j, k)] : 0.;
    const float pf = (float)p, af = d ? pf : 0.f, df = (float)(a - q);
    prev[c] = p;
    prev32[c] = pf;
    ex[c] = 2. * a - q;
    f0[c] = af;
    f1[c] = df;
    f3[c] = d ? 1.f : 0.f;
    s0 = fmaf(af, af, s0);
    s1 = fmaf(df, df, s1);
    s3 += d ? 1 : 0;
  }
  block_add((double)s0, sums);
  block_add((double)s1, sums + 1);
  block_add((double)s3, sums + 3);
}
// f2 = aj * (b - A ex): the extrapolation residual of the aj-scaled system
__global__ void k_guess_f2(size_t n, const uint8_t *rt, const double *aj, const double *r, float *f2, double *sums) {
  double s = 0.;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const double v = rt[c] == 1 ? aj[c] * r[c] : 0.;
    f2[c] = (float)v;
    s += v * v;
  }
  block_add(s, sums + 2);
}
// The two candidates the solver judges: ra = b - A xa in FP64 (stored: the
// residual FGMRES starts from when xa is chosen) and the norm of
// rb = b - A xb estimated in FP32 from the packed level-0 operator (its rows
// are the aj-scaled ones, so each is divided by its row scale) with xb in
// FP32 -- FP64 arithmetic is the scarce pipe and a judgement needs a few
// digits.  ||ra||^2, the estimate of ||rb||^2 and ||b||^2 go to rows 0..2
// of `partial` (grid guess_grid: a thread takes kGuessRows j-rows of one
// column, one partial per block).
constexpr int kGuessRows = 8;
__global__ void __launch_bounds__(128) k_guess_residuals(Box b, const double *__restrict__ A,
                                                          const __half2 *__restrict__ C, const float *__restrict__ D,
                                                          const float *__restrict__ scale, const double *__restrict__ xa,
                                                          const float *__restrict__ xb, const double *__restrict__ rhs,
                                                          double *__restrict__ ra, double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.z;
  double s0 = 0., s2 = 0.;
  float s1 = 0.f;
  const uint32_t n = (uint32_t)b.n();
  for (int j = blockIdx.y * kGuessRows; i < b.nx && j < min(b.ny, (int)(blockIdx.y + 1) * kGuessRows); j++) {
    uint32_t idx[NSLOT];
    stencil_index(b, i, j, k, idx);
    const uint32_t c = idx[CP], cs = c - i + split_pos(i, b.nx);
    double ya = 0.;
#pragma unroll
    for (int q = 0; q < NSLOT; q++) ya = fma(__ldcs(&A[(size_t)q * n + c]), __ldg(&xa[idx[q]]), ya);
    const float xc = __ldg(&xb[c]);
    float t = 0.f;
#pragma unroll
    for (int m = 0; m < 9; m++) {
      const float2 f = __half22float2(__ldcs(&C[(size_t)m * n + cs]));
      t = fmaf(f.x, __ldg(&xb[idx[2 * m + 1]]) - xc, t);
      t = fmaf(f.y, __ldg(&xb[idx[2 * m + 2]]) - xc, t);
    }
    t = fmaf(__half22float2(__ldcs(&C[(size_t)9 * n + cs])).x, xc, t);
    const double bv = rhs[c], va = bv - ya;
    const float sc = scale[c];
    const float vb = sc != 0.f ? (float)bv - __ldcs(&D[cs]) * t / sc : (float)bv;
    ra[c] = va;
    s0 += va * va;
    s1 = fmaf(vb, vb, s1);
    s2 += bv * bv;
  }
  const double t0 = block_sum(s0), t1 = block_sum((double)s1), t2 = block_sum(s2);
  if (threadIdx.x == 0) {
    const size_t nb = (size_t)gridDim.x * gridDim.y * gridDim.z;
    const size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
    partial[blk] = t0;
    partial[nb + blk] = t1;
    partial[2 * nb + blk] = t2;
  }
}
__device__ inline double plane_rms(const double *sums, int q) {
  const double cnt = sums[3] > 1. ? sums[3] : 1.;
  return sqrt(sums[q] / cnt);
}
// planes 0..2 divided by their fluid RMS
__global__ void k_guess_scale(size_t n, float *f, const double *sums) {
  float inv[3];
  for (int q = 0; q < 3; q++) {
    const double r = plane_rms(sums, q);
    inv[q] = r > 0. ? (float)(1. / r) : 0.f;
  }
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    for (int q = 0; q < 3; q++) f[q * n + c] *= inv[q];
}
// training target (phi_n - ex) / rms(f2) and loss weight (dof flag)
__global__ void k_guess_target(Grid g, Box b, const uint8_t *rt, const double *phi, const double *ex,
                               const double *sums, float *tgt, float *wt) {
  const double s2 = plane_rms(sums, 2), inv = s2 > 0. ? 1. / s2 : 0.;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < b.n(); c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    const bool d = rt[c] == 1;
    tgt[c] = d ? (float)((phi[g.at(i, j, k)] - ex[c]) * inv) : 0.f;
    wt[c] = d ? 1.f : 0.f;
  }
}
// 2x2x2 restriction of the fine planes to the network's half-resolution
// grid: planes 0..2 (and the target) average over the dof children, plane
// 3 (and the loss weight) is the dof fraction.
__global__ void k_guess_restrict(Box b, const float *ff, const float *tf, float *fc, float *tc, float *wc) {
  const int cx = b.nx / 2, cy = b.ny / 2, cz = b.nz / 2;
  const size_t nc = (size_t)cx * cy * cz, nf = b.n();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < nc; c += (size_t)gridDim.x * blockDim.x) {
    const uint32_t row = (uint32_t)c / (uint32_t)cx;
    const int I = (int)((uint32_t)c - row * (uint32_t)cx), J = (int)(row % (uint32_t)cy), K = (int)(row / (uint32_t)cy);
    float w = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f, st = 0.f;
    for (int q = 0; q < 8; q++) {
      const size_t f = b.at(2 * I + (q & 1), 2 * J + ((q >> 1) & 1), 2 * K + (q >> 2));
      const float d = ff[3 * nf + f];
      w += d;
      s0 += d * ff[f];
      s1 += d * ff[nf + f];
      s2 += d * ff[2 * nf + f];
      if (tf) st += d * tf[f];
    }
    const float inv = w > 0.f ? 1.f / w : 0.f;
    fc[c] = s0 * inv;
    fc[nc + c] = s1 * inv;
    fc[2 * nc + c] = s2 * inv;
    fc[3 * nc + c] = 0.125f * w;
    if (tc) {
      tc[c] = st * inv;
      wc[c] = 0.125f * w;
    }
  }
}
// cell-centred trilinear prolongation of the half-resolution output
__global__ void k_guess_prolong(Box b, const float *oc, float *of) {
  const int cx = b.nx / 2, cy = b.ny / 2, cz = b.nz / 2;
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < b.n(); f += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, f, i, j, k);
    int I[2] = {i >> 1, (i & 1) ? (i >> 1) + 1 : (i >> 1) - 1};
    int J[2] = {j >> 1, (j & 1) ? (j >> 1) + 1 : (j >> 1) - 1};
    int K[2] = {k >> 1, (k & 1) ? (k >> 1) + 1 : (k >> 1) - 1};
    I[1] = min(max(I[1], 0), cx - 1);
    J[1] = min(max(J[1], 0), cy - 1);
    K[1] = min(max(K[1], 0), cz - 1);
    const float w[2] = {0.75f, 0.25f};
    float s = 0.f;
    for (int q = 0; q < 8; q++) {
      const int a = q & 1, bb = (q >> 1) & 1, c = q >> 2;
      s += w[a] * w[bb] * w[c] * oc[((size_t)K[c] * cy + J[bb]) * cx + I[a]];
    }
    of[f] = s;
  }
}
// one pass of the binomial filter (1/4, 1/2, 1/4, clamped at the box
// faces) along direction `dir` (0 x, 1 y, 2 z; -1 copies); `mask` (may be
// null) zeroes the output off the dofs
__global__ void k_guess_smooth(Box b, const float *in, float *out, int dir, const uint8_t *mask) {
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < b.n(); f += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, f, i, j, k);
    size_t m = f, p = f;
    if (dir < 0) {
    } else if (dir == 0) {
      m = i > 0 ? f - 1 : f;
      p = i < b.nx - 1 ? f + 1 : f;
    } else if (dir == 1) {
      m = j > 0 ? f - b.nx : f;
      p = j < b.ny - 1 ? f + b.nx : f;
    } else {
      const size_t sl = (size_t)b.nx * b.ny;
      m = k > 0 ? f - sl : f;
      p = k < b.nz - 1 ? f + sl : f;
    }
    const float v = dir < 0 ? in[f] : 0.25f * in[m] + 0.5f * in[f] + 0.25f * in[p];
    out[f] = (mask && mask[f] != 1) ? 0.f : v;
  }
}
// One pass of the 27-point binomial filter (the tensor product of
// (1/4, 1/2, 1/4) along x, y and z, clamped at the box faces); `mask` (may
// be null) zeroes the output off the dofs.
__global__ void __launch_bounds__(128) k_guess_smooth3(Box b, const float *__restrict__ in, float *__restrict__ out,
                                                        const uint8_t *__restrict__ mask) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= b.nx) return;
  const int xs[3] = {max(i - 1, 0), i, min(i + 1, b.nx - 1)};
  const int ys[3] = {max(j - 1, 0), j, min(j + 1, b.ny - 1)};
  const int zs[3] = {max(k - 1, 0), k, min(k + 1, b.nz - 1)};
  const float w[3] = {0.25f, 0.5f, 0.25f};
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    float sy = 0.f;
#pragma unroll
    for (int bb = 0; bb < 3; bb++) {
      const float *row = in + ((size_t)zs[c] * b.ny + ys[bb]) * b.nx;
      sy += w[bb] * (0.25f * __ldg(&row[xs[0]]) + 0.5f * __ldg(&row[xs[1]]) + 0.25f * __ldg(&row[xs[2]]));
    }
    s += w[c] * sy;
  }
  const size_t f = ((size_t)k * b.ny + j) * b.nx + i;
  out[f] = (mask && mask[f] != 1) ? 0.f : s;
}
// The learned correction enters the guess band by band: cells are grouped
// by their index distance to the nearest non-periodic y wall (where
// stretched grids put their thinnest cells and stiffest rows), and each
// band gets its own weight, chosen by least squares on the FP64 residual.
constexpr int kGuessBands = 4;
struct BandWeights {
  double a[kGuessBands];
};
__device__ inline int guess_band(const Box &b, int j) {
  if (b.py) return kGuessBands - 1;
  const int d = min(j, b.ny - 1 - j);
  return d < 2 ? 0 : (d < 8 ? 1 : (d < 32 ? 2 : 3));
}
// y_k = A (s c [band k]) per row (c already zero off the dofs), formed in
// FP32 from the level-0 multigrid operator (aj-scaled rows, parity-split
// layout) and unscaled by the row scale; block partials of
// G_kl = <y_k, y_l> (k <= l, 10 rows) and g_k = <y_k, r> (4 rows),
// r = b - A ex.  A neighbour's band follows from its j offset.  The fit
// only has to be good, not exact: the candidate it produces is then
// measured by its FP64 residual.  The sums run over every kstride-th
// k-plane (each plane holds every band, which depend on j only).
__global__ void __launch_bounds__(128) k_guess_gram(Box b, const float *__restrict__ A, const float *__restrict__ scale,
                                                     const float *__restrict__ c, const double *__restrict__ r,
                                                     double kappa, const double *sums, int kstride, double *partial) {
  const float sc = (float)(kappa * plane_rms(sums, 2));
  float acc[14];
  for (int q = 0; q < 14; q++) acc[q] = 0.f;
  const int p = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.z * kstride;
  const uint32_t n = (uint32_t)b.n();
  for (int j = blockIdx.y * kGuessRows; p < b.nx && j < min(b.ny, (int)(blockIdx.y + 1) * kGuessRows); j++) {
    const int i = split_cell(p, b.nx);
    uint32_t idx[NSLOT];
    stencil_index(b, i, j, k, idx);
    const uint32_t cs = idx[CP] - i + p;
    const float sr = scale[idx[CP]];
    if (sr != 0.f) {
      const int bm = guess_band(b, j > 0 ? j - 1 : j), b0 = guess_band(b, j),
                bp = guess_band(b, j < b.ny - 1 ? j + 1 : j);
      float y[kGuessBands] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int t = 0; t < NSLOT; t++) {
        int di, dj, dk;
        slot_offset(t, di, dj, dk);
        const int bt = dj < 0 ? bm : (dj > 0 ? bp : b0);
        const float term = __ldcs(&A[(size_t)t * n + cs]) * __ldg(&c[idx[t]]);
#pragma unroll
        for (int u = 0; u < kGuessBands; u++) y[u] += bt == u ? term : 0.f;
      }
      const float inv = 1.f / sr, rv = (float)r[idx[CP]];
      int q = 0;
#pragma unroll
      for (int u = 0; u < kGuessBands; u++) {
        y[u] *= sc * inv;
#pragma unroll
        for (int v = u; v < kGuessBands; v++) acc[q++] += y[u] * y[v];
      }
#pragma unroll
      for (int u = 0; u < kGuessBands; u++) acc[10 + u] += y[u] * rv;
    }
  }
  const size_t nb = (size_t)gridDim.x * gridDim.y * gridDim.z;
  const size_t blk = blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
  for (int q = 0; q < 14; q++) {
    const double t = block_sum((double)acc[q]);
    if (threadIdx.x == 0) partial[(size_t)q * nb + blk] = t;
  }
}
// learned guess x = ex + kappa * rms(f2) * alpha[band] * out on dofs
__global__ void k_guess_compose(Box b, const uint8_t *rt, const double *ex, const float *out, double kappa,
                                const double *sums, BandWeights w, double *x) {
  const double s = kappa * plane_rms(sums, 2);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < b.n(); c += (size_t)gridDim.x * blockDim.x)
    x[c] = rt[c] == 1 ? ex[c] + s * w.a[guess_band(b, (int)(((uint32_t)c / (uint32_t)b.nx) % (uint32_t)b.ny))] * (double)out[c] : 0.;
}

__device__ inline void atomic_max_pos(double *addr, double v) {
  // non-negative doubles order like their bit patterns
  atomicMax((unsigned long long *)addr, (unsigned long long)__double_as_longlong(v));
}
__global__ void k_max_spacing(Grid g, const double *coor, double *H) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y + 1, k = blockIdx.z + 1;
  const bool in = i >= 1 && i < g.mx - 1;
  if (!in) i = 1;  // every thread joins the block reduction
#define CO(a, b, c, q) coor[g.at(a, b, c) * 3 + (q)]
  double d[3] = {0, 0, 0};
  for (int q = 0; q < 3; q++) {
    double fp0 = 0.25 * (CO(i, j, k, q) + CO(i, j - 1, k, q) + CO(i, j, k - 1, q) + CO(i, j - 1, k - 1, q));
    double fm0 = 0.25 * (CO(i - 1, j, k, q) + CO(i - 1, j - 1, k, q) + CO(i - 1, j, k - 1, q) + CO(i - 1, j - 1, k - 1, q));
    double fp1 = 0.25 * (CO(i, j, k, q) + CO(i - 1, j, k, q) + CO(i, j, k - 1, q) + CO(i - 1, j, k - 1, q));
    double fm1 = 0.25 * (CO(i, j - 1, k, q) + CO(i - 1, j - 1, k, q) + CO(i, j - 1, k - 1, q) + CO(i - 1, j - 1, k - 1, q));
    double fp2 = 0.25 * (CO(i, j, k, q) + CO(i - 1, j, k, q) + CO(i, j - 1, k, q) + CO(i - 1, j - 1, k, q));
    double fm2 = 0.25 * (CO(i, j, k - 1, q) + CO(i - 1, j, k - 1, q) + CO(i, j - 1, k - 1, q) + CO(i - 1, j - 1, k - 1, q));
    d[0] += (fp0 - fm0) * (fp0 - fm0);
    d[1] += (fp1 - fm1) * (fp1 - fm1);
    d[2] += (fp2 - fm2) * (fp2 - fm2);
  }
  if (!in) d[0] = d[1] = d[2] = 0.;
#undef CO
  for (int q = 0; q < 3; q++) {
    double m = block_max(sqrt(d[q]));
    if (threadIdx.x == 0) atomic_max_pos(&H[q], m);
  }
}

struct Level {
  Grid g{};
  Box b{};
  int cx = 0, cy = 0, cz = 0;
  double *coor = nullptr, *nvert = nullptr;
  double *nvert_prev = nullptr;  // the restricted mask of the previous fill (coarse levels, incremental refill)
  MetricPtrs met{};
  bool own_met = false;
  double *A64 = nullptr;
  float *A32 = nullptr;
  __half2 *C16 = nullptr;  // the FP32 V-cycle's residual operator (k_pack16)
  float *D32 = nullptr;
  uint8_t *rowtype = nullptr, *blank = nullptr;
  double *inv64 = nullptr, *cp64 = nullptr, *w64 = nullptr;
  float *inv32 = nullptr, *cp32 = nullptr, *w32 = nullptr;
  double *v64[4] = {};  // x, b, r, t
  float *v32[4] = {};
  int nd = 0;
  int *didx = nullptr, *dmap = nullptr;
  double *dinv = nullptr;
  double *rho = nullptr, *level = nullptr;  // level-set fields of this level (DA layout)
  double *xfinal64 = nullptr;  // where x lives after a V-cycle (set at capture)
  float *xfinal32 = nullptr;
};

}  // namespace

struct vfs_poisson {
  vfs_grid_desc desc{};
  Grid g{};
  Box box{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  int64_t launches = 0;
  bool capturing = false;
  // DA-layout inputs and outputs
  double *coor = nullptr, *nvert = nullptr, *ucont = nullptr, *phi_da = nullptr, *p_da = nullptr;
  double *stage = nullptr;  // DA-sized staging, 3 components
  MetricPtrs met{};
  // fine operator and masks (box layout)
  double *A0 = nullptr, *scale = nullptr, *pc = nullptr, *aj_box = nullptr;
  float *scale32 = nullptr;  // the row scale in FP32 (the FP32 V-cycle's right-hand side)
  uint8_t *rowtype0 = nullptr, *fluid = nullptr;
  int *gid_box = nullptr, *gid_da = nullptr, *blk = nullptr, *total = nullptr;
  int ndof = 0;
  double *b = nullptr, *x = nullptr, *r = nullptr;
  // Krylov basis
  int m_alloc = 0;
  std::vector<double *> V, Z;
  double **dV = nullptr, **dZ = nullptr;
  // dsv[2q] = ||V_q||^2 and dsv[2q+1] = 1 / ||V_q||; dsv32[q] the latter in FP32
  double *partial = nullptr, *red = nullptr, *coef = nullptr, *dsv = nullptr;
  float *dsv32 = nullptr;
  size_t partial_len = 0;
  double *hbuf = nullptr;  // pinned host readback
  // learned initial guess: extrapolated phi, plane sums, feature planes and
  // network output (box layout, allocated on first use)
  double *gex = nullptr, *gsum = nullptr, *gnet = nullptr;  // gnet: the network's guess
  float *gfeat = nullptr, *gtgt = nullptr, *gfc = nullptr, *gout = nullptr, *gof[2] = {nullptr, nullptr};
  int gsmooth = 2;  // binomial passes over the prolonged correction
  std::vector<IbmBody> ibm_bodies;  // IB node records per body (ibm.cu)
  double *ibm_work = nullptr;        // 5 N words + the surface velocities (allocated on first use)
  IbmScratch ibm_scratch;            // the surface search's buffers
  size_t ibm_work_len = 0;
  // residual of the iterate installed by the learned guess, handed to the
  // next solve (warm_start 2) so that it does not form it again
  double *rprev = nullptr, *rlearn = nullptr, *r0 = nullptr;
  float *prev32 = nullptr;
  double *ucat = nullptr;  // Contra2Cart output staging (3 per DA point)
  // level-set variant of the operator and projection (vfs_poisson_set_levelset)
  double *ls_rho = nullptr, *ls_level = nullptr;
  int ls_on = 0, ls_bc3 = 0, ls_bc4 = 0, ls_bc5 = 0;
  int line_cols_cap = 0;  // cap on the line kernels' columns per block (0: none)
  // V-cycle kernels start during their predecessor's last wave (programmatic
  // dependent launch; VFS_PDL=0 at create turns it off); pdl_prev: the last
  // operation issued on the stream was such a kernel
  bool pdl = true, pdl_prev = false;
  // incremental refill of the finest level on a new mask (VFS_INCREMENTAL=0
  // at create turns it off): the mask the hierarchy was last filled with
  // (nvert_prev after the swap), the changed DA points, the rows to refill
  // (natural box indices, count on the device) and their j-columns;
  // inc_rows: the level-0 refill in progress uses that list
  bool inc_enable = true, nvert_prev_valid = false, inc_rows = false;
  double *nvert_prev = nullptr;
  uint8_t *chg_a = nullptr, *chg_b = nullptr, *colflag = nullptr;
  int *rows = nullptr, *nrows = nullptr;
  // history of the last hist_cnt (at most hist_cap) converged solutions for
  // the initial guess, held as the newest one X_n (the FGMRES iterate before
  // the mean removal) with its image Y_n = A X_n (b - r of its solve), stored
  // under the operator assembly hist_vn, and the differences of consecutive
  // solutions before it, D_j = X_j - X_{j-1} with images E_j = Y_j - Y_{j-1},
  // in a ring of hist_cap - 1 slots with the newest at hist_head - 1.
  // hist_ver[j]: the assembly both ends of D_j were stored under (kHistMixed
  // when they differ).  Gram entries (host): hist_Gnn = Y_n . Y_n,
  // hist_Gn[j] = Y_n . E_j, hist_G[i][j] = E_i . E_j.  The projection uses
  // the basis Y_n, E_newest, ... of the current assembly; the extrapolation
  // X_n + D_newest = 2 X_n - X_{n-1}.
  int hist_cap = 0, hist_cnt = 0, hist_head = 0;
  double *hist_Xn = nullptr, *hist_Yn = nullptr;
  uint64_t hist_vn = 0;
  double *hist_X[kHistMax] = {}, *hist_Y[kHistMax] = {};
  uint64_t hist_ver[kHistMax] = {};
  double hist_Gnn = 0., hist_Gn[kHistMax] = {}, hist_G[kHistMax][kHistMax] = {};
  double *hist_x = nullptr, *hist_r = nullptr;    // the projection and its residual
  double *hist_ex = nullptr, *hist_er = nullptr;  // the extrapolation and its residual
  double *hist_coef = nullptr;                    // combination coefficients (device)
  uint64_t op_version = 0;                        // operator assemblies seen
  // the learned guess runs its network on every net_period-th call while
  // its candidate keeps losing (net_wait: calls left to skip)
  int net_period = 1, net_wait = 0;
  bool hist_record = true;  // converged solves append to the history
  double r0_norm = 0.;
  bool r0_valid = false;
  // Z_0 of the next solve formed by the guess's judge: one V-cycle of the
  // installed residual divided by its norm, under the options z0_opts
  bool z0_valid = false;
  vfs_solve_opts z0_opts{};
  // FullyBlocked of the current nvert: first blocked k per (i, j) column
  // (device, mx * my) and the multiple-null-space flag (-1: not formed)
  int *ksk = nullptr, *ksk_count = nullptr;
  int multinull = -1;
  uint64_t ksk_version = 0;
  // what the last guess installed (vfs_poisson_guess_report)
  int guess_chosen = -1;
  double guess_rel[3] = {-1., -1., -1.}, guess_est[3] = {-1., -1., -1.};
  // Speculative first Arnoldi step: a learned guess that expects the plain
  // extrapolation to win (the previous guess did, with every band weight 0)
  // enqueues step 0 of the next solve on the handle's stream while the
  // network and the band fit run on a side stream.  The solve resumes at
  // step 1 when the guess installs that extrapolation and the solve's
  // options are the ones the step used; otherwise the step is dropped.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_feat = nullptr;
  // the solve's copy of phi to a host array, beside the history push
  cudaStream_t dl_stream = nullptr;
  cudaEvent_t dl_ev[2] = {nullptr, nullptr};
  double *spartial = nullptr, *sred = nullptr;  // side-stream reductions
  bool spec_enable = true;                      // VFS_GUESS_SPECULATE=0 turns it off
  bool spec_next = false, spec_valid = false;
  vfs_solve_opts spec_opts{};
  std::vector<Level> L;
  // the hierarchy's build parameters (a new mask with the same ones refills
  // the levels in place)
  int hier_cmax = -1;
  bool hier_ls = false;
  bool have_grid = false, have_nvert = false, have_rhs = false, have_phi = false;
  // graphs of the V-cycle per precision and parameters they were built for
  // captured V-cycles per precision, a few parameter sets each (least
  // recently used one replaced)
  struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    void *xfinal0 = nullptr;  // where this V-cycle leaves the finest level's x
    int64_t nodes = 0;
    int params[4] = {-1, -1, -1, -1};
    double omega = 0.;
    uint64_t used = 0;
  };
  static constexpr int kGraphSlots = 4;
  GraphSlot gslot[2][kGraphSlots];
  uint64_t gclock = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool own_stream = true;
  // live timing of the level-0 line sweeps (the dominant kernel)
  bool prof = false;
  cudaEvent_t pev[2][16] = {};
  int pcount = 0;            // sweeps recorded in the V-cycle in flight
  double pbytes[16] = {};    // algorithmic bytes of each recorded sweep
  double prof_ms = 0., prof_bytes = 0.;
  int64_t prof_launches = 0;
  // optional per-phase timing of the outer iteration (environment variable
  // VFS_PHASE_TIMING=1): preconditioner, operator apply, Gram-Schmidt
  bool phase = false;
  cudaEvent_t phev[4] = {};
  double phase_ms[3] = {0., 0., 0.};
  double host_ms[4] = {0., 0., 0., 0.};  // enqueue, (unused), wait, host work
};

namespace {

template <typename T>
int dalloc(vfs_poisson *h, T **p, size_t count) {
  void *q = nullptr;
  size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(VFS_ENOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
  }
  h->allocs.push_back(q);
  *p = (T *)q;
  return VFS_OK;
}
void dfree(vfs_poisson *h, void *p) {
  if (!p) return;
  auto it = std::find(h->allocs.begin(), h->allocs.end(), p);
  if (it != h->allocs.end()) h->allocs.erase(it);
  cudaFree(p);
}

bool is_device_ptr(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// copy a caller array (host or device) into a device buffer
int upload(vfs_poisson *h, double *dst, const double *src, size_t count) {
  CUDA_TRY(cudaMemcpyAsync(dst, src, count * sizeof(double),
                           is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
  return VFS_OK;
}
// device memory is read where it lies; host memory is staged
int device_view(vfs_poisson *h, const double *src, double *stage, size_t count, const double **out) {
  if (is_device_ptr(src)) {
    *out = src;
    return VFS_OK;
  }
  *out = stage;
  return upload(h, stage, src, count);
}
int download(vfs_poisson *h, double *dst, const double *src, size_t count) {
  CUDA_TRY(cudaMemcpyAsync(dst, src, count * sizeof(double),
                           is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
  return VFS_OK;
}
int sync(vfs_poisson *h) {
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return VFS_OK;
}

dim3 da_grid(const Grid &g, int bx = 128) { return dim3((g.mx + bx - 1) / bx, g.my, g.mz); }
dim3 box_grid(const Box &b, int bx = 128) { return dim3((b.nx + bx - 1) / bx, b.ny, b.nz); }
unsigned lin_grid(size_t n, int bx = 256) { return (unsigned)((n + bx - 1) / bx); }
// grid of the guess's reduction kernels: 128 columns x kGuessRows j-rows
dim3 guess_grid(const Box &b) { return dim3((b.nx + 127) / 128, (b.ny + kGuessRows - 1) / kGuessRows, b.nz); }

#define LAUNCH(h, kern, grid, block, ...)                          \
  do {                                                             \
    kern<<<(grid), (block), 0, (h)->stream>>>(__VA_ARGS__);        \
    (h)->launches++;                                               \
  } while (0)

#define LAUNCH_SM(h, kern, grid, block, smem, ...)                 \
  do {                                                             \
    kern<<<(grid), (block), (smem), (h)->stream>>>(__VA_ARGS__);   \
    (h)->launches++;                                               \
  } while (0)

// A kernel of the V-cycle.  When the previous operation on the stream was
// one too, the launch carries programmatic stream serialization: its blocks
// may start as the previous kernel's last blocks run, load the level's
// operator planes and wait (griddepcontrol.wait) for that kernel's results.
// Only kernels that wait before reading anything the V-cycle writes go
// through here.  A memset or an event in between (vmemset, the profiling
// events) makes the next launch an ordinary one.
template <typename... P, typename... A>
void launch_v(vfs_poisson *h, void (*kern)(P...), dim3 grid, dim3 block, size_t smem, A &&...args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cfg.attrs = at;
  cfg.numAttrs = h->pdl && h->pdl_prev ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
  h->pdl_prev = true;
  h->launches++;
}
void vmemset(vfs_poisson *h, void *p, size_t bytes) {
  cudaMemsetAsync(p, 0, bytes, h->stream);
  h->pdl_prev = false;
}

int alloc_metrics(vfs_poisson *h, const Grid &g, MetricPtrs &m) {
  size_t n = g.n();
  double **vec[] = {&m.cent, &m.csi, &m.eta, &m.zet, &m.icsi, &m.ieta, &m.izet, &m.jcsi, &m.jeta, &m.jzet,
                    &m.kcsi, &m.keta, &m.kzet};
  double **sca[] = {&m.aj, &m.iaj, &m.jaj, &m.kaj};
  for (auto p : vec) { TRY(dalloc(h, p, 3 * n)); CUDA_TRY(cudaMemsetAsync(*p, 0, 3 * n * 8, h->stream)); }
  for (auto p : sca) { TRY(dalloc(h, p, n)); CUDA_TRY(cudaMemsetAsync(*p, 0, n * 8, h->stream)); }
  m.gface = nullptr;  // formed by face_coef once the metrics are final
  return VFS_OK;
}
// the operator's face coefficients of a grid's final metrics (every later
// assembly reads them instead of forming them from the metrics)
int face_coef(vfs_poisson *h, const Grid &g, MetricPtrs &m) {
  if (!m.gface) TRY(dalloc(h, &m.gface, 9 * g.n()));
  MetricPtrs src = m;
  src.gface = nullptr;
  LAUNCH(h, k_face_coef, da_grid(g), 128, g, src, m.gface);
  return VFS_OK;
}
void free_metrics(vfs_poisson *h, MetricPtrs &m) {
  double *all[] = {m.cent, m.csi, m.eta, m.zet, m.icsi, m.ieta, m.izet, m.jcsi, m.jeta, m.jzet,
                   m.kcsi, m.keta, m.kzet, m.aj, m.iaj, m.jaj, m.kaj, m.gface};
  for (auto p : all) dfree(h, p);
  m = MetricPtrs{};
}

// FormMetrics on the device, in the reference's order of passes.
int form_metrics(vfs_poisson *h, const Grid &g, const double *coor, MetricPtrs &m) {
  LAUNCH(h, k_metrics_cell, da_grid(g), 128, g, coor, m);
  LAUNCH(h, k_metrics_mirror, dim3((g.my + 127) / 128, g.mz), 128, g, m, 0);
  LAUNCH(h, k_metrics_mirror, dim3((g.mx + 127) / 128, g.mz), 128, g, m, 1);
  LAUNCH(h, k_metrics_mirror, dim3((g.mx + 127) / 128, g.my), 128, g, m, 2);
  LAUNCH(h, k_metrics_periodic, da_grid(g), 128, g, m, 0);
  for (int d = 0; d < 3; d++) LAUNCH(h, k_metrics_face, da_grid(g), 128, g, m, d);
  LAUNCH(h, k_metrics_periodic, da_grid(g), 128, g, m, 1);
  return VFS_OK;
}

// Coarsening choice (same rule as the CPU baseline): coarsen a direction with
// an even count >= 4 whose largest cell extent is at most twice the smallest
// largest-extent of the other directions; fall back to the finest direction.
bool choose_coarsening(const double H[3], const int n[3], int c[3]) {
  bool any = false;
  for (int q = 0; q < 3; q++) {
    c[q] = 0;
    if (n[q] % 2 || n[q] < 4) continue;
    double mn = 1e300;
    for (int e = 0; e < 3; e++)
      if (e != q && n[e] >= 2 && H[e] < mn) mn = H[e];
    if (H[q] <= 2.0 * mn) { c[q] = 1; any = true; }
  }
  if (!any) {
    int best = -1;
    for (int q = 0; q < 3; q++)
      if (n[q] % 2 == 0 && n[q] >= 4 && (best < 0 || H[q] < H[best])) best = q;
    if (best >= 0) { c[best] = 1; any = true; }
  }
  return any;
}

// Dense inverse of the coarsest operator with one pinned row per connected
// component (the singular Neumann / periodic system becomes regular).
int build_coarsest(vfs_poisson *h, Level &l) {
  const size_t n = l.b.n();
  std::vector<double> A(n * NSLOT);
  std::vector<uint8_t> rt(n);
  CUDA_TRY(cudaMemcpyAsync(A.data(), l.A64, n * NSLOT * 8, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaMemcpyAsync(rt.data(), l.rowtype, n, cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  std::vector<int> map(n, -1), idx;
  for (size_t c = 0; c < n; c++)
    if (rt[c]) { map[c] = (int)idx.size(); idx.push_back((int)c); }
  const int nd = (int)idx.size();
  if (nd > 1024) return fail(VFS_EINVAL, "coarsest level has more than 1024 dofs");
  std::vector<double> M((size_t)nd * nd, 0.), I((size_t)nd * nd, 0.);
  const Box &b = l.b;
  for (int r = 0; r < nd; r++) {
    int c = idx[r];
    int i = c % b.nx, j = (c / b.nx) % b.ny, k = c / (b.nx * b.ny);
    const size_t cs = b.at(split_pos(i, b.nx), j, k);  // level operators are stored split
    for (int s = 0; s < NSLOT; s++) {
      int di, dj, dk;
      slot_offset(s, di, dj, dk);
      int a = i + di, bb = j + dj, cc = k + dk;
      if (a < 0) { if (!b.px) continue; a += b.nx; }
      if (a >= b.nx) { if (!b.px) continue; a -= b.nx; }
      if (bb < 0) { if (!b.py) continue; bb += b.ny; }
      if (bb >= b.ny) { if (!b.py) continue; bb -= b.ny; }
      if (cc < 0) { if (!b.pz) continue; cc += b.nz; }
      if (cc >= b.nz) { if (!b.pz) continue; cc -= b.nz; }
      int q = map[b.at(a, bb, cc)];
      if (q < 0) continue;
      M[(size_t)r * nd + q] += A[(size_t)s * n + cs];
    }
  }
  std::vector<int> comp(nd, -1), queue(nd), first;
  // a row whose coefficients do not sum to zero (a Dirichlet boundary of
  // the level-set variant) makes its component regular: no pinned row there
  std::vector<char> regular_row(nd, 0);
  for (int r = 0; r < nd; r++) {
    double sum = 0., dg = std::fabs(M[(size_t)r * nd + r]);
    for (int q = 0; q < nd; q++) sum += M[(size_t)r * nd + q];
    regular_row[r] = std::fabs(sum) > 1e-8 * dg;
  }
  int ncomp = 0;
  std::vector<int> pin_comp;                  // component of each pinned row
  std::vector<std::vector<double>> pin_row;   // its equation before pinning
  for (int r0 = 0; r0 < nd; r0++) {
    if (comp[r0] >= 0) continue;
    int hd = 0, tl = 0;
    queue[tl++] = r0;
    comp[r0] = ncomp;
    bool regular = false;
    while (hd < tl) {
      int r = queue[hd++];
      regular = regular || regular_row[r];
      for (int q = 0; q < nd; q++)
        if (comp[q] < 0 && (M[(size_t)r * nd + q] != 0. || M[(size_t)q * nd + r] != 0.)) {
          comp[q] = ncomp;
          queue[tl++] = q;
        }
    }
    if (!regular) {
      pin_comp.push_back(ncomp);
      pin_row.emplace_back(M.begin() + (size_t)r0 * nd, M.begin() + (size_t)(r0 + 1) * nd);
      for (int q = 0; q < nd; q++) M[(size_t)r0 * nd + q] = 0.;
      M[(size_t)r0 * nd + r0] = 1.;
      first.push_back(r0);
    }
    ncomp++;
  }
  for (int r = 0; r < nd; r++) I[(size_t)r * nd + r] = 1.;
  for (int c = 0; c < nd; c++) {  // Gauss-Jordan, partial pivoting
    int p = c;
    for (int r = c + 1; r < nd; r++)
      if (std::fabs(M[(size_t)r * nd + c]) > std::fabs(M[(size_t)p * nd + c])) p = r;
    if (p != c)
      for (int q = 0; q < nd; q++) {
        std::swap(M[(size_t)c * nd + q], M[(size_t)p * nd + q]);
        std::swap(I[(size_t)c * nd + q], I[(size_t)p * nd + q]);
      }
    double piv = M[(size_t)c * nd + c];
    double ip = piv != 0. ? 1. / piv : 0.;
    for (int q = 0; q < nd; q++) { M[(size_t)c * nd + q] *= ip; I[(size_t)c * nd + q] *= ip; }
    const double *__restrict__ mc = &M[(size_t)c * nd];
    const double *__restrict__ ic = &I[(size_t)c * nd];
    for (int r = 0; r < nd; r++) {
      if (r == c) continue;
      double f = M[(size_t)r * nd + c];
      if (f == 0.) continue;
      // distinct rows: the restrict pointers let the compiler vectorise
      double *__restrict__ mr = &M[(size_t)r * nd];
      double *__restrict__ ir = &I[(size_t)r * nd];
      for (int q = 0; q < nd; q++) {
        mr[q] -= f * mc[q];
        ir[q] -= f * ic[q];
      }
    }
  }
  // Left null vector w of each singular component (w^T M = 0 on it): with
  // M_p the matrix with row r0 pinned to e_r0 and I = M_p^-1, M_p 1 = e_r0
  // (the rows sum to zero), and w^T = e_r0^T I - m_r0^T I has w_r0 = 1.
  std::vector<std::vector<double>> wv;
  for (size_t t = 0; t < first.size(); t++) {
    const int r0 = first[t];
    std::vector<double> w(I.begin() + (size_t)r0 * nd, I.begin() + (size_t)(r0 + 1) * nd);
    for (int p = 0; p < nd; p++) {
      const double m = pin_row[t][p];
      if (m == 0.) continue;
      for (int q = 0; q < nd; q++) w[q] -= m * I[(size_t)p * nd + q];
    }
    wv.push_back(std::move(w));
  }
  for (int r0 : first)  // pinned rows see a zero right-hand side
    for (int r = 0; r < nd; r++) I[(size_t)r * nd + r0] = 0.;
  // A restricted right-hand side need not be consistent (w^T b != 0 on a
  // singular component); pinning alone would put the whole inconsistency
  // into the pinned cell's equation.  The solve projects it out evenly
  // first: dinv = I_z (1 - 1_c w^T / w^T 1_c) on every such component c.
  for (size_t t = 0; t < first.size(); t++) {
    const int cid = pin_comp[t];
    const std::vector<double> &w = wv[t];
    double s1 = 0.;
    for (int q = 0; q < nd; q++)
      if (comp[q] == cid) s1 += w[q];
    if (!(std::fabs(s1) > 0.)) continue;
    for (int r = 0; r < nd; r++) {
      double rs = 0.;
      for (int p = 0; p < nd; p++)
        if (comp[p] == cid) rs += I[(size_t)r * nd + p];
      if (rs == 0.) continue;
      const double f = rs / s1;
      for (int q = 0; q < nd; q++)
        if (comp[q] == cid) I[(size_t)r * nd + q] -= f * w[q];
    }
  }
  l.nd = nd;
  dfree(h, l.didx);
  dfree(h, l.dmap);
  dfree(h, l.dinv);
  TRY(dalloc(h, &l.didx, nd));
  TRY(dalloc(h, &l.dmap, n));
  TRY(dalloc(h, &l.dinv, (size_t)nd * nd));
  CUDA_TRY(cudaMemcpyAsync(l.didx, idx.data(), nd * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(l.dmap, map.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(l.dinv, I.data(), (size_t)nd * nd * 8, cudaMemcpyHostToDevice, h->stream));
  return sync(h);
}

void free_level(vfs_poisson *h, Level &l, bool level0) {
  if (!level0) { dfree(h, l.coor); dfree(h, l.nvert); dfree(h, l.nvert_prev); dfree(h, l.rho); dfree(h, l.level); }
  if (l.own_met) free_metrics(h, l.met);
  dfree(h, l.A64); dfree(h, l.A32); dfree(h, l.C16); dfree(h, l.D32); dfree(h, l.rowtype); dfree(h, l.blank);
  dfree(h, l.inv64); dfree(h, l.cp64); dfree(h, l.w64); dfree(h, l.inv32); dfree(h, l.cp32); dfree(h, l.w32);
  for (int q = 0; q < 4; q++) { dfree(h, l.v64[q]); dfree(h, l.v32[q]); }
  dfree(h, l.didx); dfree(h, l.dmap); dfree(h, l.dinv);
  l = Level{};
}

void drop_graphs(vfs_poisson *h) {
  for (int p = 0; p < 2; p++) {
    for (auto &g : h->gslot[p]) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g = vfs_poisson::GraphSlot{};
    }
  }
}

LevelSet level_set(const vfs_poisson *h, const Level &l) {
  LevelSet ls;
  if (h->ls_on) {
    ls.rho = l.rho;
    ls.level = l.level;
    ls.on = 1;
    ls.bc3 = h->ls_bc3;
    ls.bc4 = h->ls_bc4;
    ls.bc5 = h->ls_bc5;
  }
  return ls;
}

// Operator, masks and line factors of one level (assembled from its
// metrics, unless `assembled`: the fine level's operator formed together
// with the FGMRES operator) into its buffers, allocated on the first build.
int build_level_operator(vfs_poisson *h, Level &l, bool assembled = false) {
  const size_t n = l.b.n();
  if (!l.A64) {
    TRY(dalloc(h, &l.A64, n * NSLOT));
    TRY(dalloc(h, &l.A32, n * NSLOT));
    TRY(dalloc(h, &l.C16, n * 10));
    TRY(dalloc(h, &l.D32, n));
    TRY(dalloc(h, &l.rowtype, n));
    TRY(dalloc(h, &l.blank, n));
    TRY(dalloc(h, &l.w64, n));
    TRY(dalloc(h, &l.w32, n));
    TRY(dalloc(h, &l.inv64, n)); TRY(dalloc(h, &l.cp64, n));
    TRY(dalloc(h, &l.inv32, n)); TRY(dalloc(h, &l.cp32, n));
    for (int q = 0; q < 4; q++) { TRY(dalloc(h, &l.v64[q], n)); TRY(dalloc(h, &l.v32[q], n)); }
  }
  if (!assembled && h->inc_rows)
    LAUNCH(h, k_assemble_rows, kRedBlocks, 256, l.g, l.b, l.nvert, l.met, 1, 0, 1, l.A64, l.rowtype, level_set(h, l),
           (const int *)h->rows, (const int *)h->nrows);
  else if (!assembled)
    LAUNCH(h, k_assemble, box_grid(l.b), 128, l.g, l.b, l.nvert, l.met, 1, 0, 1, l.A64, l.rowtype, level_set(h, l));
  LAUNCH(h, k_level_masks, lin_grid(n), 256, l.g, l.b, l.nvert, l.blank, l.w64, l.w32, (double *)nullptr,
         (const double *)nullptr);
  // a level of an incremental refill: only the listed rows' copies and the
  // j-columns that hold one are formed again
  const uint8_t *cols = h->inc_rows ? h->colflag : nullptr;
  LAUNCH(h, k_line_lu_f64, dim3((l.b.nx + 127) / 128, l.b.nz), 128, l.b, l.A64, l.inv64, l.cp64, cols);
  LAUNCH(h, k_line_lu_f32, dim3((l.b.nx + 127) / 128, l.b.nz), 128, l.b, l.A64, l.inv32, l.cp32, cols);
  if (cols) {
    LAUNCH(h, k_pack16_rows, kRedBlocks, 256, l.b, (const double *)l.A64, l.C16, l.D32, l.A32, (const int *)h->rows,
           (const int *)h->nrows);
  } else {
    LAUNCH(h, k_cast_planes_f32, kRedBlocks, 256, l.A64, l.A32, n * NSLOT);
    LAUNCH(h, k_pack16, kRedBlocks, 256, n, l.A64, l.C16, l.D32);
  }
  return VFS_OK;
}

// A new mask on the hierarchy's grid: the levels' shapes, coarsening,
// coordinates and metrics do not depend on nvert, so every level keeps its
// buffers; its mask is restricted again and its operator, line factors and
// packed copy are refilled in place.  Only the coarsest level's dense
// inverse (its size follows the dof count) is formed anew, and the V-cycle
// graphs (which hold that count) are captured again at their next use.
int refresh_hierarchy(vfs_poisson *h) {
  drop_graphs(h);
  h->L[0].nvert = h->nvert;
  h->L[0].rho = h->ls_rho;
  h->L[0].level = h->ls_level;
  // an incremental refill keeps each coarse level's previous mask to find
  // the rows to refill there too
  const bool incremental = h->inc_rows;
  for (size_t li = 1; li < h->L.size(); li++) {
    Level &f = h->L[li - 1], &q = h->L[li];
    if (incremental) {
      if (!q.nvert_prev) TRY(dalloc(h, &q.nvert_prev, q.g.n()));
      std::swap(q.nvert, q.nvert_prev);
    }
    LAUNCH(h, k_nvert_restrict, da_grid(q.g), 128, f.g, q.g, f.cx, f.cy, f.cz, f.nvert, h->stage);
    LAUNCH(h, k_nvert_fill, da_grid(q.g), 128, q.g, h->stage, q.nvert);
    if (h->ls_on) {
      LAUNCH(h, k_cellfield_restrict, da_grid(q.g), 128, f.g, q.g, f.cx, f.cy, f.cz, f.rho, q.rho);
      LAUNCH(h, k_cellfield_restrict, da_grid(q.g), 128, f.g, q.g, f.cx, f.cy, f.cz, f.level, q.level);
    }
  }
  const auto t0 = std::chrono::steady_clock::now();
  for (size_t li = 0; li < h->L.size(); li++) {
    Level &l = h->L[li];
    if (li > 0 && incremental) {
      // the rows of this level within two points of a changed restricted
      // mask value (the list buffers of the finest level, consumed by its
      // launches above, are reused in stream order)
      LAUNCH(h, k_mask_changed, kRedBlocks, 256, l.g.n(), (const double *)l.nvert, (const double *)l.nvert_prev,
             h->chg_a);
      LAUNCH(h, k_dilate_axis, da_grid(l.g), 128, l.g, 0, 2, (const uint8_t *)h->chg_a, h->chg_b);
      LAUNCH(h, k_dilate_axis, da_grid(l.g), 128, l.g, 1, 2, (const uint8_t *)h->chg_b, h->chg_a);
      LAUNCH(h, k_dilate_axis, da_grid(l.g), 128, l.g, 2, 2, (const uint8_t *)h->chg_a, h->chg_b);
      CUDA_TRY(cudaMemsetAsync(h->nrows, 0, sizeof(int), h->stream));
      CUDA_TRY(cudaMemsetAsync(h->colflag, 0, (size_t)l.b.nx * l.b.nz, h->stream));
      LAUNCH(h, k_list_rows, kRedBlocks, 256, l.g, l.b, (const uint8_t *)h->chg_b, h->rows, h->nrows, h->colflag);
    }
    TRY(build_level_operator(h, l, li == 0));
  }
  h->inc_rows = false;
  if (h->phase) TRY(sync(h));
  const auto t1 = std::chrono::steady_clock::now();
  Level &c = h->L.back();
  // an incremental refill that listed no row of the coarsest level (the
  // last list formed above) leaves its operator, and so its inverse, as it was
  bool same = false;
  if (incremental && c.dinv) {
    int nr = -1;
    CUDA_TRY(cudaMemcpyAsync(&nr, h->nrows, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    same = nr == 0;
  }
  if (!same) {
    dfree(h, c.didx); dfree(h, c.dmap); dfree(h, c.dinv);
    c.didx = c.dmap = nullptr;
    c.dinv = nullptr;
    TRY(build_coarsest(h, c));
  }
  TRY(sync(h));
  if (h->phase)
    fprintf(stderr, "vfs refill ms: level operators %.3f coarsest %.3f\n",
            std::chrono::duration<double, std::milli>(t1 - t0).count(),
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count());
  return VFS_OK;
}

// a new mask refills the existing hierarchy (its level-0 operator then
// assembled by vfs_poisson_set_nvert together with the FGMRES operator)
bool hierarchy_refills(const vfs_poisson *h, int coarsest_max) {
  return !h->L.empty() && h->hier_cmax == coarsest_max && h->hier_ls == (h->ls_on != 0);
}

int build_hierarchy(vfs_poisson *h, int coarsest_max) {
  if (hierarchy_refills(h, coarsest_max)) return refresh_hierarchy(h);
  for (size_t li = 0; li < h->L.size(); li++) free_level(h, h->L[li], li == 0);
  h->L.clear();
  drop_graphs(h);
  Level l0;
  l0.g = h->g;
  l0.b = h->box;
  l0.coor = h->coor;
  l0.nvert = h->nvert;
  l0.met = h->met;
  l0.rho = h->ls_rho;
  l0.level = h->ls_level;
  h->L.push_back(l0);
  double *H;
  TRY(dalloc(h, &H, 3));
  for (;;) {
    Level &f = h->L.back();
    if (f.b.n() <= (size_t)coarsest_max || (int)h->L.size() >= kMaxLevels) break;
    double Hh[3];
    CUDA_TRY(cudaMemsetAsync(H, 0, 3 * 8, h->stream));
    LAUNCH(h, k_max_spacing, dim3((f.g.mx + 127) / 128, f.g.my - 2, f.g.mz - 2), 128, f.g, f.coor, H);
    CUDA_TRY(cudaMemcpyAsync(Hh, H, 24, cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    int n3[3] = {f.b.nx, f.b.ny, f.b.nz}, c[3];
    if (!choose_coarsening(Hh, n3, c)) break;
    f.cx = c[0]; f.cy = c[1]; f.cz = c[2];
    Level q;
    q.b = f.b;
    q.b.nx = c[0] ? f.b.nx / 2 : f.b.nx;
    q.b.ny = c[1] ? f.b.ny / 2 : f.b.ny;
    q.b.nz = c[2] ? f.b.nz / 2 : f.b.nz;
    q.g = f.g;
    q.g.mx = q.b.nx + 2; q.g.my = q.b.ny + 2; q.g.mz = q.b.nz + 2;
    TRY(dalloc(h, &q.coor, q.g.n() * 3));
    TRY(dalloc(h, &q.nvert, q.g.n()));
    double *tmp;
    TRY(dalloc(h, &tmp, q.g.n()));
    LAUNCH(h, k_coarse_nodes, da_grid(q.g), 128, f.g, q.g, c[0], c[1], c[2], f.coor, q.coor);
    LAUNCH(h, k_nvert_restrict, da_grid(q.g), 128, f.g, q.g, c[0], c[1], c[2], f.nvert, tmp);
    LAUNCH(h, k_nvert_fill, da_grid(q.g), 128, q.g, tmp, q.nvert);
    if (h->ls_on) {  // level-set fields of the coarse level: child averages
      TRY(dalloc(h, &q.rho, q.g.n()));
      TRY(dalloc(h, &q.level, q.g.n()));
      LAUNCH(h, k_cellfield_restrict, da_grid(q.g), 128, f.g, q.g, c[0], c[1], c[2], f.rho, q.rho);
      LAUNCH(h, k_cellfield_restrict, da_grid(q.g), 128, f.g, q.g, c[0], c[1], c[2], f.level, q.level);
    }
    TRY(sync(h));
    dfree(h, tmp);
    h->L.push_back(q);
  }
  dfree(h, H);
  for (size_t li = 0; li < h->L.size(); li++) {
    Level &l = h->L[li];
    if (li > 0) {
      TRY(alloc_metrics(h, l.g, l.met));
      l.own_met = true;
      TRY(form_metrics(h, l.g, l.coor, l.met));
      TRY(face_coef(h, l.g, l.met));
    }
    TRY(build_level_operator(h, l));
    TRY(sync(h));
    // the coarse metrics stay for the assembly of later masks
  }
  TRY(build_coarsest(h, h->L.back()));
  h->hier_cmax = coarsest_max;
  h->hier_ls = h->ls_on != 0;
  return VFS_OK;
}

// ---- V-cycle (issued on the stream; captured into a graph when enabled) ----
template <typename T>
struct Prec;
template <>
struct Prec<float> {
  static constexpr auto sweep = k_line_sweep_f32;
  static void residual(vfs_poisson *h, Level &l, dim3 g, const float *x, const float *bb, float *r, int color,
                       bool split) {
    if (split) launch_v(h, k_residual16_split, g, 128, 0, l.b, l.C16, l.D32, x, bb, r, color);
    else launch_v(h, k_residual16, g, 128, 0, l.b, l.C16, l.D32, x, bb, r, color);
  }
  static constexpr auto restrict_ = k_restrict_f32;
  static constexpr auto prolong = k_prolong_f32;
  static constexpr auto prolong_split = k_prolong_f32_split;
  static constexpr auto coarsest = k_coarsest_f32;
  static constexpr auto tri = k_line_tri_f32;
  static constexpr auto tri_split = k_line_tri_f32_split;
  static void fused(vfs_poisson *h, Level &l, dim3 g, dim3 blk, size_t sm, const float *xo, const float *xn,
                    const float *bb, float *xd, float omega, bool own_zero, bool both_zero, int color) {
    const auto kern = both_zero ? k_line_fused16_z : own_zero ? k_line_fused16_oz : k_line_fused16;
    launch_v(h, kern, g, blk, sm, l.b, l.C16, l.D32, xo, xn, bb, l.A32 + (size_t)SP * l.b.n(), l.inv32, l.cp32, xd,
             omega, color);
  }
  static float *A(Level &l) { return l.A32; }
  static float *inv(Level &l) { return l.inv32; }
  static float *cp(Level &l) { return l.cp32; }
  static float *w(Level &l) { return l.w32; }
  static float **v(Level &l) { return l.v32; }
  static float *&xfinal(Level &l) { return l.xfinal32; }
};
template <>
struct Prec<double> {
  static constexpr auto sweep = k_line_sweep_f64;
  static void residual(vfs_poisson *h, Level &l, dim3 g, const double *x, const double *bb, double *r, int color,
                       bool) {
    launch_v(h, k_residual_f64, g, 128, 0, l.b, l.A64, x, bb, r, color);
  }
  static constexpr auto restrict_ = k_restrict_f64;
  static constexpr auto prolong = k_prolong_f64;
  static constexpr auto prolong_split = k_prolong_f64;  // (the FP64 V-cycle keeps natural vectors)
  static constexpr auto coarsest = k_coarsest_f64;
  static constexpr auto tri = k_line_tri_f64;
  static constexpr auto tri_split = k_line_tri_f64;
  // no FP64 variant of the fused sweep (smoother 4 runs smoother 3's kernels)
  static void fused(vfs_poisson *, Level &, dim3, dim3, size_t, const double *, const double *, const double *,
                    double *, double, bool, bool, int) {}
  static double *A(Level &l) { return l.A64; }
  static double *inv(Level &l) { return l.inv64; }
  static double *cp(Level &l) { return l.cp64; }
  static double *w(Level &l) { return l.w64; }
  static double **v(Level &l) { return l.v64; }
  static double *&xfinal(Level &l) { return l.xfinal64; }
};

// Event pairs around the level-0 sweeps of one V-cycle (recorded as graph
// nodes when the V-cycle is captured); read after the next stream sync.
// Algorithmic bytes of a sweep per cell, in words of T: the fused sweep
// reads 16 off-line coefficients, the S slot, inv and cp, the right-hand
// side and x and writes x (22 words), or 5 words from a zero guess (S, inv,
// cp, rhs, x out).  The correction-form sweeps (residual kernel +
// tridiagonal kernel) move R + 6 words per cell: the residual's operator, x,
// rhs and r (R = 22 with 19 coefficients of T; R = 14 for the FP32 packed
// operator, 10 half2 words and the diagonal), then r, S slot, inv, cp and x
// read and written.  A zero-guess zebra sweep skips the first colour's
// residual and reads rhs, S, inv, cp and writes x there.
// Smoother 4 forms the residual inside the line kernel on levels of at most
// kFusedMaxCells cells (FP32).  Finer levels run smoother 3's kernels: they
// are bandwidth-bound, and there the separate residual kernel (high
// occupancy) and line kernel move their larger byte count faster than the
// fused kernel (one 168-register block per SM) moves its smaller one.  The
// coarse levels are latency-bound and gain from half the launches.
constexpr size_t kFusedMaxCells = size_t(1) << 20;
template <typename T>
bool fused_level(const Level &l, int smoother) {
  return smoother == 4 && std::is_same<T, float>::value && l.b.n() <= kFusedMaxCells;
}
// The finest FP32 level under the two-kernel checkerboard sweep keeps x and
// its right-hand side in the parity-split row layout: each colour's launches
// then read and write whole sectors of them (natural vectors give every
// other float of a sector).  The residual handed to the restriction stays
// natural, so the coarser levels are unaffected.
template <typename T>
bool split_level(const vfs_poisson *h, int li, int smoother) {
  return std::is_same<T, float>::value && li == 0 && h->L.size() > 1 && smoother >= 3 &&
         !fused_level<T>(h->L[0], smoother);
}

template <typename T>
void prof_begin(vfs_poisson *h, int li, bool zero_guess, int smoother) {
  if (!h->prof || li != 0 || h->pcount >= 16) return;
  cudaEventRecord(h->pev[0][h->pcount], h->stream);
  h->pdl_prev = false;
  const double R = std::is_same<T, float>::value ? 14.0 : 22.0;
  double words = zero_guess ? (smoother >= 2 ? 0.5 * (5.0 + R + 6.0) : 5.0)
                            : (smoother == 0 ? 22.0 : R + 6.0);
  // residual formed in the line kernel (FP32): 10 half2 words and the
  // diagonal, x, rhs, S slot, inv, cp and x written; from a zero guess the
  // first colour streams rhs, S, inv, cp and x written
  if (fused_level<T>(h->L[li], smoother)) words = zero_guess ? 0.5 * (5.0 + 17.0) : 17.0;
  h->pbytes[h->pcount] = (double)h->box.n() * sizeof(T) * words;
}
void prof_end(vfs_poisson *h, int li) {
  if (!h->prof || li != 0 || h->pcount >= 16) return;
  cudaEventRecord(h->pev[1][h->pcount], h->stream);
  h->pdl_prev = false;
  h->pcount++;
}

// Columns per block of the line kernels for lines of P chunks.  The
// kernels are compiled for at most kLineMaxThreads threads per block (a
// whole chunk stays in registers): 16 columns in FP32 and 4 in FP64, where
// more, smaller blocks per SM measured faster (warm FP64 solve 31.5 -> 30.3
// ms on the 256x192x256 towers grid; FP32 unchanged), halved while the block
// would exceed the limit (8 columns for j-lines of 193..384 cells in FP32).
// Every column is solved independently, so the width changes no result bit.
// VFS_LINE_COLUMNS caps the width (read at create).
int line_columns(const vfs_poisson *h, int P, bool fp64) {
  int ti = fp64 ? 4 : 16;
  if (h->line_cols_cap > 0 && ti > h->line_cols_cap) ti = h->line_cols_cap;
  while (ti > 1 && ti * P > kLineMaxThreads) ti >>= 1;
  return ti;
}

// One smoothing sweep on level l.  smoother 0: fused j-line Jacobi kernel;
// 1: j-line Jacobi in correction form (residual kernel + tridiagonal
// kernel); 2: zebra j-line Gauss-Seidel over even then odd k-planes in
// correction form; 3: zebra over checkerboard columns in correction form;
// 4: the same sweep with each colour's residual formed in the line kernel
// on the levels fused_level selects (3 elsewhere).  x/t are swapped by the
// sweeps that write t (0 and the fused 4).
template <typename T>
void smooth(vfs_poisson *h, Level &l, int li, int smoother, bool zero_guess, T omega, T *&x, T *&t, T *bb, T *r) {
  const int P = (l.b.ny + kLineChunk - 1) / kLineChunk;
  const int TI = line_columns(h, P, std::is_same<T, double>::value);
  dim3 lb(TI, P), lg((l.b.nx + TI - 1) / TI, l.b.nz);
  const size_t lsm = 2 * TI * P * sizeof(T);
  T *Asp = Prec<T>::A(l) + (size_t)SP * l.b.n();
  prof_begin<T>(h, li, zero_guess, smoother);
  if (smoother == 0) {
    launch_v(h, Prec<T>::sweep, lg, lb, lsm, l.b, Prec<T>::A(l), Prec<T>::inv(l), Prec<T>::cp(l), x, bb, t, omega,
             zero_guess ? 1 : 0);
    std::swap(x, t);
  } else if (smoother == 1) {
    if (!zero_guess) Prec<T>::residual(h, l, box_grid(l.b), x, bb, r, -1, false);
    launch_v(h, Prec<T>::tri, lg, lb, lsm, l.b, zero_guess ? bb : r, Asp, Prec<T>::inv(l), Prec<T>::cp(l), x,
             omega, zero_guess ? 1 : 0, -1);
  } else if (smoother == 2) {
    if (zero_guess) vmemset(h, x, l.b.n() * sizeof(T));
    for (int color = 0; color < 2; color++) {
      const bool skip_res = zero_guess && color == 0;  // x = 0: r = rhs
      if (!skip_res) Prec<T>::residual(h, l, box_grid(l.b), x, bb, r, color, false);
      launch_v(h, Prec<T>::tri, lg, lb, lsm, l.b, skip_res ? bb : r, Asp, Prec<T>::inv(l), Prec<T>::cp(l), x,
               omega, 0, color);
    }
  } else if (fused_level<T>(l, smoother)) {
    // checkerboard zebra, residual in the line kernel: the first colour reads
    // x and writes its columns to t, the second reads its own colour from x
    // and the first colour from t and writes its columns to t
    const int nh = (l.b.nx + 1) / 2;
    dim3 cg((nh + TI - 1) / TI, l.b.nz);
    Prec<T>::fused(h, l, cg, lb, lsm, x, x, bb, t, omega, zero_guess, zero_guess, 2);
    Prec<T>::fused(h, l, cg, lb, lsm, x, t, bb, t, omega, zero_guess, false, 3);
    std::swap(x, t);
  } else {
    // zebra by checkerboard columns: colour (i + k) % 2 == c; the colour's
    // residuals go to split positions (r of the natural rhs when x = 0).
    // From a zero guess the first colour's line kernel does not read x; on
    // a split level it also writes the other colour's zeros (no clearing
    // pass), elsewhere x is cleared first.
    const bool split = split_level<T>(h, li, smoother);
    if (zero_guess && !split) vmemset(h, x, l.b.n() * sizeof(T));
    const int nh = (l.b.nx + 1) / 2;
    dim3 cg((nh + TI - 1) / TI, l.b.nz), rg((nh + 127) / 128, l.b.ny, l.b.nz);
    for (int color = 0; color < 2; color++) {
      const bool skip_res = zero_guess && color == 0;
      if (!skip_res) Prec<T>::residual(h, l, rg, x, bb, r, 2 + color, split);
      const auto tri = split ? Prec<T>::tri_split : Prec<T>::tri;
      launch_v(h, tri, cg, lb, lsm, l.b, skip_res ? bb : r, Asp, Prec<T>::inv(l), Prec<T>::cp(l), x, omega,
               skip_res ? (split ? 2 : 1) : 0, (skip_res ? 4 : 2) + color);
    }
  }
  prof_end(h, li);
}

template <typename T>
void vcycle(vfs_poisson *h, int li, int nu1, int nu2, T omega, int smoother) {
  Level &l = h->L[li];
  T **v = Prec<T>::v(l);
  T *x = v[0], *bb = v[1], *r = v[2], *t = v[3];
  if (li == (int)h->L.size() - 1) {
    launch_v(h, Prec<T>::coarsest, (int)((l.b.n() + 7) / 8), 256, 0, l.nd, l.dmap, l.didx, l.dinv, bb, x,
             (int)l.b.n());
    Prec<T>::xfinal(l) = x;
    return;
  }
  if (nu1 == 0) vmemset(h, x, l.b.n() * sizeof(T));
  for (int s = 0; s < nu1; s++) smooth<T>(h, l, li, smoother, s == 0, omega, x, t, bb, r);
  if ((smoother == 3 || smoother == 4) && nu1 > 0 && omega == (T)1) {
    // the second colour's lines were just solved exactly (omega 1), so its
    // residual is zero up to rounding: form the first colour's only
    const int nh = (l.b.nx + 1) / 2;
    vmemset(h, r, l.b.n() * sizeof(T));
    Prec<T>::residual(h, l, dim3((nh + 127) / 128, l.b.ny, l.b.nz), x, bb, r, 6, split_level<T>(h, li, smoother));
  } else {
    Prec<T>::residual(h, l, box_grid(l.b), x, bb, r, -1, split_level<T>(h, li, smoother));
  }
  Level &q = h->L[li + 1];
  launch_v(h, Prec<T>::restrict_, box_grid(q.b), 128, 0, l.b, q.b, l.cx, l.cy, l.cz, r, Prec<T>::w(l), q.blank,
           Prec<T>::v(q)[1]);
  vcycle<T>(h, li + 1, nu1, nu2, omega, smoother);
  const auto prolong = split_level<T>(h, li, smoother) ? Prec<T>::prolong_split : Prec<T>::prolong;
  launch_v(h, prolong, dim3((l.b.nx + 127) / 128, (l.b.ny + 1) / 2, l.b.nz), 128, 0, l.b, q.b, l.cx, l.cy, l.cz,
           (const T *)Prec<T>::xfinal(q), q.blank, l.blank, x, 1);
  for (int s = 0; s < nu2; s++) smooth<T>(h, l, li, smoother, false, omega, x, t, bb, r);
  Prec<T>::xfinal(l) = x;
}

// Run one V-cycle on level 0 (rhs already in level 0's b buffer).
template <typename T>
int run_vcycle(vfs_poisson *h, const vfs_solve_opts &o) {
  const int p = std::is_same<T, float>::value ? 0 : 1;
  h->pdl_prev = false;  // the V-cycle's first kernel waits for all earlier work
  if (!o.use_graphs || h->prof) {  // live kernel timing runs the V-cycle without a graph
    h->pcount = 0;
    vcycle<T>(h, 0, o.nu1, o.nu2, (T)o.omega, o.smoother);
    return VFS_OK;
  }
  const int key[4] = {o.nu1, o.nu2, (int)h->prof, o.smoother};
  vfs_poisson::GraphSlot *slot = nullptr, *victim = &h->gslot[p][0];
  for (auto &g : h->gslot[p]) {
    if (g.exec && g.omega == o.omega && std::equal(key, key + 4, g.params)) { slot = &g; break; }
    if (!g.exec || (victim->exec && g.used < victim->used)) victim = &g;
  }
  if (!slot) {
    slot = victim;
    h->pcount = 0;
    if (slot->exec) cudaGraphExecDestroy(slot->exec);
    *slot = vfs_poisson::GraphSlot{};
    cudaGraph_t graph;
    int64_t before = h->launches;
    CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    vcycle<T>(h, 0, o.nu1, o.nu2, (T)o.omega, o.smoother);
    CUDA_TRY(cudaStreamEndCapture(h->stream, &graph));
    slot->nodes = h->launches - before;
    h->launches = before;
    cudaError_t e = cudaGraphInstantiate(&slot->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      cudaGetLastError();
      slot->exec = nullptr;
      return fail(VFS_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    std::copy(key, key + 4, slot->params);
    slot->omega = o.omega;
    slot->xfinal0 = Prec<T>::xfinal(h->L[0]);
  }
  // the buffer holding the result depends on the captured sweeps (the fused
  // ones swap x and t): each graph's own
  Prec<T>::xfinal(h->L[0]) = static_cast<T *>(slot->xfinal0);
  slot->used = ++h->gclock;
  CUDA_TRY(cudaGraphLaunch(slot->exec, h->stream));
  h->launches += slot->nodes;
  return VFS_OK;
}

// z = M (s v): aj row scaling, one V-cycle of the chosen precision, back to
// FP64.  With sinv64 / sinv32 (device) set, v is also multiplied by
// sinv64[0] (FP64 V-cycle) or sinv32[0] (FP32 V-cycle).
int precondition(vfs_poisson *h, const double *v, double s, const double *sinv64, const float *sinv32, double *z,
                 const vfs_solve_opts &o) {
  Level &l0 = h->L[0];
  const size_t n = h->box.n();
  if (o.precision == 0) {
    const int snx = split_level<float>(h, 0, o.smoother) ? l0.b.nx : 0;
    LAUNCH(h, k_scale_to32, lin_grid(n), 256, n, v, (float)s, sinv32, h->scale32, l0.v32[1], snx);
    TRY(run_vcycle<float>(h, o));
    LAUNCH(h, k_to64, lin_grid(n), 256, n, (const float *)l0.xfinal32, (const double *)nullptr, z, snx);
  } else {
    LAUNCH(h, k_scale_to, kRedBlocks, 256, n, v, s, sinv64, h->scale, l0.v64[1]);
    TRY(run_vcycle<double>(h, o));
    LAUNCH(h, k_to64, lin_grid(n), 256, n, (const float *)nullptr, (const double *)l0.xfinal64, z, 0);
  }
  return VFS_OK;
}

// Add the level-0 sweep timings of the last V-cycle (the stream has been
// synchronised since it ran).
void prof_collect(vfs_poisson *h) {
  if (!h->prof) return;
  for (int q = 0; q < h->pcount; q++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->pev[0][q], h->pev[1][q]) == cudaSuccess) {
      h->prof_ms += ms;
      h->prof_bytes += h->pbytes[q];
      h->prof_launches++;
    } else {
      cudaGetLastError();
    }
  }
}

// reduce `nrow` rows of `nb` partials on the device and read them back
int reduce_read(vfs_poisson *h, int nb, int nrow, double *out) {
  LAUNCH(h, k_reduce_rows, nrow, 1024, h->partial, nb, nrow, h->red);
  CUDA_TRY(cudaMemcpyAsync(h->hbuf, h->red, nrow * 8, cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  for (int q = 0; q < nrow; q++) out[q] = h->hbuf[q];
  return VFS_OK;
}

// r = b - A x in FP64 and ||r||: the residual kernel without a reduction,
// then the fixed-shape sum of squares (faster than block partials formed in
// the stencil kernel, whose barriers hold its loads back)
int residual_norm(vfs_poisson *h, const double *x, double *r, double *norm) {
  LAUNCH(h, k_residual64r, box_grid(h->box), 128, h->box, h->A0, x, h->b, r);
  LAUNCH(h, k_sumsq, kRedBlocks, 256, h->box.n(), r, h->partial);
  double s;
  TRY(reduce_read(h, kRedBlocks, 1, &s));
  *norm = std::sqrt(s);
  return VFS_OK;
}

int ensure_krylov(vfs_poisson *h, int m);
void resolve_opts(vfs_solve_opts &o);
// hbuf offset of the history combinations' coefficients (kHistMax + 2)
constexpr int kHistStage = 960;

// ---- history projection of the initial guess (Fischer's projection for
// successive right-hand sides, CMAME 163 (1998) 193-204) ----
HistPtrs hist_ptrs(double *const *a, int k) {
  HistPtrs p{};
  for (int j = 0; j < k; j++) p.p[j] = a[j];
  return p;
}

constexpr uint64_t kHistMixed = ~uint64_t(0);

// difference slot of the i-th newest difference
int hist_slot(const vfs_poisson *h, int i) {
  const int nd = h->hist_cap - 1;
  return ((h->hist_head - 1 - i) % nd + nd) % nd;
}

// the projection's basis under the current operator assembly: Y_n, then the
// differences whose ends both belong to it, newest first (their slots in
// sl); returns its size, 0 when the newest solution is of another assembly
// (a moving mask makes the stored images stale: they are not recomputed)
int hist_fresh(const vfs_poisson *h, int *sl) {
  if (!h->hist_cnt || h->hist_vn != h->op_version) return 0;
  int nf = 1;
  for (int i = 0; i < h->hist_cnt - 1; i++) {
    const int q = hist_slot(h, i);
    if (h->hist_ver[q] != h->op_version) break;
    sl[nf++ - 1] = q;
  }
  return nf;
}

// store a converged solve: the iterate x and its image b - r (V_0 holds the
// solve's final FP64 residual r = b - A x) under the current assembly, as
// the new X_n, Y_n and, from the second solve on, the difference from the
// previous newest in the ring (over the oldest difference when it is full)
int hist_push(vfs_poisson *h) {
  if (!h->hist_cap) return VFS_OK;
  const size_t n = h->box.n();
  HistPtrs E{};
  if (h->hist_cnt == 0 || h->hist_cap == 1) {
    launch_hist_push(h->stream, kRedBlocks, n, h->x, h->b, h->V[0], h->hist_Xn, h->hist_Yn, nullptr, nullptr, E, 0,
                     true, h->partial);
    h->launches++;
    TRY(reduce_read(h, kRedBlocks, 1, &h->hist_Gnn));
    h->hist_vn = h->op_version;
    h->hist_cnt = 1;
    return VFS_OK;
  }
  const int s = h->hist_head, nd = h->hist_cap - 1;
  // the differences that stay: all stored ones but the slot written now
  const int keep = std::min(h->hist_cnt - 1, nd - 1);
  int win[kHistMax];
  for (int i = 0; i < keep; i++) {
    win[i] = hist_slot(h, i);
    E.p[i] = h->hist_Y[win[i]];
  }
  launch_hist_push(h->stream, kRedBlocks, n, h->x, h->b, h->V[0], h->hist_Xn, h->hist_Yn, h->hist_X[s],
                   h->hist_Y[s], E, keep, false, h->partial);
  h->launches++;
  double d[kHistMax + 3];
  TRY(reduce_read(h, kRedBlocks, keep + 3, d));
  const double ee = d[keep], ye = d[keep + 1];
  for (int i = 0; i < keep; i++) {
    h->hist_G[s][win[i]] = h->hist_G[win[i]][s] = d[i];
    h->hist_Gn[win[i]] += d[i];  // Y_new . E_j = Y_old . E_j + E_new . E_j
  }
  h->hist_G[s][s] = ee;
  h->hist_Gn[s] = ye + ee;
  h->hist_Gnn = d[keep + 2];
  h->hist_ver[s] = h->hist_vn == h->op_version ? h->op_version : kHistMixed;
  h->hist_vn = h->op_version;
  h->hist_head = (s + 1) % nd;
  if (h->hist_cnt < h->hist_cap) h->hist_cnt++;
  return VFS_OK;
}

// the projection x = X c, r = b - Y c minimising ||b - Y c|| over the span of
// the stored images of the current assembly, in the basis Y_n, E_newest, ...:
// normal equations G c = B^T b by a Cholesky factorisation in that order,
// where a vector whose pivot falls below 1e-13 of its Gram diagonal adds
// nothing new and keeps the coefficient 0.  The images of successive
// solutions are nearly parallel; their differences are not, and their Gram
// entries were formed from the differences themselves, so that the
// factorisation resolves the directions a least-squares fit by orthogonal
// factors resolves (the raw images' Gram matrix loses them from about eight
// solutions on).  Y_n alone is in the span, so the result's residual is
// never above the previous step's phi's.  *rext receives the residual norm
// of the extrapolation 2 X_n - X_{n-1}, predicted from the Gram entries when
// both solutions are of the current assembly (else -1).
int hist_project(vfs_poisson *h, double *rnorm, double *bnorm, double *rext) {
  int sl[kHistMax];
  const int k = hist_fresh(h, sl);
  *rext = -1.;
  if (k == 0) return fail(VFS_ESTATE, "no stored solution of the current operator");
  const size_t n = h->box.n();
  double *Xp[kHistMax], *Yp[kHistMax];
  Xp[0] = h->hist_Xn;
  Yp[0] = h->hist_Yn;
  for (int i = 1; i < k; i++) {
    Xp[i] = h->hist_X[sl[i - 1]];
    Yp[i] = h->hist_Y[sl[i - 1]];
  }
  launch_hist_dots(h->stream, kRedBlocks, n, hist_ptrs(Yp, k), k, h->b, h->partial);
  h->launches++;
  double g[kHistMax + 1];
  TRY(reduce_read(h, kRedBlocks, k + 1, g));
  // the basis Gram matrix
  double G[kHistMax][kHistMax];
  G[0][0] = h->hist_Gnn;
  for (int i = 1; i < k; i++) {
    G[0][i] = G[i][0] = h->hist_Gn[sl[i - 1]];
    for (int j = 1; j < k; j++) G[i][j] = h->hist_G[sl[i - 1]][sl[j - 1]];
  }
  int ord[kHistMax], na = 0;
  double L[kHistMax][kHistMax] = {};
  for (int i = 0; i < k; i++) {
    double row[kHistMax];
    for (int q = 0; q < na; q++) {
      double v = G[i][ord[q]];
      for (int t = 0; t < q; t++) v -= row[t] * L[q][t];
      row[q] = v / L[q][q];
    }
    double piv = G[i][i];
    for (int t = 0; t < na; t++) piv -= row[t] * row[t];
    if (!(piv > 1e-13 * G[i][i])) continue;
    for (int t = 0; t < na; t++) L[na][t] = row[t];
    L[na][na] = std::sqrt(piv);
    ord[na++] = i;
  }
  double z[kHistMax], cc[kHistMax] = {}, c[kHistMax] = {};
  for (int p = 0; p < na; p++) {
    double v = g[ord[p]];
    for (int t = 0; t < p; t++) v -= L[p][t] * z[t];
    z[p] = v / L[p][p];
  }
  for (int p = na - 1; p >= 0; p--) {
    double v = z[p];
    for (int t = p + 1; t < na; t++) v -= L[t][p] * cc[t];
    cc[p] = v / L[p][p];
  }
  for (int p = 0; p < na; p++) c[ord[p]] = cc[p];
  if (h->phase) {
    // the coefficients of the stored solutions themselves: X_n gets c_0 + c_1,
    // X_{n-m} gets c_{m+1} - c_m (D_m = X_{n-m+1} - X_{n-m})
    double s1 = 0.;
    for (int m = 0; m < k; m++) s1 += std::fabs((m == 0 ? c[0] : -c[m]) + (m + 1 < k ? c[m + 1] : 0.));
    fprintf(stderr, "vfs history: basis %d, used %d, sum |c| over the solutions %.3g\n", k, na, s1);
  }
  for (int j = 0; j < k; j++) h->hbuf[kHistStage + j] = c[j];
  CUDA_TRY(cudaMemcpyAsync(h->hist_coef, h->hbuf + kHistStage, k * 8, cudaMemcpyHostToDevice, h->stream));
  launch_hist_combine(h->stream, kRedBlocks, n, hist_ptrs(Xp, k), hist_ptrs(Yp, k), k, h->hist_coef, h->b,
                      h->hist_x, h->hist_r, h->partial);
  h->launches++;
  double rr;
  TRY(reduce_read(h, kRedBlocks, 1, &rr));
  *rnorm = std::sqrt(std::max(rr, 0.));
  *bnorm = std::sqrt(std::max(g[k], 0.));
  if (k >= 2 && sl[0] == hist_slot(h, 0)) {
    // ||b - Y_n - E_newest||^2
    const double e2 = g[k] - 2. * (g[0] + g[1]) + G[0][0] + 2. * G[0][1] + G[1][1];
    *rext = std::sqrt(std::max(e2, 0.));
  }
  return VFS_OK;
}

// hist_er: from the stored images when both belong to the current
// assembly, otherwise by an operator apply
int hist_extrap(vfs_poisson *h, double *rnorm) {
  const int k = std::min(h->hist_cnt, 2);
  if (k == 0) return fail(VFS_ESTATE, "no stored solution");
  const size_t n = h->box.n();
  // X_n + D_newest (X_n alone with one stored solution)
  const int s0 = k > 1 ? hist_slot(h, 0) : 0;
  double *Xp[2] = {h->hist_Xn, k > 1 ? h->hist_X[s0] : nullptr};
  double *Yp[2] = {h->hist_Yn, k > 1 ? h->hist_Y[s0] : nullptr};
  const bool fresh = h->hist_vn == h->op_version && (k == 1 || h->hist_ver[s0] == h->op_version);
  h->hbuf[kHistStage + kHistMax] = 1.;
  h->hbuf[kHistStage + kHistMax + 1] = 1.;
  CUDA_TRY(cudaMemcpyAsync(h->hist_coef + kHistMax, h->hbuf + kHistStage + kHistMax, 2 * 8, cudaMemcpyHostToDevice,
                           h->stream));
  // (with stale images the combination's residual is formed again below)
  launch_hist_combine(h->stream, kRedBlocks, n, hist_ptrs(Xp, k), hist_ptrs(Yp, k), k, h->hist_coef + kHistMax,
                      h->b, h->hist_ex, h->hist_er, h->partial);
  h->launches++;
  if (fresh) {
    double rr;
    TRY(reduce_read(h, kRedBlocks, 1, &rr));
    *rnorm = std::sqrt(std::max(rr, 0.));
    return VFS_OK;
  }
  // cells that are no fluid rows under the current mask (a body moved over
  // them) drop the old solutions' values: 0 is their solution
  LAUNCH(h, k_mask_fluid, lin_grid(n), 256, n, h->rowtype0, h->hist_ex);
  return residual_norm(h, h->hist_ex, h->hist_er, rnorm);
}

// A candidate initial guess: its iterate, its FP64 residual and norm, the
// code reported for it (0 projection or previous phi, 1 network, 2
// extrapolation), and a V-cycle of its residual already formed (or null).
struct GuessCand {
  double *x, *r;
  double beta;
  int code;
  const double *zready;
  double est;
};

// The judge among candidate guesses.  Their FP64 residuals alone mislead:
// a least-squares fit of the residual can leave a large smooth error that
// has a small residual and that the preconditioned iteration removes
// slowly, while an extrapolation's larger residual can sit in components
// the first V-cycle removes.  Each candidate within kJudgeGate of the
// smallest residual is therefore rated by its estimated error: one V-cycle
// of its residual (the solver's default preconditioner), the fluid mean
// removed (the operator's constant null space), 2-norm.  The winner's
// V-cycle, divided by its residual norm, is Z_0 of the next solve.
constexpr double kJudgeGate = 32.;
int judge(vfs_poisson *h, GuessCand *c, int nc, int *win) {
  double bmin = c[0].beta;
  for (int i = 1; i < nc; i++) bmin = std::min(bmin, c[i].beta);
  int live[4], nl = 0;
  for (int i = 0; i < nc; i++) {
    c[i].est = -1.;
    if (c[i].beta <= kJudgeGate * bmin) live[nl++] = i;
  }
  h->z0_valid = false;
  if (nl == 1 || bmin == 0.) {
    int b = 0;
    for (int i = 1; i < nc; i++) if (c[i].beta < c[b].beta) b = i;
    *win = b;
    return VFS_OK;
  }
  vfs_solve_opts so;
  vfs_poisson_default_opts(&so);
  resolve_opts(so);
  TRY(ensure_krylov(h, std::max(h->m_alloc, 20)));
  const size_t n = h->box.n();
  int best = -1;
  const double *zbest = nullptr;
  for (int q = 0; q < nl; q++) {
    GuessCand &cd = c[live[q]];
    const double *z = cd.zready;
    if (!z) {
      TRY(precondition(h, cd.r, 1.0 / cd.beta, nullptr, nullptr, h->Z[1 + q], so));
      z = h->Z[1 + q];
    }
    LAUNCH(h, k_fluid_moments, kRedBlocks, 256, n, (const uint8_t *)h->fluid, z, 0., 0, h->partial);
    double m[2];
    TRY(reduce_read(h, kRedBlocks, 2, m));
    LAUNCH(h, k_fluid_moments, kRedBlocks, 256, n, (const uint8_t *)h->fluid, z, m[1] > 0. ? m[0] / m[1] : 0., 1,
           h->partial);
    double d;
    TRY(reduce_read(h, kRedBlocks, 1, &d));
    cd.est = cd.beta * std::sqrt(std::max(d, 0.));
    if (best < 0 || cd.est < c[best].est) {
      best = live[q];
      zbest = z;
    }
  }
  if (zbest != h->Z[0]) CUDA_TRY(cudaMemcpyAsync(h->Z[0], zbest, n * 8, cudaMemcpyDeviceToDevice, h->stream));
  h->z0_valid = true;
  h->z0_opts = so;
  *win = best;
  return VFS_OK;
}

// make candidate c the solver's iterate (warm_start 2): its buffer trades
// places with x (queued work holds the pointers it was launched with; none
// writes these buffers later) and its residual becomes FGMRES's start
void install_guess(vfs_poisson *h, GuessCand &c) {
  if (c.x != h->x) {
    double *old = h->x;
    h->x = c.x;
    if (h->gex == c.x) h->gex = old;
    else if (h->gnet == c.x) h->gnet = old;
    else if (h->hist_x == c.x) h->hist_x = old;
    else if (h->hist_ex == c.x) h->hist_ex = old;
  }
  h->r0 = c.r;
  h->r0_norm = c.beta;
  h->r0_valid = true;
}

// The history's candidates for the next solve's guess: the projection over
// the slots of the current assembly (code 0) and the extrapolation of the
// newest two solutions (code 2).  The extrapolation is formed only when it
// can pass the judge's gate: its residual, predicted from the Gram matrix
// when both solutions are of the current assembly, within kJudgeGate of the
// projection's.  *far: the prediction exceeds the projection's residual by
// more than kNetGate.  *bnorm: ||b||.
constexpr double kNetGate = 1024.;
int history_candidates(vfs_poisson *h, GuessCand *c, int *nc, double *bnorm, bool *far) {
  int sl[kHistMax];
  const int nf = hist_fresh(h, sl);
  *nc = 0;
  *far = false;
  if (nf) {
    double rp, re;
    TRY(hist_project(h, &rp, bnorm, &re));
    c[(*nc)++] = GuessCand{h->hist_x, h->hist_r, rp, 0, nullptr, -1.};
    if (h->hist_cnt < 2) return VFS_OK;  // the extrapolation would be the projection's vector
    if (re >= 0.) {
      *far = re > kNetGate * rp;
      if (re > kJudgeGate * rp) return VFS_OK;
    }
  } else {
    LAUNCH(h, k_sumsq, kRedBlocks, 256, h->box.n(), h->b, h->partial);
    double bb;
    TRY(reduce_read(h, kRedBlocks, 1, &bb));
    *bnorm = std::sqrt(std::max(bb, 0.));
  }
  double rex;
  TRY(hist_extrap(h, &rex));
  c[(*nc)++] = GuessCand{h->hist_ex, h->hist_er, rex, 2, nullptr, -1.};
  return VFS_OK;
}

// what the guess installed, for vfs_poisson_guess_report: per candidate
// code its residual relative to ||b|| and its estimated error
void guess_report(vfs_poisson *h, const GuessCand *c, int nc, int w, double bnorm) {
  for (int q = 0; q < 3; q++) h->guess_rel[q] = h->guess_est[q] = -1.;
  for (int i = 0; i < nc; i++) {
    h->guess_rel[c[i].code] = bnorm > 0. ? c[i].beta / bnorm : 0.;
    h->guess_est[c[i].code] = c[i].est;
  }
  h->guess_chosen = c[w].code;
}

int ensure_krylov(vfs_poisson *h, int m) {
  if (m <= h->m_alloc) return VFS_OK;
  for (auto p : h->V) dfree(h, p);
  for (auto p : h->Z) dfree(h, p);
  h->V.assign(m + 1, nullptr);
  h->Z.assign(m, nullptr);
  const size_t n = h->box.n();
  for (int q = 0; q <= m; q++) TRY(dalloc(h, &h->V[q], n));
  for (int q = 0; q < m; q++) TRY(dalloc(h, &h->Z[q], n));
  dfree(h, h->dV); dfree(h, h->dZ); dfree(h, h->coef); dfree(h, h->dsv); dfree(h, h->dsv32);
  TRY(dalloc(h, &h->dsv, 2 * (m + 1)));
  TRY(dalloc(h, &h->dsv32, m + 1));
  TRY(dalloc(h, &h->dV, m + 1));
  TRY(dalloc(h, &h->dZ, m));
  TRY(dalloc(h, &h->coef, m + 1));
  CUDA_TRY(cudaMemcpyAsync(h->dV, h->V.data(), (m + 1) * sizeof(double *), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->dZ, h->Z.data(), m * sizeof(double *), cudaMemcpyHostToDevice, h->stream));
  if (h->hbuf) cudaFreeHost(h->hbuf);
  CUDA_TRY(cudaMallocHost(&h->hbuf, 1024 * 8));
  h->m_alloc = m;
  return sync(h);
}

// omega 0 selects the smoother's own damping: 1 for the zebra
// Gauss-Seidel variants, 0.8 for line Jacobi (undamped line Jacobi does not
// converge as a smoother on the stretched curvilinear grids)
void resolve_opts(vfs_solve_opts &o) {
  if (o.omega == 0.) o.omega = o.smoother >= 2 ? 1.0 : 0.8;
}

int check_opts(const vfs_solve_opts &o) {
  if (!(o.rtol > 0) || o.max_it < 1 || o.restart < 1 || o.restart > 64 || o.nu1 < 0 || o.nu2 < 0 ||
      o.nu1 + o.nu2 < 1 || o.nu1 > 8 || o.nu2 > 8 || !(o.omega > 0 && o.omega <= 1.5) ||
      (o.precision != 0 && o.precision != 1) || o.smoother < 0 || o.smoother > 4 || (o.orth != 0 && o.orth != 1))
    return fail(VFS_EINVAL, "invalid solver options");
  return VFS_OK;
}

// One DCGS2 dots launch over basis vectors v0 .. v0+nv-1 (nv <= 8).
void gs_dots(vfs_poisson *h, int nv, int nb, size_t n, int v0, const double *u, const double *w, int first) {
  const double *const *Q = (const double *const *)h->dV;
  switch (nv) {
#define CASE(NV) \
  case NV: LAUNCH(h, k_gs_dots##NV, nb, 256, n, v0, Q, u, w, first, h->partial); break;
    CASE(0) CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8)
#undef CASE
  }
}

// One classical Gram-Schmidt dots launch over basis vectors v0 .. v0+nv-1
// (1 <= nv <= 8).
void cgs_dots(vfs_poisson *h, int nv, int nb, size_t n, int v0, const double *w) {
  const double *const *Q = (const double *const *)h->dV;
  switch (nv) {
#define CASE(NV) \
  case NV: LAUNCH(h, k_cgs_dots##NV, nb, 256, n, v0, Q, w, h->partial); break;
    CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8)
#undef CASE
  }
}

// hbuf offsets: the read-back of the speculative step 0 and its staging of
// the first basis norm (apart from the rows reduce_read and FGMRES use)
constexpr int kSpecHb = 620, kSpecStage = 610;

// Enqueue Arnoldi step jj of FGMRES: precondition V_jj (unless Z_jj holds it
// already: have_z), apply A, orthogonalise (orth 0 or DCGS2), reduce the new
// vector's norm and copy the Hessenberg data to hbuf + hb (orth 0: h at
// hb + 0..jj; the norm^2 at hb + kGsR + 3).
int arnoldi_enqueue(vfs_poisson *h, int jj, int nbd, const vfs_solve_opts &o, int hb, bool have_z = false) {
  const size_t n = h->box.n();
  const double *const *dV = (const double *const *)h->dV;
  if (!have_z) TRY(precondition(h, h->V[jj], 1.0, h->dsv + 2 * jj + 1, h->dsv32 + jj, h->Z[jj], o));
  if (h->phase && hb == 0) cudaEventRecord(h->phev[1], h->stream);
  double *w = h->V[jj + 1];
  LAUNCH(h, k_apply64, box_grid(h->box), 128, h->box, h->A0, h->Z[jj], w);
  if (h->phase && hb == 0) cudaEventRecord(h->phev[2], h->stream);
  if (o.orth == 0) {
    for (int v0 = 0; v0 <= jj; v0 += 8) cgs_dots(h, std::min(8, jj + 1 - v0), nbd, n, v0, w);
    LAUNCH(h, k_cgs_reduce, jj + 1, 1024, h->partial, nbd, h->dsv, h->red);
    LAUNCH(h, k_cgs_update, nbd, 256, n, jj + 1, dV, h->red, w, h->partial);
  } else {
    for (int v0 = 0; v0 == 0 || v0 < jj; v0 += 8)
      gs_dots(h, std::min(8, jj - v0), nbd, n, v0, h->V[jj], w, v0 == 0);
    LAUNCH(h, k_gs_reduce, 2 * jj + 2, 1024, h->partial, nbd, jj, h->red);
    LAUNCH(h, k_gs_coef, 1, 32, jj, h->red);
    LAUNCH(h, k_gs_update, nbd, 256, n, jj, dV, h->red, h->V[jj], w, h->partial);
  }
  LAUNCH(h, k_reduce_norm, 1, 1024, h->partial, nbd, h->dsv + 2 * (jj + 1), h->dsv32 + jj + 1);
  if (h->phase && hb == 0) cudaEventRecord(h->phev[3], h->stream);
  CUDA_TRY(cudaMemcpyAsync(h->hbuf + hb, h->red, (o.orth == 0 ? jj + 1 : kGsR + 3) * 8, cudaMemcpyDeviceToHost,
                           h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->hbuf + hb + kGsR + 3, h->dsv + 2 * (jj + 1), 8, cudaMemcpyDeviceToHost, h->stream));
  return VFS_OK;
}

// A solve whose initial residual is within this factor of rtol runs its
// V-cycles with opts.nu2_near post sweeps.
constexpr double kNearStart = 32.;

// The options of a solve that may resume from the speculative step 0: the
// same preconditioner and orthogonalisation.
bool spec_matches(const vfs_solve_opts &a, const vfs_solve_opts &b) {
  return a.precision == b.precision && a.nu1 == b.nu1 && a.nu2 == b.nu2 && a.omega == b.omega &&
         a.smoother == b.smoother && a.orth == b.orth && a.restart >= 1 && a.max_it >= 1;
}

// FGMRES(m) (flexible GMRES: the preconditioned vectors Z_j are kept and
// x = x0 + Z y).  The basis vectors stay unnormalised in memory; their
// norms and inverse norms are reduced on the device (dsv) and every use
// scales by them.
// orth 0, classical Gram-Schmidt in one pass: step j preconditions
// V_j / ||V_j||, applies A, forms h_i = Q_i.w / ||Q_i|| for i <= j in one
// pass and w - sum h_i Q_i / ||Q_i|| with its norm in another; column j is
// final at once.
// orth 1, delayed reorthogonalisation (DCGS2):
// step j preconditions the pending vector V_j (projected once, divided by its
// norm reduced on the device), applies A, and one Gram-Schmidt round
// finishes V_j (reorthogonalised, normalised) and projects A z_j into
// V_{j+1}.  Finishing V_j = (u - Q a) / r corrects Hessenberg column j-1
// (H[0..j-1, j-1] += a, H[j, j-1] = r) and its Givens rotation is formed
// again; column j enters with the norm of the once-projected vector, which
// gives the residual estimate of the convergence test.  One host read-back
// per step.
int fgmres(vfs_poisson *h, const vfs_solve_opts &oin, vfs_solve_stats *st) {
  // the options of this solve: nu2_near post sweeps when it starts within
  // kNearStart x rtol (set once the initial residual is known)
  vfs_solve_opts o = oin;
  const size_t n = h->box.n();
  const int m = o.restart;
  // a larger basis is allocated afresh: the speculative step's vectors go
  if (m > h->m_alloc) h->spec_valid = h->z0_valid = false;
  TRY(ensure_krylov(h, m));
  const int nbd = (int)((n + 256 * kGsTile - 1) / (256 * kGsTile));
  double bn2;
  LAUNCH(h, k_sumsq, kRedBlocks, 256, n, h->b, h->partial);
  TRY(reduce_read(h, kRedBlocks, 1, &bn2));
  const double bn = std::sqrt(bn2);
  int it = 0;
  double rel = 0., beta = 0.;
  // Hraw: Hessenberg columns as formed; R: the same after the Givens rotations
  std::vector<double> Hraw((size_t)(m + 1) * m, 0.), R((size_t)(m + 1) * m, 0.), cs(m), sn(m), gv(m + 1),
      gsave(m + 1), y(m);
  if (bn == 0.) {
    CUDA_TRY(cudaMemsetAsync(h->x, 0, n * 8, h->stream));
    st->initial_rel_residual = 0.;
    st->rel_residual = 0.;
    st->iterations = 0;
    return VFS_OK;
  }
  // step 0 enqueued by the learned guess (V_0 = the guess's residual)
  const bool resume = o.warm_start == 2 && h->r0_valid && h->spec_valid && spec_matches(o, h->spec_opts);
  // Z_0 formed by the guess's judge (one V-cycle of the installed residual)
  const bool have_z0 = !resume && o.warm_start == 2 && h->r0_valid && h->z0_valid && spec_matches(o, h->z0_opts);
  h->spec_valid = false;
  h->z0_valid = false;
  if (resume) {
    beta = h->r0_norm;
  } else if (o.warm_start == 2 && h->r0_valid) {  // residual formed by the guess
    CUDA_TRY(cudaMemcpyAsync(h->V[0], h->r0, n * 8, cudaMemcpyDeviceToDevice, h->stream));
    beta = h->r0_norm;
  } else if (o.warm_start) {
    TRY(residual_norm(h, h->x, h->V[0], &beta));
  } else {  // zero initial guess: r = b
    CUDA_TRY(cudaMemcpyAsync(h->V[0], h->b, n * 8, cudaMemcpyDeviceToDevice, h->stream));
    beta = bn;
  }
  rel = beta / bn;
  st->initial_rel_residual = rel;
  if (o.nu2_near > 0 && rel <= kNearStart * o.rtol) o.nu2 = o.nu2_near;
  // rotate the formed column j by rotations 0..j-1, form rotation j and
  // apply it to the right-hand side gv
  auto rotate = [&](int j) {
    for (int i = 0; i <= j + 1; i++) R[(size_t)i * m + j] = Hraw[(size_t)i * m + j];
    for (int i = 0; i < j; i++) {
      const double a = R[(size_t)i * m + j], b2 = R[(size_t)(i + 1) * m + j];
      R[(size_t)i * m + j] = cs[i] * a + sn[i] * b2;
      R[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * b2;
    }
    const double a = R[(size_t)j * m + j], b2 = R[(size_t)(j + 1) * m + j];
    const double den = std::sqrt(a * a + b2 * b2);
    cs[j] = den != 0. ? a / den : 1.;
    sn[j] = den != 0. ? b2 / den : 0.;
    R[(size_t)j * m + j] = den;
    R[(size_t)(j + 1) * m + j] = 0.;
    gv[j + 1] = -sn[j] * gv[j];
    gv[j] = cs[j] * gv[j];
  };
  while (rel > o.rtol && it < o.max_it) {
    h->hbuf[400] = beta * beta;  // pinned staging: pageable copies cost ~0.5 ms each
    h->hbuf[401] = 1.0 / beta;
    reinterpret_cast<float *>(h->hbuf + 402)[0] = (float)(1.0 / beta);
    CUDA_TRY(cudaMemcpyAsync(h->dsv, h->hbuf + 400, 16, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->dsv32, h->hbuf + 402, 4, cudaMemcpyHostToDevice, h->stream));
    std::fill(gv.begin(), gv.end(), 0.);
    std::fill(Hraw.begin(), Hraw.end(), 0.);
    gv[0] = beta;
    int jj = 0;
    for (; jj < m && it < o.max_it; jj++) {
      const auto t0 = h->phase ? std::chrono::steady_clock::now() : std::chrono::steady_clock::time_point();
      if (h->phase) cudaEventRecord(h->phev[0], h->stream);
      const bool pre = resume && it == 0 && jj == 0;  // enqueued by the guess
      const int hb = pre ? kSpecHb : 0;
      if (!pre) TRY(arnoldi_enqueue(h, jj, nbd, o, 0, have_z0 && it == 0 && jj == 0));
      const auto t2 = h->phase ? std::chrono::steady_clock::now() : t0;
      TRY(sync(h));
      const auto t3 = h->phase ? std::chrono::steady_clock::now() : t0;
      if (h->phase && !pre) {
        h->host_ms[0] += std::chrono::duration<double, std::milli>(t2 - t0).count();
        h->host_ms[2] += std::chrono::duration<double, std::milli>(t3 - t2).count();
        float a = 0.f, b = 0.f, c = 0.f;
        cudaEventElapsedTime(&a, h->phev[0], h->phev[1]);
        cudaEventElapsedTime(&b, h->phev[1], h->phev[2]);
        cudaEventElapsedTime(&c, h->phev[2], h->phev[3]);
        h->phase_ms[0] += a; h->phase_ms[1] += b; h->phase_ms[2] += c;
      }
      prof_collect(h);
      it++;
      const double *rb = h->hbuf + hb;
      const double wn = std::sqrt(std::max(rb[kGsR + 3], 0.));
      if (o.orth == 0) {  // column jj is final: H[i, jj] = Q_i.w / ||Q_i||
        for (int i = 0; i <= jj; i++) Hraw[(size_t)i * m + jj] = rb[i];
      } else {
        const double r = h->hbuf[kGsR], hj = h->hbuf[kGsR + 1];
        if (jj > 0) {
          // V_jj lies in the span of the finished vectors: column jj-1 was a
          // breakdown; the cycle ends with the columns before this step
          if (!(r > 0.)) break;
          for (int i = 0; i < jj; i++) Hraw[(size_t)i * m + jj - 1] += h->hbuf[i];
          Hraw[(size_t)jj * m + jj - 1] = r;
          gv = gsave;
          rotate(jj - 1);
        }
        for (int i = 0; i < jj; i++) Hraw[(size_t)i * m + jj] = h->hbuf[kGsB + i];
        Hraw[(size_t)jj * m + jj] = hj;
        gsave = gv;
      }
      Hraw[(size_t)(jj + 1) * m + jj] = wn;
      rotate(jj);
      if (h->phase) h->host_ms[3] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (std::fabs(gv[jj + 1]) / bn <= o.rtol || wn == 0.) { jj++; break; }
    }
    for (int i = jj - 1; i >= 0; i--) {
      double s = gv[i];
      for (int q = i + 1; q < jj; q++) s -= R[(size_t)i * m + q] * y[q];
      y[i] = R[(size_t)i * m + i] != 0. ? s / R[(size_t)i * m + i] : 0.;
    }
    for (int i = 0; i < jj; i++) h->hbuf[400 + 64 + i] = y[i];
    CUDA_TRY(cudaMemcpyAsync(h->coef, h->hbuf + 464, jj * 8, cudaMemcpyHostToDevice, h->stream));
    LAUNCH(h, k_axpy_multi, kRedBlocks, 256, n, jj, (const double *const *)h->dZ, h->coef, h->x);
    TRY(residual_norm(h, h->x, h->V[0], &beta));
    rel = beta / bn;
  }
  st->iterations = it;
  st->rel_residual = rel;
  if (h->phase) {
    fprintf(stderr, "vfs phase ms: precondition %.3f apply %.3f gram-schmidt %.3f (iterations %d)\n",
            h->phase_ms[0], h->phase_ms[1], h->phase_ms[2], it);
    fprintf(stderr, "vfs host ms: enqueue %.3f wait %.3f iteration-wall %.3f\n", h->host_ms[0], h->host_ms[2],
            h->host_ms[3]);
    h->phase_ms[0] = h->phase_ms[1] = h->phase_ms[2] = 0.;
    for (double &v : h->host_ms) v = 0.;
  }
  return VFS_OK;
}

}  // namespace

namespace vfs {
void set_last_error(const std::string &msg) { g_err = msg; }

int ibm_context(vfs_poisson *h, IbmContext *c) {
  if (!h->have_grid) return fail(VFS_ESTATE, "set_grid must come before the surface search");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(VFS_ECUDA, "cudaSetDevice failed");
  c->stream = h->stream;
  c->g = h->g;
  c->cent = h->met.cent;
  c->launches = &h->launches;
  c->bodies = &h->ibm_bodies;
  c->scratch = &h->ibm_scratch;
  return VFS_OK;
}
}  // namespace vfs

// ============================== C ABI =====================================

extern "C" {

const char *vfs_last_error(void) { return g_err.c_str(); }

void vfs_poisson_default_opts(vfs_solve_opts *o) {
  o->rtol = 1e-8;
  o->max_it = 200;
  o->restart = 20;
  o->precision = 0;
  o->nu1 = 1;
  o->nu2 = 2;
  o->omega = 0.0;
  o->use_graphs = 1;
  o->coarsest_max = 256;
  o->warm_start = 0;
  o->smoother = 4;
  o->orth = 0;
  o->nu2_near = 0;
}

int vfs_poisson_create(const vfs_grid_desc *gd, vfs_poisson **out) {
  if (!gd || !out) return fail(VFS_EINVAL, "null argument");
  *out = nullptr;
  if (gd->mx < 3 || gd->my < 3 || gd->mz < 3) return fail(VFS_EINVAL, "grid needs at least one interior cell per direction");
  const int nx = gd->mx - 2, ny = gd->my - 2, nz = gd->mz - 2;
  const bool px = gd->i_periodic || gd->ii_periodic, py = gd->j_periodic || gd->jj_periodic,
             pz = gd->k_periodic || gd->kk_periodic;
  if ((px && nx < 3) || (py && ny < 3) || (pz && nz < 3))
    return fail(VFS_EINVAL, "a periodic direction needs at least 3 interior cells");
  if (ny > kLineMaxThreads * kLineChunk)
    return fail(VFS_EINVAL, "j-lines longer than " + std::to_string(kLineMaxThreads * kLineChunk) +
                                " cells are not supported");
  if ((size_t)gd->mx * gd->my * gd->mz * NSLOT >= ((size_t)1 << 32))
    return fail(VFS_EINVAL, "grid too large: 19 operator planes must stay below 2^32 entries");
  vfs_poisson *h = new vfs_poisson();
  h->desc = *gd;
  h->g = Grid{gd->mx, gd->my, gd->mz, px, py, pz};
  h->box = Box{nx, ny, nz, px, py, pz};
  cudaGetDevice(&h->device);
  auto bail = [&](int rc) { vfs_poisson_destroy(h); return rc; };
  // a blocking stream: work the caller queued on the legacy default stream
  // (e.g. filling a device input array) completes before ours starts
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamDefault) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return fail(VFS_ECUDA, "cudaStreamCreate failed (no usable GPU?)");
  }
  cudaEventCreate(&h->ev0);
  cudaEventCreate(&h->ev1);
  for (int a = 0; a < 2; a++)
    for (int q = 0; q < 16; q++) cudaEventCreate(&h->pev[a][q]);
  for (int q = 0; q < 4; q++) cudaEventCreate(&h->phev[q]);
  {
    const char *e = getenv("VFS_PHASE_TIMING");
    h->phase = e && e[0] == '1';
    const char *sp = getenv("VFS_GUESS_SPECULATE");
    h->spec_enable = !(sp && sp[0] == '0');
    const char *lc = getenv("VFS_LINE_COLUMNS");
    h->line_cols_cap = lc ? atoi(lc) : 0;
    const char *pd = getenv("VFS_PDL");
    h->pdl = !(pd && pd[0] == '0');
    const char *inc = getenv("VFS_INCREMENTAL");
    h->inc_enable = !(inc && inc[0] == '0');
  }
  const size_t N = h->g.n(), n = h->box.n();
  int rc;
  if ((rc = dalloc(h, &h->coor, 3 * N)) || (rc = dalloc(h, &h->nvert, N)) || (rc = dalloc(h, &h->ucont, 3 * N)) ||
      (rc = dalloc(h, &h->phi_da, N)) || (rc = dalloc(h, &h->p_da, N)) || (rc = dalloc(h, &h->stage, 3 * N)) ||
      (rc = alloc_metrics(h, h->g, h->met)) || (rc = dalloc(h, &h->A0, n * NSLOT)) ||
      (rc = dalloc(h, &h->scale, n)) || (rc = dalloc(h, &h->scale32, n)) || (rc = dalloc(h, &h->pc, 12 * n)) ||
      (rc = dalloc(h, &h->aj_box, n)) ||
      (rc = dalloc(h, &h->rowtype0, n)) || (rc = dalloc(h, &h->fluid, n)) || (rc = dalloc(h, &h->gid_box, n)) ||
      (rc = dalloc(h, &h->gid_da, N)) || (rc = dalloc(h, &h->b, n)) || (rc = dalloc(h, &h->x, n)) ||
      (rc = dalloc(h, &h->r, n)) || (rc = dalloc(h, &h->red, 512)) || (rc = dalloc(h, &h->total, 1)))
    return bail(rc);
  const int nblk = (int)((n + 1023) / 1024);
  if ((rc = dalloc(h, &h->blk, nblk))) return bail(rc);
  {
    const dim3 gb = guess_grid(h->box);  // 14 rows of per-block partials (k_guess_gram)
    h->partial_len = std::max<size_t>({n / 16 + 65536, (size_t)(kGsUU + 2) * ((n + 2047) / 2048) + 4096,
                                       (size_t)16 * gb.x * gb.y * gb.z + 4096});
  }
  if ((rc = dalloc(h, &h->partial, h->partial_len))) return bail(rc);
  if (cudaMallocHost(&h->hbuf, 1024 * 8) != cudaSuccess) { cudaGetLastError(); return bail(fail(VFS_ENOMEM, "pinned alloc")); }
  cudaMemsetAsync(h->phi_da, 0, N * 8, h->stream);
  cudaMemsetAsync(h->x, 0, n * 8, h->stream);
  if ((rc = sync(h))) return bail(rc);
  *out = h;
  return VFS_OK;
}

void vfs_poisson_destroy(vfs_poisson *h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  for (void *p : h->allocs) cudaFree(p);
  h->allocs.clear();
  for (void *p : h->ibm_scratch.buf)
    if (p) cudaFree(p);
  if (h->ibm_scratch.bbox) cudaFree(h->ibm_scratch.bbox);
  if (h->ibm_scratch.hits) cudaFree(h->ibm_scratch.hits);
  for (auto &b : h->ibm_bodies) {
    if (b.nodes) cudaFree(b.nodes);
    if (b.tri) cudaFree(b.tri);
  }
  if (h->hbuf) cudaFreeHost(h->hbuf);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (int a = 0; a < 2; a++)
    for (int q = 0; q < 16; q++)
      if (h->pev[a][q]) cudaEventDestroy(h->pev[a][q]);
  for (int q = 0; q < 4; q++)
    if (h->phev[q]) cudaEventDestroy(h->phev[q]);
  if (h->ev_feat) cudaEventDestroy(h->ev_feat);
  if (h->side) cudaStreamDestroy(h->side);
  for (cudaEvent_t e : h->dl_ev)
    if (e) cudaEventDestroy(e);
  if (h->dl_stream) cudaStreamDestroy(h->dl_stream);
  if (h->stream && h->own_stream) cudaStreamDestroy(h->stream);
  cudaGetLastError();
  delete h;
}

int vfs_poisson_set_grid(vfs_poisson *h, const double *coor, const double *const *fm) {
  if (!h || !coor) return fail(VFS_EINVAL, "null argument");
  h->hier_cmax = -1;  // new coordinates: the next mask builds the hierarchy afresh
  h->ibm_scratch.bbox_valid = false;  // and the next search bounds the new centres
  h->nvert_prev_valid = false;        // and the next mask fills every row
  const size_t N = h->g.n();
  TRY(upload(h, h->coor, coor, 3 * N));
  TRY(form_metrics(h, h->g, h->coor, h->met));
  if (fm) {
    double *vec[9] = {h->met.icsi, h->met.ieta, h->met.izet, h->met.jcsi, h->met.jeta,
                      h->met.jzet, h->met.kcsi, h->met.keta, h->met.kzet};
    double *sca[4] = {h->met.iaj, h->met.jaj, h->met.kaj, h->met.aj};
    for (int q = 0; q < 9; q++) if (fm[q]) TRY(upload(h, vec[q], fm[q], 3 * N));
    for (int q = 0; q < 4; q++) if (fm[9 + q]) TRY(upload(h, sca[q], fm[9 + q], N));
  }
  TRY(face_coef(h, h->g, h->met));
  LAUNCH(h, k_projection_coef, box_grid(h->box), 128, h->g, h->box, h->met, h->pc);
  TRY(sync(h));
  h->have_grid = true;
  h->have_nvert = false;
  return VFS_OK;
}

int vfs_poisson_set_nvert(vfs_poisson *h, const double *nvert) {
  if (!h || !nvert) return fail(VFS_EINVAL, "null argument");
  if (!h->have_grid) return fail(VFS_ESTATE, "set_grid must come before set_nvert");
  const size_t N = h->g.n(), n = h->box.n();
  const auto tp0 = std::chrono::steady_clock::now();
  vfs_solve_opts o;
  vfs_poisson_default_opts(&o);
  const bool refills = hierarchy_refills(h, o.coarsest_max);
  // a new mask on a filled hierarchy without a level set refills only the
  // finest-level rows next to the changed points; the mask it was filled
  // with is kept (two buffers, swapped) to find them
  const bool incremental = refills && h->inc_enable && !h->ls_on && h->nvert_prev_valid;
  h->nvert_prev_valid = false;
  h->inc_rows = false;
  if (h->inc_enable && !h->nvert_prev) {
    TRY(dalloc(h, &h->nvert_prev, N));
    TRY(dalloc(h, &h->chg_a, N));
    TRY(dalloc(h, &h->chg_b, N));
    TRY(dalloc(h, &h->colflag, (size_t)h->box.nx * h->box.nz));
    TRY(dalloc(h, &h->rows, n));
    TRY(dalloc(h, &h->nrows, 1));
  }
  if (incremental) std::swap(h->nvert, h->nvert_prev);
  TRY(upload(h, h->nvert, nvert, N));
  // setup_lidx2: dof numbering in k-j-i order
  const int nblk = (int)((n + 1023) / 1024);
  LAUNCH(h, k_count_dofs, nblk, 1024, h->g, h->box, h->nvert, h->blk);
  LAUNCH(h, k_scan_blocks, 1, 1024, h->blk, nblk, h->total);
  LAUNCH(h, k_number_dofs, nblk, 1024, h->g, h->box, h->nvert, h->blk, h->gid_box);
  LAUNCH(h, k_gid_da, da_grid(h->g), 128, h->g, h->box, h->gid_box, h->gid_da);
  LAUNCH(h, k_fluid_mask, lin_grid(n), 256, h->g, h->box, h->nvert, h->fluid);
  // PoissonLHSNew: unscaled operator with the reference's insertion filter
  LevelSet fls;
  if (h->ls_on) {
    fls.rho = h->ls_rho; fls.level = h->ls_level; fls.on = 1;
    fls.bc3 = h->ls_bc3; fls.bc4 = h->ls_bc4; fls.bc5 = h->ls_bc5;
  }
  if (incremental) {
    LAUNCH(h, k_mask_changed, kRedBlocks, 256, N, (const double *)h->nvert, (const double *)h->nvert_prev, h->chg_a);
    LAUNCH(h, k_dilate_axis, da_grid(h->g), 128, h->g, 0, 2, (const uint8_t *)h->chg_a, h->chg_b);
    LAUNCH(h, k_dilate_axis, da_grid(h->g), 128, h->g, 1, 2, (const uint8_t *)h->chg_b, h->chg_a);
    LAUNCH(h, k_dilate_axis, da_grid(h->g), 128, h->g, 2, 2, (const uint8_t *)h->chg_a, h->chg_b);
    CUDA_TRY(cudaMemsetAsync(h->nrows, 0, sizeof(int), h->stream));
    CUDA_TRY(cudaMemsetAsync(h->colflag, 0, (size_t)h->box.nx * h->box.nz, h->stream));
    LAUNCH(h, k_list_rows, kRedBlocks, 256, h->g, h->box, (const uint8_t *)h->chg_b, h->rows, h->nrows, h->colflag);
    LAUNCH(h, k_assemble_fine_rows, kRedBlocks, 256, h->g, h->box, h->nvert, h->met, h->A0, h->rowtype0,
           h->L[0].A64, h->L[0].rowtype, fls, (const int *)h->rows, (const int *)h->nrows);
    h->inc_rows = true;
  } else if (refills) {  // both fine operators from one evaluation of each row
    LAUNCH(h, k_assemble_fine, box_grid(h->box), 128, h->g, h->box, h->nvert, h->met, h->A0, h->rowtype0,
           h->L[0].A64, h->L[0].rowtype, fls);
  } else
    LAUNCH(h, k_assemble, box_grid(h->box), 128, h->g, h->box, h->nvert, h->met, 0, 1, 0, h->A0, h->rowtype0, fls);
  // aj at the box cells for the row scale (each level forms its own masks)
  LAUNCH(h, k_level_masks, lin_grid(n), 256, h->g, h->box, h->nvert, (uint8_t *)nullptr, (double *)nullptr,
         (float *)nullptr, h->aj_box, (const double *)h->met.aj);
  LAUNCH(h, k_row_scale, lin_grid(n), 256, n, h->rowtype0, h->aj_box, h->scale);
  LAUNCH(h, k_cast_planes_f32, kRedBlocks, 256, h->scale, h->scale32, n);
  int tot = 0;
  CUDA_TRY(cudaMemcpyAsync(&tot, h->total, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  h->ndof = tot;
  const auto tp1 = std::chrono::steady_clock::now();
  TRY(build_hierarchy(h, o.coarsest_max));
  h->inc_rows = false;
  h->nvert_prev_valid = h->inc_enable;  // nvert now holds the mask every row was filled with
  if (h->phase)
    fprintf(stderr, "vfs set_nvert ms: numbering+fine operators+masks %.3f hierarchy %.3f\n",
            std::chrono::duration<double, std::milli>(tp1 - tp0).count(),
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tp1).count());
  CUDA_TRY(cudaMemsetAsync(h->x, 0, n * 8, h->stream));
  TRY(sync(h));
  h->have_nvert = true;
  h->have_rhs = false;
  h->r0_valid = false;
  h->op_version++;  // stored history images belong to the previous assembly
  return VFS_OK;
}

int vfs_poisson_rhs(vfs_poisson *h, const double *ucont, double dt, double st, double coeff) {
  if (!h || !ucont) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before rhs");
  if (!(dt != 0.) || !(coeff != 0.)) return fail(VFS_EINVAL, "dt and coeff must be non-zero");
  const size_t N = h->g.n();
  TRY(upload(h, h->ucont, ucont, 3 * N));
  LAUNCH(h, k_rhs, kRedBlocks, 256, h->g, h->box, h->nvert, h->ucont, h->met.aj, dt, st, coeff, h->b, h->partial);
  // Remove_Nullspace_Scale, skipped for bctype[3] == -10 and for a level
  // set with the Dirichlet top bctype[5] == 4 (poisson_hypre.c:120, :375)
  if (h->desc.bctype3 != -10 && !(h->ls_on && h->ls_bc5 == 4)) {
    LAUNCH(h, k_reduce_rows, 2, 1024, h->partial, kRedBlocks, 2, h->red);
    LAUNCH(h, k_rhs_nullspace, kRedBlocks, 256, h->g, h->box, h->nvert, h->met.aj, h->red, h->b);
  }
  TRY(sync(h));
  h->have_rhs = true;
  h->r0_valid = false;
  return VFS_OK;
}

int vfs_poisson_set_levelset(vfs_poisson *h, const double *rho, const double *level, const int *bctype, int enable) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  if (!enable) {
    if (h->ls_on) {
      // the assembled operator and right-hand side carry the density
      // weights: both have to be formed again without them
      h->have_nvert = false;
      h->have_rhs = false;
      h->r0_valid = false;
    }
    h->ls_on = 0;
    return VFS_OK;
  }
  if (!rho || !bctype) return fail(VFS_EINVAL, "density and bctype are required");
  const size_t N = h->g.n();
  if (!h->ls_rho) {
    TRY(dalloc(h, &h->ls_rho, N));
    TRY(dalloc(h, &h->ls_level, N));
  }
  TRY(upload(h, h->ls_rho, rho, N));
  if (level) TRY(upload(h, h->ls_level, level, N));
  else CUDA_TRY(cudaMemsetAsync(h->ls_level, 0, N * 8, h->stream));
  h->ls_on = 1;
  h->ls_bc3 = bctype[3];
  h->ls_bc4 = bctype[4];
  h->ls_bc5 = bctype[5];
  TRY(sync(h));
  h->have_nvert = false;  // the operator has to be assembled again
  h->have_rhs = false;
  return VFS_OK;
}

int vfs_poisson_rhs2(vfs_poisson *h, const double *ucont, double dt, double st, double coeff, int poisson) {
  if (!h || !ucont) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before rhs");
  if (!(dt != 0.) || !(coeff != 0.)) return fail(VFS_EINVAL, "dt and coeff must be non-zero");
  if (poisson != 0 && poisson != -1) return fail(VFS_EINVAL, "poisson must be 0 or -1");
  const size_t N = h->g.n();
  TRY(upload(h, h->ucont, ucont, 3 * N));
  LAUNCH(h, k_rhs2, kRedBlocks, 256, h->g, h->box, h->nvert, h->rowtype0, h->ucont, h->met.aj, dt, st, coeff,
         poisson, h->b, h->partial);
  LAUNCH(h, k_reduce_rows, 2, 1024, h->partial, kRedBlocks, 2, h->red);
  LAUNCH(h, k_rhs2_shift, kRedBlocks, 256, h->g, h->box, h->nvert, h->met.aj, h->red, poisson, h->b);
  TRY(sync(h));
  h->have_rhs = true;
  h->r0_valid = false;
  return VFS_OK;
}

int vfs_poisson_volume_flux(vfs_poisson *h, double *ucont, int flg, double flux_intp_sum, double *ibm_flux,
                            double *ibm_area) {
  if (!h || !ucont) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before volume_flux");
  if (flg < 0 || flg > 3) return fail(VFS_EINVAL, "flg must be 0..3");
  const size_t N = h->g.n();
  TRY(upload(h, h->ucont, ucont, 3 * N));
  double sums[3];
  LAUNCH(h, k_vflux_sum, kRedBlocks, 256, h->g, h->nvert, h->met, h->ucont, flg, 0, h->partial);
  TRY(reduce_read(h, kRedBlocks, 3, sums));
  double corr = 0.;
  if (sums[2] > 1.e-15) {
    if (flg > 1) corr = (sums[0] + flux_intp_sum) / sums[1];
    else if (flg) corr = (sums[0] + flux_intp_sum) / sums[2];
    else corr = sums[0] / sums[2];
  }
  LAUNCH(h, k_vflux_apply, kRedBlocks, 256, h->g, h->nvert, h->met, h->ucont, flg, corr);
  LAUNCH(h, k_vflux_sum, kRedBlocks, 256, h->g, h->nvert, h->met, h->ucont, flg, 2, h->partial);
  TRY(reduce_read(h, kRedBlocks, 3, sums));
  if (ibm_flux) *ibm_flux = sums[0];
  if (ibm_area) *ibm_area = sums[2];
  TRY(download(h, ucont, h->ucont, 3 * N));
  return sync(h);
}

int vfs_poisson_volume_flux0(vfs_poisson *h, double *ucont, int immersed, double *flux, double *area) {
  if (!h || !ucont) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before volume_flux0");
  if (immersed == 1) return fail(VFS_EINVAL, "immersed 1 takes the other VolumeFlux (vfs_poisson_volume_flux)");
  const size_t N = h->g.n();
  TRY(upload(h, h->ucont, ucont, 3 * N));
  double sums[2];
  LAUNCH(h, k_vflux0_sum, kRedBlocks, 256, h->g, h->nvert, h->met, h->ucont, h->partial);
  TRY(reduce_read(h, kRedBlocks, 2, sums));
  if (immersed != 2) {
    const double corr = sums[1] > 1.e-15 ? sums[0] / sums[1] : 0.;
    LAUNCH(h, k_vflux0_apply, kRedBlocks, 256, h->g, h->nvert, h->met, h->ucont, corr,
           (immersed == 0 || immersed == 3) ? 1 : 0);
  }
  LAUNCH(h, k_vflux0_sum, kRedBlocks, 256, h->g, h->nvert, h->met, h->ucont, h->partial);
  TRY(reduce_read(h, kRedBlocks, 2, sums));
  if (flux) *flux = sums[0];
  if (area) *area = sums[1];
  TRY(download(h, ucont, h->ucont, 3 * N));
  return sync(h);
}

int vfs_poisson_contra2cart(vfs_poisson *h, const double *ucont, double *ucat, int zero_solid) {
  if (!h || !ucont || !ucat) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before contra2cart");
  const size_t N = h->g.n();
  if (!h->ucat) TRY(dalloc(h, &h->ucat, 3 * N));
  TRY(upload(h, h->ucont, ucont, 3 * N));
  TRY(upload(h, h->ucat, ucat, 3 * N));
  LAUNCH(h, k_periodic_cmpnts, da_grid(h->g), 128, h->g, h->ucont, h->stage);
  LAUNCH(h, k_contra2cart, dim3((h->g.mx - 2 + 127) / 128, h->g.my - 2, h->g.mz - 2), 128, h->g, h->nvert, h->met,
         h->stage, h->ucat);
  LAUNCH(h, k_periodic_cmpnts, da_grid(h->g), 128, h->g, h->ucat, h->stage);
  if (zero_solid) LAUNCH(h, k_zero_solid, kRedBlocks, 256, h->g, h->nvert, h->stage);
  TRY(download(h, ucat, h->stage, 3 * N));
  return sync(h);
}

int vfs_poisson_ibm_interpolate(vfs_poisson *h, int ibi, const double *u_surf, int immersed, const int *bctype,
                                double *ucat, double *p, double *ucont) {
  if (!h || !ucat || !p || !ucont) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before the IB interpolation");
  if (ibi < 0 || ibi >= (int)h->ibm_bodies.size() || !h->ibm_bodies[ibi].nodes)
    return fail(VFS_ESTATE, "vfs_poisson_ibm_search_nodes must run for this body first");
  const IbmBody &B = h->ibm_bodies[ibi];
  const size_t N = h->g.n();
  if (!h->ucat) TRY(dalloc(h, &h->ucat, 3 * N));
  // device work space: ucat (h->ucat) and ucont (h->ucont); the copies of
  // the inputs as read, p and the surface velocities in ibm_work
  const size_t need = 5 * N + (size_t)B.n_v * 3;
  if (h->ibm_work_len < need) {
    if (h->ibm_work) dfree(h, h->ibm_work);
    h->ibm_work = nullptr;
    h->ibm_work_len = 0;
    TRY(dalloc(h, &h->ibm_work, need));
    h->ibm_work_len = need;
  }
  double *lucat = h->ibm_work, *lpr = h->ibm_work + 3 * N, *pd = h->ibm_work + 4 * N, *us = nullptr;
  TRY(upload(h, h->ucat, ucat, 3 * N));
  TRY(upload(h, pd, p, N));
  TRY(upload(h, h->ucont, ucont, 3 * N));
  CUDA_TRY(cudaMemcpyAsync(lucat, h->ucat, 3 * N * 8, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(lpr, pd, N * 8, cudaMemcpyDeviceToDevice, h->stream));
  if (u_surf) {
    if (is_device_ptr(u_surf)) {
      us = const_cast<double *>(u_surf);
    } else {
      us = h->ibm_work + 5 * N;
      CUDA_TRY(cudaMemcpyAsync(us, u_surf, (size_t)B.n_v * 3 * 8, cudaMemcpyHostToDevice, h->stream));
    }
  }
  if (B.n_nodes > 0)
    LAUNCH(h, k_ibm_apply, (B.n_nodes + 127) / 128, 128, h->g, B.nodes, B.n_nodes, B.tri, us, h->nvert, lucat, lpr,
           h->ucat, pd);
  // the new ucat with periodic ghosts (the local copy the flux loop reads)
  LAUNCH(h, k_periodic_cmpnts, da_grid(h->g), 128, h->g, h->ucat, h->stage);
  int b[6] = {0, 0, 0, 0, 0, 0};
  if (bctype)
    for (int q = 0; q < 6; q++) b[q] = bctype[q];
  LAUNCH(h, k_ibm_faces, dim3((h->g.mx - 2 + 127) / 128, h->g.my - 2, h->g.mz - 2), 128, h->g, h->nvert, h->stage,
         h->met.icsi, h->met.jeta, h->met.kzet, immersed == 3 ? 0. : 1., b[0], b[1], b[2], b[3], b[4], b[5],
         h->ucont);
  // Contra2Cart with the solid zeroing
  LAUNCH(h, k_periodic_cmpnts, da_grid(h->g), 128, h->g, h->ucont, h->stage);
  LAUNCH(h, k_contra2cart, dim3((h->g.mx - 2 + 127) / 128, h->g.my - 2, h->g.mz - 2), 128, h->g, h->nvert, h->met,
         h->stage, h->ucat);
  LAUNCH(h, k_periodic_cmpnts, da_grid(h->g), 128, h->g, h->ucat, h->stage);
  LAUNCH(h, k_zero_solid, kRedBlocks, 256, h->g, h->nvert, h->stage);
  TRY(download(h, ucat, h->stage, 3 * N));
  TRY(download(h, p, pd, N));
  TRY(download(h, ucont, h->ucont, 3 * N));
  return sync(h);
}

int vfs_poisson_ib_bc(vfs_poisson *h, int immersed, const int *bctype, double *ucat, double *ucont) {
  if (!h || !ucat || !ucont) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before IB_BC");
  const size_t N = h->g.n();
  if (!h->ucat) TRY(dalloc(h, &h->ucat, 3 * N));
  TRY(upload(h, h->ucat, ucat, 3 * N));
  TRY(upload(h, h->ucont, ucont, 3 * N));
  int b[6] = {0, 0, 0, 0, 0, 0};
  if (bctype)
    for (int q = 0; q < 6; q++) b[q] = bctype[q];
  // periodic ghosts of ucat from their partners (written back: the
  // reference writes them into lUcat)
  LAUNCH(h, k_periodic_cmpnts, da_grid(h->g), 128, h->g, h->ucat, h->stage);
  LAUNCH(h, k_ib_bc_faces, dim3((h->g.mx - 2 + 127) / 128, h->g.my - 2, h->g.mz - 2), 128, h->g, h->nvert,
         h->stage, h->met.icsi, h->met.jeta, h->met.kzet, immersed, b[0], b[1], b[2], b[3], h->ucont);
  if (h->ibm_work_len < 3 * N) {
    if (h->ibm_work) dfree(h, h->ibm_work);
    h->ibm_work = nullptr;
    h->ibm_work_len = 0;
    TRY(dalloc(h, &h->ibm_work, 3 * N));
    h->ibm_work_len = 3 * N;
  }
  double *uold = h->ibm_work;
  CUDA_TRY(cudaMemcpyAsync(uold, h->ucont, 3 * N * 8, cudaMemcpyDeviceToDevice, h->stream));
  LAUNCH(h, k_ib_bc_edges, da_grid(h->g), 128, h->g, uold, b[0], b[1], b[2], b[3], b[4], b[5], h->ucont);
  TRY(download(h, ucat, h->stage, 3 * N));
  TRY(download(h, ucont, h->ucont, 3 * N));
  return sync(h);
}

int vfs_poisson_solve(vfs_poisson *h, double *phi, const vfs_solve_opts *opts, vfs_solve_stats *stats) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  if (!h->have_rhs) return fail(VFS_ESTATE, "rhs must come before solve");
  vfs_solve_opts o;
  if (opts) o = *opts; else vfs_poisson_default_opts(&o);
  resolve_opts(o);
  TRY(check_opts(o));
  vfs_solve_stats st{};
  const size_t n = h->box.n();
  CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
  if (o.warm_start == 1 && phi) {
    TRY(upload(h, h->stage, phi, h->g.n()));
    LAUNCH(h, k_da_to_box, lin_grid(n), 256, h->g, h->box, h->stage, h->x);
    LAUNCH(h, k_mask_box, lin_grid(n), 256, n, h->rowtype0, h->x);
  } else if (!o.warm_start) {
    CUDA_TRY(cudaMemsetAsync(h->x, 0, n * 8, h->stream));
  }
  const auto tf0 = std::chrono::steady_clock::now();
  TRY(fgmres(h, o, &st));
  const auto tf1 = std::chrono::steady_clock::now();
  if (h->phase) cudaEventRecord(h->phev[0], h->stream);
  // Remove_Nullspace of phi (:604-608), its shift applied by the DA output
  const bool shift = h->desc.bctype3 != -10 && !(h->ls_on && h->ls_bc5 == 4);
  if (shift) {
    LAUNCH(h, k_mean_partial, kRedBlocks, 256, h->box, h->fluid, h->x, h->partial);
    LAUNCH(h, k_reduce_rows, 2, 1024, h->partial, kRedBlocks, 2, h->red);
    LAUNCH(h, k_mean_shift, 1, 32, h->red);
  }
  LAUNCH(h, k_box_to_da_phi, da_grid(h->g), 128, h->g, h->box, h->nvert, h->x, h->phi_da,
         shift ? (const double *)h->red + 2 : nullptr);
  // phi to a host array on a side stream, while the solution enters the
  // history on the handle's stream (it reads x, b and the residual, not
  // phi); the handle's stream waits for the copy before the call returns
  const bool host_out = phi && !is_device_ptr(phi);
  if (host_out) {
    if (!h->dl_stream) {
      CUDA_TRY(cudaStreamCreateWithFlags(&h->dl_stream, cudaStreamNonBlocking));
      CUDA_TRY(cudaEventCreateWithFlags(&h->dl_ev[0], cudaEventDisableTiming));
      CUDA_TRY(cudaEventCreateWithFlags(&h->dl_ev[1], cudaEventDisableTiming));
    }
    CUDA_TRY(cudaEventRecord(h->dl_ev[0], h->stream));
    CUDA_TRY(cudaStreamWaitEvent(h->dl_stream, h->dl_ev[0], 0));
    CUDA_TRY(cudaMemcpyAsync(phi, h->phi_da, h->g.n() * sizeof(double), cudaMemcpyDeviceToHost, h->dl_stream));
    if (h->phase) cudaEventRecord(h->phev[2], h->dl_stream);
    CUDA_TRY(cudaEventRecord(h->dl_ev[1], h->dl_stream));
  } else if (phi) {
    TRY(download(h, phi, h->phi_da, h->g.n()));
  }
  if (h->hist_cap && h->hist_record && st.initial_rel_residual > 0. && st.rel_residual <= o.rtol)
    TRY(hist_push(h));
  if (h->phase) cudaEventRecord(h->phev[1], h->stream);
  const auto tf2 = std::chrono::steady_clock::now();
  if (host_out) CUDA_TRY(cudaStreamWaitEvent(h->stream, h->dl_ev[1], 0));
  CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
  TRY(sync(h));
  if (h->phase) {
    // host: the FGMRES call, the tail's launches (with the push's Gram read)
    // and the final wait; device: from the end of FGMRES to the end of the
    // push and of the host copy
    const auto tf3 = std::chrono::steady_clock::now();
    float a = 0.f, c = -1.f;
    cudaEventElapsedTime(&a, h->phev[0], h->phev[1]);
    if (host_out) cudaEventElapsedTime(&c, h->phev[0], h->phev[2]);
    fprintf(stderr, "vfs solve tail ms: host fgmres %.3f tail %.3f wait %.3f; device to push end %.3f, to copy end %.3f\n",
            std::chrono::duration<double, std::milli>(tf1 - tf0).count(),
            std::chrono::duration<double, std::milli>(tf2 - tf1).count(),
            std::chrono::duration<double, std::milli>(tf3 - tf2).count(), a, c);
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  st.ms_total = ms;
  st.levels = (int)h->L.size();
  st.status = st.rel_residual <= o.rtol ? VFS_OK : VFS_ENOCONV;
  if (stats) *stats = st;
  h->have_phi = true;
  h->r0_valid = false;
  if (st.status != VFS_OK)
    return fail(VFS_ENOCONV, "solver stopped at relative residual " + std::to_string(st.rel_residual));
  return VFS_OK;
}

}  // extern "C"

namespace {
int guess_buffers(vfs_poisson *h) {
  const size_t n = h->box.n();
  if (!h->gex) {
    TRY(dalloc(h, &h->gex, n));
    TRY(dalloc(h, &h->gsum, 8));
    TRY(dalloc(h, &h->gfeat, 4 * n));
    TRY(dalloc(h, &h->gtgt, n));
    TRY(dalloc(h, &h->gfc, 4 * (n / 8 + 1)));
    TRY(dalloc(h, &h->gout, n / 8 + 1));
    TRY(dalloc(h, &h->gof[0], n));
    TRY(dalloc(h, &h->gof[1], n));
    TRY(dalloc(h, &h->rprev, n));
    TRY(dalloc(h, &h->rlearn, n));
    TRY(dalloc(h, &h->gnet, n));
    TRY(dalloc(h, &h->prev32, n));
    const char *e = getenv("VFS_GUESS_SMOOTH");
    if (e) h->gsmooth = std::max(0, std::min(8, atoi(e)));
  }
  return VFS_OK;
}

// fine feature planes of the current right-hand side into h->gfeat; also
// phi_{n-1} as a box vector in the last Z and the squared norms of b - A ex,
// b - A phi_{n-1} (an FP32 estimate) and b in norms[0..2]
int guess_features(vfs_poisson *h, const double *phi_nm1, const double *phi_nm2, double *norms) {
  if (!h || !phi_nm1 || !phi_nm2) return fail(VFS_EINVAL, "null argument");
  if (!h->have_rhs) return fail(VFS_ESTATE, "rhs must come before the guess");
  if (h->box.nx % 8 || h->box.ny % 8 || h->box.nz % 8)
    return fail(VFS_EINVAL, "the learned guess needs box dims that are multiples of 8");
  TRY(guess_buffers(h));
  float *feat = h->gfeat;
  const size_t n = h->box.n(), N = h->g.n();
  const double *p1, *p2;
  TRY(device_view(h, phi_nm1, h->stage, N, &p1));
  TRY(device_view(h, phi_nm2, h->stage + N, N, &p2));
  CUDA_TRY(cudaMemsetAsync(h->gsum, 0, 8 * sizeof(double), h->stream));
  TRY(ensure_krylov(h, std::max(h->m_alloc, 20)));
  // phi_{n-1} (box layout) in the last preconditioned vector, free until the
  // next solve (the speculative step 0 writes Z_0)
  double *prev = h->Z[h->m_alloc - 1];
  LAUNCH(h, k_guess_prep, kRedBlocks, 256, h->g, h->box, h->rowtype0, p1, p2, h->gex, prev, h->prev32, feat,
         feat + n, feat + 3 * n, h->gsum);
  const dim3 gr = guess_grid(h->box);
  const int nbox = (int)(gr.x * gr.y * gr.z);
  LAUNCH(h, k_guess_residuals, gr, 128, h->box, h->A0, h->L[0].C16, h->L[0].D32, h->scale32, h->gex, h->prev32,
         h->b, h->r, h->partial);
  LAUNCH(h, k_guess_f2, kRedBlocks, 256, n, h->rowtype0, (const double *)h->aj_box, h->r, feat + 2 * n, h->gsum);
  LAUNCH(h, k_guess_scale, kRedBlocks, 256, n, feat, h->gsum);
  double nr[3];
  TRY(reduce_read(h, nbox, 3, nr));
  if (norms) for (int q = 0; q < 3; q++) norms[q] = nr[q];
  return VFS_OK;
}
}  // namespace

extern "C" {

int vfs_poisson_guess_sample(vfs_poisson *h, const double *phi_n, const double *phi_nm1, const double *phi_nm2,
                             float *features, float *target, float *weight) {
  if (!phi_n || !target || !weight) return fail(VFS_EINVAL, "null argument");
  if (!is_device_ptr(features) || !is_device_ptr(target) || !is_device_ptr(weight))
    return fail(VFS_EINVAL, "features, target and weight must be device memory");
  TRY(guess_features(h, phi_nm1, phi_nm2, nullptr));
  const size_t N = h->g.n();
  TRY(upload(h, h->stage + 2 * N, phi_n, N));
  LAUNCH(h, k_guess_target, kRedBlocks, 256, h->g, h->box, h->rowtype0, h->stage + 2 * N, h->gex, h->gsum, h->gtgt,
         h->gof[0]);
  LAUNCH(h, k_guess_restrict, kRedBlocks, 256, h->box, h->gfeat, h->gtgt, features, target, weight);
  return sync(h);
}

int vfs_poisson_get_operator32(vfs_poisson *h, float *planes) {
  if (!h || !planes) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert || h->L.empty() || !h->L[0].A32) return fail(VFS_ESTATE, "set_nvert must come first");
  // the level operator is stored in the parity-split row layout: one plane
  // at a time back to the natural layout (through the staging buffer when
  // the destination is host memory)
  const size_t n = h->box.n();
  const bool dev = is_device_ptr(planes);
  float *tmp = reinterpret_cast<float *>(h->stage);
  for (int q = 0; q < NSLOT; q++) {
    float *dst = dev ? planes + (size_t)q * n : tmp;
    LAUNCH(h, k_unsplit_plane, lin_grid(n), 256, h->box, h->L[0].A32 + (size_t)q * n, dst);
    if (!dev) CUDA_TRY(cudaMemcpyAsync(planes + (size_t)q * n, tmp, n * sizeof(float), cudaMemcpyDeviceToHost,
                                       h->stream));
  }
  return sync(h);
}

int vfs_poisson_set_history(vfs_poisson *h, int k) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  if (k < 0 || k > kHistMax) return fail(VFS_EINVAL, "history length must be 0.." + std::to_string(kHistMax));
  TRY(sync(h));
  for (int j = 0; j < kHistMax; j++) {
    dfree(h, h->hist_X[j]);
    dfree(h, h->hist_Y[j]);
    h->hist_X[j] = h->hist_Y[j] = nullptr;
  }
  if (h->r0 == h->hist_r) h->r0_valid = false;
  if (h->r0 == h->hist_er) h->r0_valid = false;
  for (double **p : {&h->hist_Xn, &h->hist_Yn, &h->hist_x, &h->hist_r, &h->hist_ex, &h->hist_er, &h->hist_coef}) {
    dfree(h, *p);
    *p = nullptr;
  }
  h->hist_cap = h->hist_cnt = h->hist_head = 0;
  const size_t n = h->box.n();
  for (int j = 0; j + 1 < k; j++) {  // k - 1 difference slots
    TRY(dalloc(h, &h->hist_X[j], n));
    TRY(dalloc(h, &h->hist_Y[j], n));
  }
  if (k) {
    TRY(dalloc(h, &h->hist_Xn, n));
    TRY(dalloc(h, &h->hist_Yn, n));
    TRY(dalloc(h, &h->hist_x, n));
    TRY(dalloc(h, &h->hist_r, n));
    TRY(dalloc(h, &h->hist_ex, n));
    TRY(dalloc(h, &h->hist_er, n));
    TRY(dalloc(h, &h->hist_coef, 2 * kHistMax));
  }
  h->hist_cap = k;
  return VFS_OK;
}

int vfs_poisson_history_record(vfs_poisson *h, int on) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  h->hist_record = on != 0;
  return VFS_OK;
}

int vfs_poisson_set_network_period(vfs_poisson *h, int period) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  if (period < 1) return fail(VFS_EINVAL, "period must be at least 1");
  h->net_period = period;
  h->net_wait = 0;
  return VFS_OK;
}

int vfs_poisson_fully_blocked(vfs_poisson *h, int *multinullspace, int32_t *ksk) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come first");
  const Grid &g = h->g;
  const size_t nc = (size_t)g.mx * g.my;
  if (!h->ksk) {
    TRY(dalloc(h, &h->ksk, nc));
    TRY(dalloc(h, &h->ksk_count, 1));
  }
  if (h->multinull < 0 || h->ksk_version != h->op_version) {
    CUDA_TRY(cudaMemsetAsync(h->ksk_count, 0, sizeof(int), h->stream));
    LAUNCH(h, k_fully_blocked, dim3((g.mx + 127) / 128, g.my), 128, g, (const double *)h->nvert, h->ksk, h->ksk_count);
    int cnt = 0;
    CUDA_TRY(cudaMemcpyAsync(h->hbuf, h->ksk_count, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    memcpy(&cnt, h->hbuf, sizeof(int));
    h->multinull = cnt == 0 ? 1 : 0;
    h->ksk_version = h->op_version;
  }
  if (multinullspace) *multinullspace = h->multinull;
  if (ksk) {
    CUDA_TRY(cudaMemcpyAsync(ksk, h->ksk, nc * sizeof(int32_t),
                             is_device_ptr(ksk) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
  }
  return VFS_OK;
}

int vfs_poisson_nullspace_original(vfs_poisson *h, double *x) {
  if (!h || !x) return fail(VFS_EINVAL, "null argument");
  TRY(vfs_poisson_fully_blocked(h, nullptr, nullptr));
  const Grid &g = h->g;
  const size_t N = g.n();
  const bool dev = is_device_ptr(x);
  double *xd = dev ? x : h->stage;
  if (!dev) TRY(upload(h, xd, x, N));
  LAUNCH(h, k_nullspace_sums, kRedBlocks, 256, g, (const double *)h->nvert, (const int *)h->ksk, h->multinull,
         (const double *)xd, h->partial);
  double sm[4];
  TRY(reduce_read(h, kRedBlocks, 4, sm));
  // the reference's shift per region: sum / (-num) (poisson.c:813, 840, 865)
  const double s0 = sm[0] / (-1.0 * sm[1]), s1 = h->multinull ? sm[2] / (-1.0 * sm[3]) : 0.;
  LAUNCH(h, k_nullspace_apply, da_grid(g), 128, g, (const double *)h->nvert, (const int *)h->ksk, h->multinull, s0,
         s1, xd);
  if (!dev) TRY(download(h, x, xd, N));
  return sync(h);
}

int vfs_poisson_guess_report(vfs_poisson *h, int *chosen, double *rel_res, double *est) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  if (h->guess_chosen < 0) return fail(VFS_ESTATE, "no guess installed yet");
  if (chosen) *chosen = h->guess_chosen;
  for (int q = 0; q < 3; q++) {
    if (rel_res) rel_res[q] = h->guess_rel[q];
    if (est) est[q] = h->guess_est[q];
  }
  return VFS_OK;
}

int vfs_poisson_history_guess(vfs_poisson *h, double *rel_res) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  if (!h->have_rhs) return fail(VFS_ESTATE, "rhs must come before the guess");
  if (!h->hist_cnt) return fail(VFS_ESTATE, "no stored solution (vfs_poisson_set_history, then a solve)");
  h->r0_valid = h->spec_valid = h->spec_next = h->z0_valid = false;
  GuessCand c[2];
  int nc = 0;
  double bn = 0.;
  bool far = false;
  TRY(history_candidates(h, c, &nc, &bn, &far));
  int w = 0;
  TRY(judge(h, c, nc, &w));
  install_guess(h, c[w]);
  guess_report(h, c, nc, w, bn);
  if (rel_res) *rel_res = bn > 0. ? c[w].beta / bn : 0.;
  return sync(h);
}

int vfs_poisson_learned_guess(vfs_poisson *h, vfs_unet *u, const double *phi_nm1, const double *phi_nm2,
                              double kappa, int *chosen, double *rel_res) {
  if (!h || !u) return fail(VFS_EINVAL, "null argument");
  const Box b = h->box;
  h->r0_valid = h->spec_valid = h->z0_valid = false;
  if (h->phase) cudaEventRecord(h->phev[0], h->stream);
  // with a solution history the network's candidate competes with the
  // projection and the extrapolation of the stored solutions
  const bool use_hist = h->hist_cnt > 0;
  GuessCand hc[2];
  int nh = 0;
  double bn_h = 0.;
  bool far = false;
  if (use_hist) {
    if (!h->have_rhs) return fail(VFS_ESTATE, "rhs must come before the guess");
    TRY(history_candidates(h, hc, &nh, &bn_h, &far));
  }
  // the network sits this call out: between its periodic runs while it
  // loses, or when the projection's residual is below the extrapolation's
  // by more than kNetGate (the network's correction of the extrapolation
  // would have to cut its residual by more than the judge's gate)
  if (use_hist && (far || h->net_wait > 0)) {
    if (!far) h->net_wait--;
    int w = 0;
    TRY(judge(h, hc, nh, &w));
    install_guess(h, hc[w]);
    h->spec_next = false;
    guess_report(h, hc, nh, w, bn_h);
    if (chosen) *chosen = hc[w].code;
    if (rel_res) {
      rel_res[0] = bn_h > 0. ? hc[w].beta / bn_h : 0.;
      rel_res[1] = -1.;
    }
    return sync(h);
  }
  double nrm[3];
  TRY(guess_features(h, phi_nm1, phi_nm2, nrm));
  const size_t n = b.n();
  // speculative step 0 of the next solve on the handle's stream; the network
  // and the band fit then run on the side stream with their own reduction
  // buffers (the step's V-cycle, apply and Gram-Schmidt use V_0, V_1, Z_0,
  // dsv, partial, red and the level buffers; the guess reads r and writes
  // its own planes)
  const bool spec = h->spec_enable && h->spec_next && !h->phase && !h->prof && nrm[0] > 0.;
  // puts the handle's stream and reduction buffers back on every exit
  struct SideScope {
    vfs_poisson *h;
    vfs_unet *u;
    cudaStream_t main;
    bool on = false;
    void leave() {
      if (!on) return;
      h->stream = main;
      std::swap(h->partial, h->spartial);
      std::swap(h->red, h->sred);
      vfs_unet_set_stream(u, main);
      on = false;
    }
    ~SideScope() { leave(); }
  } side_scope{h, u, h->stream};
  if (spec) {
    if (!h->side) {
      CUDA_TRY(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
      CUDA_TRY(cudaEventCreateWithFlags(&h->ev_feat, cudaEventDisableTiming));
      const dim3 gb = guess_grid(h->box);
      TRY(dalloc(h, &h->spartial, (size_t)16 * gb.x * gb.y * gb.z + 4096));
      TRY(dalloc(h, &h->sred, 32));
    }
    vfs_solve_opts so;
    vfs_poisson_default_opts(&so);
    resolve_opts(so);
    h->spec_opts = so;
    const double beta = std::sqrt(nrm[0]);
    CUDA_TRY(cudaEventRecord(h->ev_feat, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->V[0], h->r, n * 8, cudaMemcpyDeviceToDevice, h->stream));
    h->hbuf[kSpecStage] = beta * beta;
    h->hbuf[kSpecStage + 1] = 1.0 / beta;
    reinterpret_cast<float *>(h->hbuf + kSpecStage + 2)[0] = (float)(1.0 / beta);
    CUDA_TRY(cudaMemcpyAsync(h->dsv, h->hbuf + kSpecStage, 16, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->dsv32, h->hbuf + kSpecStage + 2, 4, cudaMemcpyHostToDevice, h->stream));
    const int nbd = (int)((n + 256 * kGsTile - 1) / (256 * kGsTile));
    TRY(arnoldi_enqueue(h, 0, nbd, so, kSpecHb));
    CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_feat, 0));
    h->stream = h->side;
    std::swap(h->partial, h->spartial);
    std::swap(h->red, h->sred);
    side_scope.on = true;
  }
  if (h->phase) cudaEventRecord(h->phev[1], h->stream);
  LAUNCH(h, k_guess_restrict, kRedBlocks, 256, b, h->gfeat, nullptr, h->gfc, nullptr, nullptr);
  vfs_unet_set_stream(u, h->stream);
  const int hx = b.nx / 2, hy = b.ny / 2, hz = b.nz / 2;
  vfs_unet_batch bt{h->gfc, nullptr, nullptr, hx, hy, hz, 0, 0, 0, hx, hy, hz, nullptr, 0.f, 0.f, 0.f};
  const int64_t before = vfs_unet_kernel_launches(u);
  TRY(vfs_unet_forward(u, &bt, h->gout));
  h->launches += vfs_unet_kernel_launches(u) - before;
  if (h->phase) cudaEventRecord(h->phev[2], h->stream);
  LAUNCH(h, k_guess_prolong, kRedBlocks, 256, b, h->gout, h->gof[0]);
  int cur = 0;
  // gsmooth passes of the 27-point binomial filter; the last one also
  // zeroes the correction off the dofs (gsmooth 0: only the masking)
  if (h->gsmooth == 0) {
    LAUNCH(h, k_guess_smooth, kRedBlocks, 256, b, h->gof[cur], h->gof[cur ^ 1], -1, (const uint8_t *)h->rowtype0);
    cur ^= 1;
  }
  for (int p = 0; p < h->gsmooth; p++, cur ^= 1)
    LAUNCH(h, k_guess_smooth3, box_grid(b), 128, b, h->gof[cur], h->gof[cur ^ 1],
           p == h->gsmooth - 1 ? (const uint8_t *)h->rowtype0 : nullptr);
  // least-squares band weights: minimise ||r_ex - sum_k alpha_k y_k||
  // (alpha = 0 is the plain extrapolation, so the guess is never worse)
  // the normal equations from every kGramStride-th k-plane, scaled to the
  // whole box (the fit predicts the full ||r||^2 below)
  constexpr int kGramStride = 4;
  dim3 gg = guess_grid(b);
  gg.z = (b.nz + kGramStride - 1) / kGramStride;
  LAUNCH(h, k_guess_gram, gg, 128, b, h->L[0].A32, (const float *)h->scale32, h->gof[cur], h->r, kappa, h->gsum,
         kGramStride, h->partial);
  double gm[14];
  const int grc = reduce_read(h, (int)(gg.x * gg.y * gg.z), 14, gm);
  side_scope.leave();  // back to the handle's stream and buffers
  TRY(grc);
  for (double &v : gm) v *= (double)b.nz / gg.z;
  BandWeights bw{};
  {
    // the normal equations G alpha = g (symmetric positive semi-definite)
    // by Cholesky over the bands that carry a correction
    double G[kGuessBands][kGuessBands], g[kGuessBands];
    int q = 0;
    for (int u = 0; u < kGuessBands; u++)
      for (int v = u; v < kGuessBands; v++) G[u][v] = G[v][u] = gm[q++];
    for (int u = 0; u < kGuessBands; u++) g[u] = gm[10 + u];
    double gmax = 0.;
    for (int u = 0; u < kGuessBands; u++) gmax = std::max(gmax, G[u][u]);
    int ids[kGuessBands], na = 0;
    for (int u = 0; u < kGuessBands; u++)
      if (gmax > 0. && G[u][u] > 1e-14 * gmax) ids[na++] = u;
    double L[kGuessBands][kGuessBands] = {}, z[kGuessBands] = {}, al[kGuessBands] = {};
    bool ok = na > 0;
    for (int p = 0; p < na && ok; p++) {
      for (int r2 = 0; r2 <= p; r2++) {
        double v = G[ids[p]][ids[r2]] * (p == r2 ? 1. + 1e-10 : 1.);
        for (int t = 0; t < r2; t++) v -= L[p][t] * L[r2][t];
        if (p == r2) {
          if (!(v > 0.)) { ok = false; break; }
          L[p][p] = std::sqrt(v);
        } else {
          L[p][r2] = v / L[r2][r2];
        }
      }
    }
    if (ok) {
      for (int p = 0; p < na; p++) {
        double v = g[ids[p]];
        for (int t = 0; t < p; t++) v -= L[p][t] * z[t];
        z[p] = v / L[p][p];
      }
      for (int p = na - 1; p >= 0; p--) {
        double v = z[p];
        for (int t = p + 1; t < na; t++) v -= L[t][p] * al[t];
        al[p] = v / L[p][p];
      }
      for (int p = 0; p < na; p++) bw.a[ids[p]] = al[p];
    }
  }
  if (h->phase)
    fprintf(stderr, "vfs guess band weights: %.4g %.4g %.4g %.4g\n", bw.a[0], bw.a[1], bw.a[2], bw.a[3]);
  // the candidates: the base (the history's projection, or the previous
  // step's phi without a history), the extrapolation and, when a band
  // weight is not 0, the network's correction of it; the fit predicts the
  // last one's residual, ||r_ex||^2 - 2 alpha.g + alpha.G.alpha, and it is
  // composed only when that could pass the judge's gate
  double r2 = nrm[0];
  {
    int q = 0;
    for (int u2 = 0; u2 < kGuessBands; u2++) {
      r2 -= 2. * bw.a[u2] * gm[10 + u2];
      for (int v = u2; v < kGuessBands; v++, q++) r2 += (u2 == v ? 1. : 2.) * bw.a[u2] * bw.a[v] * gm[q];
    }
  }
  const double nb = nrm[2] > 0. ? std::sqrt(nrm[2]) : 1.;
  GuessCand c[3];
  int nc = 0;
  if (use_hist && hc[0].code == 0) {
    c[nc++] = hc[0];
  } else if (!use_hist) {
    // the previous step's phi: its FP64 residual
    CUDA_TRY(cudaMemcpyAsync(h->x, h->Z[h->m_alloc - 1], b.n() * 8, cudaMemcpyDeviceToDevice, h->stream));
    const dim3 gr = box_grid(h->box);
    LAUNCH(h, k_residual64, gr, 128, h->box, h->A0, h->x, h->b, h->rprev, h->partial);
    double s2 = 0.;
    TRY(reduce_read(h, (int)(gr.x * gr.y * gr.z), 1, &s2));
    c[nc++] = GuessCand{h->x, h->rprev, std::sqrt(s2), 0, nullptr, -1.};
  }
  const int iex = nc;
  c[nc++] = GuessCand{h->gex, h->r, std::sqrt(nrm[0]), 2, spec ? h->Z[0] : nullptr, -1.};
  bool weighted = false;
  for (int u2 = 0; u2 < kGuessBands; u2++) weighted = weighted || bw.a[u2] != 0.;
  double bmin = c[0].beta;
  for (int q = 1; q < nc; q++) bmin = std::min(bmin, c[q].beta);
  int inet = -1;
  double r_learn = std::sqrt(std::max(r2, 0.));
  if (weighted && r_learn <= kJudgeGate * bmin) {
    double *xl = h->gnet;
    LAUNCH(h, k_guess_compose, kRedBlocks, 256, b, h->rowtype0, h->gex, h->gof[cur], kappa, h->gsum, bw, xl);
    LAUNCH(h, k_residual64, box_grid(h->box), 128, h->box, h->A0, xl, h->b, h->rlearn, h->partial);
    double s2 = 0.;
    const dim3 gr = box_grid(h->box);
    TRY(reduce_read(h, (int)(gr.x * gr.y * gr.z), 1, &s2));
    r_learn = std::sqrt(s2);
    inet = nc;
    c[nc++] = GuessCand{xl, h->rlearn, r_learn, 1, nullptr, -1.};
  }
  int w = 0;
  TRY(judge(h, c, nc, &w));
  const bool learned = c[w].code == 1;
  install_guess(h, c[w]);
  if (use_hist) h->net_wait = learned ? 0 : h->net_period - 1;
  // the speculative step holds when the extrapolation is installed (its
  // residual and norm are the step's V_0 and beta)
  h->spec_valid = spec && w == iex;
  h->spec_next = w == iex;
  guess_report(h, c, nc, w, nb);
  if (chosen) *chosen = c[w].code;
  if (rel_res) {
    rel_res[0] = c[0].code == 0 ? c[0].beta / nb : -1.;
    rel_res[1] = (inet >= 0 ? r_learn : c[iex].beta) / nb;
  }
  if (h->phase) {
    fprintf(stderr, "vfs guess rel residuals: extrapolation %.4e fit %.4e learned %.4e base %.4e\n",
            std::sqrt(nrm[0]) / nb, std::sqrt(std::max(r2, 0.)) / nb, r_learn / nb,
            c[0].code == 0 ? c[0].beta / nb : -1.);
    cudaEventRecord(h->phev[3], h->stream);
    TRY(sync(h));
    float a = 0.f, c2 = 0.f, d = 0.f;
    cudaEventElapsedTime(&a, h->phev[0], h->phev[1]);
    cudaEventElapsedTime(&c2, h->phev[1], h->phev[2]);
    cudaEventElapsedTime(&d, h->phev[2], h->phev[3]);
    fprintf(stderr, "vfs guess ms: features+residuals %.3f network %.3f prolong+weights+judge %.3f\n", a, c2, d);
  }
  return sync(h);
}

int vfs_poisson_solver_hypre(vfs_poisson *h, const double *ucont, double dt, double st, double coeff, double *phi,
                             const vfs_solve_opts *opts, vfs_solve_stats *stats) {
  TRY(vfs_poisson_rhs(h, ucont, dt, st, coeff));
  return vfs_poisson_solve(h, phi, opts, stats);
}

int vfs_poisson_update_pressure(vfs_poisson *h, double *p, double *phi) {
  if (!h || !p) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before update_pressure");
  const size_t N = h->g.n();
  TRY(upload(h, h->p_da, p, N));
  if (phi) TRY(upload(h, h->phi_da, phi, N));
  LAUNCH(h, k_update_pressure, da_grid(h->g), 128, h->g, h->nvert, h->phi_da, h->p_da);
  LAUNCH(h, k_periodic_copy2, da_grid(h->g), 128, h->g, h->p_da, h->phi_da);
  TRY(download(h, p, h->p_da, N));
  if (phi) TRY(download(h, phi, h->phi_da, N));
  return sync(h);
}

int vfs_poisson_projection(vfs_poisson *h, double *ucont, double dt, double st, double coeff) {
  if (!h || !ucont) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before projection");
  if (!(coeff != 0.)) return fail(VFS_EINVAL, "coeff must be non-zero");
  const size_t N = h->g.n();
  TRY(upload(h, h->ucont, ucont, 3 * N));
  LevelSet pls;
  if (h->ls_on) {
    pls.rho = h->ls_rho; pls.level = h->ls_level; pls.on = 1;
    pls.bc3 = h->ls_bc3; pls.bc4 = h->ls_bc4; pls.bc5 = h->ls_bc5;
  }
  LAUNCH(h, k_projection, box_grid(h->box), 128, h->g, h->box, h->nvert, h->phi_da, h->pc, dt, st, coeff, h->ucont,
         h->met, pls);
  LAUNCH(h, k_periodic_faces, da_grid(h->g), 128, h->g, h->ucont);
  TRY(download(h, ucont, h->ucont, 3 * N));
  return sync(h);
}

int vfs_poisson_divergence(vfs_poisson *h, const double *ucont, double *maxdiv) {
  if (!h || !ucont || !maxdiv) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come before divergence");
  const size_t N = h->g.n();
  const double *u = ucont;
  if (!is_device_ptr(ucont)) {
    TRY(upload(h, h->stage, ucont, 3 * N));
    u = h->stage;
  }
  LAUNCH(h, k_divergence, kRedBlocks, 256, h->g, h->box, h->nvert, u, h->met.aj, h->partial);
  LAUNCH(h, k_reduce_max, 1, 1024, h->partial, kRedBlocks, h->red);
  CUDA_TRY(cudaMemcpyAsync(h->hbuf, h->red, 8, cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  *maxdiv = h->hbuf[0];
  return VFS_OK;
}

int vfs_poisson_get_numbering(vfs_poisson *h, int *ndof, int32_t *gid) {
  if (!h || !ndof) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come first");
  *ndof = h->ndof;
  if (gid) {
    CUDA_TRY(cudaMemcpyAsync(gid, h->gid_da, h->g.n() * 4,
                             is_device_ptr(gid) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream));
  }
  return sync(h);
}

int vfs_poisson_get_operator(vfs_poisson *h, double *vol, int32_t *rowtype) {
  if (!h || !vol) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come first");
  const size_t n = h->box.n();
  const Grid &g = h->g;
  const Box &b = h->box;
  std::vector<double> A(n * NSLOT);
  std::vector<uint8_t> rt(n);
  CUDA_TRY(cudaMemcpyAsync(A.data(), h->A0, n * NSLOT * 8, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaMemcpyAsync(rt.data(), h->rowtype0, n, cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  std::vector<double> out(g.n() * NSLOT, 0.);
  std::vector<int32_t> ort(g.n(), 0);
  for (int k = 0; k < b.nz; k++)
    for (int j = 0; j < b.ny; j++)
      for (int i = 0; i < b.nx; i++) {
        size_t c = b.at(i, j, k), t = g.at(i + 1, j + 1, k + 1);
        ort[t] = rt[c];
        for (int s = 0; s < NSLOT; s++) out[t * NSLOT + s] = A[(size_t)s * n + c];
      }
  bool dev = is_device_ptr(vol);
  CUDA_TRY(cudaMemcpy(vol, out.data(), out.size() * 8, dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost));
  if (rowtype)
    CUDA_TRY(cudaMemcpy(rowtype, ort.data(), ort.size() * 4,
                        is_device_ptr(rowtype) ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost));
  return VFS_OK;
}

int vfs_poisson_get_metric(vfs_poisson *h, int which, double *out) {
  if (!h || !out) return fail(VFS_EINVAL, "null argument");
  if (!h->have_grid) return fail(VFS_ESTATE, "set_grid must come first");
  double *vec[13] = {h->met.icsi, h->met.ieta, h->met.izet, h->met.jcsi, h->met.jeta, h->met.jzet, h->met.kcsi,
                     h->met.keta, h->met.kzet, h->met.csi,  h->met.eta,  h->met.zet,  h->met.cent};
  double *sca[4] = {h->met.iaj, h->met.jaj, h->met.kaj, h->met.aj};
  const size_t N = h->g.n();
  if (which >= 0 && which < 13) TRY(download(h, out, vec[which], 3 * N));
  else if (which >= 13 && which < 17) TRY(download(h, out, sca[which - 13], N));
  else return fail(VFS_EINVAL, "metric index out of range");
  return sync(h);
}

int vfs_poisson_get_rhs(vfs_poisson *h, double *b) {
  if (!h || !b) return fail(VFS_EINVAL, "null argument");
  if (!h->have_rhs) return fail(VFS_ESTATE, "rhs must come first");
  LAUNCH(h, k_box_to_da, da_grid(h->g), 128, h->g, h->box, h->b, h->stage);
  TRY(download(h, b, h->stage, h->g.n()));
  return sync(h);
}

int vfs_poisson_apply(vfs_poisson *h, const double *x, double *y) {
  if (!h || !x || !y) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come first");
  const size_t n = h->box.n();
  TRY(upload(h, h->stage, x, h->g.n()));
  double *tmp = h->L[0].v64[3];
  LAUNCH(h, k_da_to_box, lin_grid(n), 256, h->g, h->box, h->stage, h->r);
  LAUNCH(h, k_apply64, box_grid(h->box), 128, h->box, h->A0, h->r, tmp);
  LAUNCH(h, k_box_to_da, da_grid(h->g), 128, h->g, h->box, tmp, h->stage);
  TRY(download(h, y, h->stage, h->g.n()));
  return sync(h);
}

int vfs_poisson_mg_levels(vfs_poisson *h, int *nlevels) {
  if (!h || !nlevels) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come first");
  *nlevels = (int)h->L.size();
  return VFS_OK;
}

int vfs_poisson_mg_level_info(vfs_poisson *h, int level, int *d) {
  if (!h || !d) return fail(VFS_EINVAL, "null argument");
  if (level < 0 || level >= (int)h->L.size()) return fail(VFS_EINVAL, "level out of range");
  Level &l = h->L[level];
  d[0] = l.b.nx; d[1] = l.b.ny; d[2] = l.b.nz; d[3] = l.cx; d[4] = l.cy; d[5] = l.cz;
  return VFS_OK;
}

int vfs_poisson_mg_get_nvert(vfs_poisson *h, int level, double *nvert) {
  if (!h || !nvert) return fail(VFS_EINVAL, "null argument");
  if (level < 0 || level >= (int)h->L.size()) return fail(VFS_EINVAL, "level out of range");
  TRY(download(h, nvert, h->L[level].nvert, h->L[level].g.n()));
  return sync(h);
}

int vfs_poisson_mg_restrict(vfs_poisson *h, int fine, const double *xf, double *fc) {
  if (!h || !xf || !fc) return fail(VFS_EINVAL, "null argument");
  if (fine < 0 || fine + 1 >= (int)h->L.size()) return fail(VFS_EINVAL, "level out of range");
  Level &l = h->L[fine], &q = h->L[fine + 1];
  TRY(upload(h, h->stage, xf, l.g.n()));
  LAUNCH(h, k_da_to_box, lin_grid(l.b.n()), 256, l.g, l.b, h->stage, l.v64[2]);
  LAUNCH(h, k_restrict_f64, box_grid(q.b), 128, l.b, q.b, l.cx, l.cy, l.cz, l.v64[2], l.w64, q.blank, q.v64[1]);
  LAUNCH(h, k_box_to_da, da_grid(q.g), 128, q.g, q.b, q.v64[1], h->stage);
  TRY(download(h, fc, h->stage, q.g.n()));
  return sync(h);
}

int vfs_poisson_mg_interpolate(vfs_poisson *h, int fine, const double *xc, double *ff) {
  if (!h || !xc || !ff) return fail(VFS_EINVAL, "null argument");
  if (fine < 0 || fine + 1 >= (int)h->L.size()) return fail(VFS_EINVAL, "level out of range");
  Level &l = h->L[fine], &q = h->L[fine + 1];
  TRY(upload(h, h->stage, xc, q.g.n()));
  LAUNCH(h, k_da_to_box, lin_grid(q.b.n()), 256, q.g, q.b, h->stage, q.v64[0]);
  LAUNCH(h, k_prolong_f64, box_grid(l.b), 128, l.b, q.b, l.cx, l.cy, l.cz, (const double *)q.v64[0], q.blank,
         l.blank, l.v64[2], 0);
  LAUNCH(h, k_box_to_da, da_grid(l.g), 128, l.g, l.b, l.v64[2], h->stage);
  TRY(download(h, ff, h->stage, l.g.n()));
  return sync(h);
}

int vfs_poisson_mg_vcycle(vfs_poisson *h, int precision, const double *r, double *z) {
  if (!h || !r || !z) return fail(VFS_EINVAL, "null argument");
  if (!h->have_nvert) return fail(VFS_ESTATE, "set_nvert must come first");
  vfs_solve_opts o;
  vfs_poisson_default_opts(&o);
  resolve_opts(o);
  o.precision = precision ? 1 : 0;
  const size_t n = h->box.n();
  TRY(upload(h, h->stage, r, h->g.n()));
  LAUNCH(h, k_da_to_box, lin_grid(n), 256, h->g, h->box, h->stage, h->r);
  TRY(precondition(h, h->r, 1.0, nullptr, nullptr, h->r, o));
  LAUNCH(h, k_box_to_da, da_grid(h->g), 128, h->g, h->box, h->r, h->stage);
  TRY(download(h, z, h->stage, h->g.n()));
  return sync(h);
}

int64_t vfs_poisson_kernel_launches(vfs_poisson *h) { return h ? h->launches : 0; }

int vfs_poisson_set_stream(vfs_poisson *h, void *stream) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  TRY(sync(h));
  cudaStream_t st = (cudaStream_t)stream;
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  if (st) {
    h->stream = st;
    h->own_stream = false;
  } else {
    CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamDefault));
    h->own_stream = true;
  }
  return VFS_OK;
}

int vfs_poisson_profile(vfs_poisson *h, int enable) {
  if (!h) return fail(VFS_EINVAL, "null handle");
  h->prof = enable != 0;
  h->prof_ms = h->prof_bytes = 0.;
  h->prof_launches = 0;
  return VFS_OK;
}

int vfs_poisson_profile_read(vfs_poisson *h, double *ms, double *bytes, int64_t *launches) {
  if (!h || !ms || !bytes || !launches) return fail(VFS_EINVAL, "null argument");
  *ms = h->prof_ms;
  *bytes = h->prof_bytes;
  *launches = h->prof_launches;
  return VFS_OK;
}

}  // extern "C"
