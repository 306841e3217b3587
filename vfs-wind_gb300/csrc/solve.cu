// solve.cu -- kernels of the solve loop: operator apply / residual, j-line
// relaxation, coarsest-level solve and the FP64 Krylov vector kernels.
//
// All of them stream box-layout planes (i fastest) with one thread per cell
// or per j-column, so every warp load is a contiguous 128-byte (FP32) or
// 256-byte (FP64) segment; the 19-point neighbourhood is re-read through L1.
#include <cuda_fp16.h>

#include "common.cuh"
#include "kernels.cuh"

namespace vfs {

// r = rhs - A x for one level (A: 19 planes in the parity-split row layout;
// x, rhs natural).  `color`: -1 every row; 0/1 the k-planes with k % 2 ==
// color; 2/3 the checkerboard columns with (i + k) % 2 == color - 2, whose
// residuals are then written at their split positions (the layout the line
// kernel reads them in); 6/7 the same columns with (i + k) % 2 == color - 6
// written at their natural positions.  Threads walk split positions, so
// operator loads coalesce.
//
// The row a thread takes: its split position p (false when the thread has no
// row of the colour).
__device__ __forceinline__ bool colour_row(const Box &b, int color, int t, int k, int &p) {
  p = t;
  if (color >= 2) {
    const int par = ((color >= 6 ? color - 6 : color - 2) + k) & 1, nh = (b.nx + 1) >> 1;
    if (t >= (par ? b.nx - nh : nh)) return false;
    p = par ? nh + t : t;
    return true;
  }
  return t < b.nx && (color < 0 || (k & 1) == color);
}

template <typename T>
__device__ __forceinline__ void residual_body(Box b, const T *__restrict__ A, const T *__restrict__ x,
                                              const T *__restrict__ rhs, T *__restrict__ r, int color) {
  pdl_trigger();
  pdl_wait();
  const int t = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  int p;
  if (!colour_row(b, color, t, k, p)) return;
  const int i = split_cell(p, b.nx);
  uint32_t idx[NSLOT];
  stencil_index(b, i, j, k, idx);
  const uint32_t n = (uint32_t)b.n(), c = idx[CP], cs = c - i + p;
  T s = (T)0;
#pragma unroll
  for (int q = 0; q < NSLOT; q++) s += __ldcs(&A[q * n + cs]) * __ldg(&x[idx[q]]);
  r[color == 2 || color == 3 ? cs : c] = rhs[c] - s;
}

// The FP32 V-cycle's copy of a level operator (split layout): D = the
// diagonal; half2 plane m < 9 holds the couplings of slots 2m+1 and 2m+2
// divided by D, plane 9 the row sum divided by D (0 for the Neumann rows).
// Rows without a dof get D = 0 and zero couplings.
__device__ __forceinline__ void pack16_row(size_t n, const double *__restrict__ A, __half2 *__restrict__ C,
                                           float *__restrict__ D, size_t c) {
  const double d = A[CP * n + c];
  const double inv = d != 0. ? 1. / d : 0.;
  double sum = d;
  for (int q = 1; q < NSLOT; q++) sum += A[q * n + c];
  for (int m = 0; m < 9; m++)
    C[m * n + c] = __halves2half2(__double2half(A[(2 * m + 1) * n + c] * inv), __double2half(A[(2 * m + 2) * n + c] * inv));
  C[9 * n + c] = __halves2half2(__double2half(sum * inv), __double2half(0.));
  D[c] = (float)d;
}
__global__ void k_pack16(size_t n, const double *__restrict__ A, __half2 *__restrict__ C, float *__restrict__ D) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    pack16_row(n, A, C, D, c);
}
// The finest level's packed copy and FP32 planes of the listed rows only
// (natural box indices; the level's operator is stored split).
__global__ void k_pack16_rows(Box b, const double *__restrict__ A, __half2 *__restrict__ C, float *__restrict__ D,
                              float *__restrict__ A32, const int *__restrict__ rows, const int *__restrict__ nrows) {
  const size_t n = b.n();
  const int nr = *nrows;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nr; w += gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, (size_t)rows[w], i, j, k);
    const size_t c = b.at(split_pos(i, b.nx), j, k);
    pack16_row(n, A, C, D, c);
    for (int q = 0; q < NSLOT; q++) A32[q * n + c] = (float)A[q * n + c];
  }
}

// FP32 r = rhs - A x from the packed operator in difference form,
// r = rhs - D (s x_c + sum_q c_q (x_q - x_c)): rounding the couplings to half
// perturbs each one by at most 2^-11 relative and leaves the row sums (the
// constant null space of the Neumann rows) exact.  44 operator bytes per row
// instead of 76.  Colours and layouts as in residual_body; SPLIT: x and rhs
// in the parity-split row layout (r written as the colour selects).  The
// operator's 44 bytes per row are loaded before pdl_wait (no kernel of the
// V-cycle writes them), x and rhs after it.
template <bool SPLIT>
__device__ __forceinline__ void residual16_body(Box b, const __half2 *__restrict__ C, const float *__restrict__ D,
                                                const float *__restrict__ x, const float *__restrict__ rhs,
                                                float *__restrict__ r, int color) {
  pdl_trigger();
  const int t = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  int p;
  const bool ok = colour_row(b, color, t, k, p);
  if (!ok) p = 0;  // (a row without a cell of the colour loads nothing)
  const int i = split_cell(p, b.nx);
  uint32_t idx[NSLOT];
  stencil_index_t<SPLIT>(b, i, j, k, idx);
  const uint32_t n = (uint32_t)b.n(), c = idx[CP], row = c - (SPLIT ? p : i), cs = row + p, cn = row + i;
  __half2 hc[10];
  float d = 0.f;
  if (ok) {
#pragma unroll
    for (int m = 0; m < 10; m++) hc[m] = __ldcs(&C[m * n + cs]);
    d = __ldcs(&D[cs]);
  }
  pdl_wait();
  if (!ok) return;
  const float xc = __ldg(&x[c]);
  float s = 0.f;
#pragma unroll
  for (int m = 0; m < 9; m++) {
    const float2 f = __half22float2(hc[m]);
    s = fmaf(f.x, __ldg(&x[idx[2 * m + 1]]) - xc, s);
    s = fmaf(f.y, __ldg(&x[idx[2 * m + 2]]) - xc, s);
  }
  s = fmaf(__low2float(hc[9]), xc, s);
  r[color == 2 || color == 3 ? cs : cn] = rhs[SPLIT ? cs : cn] - d * s;
}
__global__ void __launch_bounds__(128) k_residual16(Box b, const __half2 *__restrict__ C,
                                                    const float *__restrict__ D, const float *__restrict__ x,
                                                    const float *__restrict__ rhs, float *__restrict__ r, int color) {
  residual16_body<false>(b, C, D, x, rhs, r, color);
}
__global__ void __launch_bounds__(128) k_residual16_split(Box b, const __half2 *__restrict__ C,
                                                          const float *__restrict__ D, const float *__restrict__ x,
                                                          const float *__restrict__ rhs, float *__restrict__ r,
                                                          int color) {
  residual16_body<true>(b, C, D, x, rhs, r, color);
}

// FP64 y = A x on the unscaled operator.
__global__ void __launch_bounds__(256) k_apply64(Box b, const double *__restrict__ A, const double *__restrict__ x,
                                                 double *__restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= b.nx) return;
  uint32_t idx[NSLOT];
  stencil_index(b, i, j, k, idx);
  const uint32_t n = (uint32_t)b.n(), c = idx[CP];
  double s = 0.;
#pragma unroll
  for (int q = 0; q < NSLOT; q++) s = fma(__ldcs(&A[q * n + c]), __ldg(&x[idx[q]]), s);
  y[c] = s;
}

// FP64 r = rhs - A x (the same products and order as k_residual64; its
// norm comes from k_sumsq over fixed blocks, so no block barrier holds the
// stencil's loads back).
__global__ void __launch_bounds__(256) k_residual64r(Box b, const double *__restrict__ A,
                                                     const double *__restrict__ x, const double *__restrict__ rhs,
                                                     double *__restrict__ r) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= b.nx) return;
  uint32_t idx[NSLOT];
  stencil_index(b, i, j, k, idx);
  const uint32_t n = (uint32_t)b.n(), c = idx[CP];
  double s = 0.;
#pragma unroll
  for (int q = 0; q < NSLOT; q++) s = fma(__ldcs(&A[q * n + c]), __ldg(&x[idx[q]]), s);
  r[c] = rhs[c] - s;
}

// FP64 r = rhs - A x with the block partial of ||r||^2.
__global__ void __launch_bounds__(256) k_residual64(Box b, const double *__restrict__ A, const double *__restrict__ x,
                                                    const double *__restrict__ rhs, double *__restrict__ r,
                                                    double *partial) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  double rr = 0.;
  if (i < b.nx) {
    uint32_t idx[NSLOT];
    stencil_index(b, i, j, k, idx);
    const uint32_t n = (uint32_t)b.n(), c = idx[CP];
    double s = 0.;
#pragma unroll
    for (int q = 0; q < NSLOT; q++) s = fma(__ldcs(&A[q * n + c]), __ldg(&x[idx[q]]), s);
    double v = rhs[c] - s;
    r[c] = v;
    rr = v * v;
  }
  rr = block_sum(rr);
  if (threadIdx.x == 0) partial[blockIdx.x + (size_t)gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z)] = rr;
}

// LU factors of the tridiagonal j-line part (S, CP, N slots) of a level
// operator, computed in FP64 and stored in T.  Rows without a dof get an
// identity line entry.  The j-periodic wrap couplings stay off the line.
template <typename T>
__device__ __forceinline__ void line_lu_body(Box b, const double *__restrict__ A, T *inv, T *cp,
                                             const uint8_t *__restrict__ colflag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (i >= b.nx) return;
  if (colflag && !colflag[(size_t)k * b.nx + i]) return;  // (a column left as it was)
  const size_t n = b.n();
  double cprev = 0.;
  const int p = split_pos(i, b.nx);
  for (int j = 0; j < b.ny; j++) {
    size_t c = b.at(p, j, k);  // split position of cell i
    double d = A[CP * n + c], a = 0., cc = 0.;
    if (d != 0.) {
      a = j > 0 ? A[SP * n + c] : 0.;
      cc = j < b.ny - 1 ? A[NP * n + c] : 0.;
    } else {
      d = 1.;
    }
    double iv = 1.0 / (d - a * cprev);
    inv[c] = (T)iv;
    cp[c] = (T)(cc * iv);
    cprev = cc * iv;
  }
}

// One damped j-line Jacobi sweep: for each (i,k) column solve the
// tridiagonal j-line system (slots S, CP, N; LU factors inv/cp of the whole
// line) with the off-line neighbours taken from x, then
// xo = x + omega (line solution - x).  zero_guess skips the x terms.
//
// The line is split into chunks of M cells, one thread per chunk, so a column
// is worked on by P = ceil(ny/M) threads (blockDim = (32 columns, P)).  Both
// Thomas recurrences are first-order linear recurrences, y_j = alpha_j +
// beta_j y_{j-1} and x_j = y_j + gamma_j x_{j+1}: each chunk runs its part
// with a zero incoming value while accumulating the product of its
// coefficients, a P-step scan over the chunk ends in shared memory supplies
// the true incoming values, and each chunk adds incoming * product.  This is
// the same arithmetic as a serial Thomas sweep up to rounding, with a
// dependent chain of about 2(M + P) steps instead of 2 ny.
template <typename T, int M>
__device__ __forceinline__ void line_sweep_body(Box b, const T *__restrict__ A, const T *__restrict__ inv,
                                                const T *__restrict__ cp, const T *__restrict__ x,
                                                const T *__restrict__ rhs, T *__restrict__ xo, T omega,
                                                int zero_guess) {
  pdl_trigger();
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tx = threadIdx.x, ty = threadIdx.y, TI = blockDim.x, P = blockDim.y;
  T *sA = (T *)smem_raw, *sB = sA + P * TI;
  const int pp = blockIdx.x * TI + tx, k = blockIdx.y;  // split position of the column
  const bool valid = pp < b.nx;
  const uint32_t n = (uint32_t)b.n();
  const int ny = b.ny, j0 = ty * M;
  const int cnt = valid ? max(0, min(M, ny - j0)) : 0;
  const int ii = valid ? split_cell(pp, b.nx) : 0;
  const uint32_t sC = (uint32_t)b.at(valid ? pp : 0, 0, k);  // operator / factor index of the column
  const int im = ii > 0 ? ii - 1 : (b.px ? b.nx - 1 : ii), ip = ii < b.nx - 1 ? ii + 1 : (b.px ? 0 : ii);
  const int km = k > 0 ? k - 1 : (b.pz ? b.nz - 1 : k), kp = k < b.nz - 1 ? k + 1 : (b.pz ? 0 : k);
  const uint32_t sj = b.nx;
  const uint32_t cC = (uint32_t)b.at(ii, 0, k), cE = (uint32_t)b.at(ip, 0, k), cW = (uint32_t)b.at(im, 0, k);
  const uint32_t cT = (uint32_t)b.at(ii, 0, kp), cB = (uint32_t)b.at(ii, 0, km);
  const uint32_t cTE = (uint32_t)b.at(ip, 0, kp), cBE = (uint32_t)b.at(ip, 0, km), cTW = (uint32_t)b.at(im, 0, kp),
                 cBW = (uint32_t)b.at(im, 0, km);
  T r[M], g[M];
  // right-hand sides of the chunk's cells (independent loads)
#pragma unroll
  for (int q = 0; q < M; q++) {
    r[q] = (T)0;
    if (q < cnt) {
      const int j = j0 + q;
      const uint32_t o = (uint32_t)j * sj, c = cC + o, ca = sC + o;
      T v = rhs[c];
      if (!zero_guess) {
        const uint32_t om = (uint32_t)(j > 0 ? j - 1 : (b.py ? ny - 1 : j)) * sj;
        const uint32_t op = (uint32_t)(j < ny - 1 ? j + 1 : (b.py ? 0 : j)) * sj;
        v -= __ldcs(&A[EP * n + ca]) * x[cE + o] + __ldcs(&A[WP * n + ca]) * x[cW + o] +
             __ldcs(&A[TP * n + ca]) * x[cT + o] + __ldcs(&A[BP * n + ca]) * x[cB + o] +
             __ldcs(&A[NE * n + ca]) * x[cE + op] + __ldcs(&A[SE * n + ca]) * x[cE + om] +
             __ldcs(&A[NW * n + ca]) * x[cW + op] + __ldcs(&A[SW * n + ca]) * x[cW + om] +
             __ldcs(&A[TN * n + ca]) * x[cT + op] + __ldcs(&A[BN * n + ca]) * x[cB + op] +
             __ldcs(&A[TS * n + ca]) * x[cT + om] + __ldcs(&A[BS * n + ca]) * x[cB + om] +
             __ldcs(&A[TE * n + ca]) * x[cTE + o] + __ldcs(&A[BE * n + ca]) * x[cBE + o] +
             __ldcs(&A[TW * n + ca]) * x[cTW + o] + __ldcs(&A[BW * n + ca]) * x[cBW + o];
        if (b.py) {
          if (j == 0) v -= A[SP * n + ca] * x[cC + (uint32_t)(ny - 1) * sj];
          if (j == ny - 1) v -= A[NP * n + ca] * x[cC];
        }
      }
      r[q] = v;
    }
  }
  // forward recurrence y_j = (r_j - a_j y_{j-1}) inv_j with y_{j0-1} = 0,
  // g_j = prod_{s=j0..j} (-a_s inv_s)
  T yp = (T)0, gp = (T)1;
#pragma unroll
  for (int q = 0; q < M; q++) {
    if (q < cnt) {
      const int j = j0 + q;
      const uint32_t c = sC + (uint32_t)j * sj;
      const T a = j > 0 ? __ldcs(&A[SP * n + c]) : (T)0;
      const T iv = __ldcs(&inv[c]);
      const T y = (r[q] - a * yp) * iv;
      gp = gp * (-a * iv);
      r[q] = y;
      g[q] = gp;
      yp = y;
    }
  }
  sA[ty * TI + tx] = yp;  // chunk-end y and coefficient product (0 and 1 when empty)
  sB[ty * TI + tx] = gp;
  __syncthreads();
  if (ty == 0) {  // incoming y_{j0-1} of every chunk
    T Y = (T)0;
    for (int t = 0; t < P; t++) {
      const T e = sA[t * TI + tx], G = sB[t * TI + tx];
      sA[t * TI + tx] = Y;
      Y = e + G * Y;
    }
  }
  __syncthreads();
  const T yin = sA[ty * TI + tx];
#pragma unroll
  for (int q = 0; q < M; q++) r[q] += g[q] * yin;
  __syncthreads();
  // backward recurrence x_j = y_j - cp_j x_{j+1} with x_{j0+cnt} = 0,
  // g_j = prod_{s=j..end} (-cp_s)
  T xn = (T)0, hp = (T)1;
#pragma unroll
  for (int q = M - 1; q >= 0; q--) {
    if (q < cnt) {
      const int j = j0 + q;
      const uint32_t c = sC + (uint32_t)j * sj;
      const T cv = j < ny - 1 ? __ldcs(&cp[c]) : (T)0;
      const T v = r[q] - cv * xn;
      hp = hp * (-cv);
      r[q] = v;
      g[q] = hp;
      xn = v;
    }
  }
  sA[ty * TI + tx] = xn;  // chunk-start x and coefficient product
  sB[ty * TI + tx] = hp;
  __syncthreads();
  if (ty == 0) {  // incoming x_{end+1} of every chunk
    T X = (T)0;
    for (int t = P - 1; t >= 0; t--) {
      const T e = sA[t * TI + tx], H = sB[t * TI + tx];
      sA[t * TI + tx] = X;
      X = e + H * X;
    }
  }
  __syncthreads();
  const T xin = sA[ty * TI + tx];
#pragma unroll
  for (int q = 0; q < M; q++) {
    if (q < cnt) {
      const uint32_t c = cC + (uint32_t)(j0 + q) * sj;
      const T v = r[q] + g[q] * xin;
      const T xold = zero_guess ? (T)0 : x[c];
      xo[c] = xold + omega * (v - xold);
    }
  }
}

// The chunked tridiagonal solve of one j-line: on entry y holds the
// chunk's right-hand side (rows j0 .. j0+cnt-1), av/ivv/cv its line
// coefficients and factors; on exit y holds the solution on the chunk.
// Chunk boundaries are joined by scans over the P chunks of the column in
// shared memory (sA, sB: P x TI words each).
template <typename T, int M>
__device__ __forceinline__ void line_tri_solve(T (&y)[M], const T (&av)[M], const T (&ivv)[M], const T (&cv)[M],
                                               int cnt, T *sA, T *sB) {
  const int tx = threadIdx.x, ty = threadIdx.y, TI = blockDim.x, P = blockDim.y;
  T g[M];
  T yp = (T)0, gp = (T)1;
#pragma unroll
  for (int q = 0; q < M; q++) {
    g[q] = (T)0;
    if (q < cnt) {
      const T v = (y[q] - av[q] * yp) * ivv[q];
      gp = gp * (-av[q] * ivv[q]);
      y[q] = v;
      g[q] = gp;
      yp = v;
    }
  }
  sA[ty * TI + tx] = yp;
  sB[ty * TI + tx] = gp;
  __syncthreads();
  if (ty == 0) {
    T Y = (T)0;
    for (int s = 0; s < P; s++) {
      const T e = sA[s * TI + tx], G = sB[s * TI + tx];
      sA[s * TI + tx] = Y;
      Y = e + G * Y;
    }
  }
  __syncthreads();
  const T yin = sA[ty * TI + tx];
#pragma unroll
  for (int q = 0; q < M; q++) y[q] += g[q] * yin;
  __syncthreads();
  T xn = (T)0, hp = (T)1;
#pragma unroll
  for (int q = M - 1; q >= 0; q--) {
    if (q < cnt) {
      const T v = y[q] - cv[q] * xn;
      hp = hp * (-cv[q]);
      y[q] = v;
      g[q] = hp;
      xn = v;
    }
  }
  sA[ty * TI + tx] = xn;
  sB[ty * TI + tx] = hp;
  __syncthreads();
  if (ty == 0) {
    T X = (T)0;
    for (int s = P - 1; s >= 0; s--) {
      const T e = sA[s * TI + tx], H = sB[s * TI + tx];
      sA[s * TI + tx] = X;
      X = e + H * X;
    }
  }
  __syncthreads();
  const T xin = sA[ty * TI + tx];
#pragma unroll
  for (int q = 0; q < M; q++) y[q] += g[q] * xin;
}

// Column of a line kernel thread: split position pp of column t of the
// launch's colour (2/3 and 4/5: checkerboard columns (i + k) % 2 == color %
// 2; 0/1: k-planes with k % 2 == color; -1: every column).
__device__ __forceinline__ bool line_column(const Box &b, int color, int t, int k, int &pp) {
  pp = t;
  if (color >= 2) {
    const int par = (color + k) & 1, nh = (b.nx + 1) >> 1;
    pp = par ? nh + t : t;
    return t < (par ? b.nx - nh : nh);
  }
  return t < b.nx && (color < 0 || (k & 1) == color);
}

// Tridiagonal j-line correction of a line-relaxation sweep in correction
// form: with r = rhs - A x already formed, solve L d = r on every (i,k)
// column (L = the line part S, CP, N of A, factors inv/cp) and update
// x += omega d (x = omega d when zero_guess, r then being the right-hand
// side).  `color`: -1 every column; 0/1 the k-planes with k % 2 == color
// (zebra by planes); 2/3 the checkerboard columns with (i + k) % 2 ==
// color % 2 (zebra by columns), whose r is read at split positions; 4/5
// the same columns with r natural (a right-hand side used as r).  A
// column's threads walk split positions, so operator and factor loads
// coalesce; x is natural.  Same chunked recurrences and scans as
// line_sweep_body; only 5 words per cell are streamed.
template <typename T, int M, bool SPLIT = false>
__device__ __forceinline__ void line_tri_body(Box b, const T *__restrict__ r, const T *__restrict__ Asp,
                                              const T *__restrict__ inv, const T *__restrict__ cp, T *x, T omega,
                                              int zero_guess, int color) {
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tx = threadIdx.x, ty = threadIdx.y, TI = blockDim.x, P = blockDim.y;
  T *sA = (T *)smem_raw, *sB = sA + P * TI;
  const int t = blockIdx.x * TI + tx, k = blockIdx.y;
  int pp;
  const bool valid = line_column(b, color, t, k, pp);
  const int ny = b.ny, j0 = ty * M;
  const int cnt = valid ? max(0, min(M, ny - j0)) : 0;
  const uint32_t sj = b.nx;
  const uint32_t cS = valid ? (uint32_t)b.at(pp, 0, k) : 0u;  // operator / factor index
  // x (and a right-hand side used as r, colours 4/5) at the split position
  // when the level's vectors are split, else natural
  const uint32_t cX = SPLIT ? cS : (valid ? (uint32_t)b.at(split_cell(pp, b.nx), 0, k) : 0u);
  const uint32_t cR = (color == 2 || color == 3) ? cS : cX;
  // the line coefficients and factors first (no kernel of the V-cycle
  // writes them), then, once the previous kernel has completed, the
  // residual and the x being corrected: each chunk's loads in one memory
  // round trip
  T y[M], av[M], ivv[M], cv[M], xv[M];
#pragma unroll
  for (int q = 0; q < M; q++) {
    const int j = j0 + q;
    const uint32_t o = (uint32_t)j * sj;
    const bool in = q < cnt;
    av[q] = in && j > 0 ? __ldcs(&Asp[cS + o]) : (T)0;
    ivv[q] = in ? __ldcs(&inv[cS + o]) : (T)0;
    cv[q] = in && j < ny - 1 ? __ldcs(&cp[cS + o]) : (T)0;
  }
  pdl_wait();
  if (SPLIT && zero_guess == 2 && color >= 2) {
    // the first colour of a sweep from a zero guess: the other colour's
    // half of each row (the same column t there) starts at 0 too, so that
    // no separate clearing pass is needed
    const int par = (color + k) & 1, nh = (b.nx + 1) >> 1;
    const int po = par ? t : nh + t;
    if (t < (par ? nh : b.nx - nh)) {
      const uint32_t co = (uint32_t)b.at(po, 0, k);
      for (int q = 0; q < M; q++)
        if (j0 + q < ny) x[co + (uint32_t)(j0 + q) * sj] = (T)0;
    }
  }
#pragma unroll
  for (int q = 0; q < M; q++) {
    const uint32_t o = (uint32_t)(j0 + q) * sj;
    const bool in = q < cnt;
    y[q] = in ? __ldcs(&r[cR + o]) : (T)0;
    xv[q] = in && !zero_guess ? x[cX + o] : (T)0;
  }
  line_tri_solve<T, M>(y, av, ivv, cv, cnt, sA, sB);
#pragma unroll
  for (int q = 0; q < M; q++) {
    if (q < cnt) {
      const uint32_t c = cX + (uint32_t)(j0 + q) * sj;
      x[c] = xv[q] + omega * y[q];
    }
  }
}

// One colour of the checkerboard zebra sweep with the residual formed in
// the line kernel (FP32 V-cycle, packed operator): for the columns with
// (i + k) % 2 == color % 2 (color 2/3),
//   r = rhs - A x   (difference form over the packed couplings, in the
//                    order of k_residual16),
//   x_new = x + omega L^-1 r   on every j-line (L, inv, cp as line_tri_body).
// x is read from two buffers and written to a third, so that no block reads
// a value another block of the same launch writes: a cell of the launch's
// colour (the columns' own cells and the same-colour diagonal columns
// i +- 1, k +- 1, or any wrap neighbour that has that parity) is read from
// xo, a cell of the other colour from xn, and the new values of the
// launch's columns go to xd.  Within one sweep the first colour runs with
// xo = xn = x and xd = t, the second with xo = x, xn = xd = t, which
// reproduces the in-place two-kernel sweep bit for bit.  own_zero: the
// launch's colour is zero (first sweep from a zero guess, xo not read);
// both_zero: every x is zero (r = rhs; xo and xn not read).
template <int M, bool OWN_ZERO, bool BOTH_ZERO>
__device__ __forceinline__ void line_fused16_body(Box b, const __half2 *__restrict__ C, const float *__restrict__ D,
                                                  const float *xo, const float *xn, const float *__restrict__ rhs,
                                                  const float *__restrict__ Asp, const float *__restrict__ inv,
                                                  const float *__restrict__ cp, float *xd, float omega, int color) {
  pdl_trigger();
  pdl_wait();  // (a wait after the factor loads would cost the kernel spills)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tx = threadIdx.x, ty = threadIdx.y, TI = blockDim.x, P = blockDim.y;
  float *sA = (float *)smem_raw, *sB = sA + P * TI;
  const int t = blockIdx.x * TI + tx, k = blockIdx.y;
  int pp;
  const bool valid = line_column(b, color, t, k, pp);
  const int ny = b.ny, j0 = ty * M;
  const int cnt = valid ? max(0, min(M, ny - j0)) : 0;
  const uint32_t sj = b.nx, n = (uint32_t)b.n();
  const int i = valid ? split_cell(pp, b.nx) : 0;
  const uint32_t cS = valid ? (uint32_t)b.at(pp, 0, k) : 0u;
  const uint32_t cX = valid ? (uint32_t)b.at(i, 0, k) : 0u;
  // slots holding a cell of the launch's colour (read from xo): decided by
  // the neighbour column's own (i + k) parity, wraps included
  uint32_t own = 0;
  {
    const Nbr q(b, i, 0, k);
    const int par = (i + k) & 1;
#pragma unroll
    for (int m = 1; m < NSLOT; m++) {
      int di, dj, dk;
      slot_offset(m, di, dj, dk);
      const int ii = di < 0 ? q.im : (di > 0 ? q.ip : i), kk = dk < 0 ? q.km : (dk > 0 ? q.kp : k);
      if (((ii + kk) & 1) == par) own |= 1u << m;
    }
  }
  float y[M], av[M], ivv[M], cv[M], xv[M];
#pragma unroll
  for (int q = 0; q < M; q++) {
    const int j = j0 + q;
    const uint32_t o = (uint32_t)j * sj;
    const bool in = q < cnt;
    av[q] = in && j > 0 ? __ldcs(&Asp[cS + o]) : 0.f;
    ivv[q] = in ? __ldcs(&inv[cS + o]) : 0.f;
    cv[q] = in && j < ny - 1 ? __ldcs(&cp[cS + o]) : 0.f;
  }
#pragma unroll
  for (int q = 0; q < M; q++) {
    // rows past the line end recompute the last row (in bounds, unused)
    const int j = j0 + min(q, max(cnt - 1, 0));
    const uint32_t o = (uint32_t)j * sj;
    if (BOTH_ZERO) {
      y[q] = __ldcs(&rhs[cX + o]);
      xv[q] = 0.f;
      continue;
    }
    uint32_t idx[NSLOT];
    stencil_index(b, i, j, k, idx);
    const uint32_t cs = cS + o;
    // every load unconditional (addresses selected, values masked after)
    float xs[NSLOT];
#pragma unroll
    for (int m = 0; m < NSLOT; m++) {
      const float *src = ((own >> m) & 1) || m == CP ? xo : xn;
      xs[m] = __ldg(&src[idx[m]]);
    }
    float2 f[10];
#pragma unroll
    for (int m = 0; m < 10; m++) f[m] = __half22float2(__ldcs(&C[m * n + cs]));
    const float rv = __ldg(&rhs[idx[CP]]), dv = __ldcs(&D[cs]);
    if (OWN_ZERO) {
#pragma unroll
      for (int m = 0; m < NSLOT; m++)
        if (((own >> m) & 1) || m == CP) xs[m] = 0.f;
    }
    const float xc = xs[CP];
    float sum = 0.f;
#pragma unroll
    for (int m = 0; m < 9; m++) {
      sum = fmaf(f[m].x, xs[2 * m + 1] - xc, sum);
      sum = fmaf(f[m].y, xs[2 * m + 2] - xc, sum);
    }
    sum = fmaf(f[9].x, xc, sum);
    y[q] = rv - dv * sum;
    xv[q] = xc;
  }
  line_tri_solve<float, M>(y, av, ivv, cv, cnt, sA, sB);
#pragma unroll
  for (int q = 0; q < M; q++) {
    if (q < cnt) {
      const uint32_t c = cX + (uint32_t)(j0 + q) * sj;
      xd[c] = xv[q] + omega * y[q];
    }
  }
}
#define LINE_FUSED(NAME, OZ, BZ, MINB)                                                                             \
  __global__ void __launch_bounds__(kLineMaxThreads, MINB) NAME(Box b, const __half2 *C, const float *D, const float *xo,         \
                                                 const float *xn, const float *rhs, const float *Asp,             \
                                                 const float *inv, const float *cp, float *xd, float omega,       \
                                                 int color) {                                                     \
    line_fused16_body<kLineChunk, OZ, BZ>(b, C, D, xo, xn, rhs, Asp, inv, cp, xd, omega, color);                 \
  }
// one 384-thread block per SM: the compiler keeps several cells' loads in
// flight (168 registers); capped at two blocks it spills and runs at half
// the speed
LINE_FUSED(k_line_fused16, false, false, 1)
LINE_FUSED(k_line_fused16_oz, true, false, 1)
LINE_FUSED(k_line_fused16_z, true, true, 1)
#undef LINE_FUSED

// Coarsest level: x = dinv * rhs over the nd dof cells, 0 elsewhere.  One
// warp per cell (8 per block): every block gathers the nd right-hand-side
// values into shared memory, and a warp forms its cell's row of dinv times
// them in FP64 (lane-strided sums, then a fixed shuffle tree).  dmap: the
// row of a cell, -1 off the dofs.
template <typename T>
__device__ __forceinline__ void coarsest_body(int nd, const int *__restrict__ dmap, const int *__restrict__ didx,
                                              const double *__restrict__ dinv, const T *__restrict__ rhs, T *x,
                                              int n) {
  pdl_trigger();
  pdl_wait();
  __shared__ double sb[1024];
  for (int q = threadIdx.x; q < nd; q += blockDim.x) sb[q] = (double)rhs[didx[q]];
  __syncthreads();
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= n) return;
  const int r = dmap[c];
  double s = 0.;
  if (r >= 0)
    for (int q = lane; q < nd; q += 32) s = fma(dinv[(size_t)r * nd + q], sb[q], s);
  s = warp_sum(s);
  if (lane == 0) x[c] = (T)s;
}

template <typename T>
__device__ __forceinline__ void cast_body(const double *__restrict__ src, T *__restrict__ dst, size_t n) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    dst[c] = (T)src[c];
}

// ---- FP64 Krylov kernels (fixed grid, deterministic block partials) ----
// Delayed classical Gram-Schmidt with reorthogonalisation (DCGS2: Bielich,
// Langou, Thomas, Swirydowicz, Yamazaki, Boman, "Low-synch Gram-Schmidt with
// delayed reorthogonalization for Krylov solvers", Parallel Computing 2022).
// Arnoldi step j holds the finished orthonormal vectors Q_0..Q_{j-1}, the
// pending vector u (step j-1's projected vector, projected once) and the new
// vector w = A z_j.  One pass forms Q.u, Q.w, u.u and u.w; one more pass
// reorthogonalises and normalises u into Q_j and projects w against
// Q_0..Q_j.  Two passes over the basis and one host read-back per step.
//
// Rows of the block partials (and of the reduced values): Q_v.u at v,
// Q_v.w at kGsB + v, u.u at kGsUU, u.w at kGsUU + 1.
template <int NV>
__device__ __forceinline__ void gs_dots_body(size_t n, int v0, const double *const *__restrict__ Q,
                                             const double *__restrict__ u, const double *__restrict__ w, int first,
                                             double *__restrict__ partial) {
  constexpr int NA = 2 * NV + 2;
  __shared__ double sh[8][NA];
  double acc[NA];
#pragma unroll
  for (int a = 0; a < NA; a++) acc[a] = 0.;
  const double *q[NV > 0 ? NV : 1];
#pragma unroll
  for (int v = 0; v < NV; v++) q[v] = Q[v0 + v];
  const size_t base = (size_t)blockIdx.x * blockDim.x * kGsTile + threadIdx.x;
#pragma unroll 2
  for (int t = 0; t < kGsTile; t++) {
    const size_t c = base + (size_t)t * blockDim.x;
    if (c < n) {
      const double uc = u[c], wc = w[c];
#pragma unroll
      for (int v = 0; v < NV; v++) {
        const double qv = __ldcs(q[v] + c);
        acc[v] = fma(qv, uc, acc[v]);
        acc[NV + v] = fma(qv, wc, acc[NV + v]);
      }
      acc[2 * NV] = fma(uc, uc, acc[2 * NV]);
      acc[2 * NV + 1] = fma(uc, wc, acc[2 * NV + 1]);
    }
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < NA; a++) {
    const double s = warp_sum(acc[a]);
    if (lane == 0) sh[wp][a] = s;
  }
  __syncthreads();
  if (threadIdx.x < NA) {
    const int a = threadIdx.x;
    double s = 0.;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k][a];
    const int row = a < NV ? v0 + a : a < 2 * NV ? kGsB + v0 + a - NV : kGsUU + a - 2 * NV;
    if (a < 2 * NV || first) partial[(size_t)row * gridDim.x + blockIdx.x] = s;
  }
}
// Classical Gram-Schmidt in one pass (the orthogonalisation of PETSc's
// GMRES with its default refinement "never"): rows kGsB + v0 + v of the
// block partials hold Q_{v0+v}.w, the basis vectors kept unnormalised.
template <int NV>
__device__ __forceinline__ void cgs_dots_body(size_t n, int v0, const double *const *__restrict__ Q,
                                              const double *__restrict__ w, double *__restrict__ partial) {
  __shared__ double sh[8][NV];
  double acc[NV];
  const double *q[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    acc[v] = 0.;
    q[v] = Q[v0 + v];
  }
  const size_t base = (size_t)blockIdx.x * blockDim.x * kGsTile + threadIdx.x;
#pragma unroll 2
  for (int t = 0; t < kGsTile; t++) {
    const size_t c = base + (size_t)t * blockDim.x;
    if (c < n) {
      const double wc = __ldg(&w[c]);
#pragma unroll
      for (int v = 0; v < NV; v++) acc[v] = fma(__ldcs(q[v] + c), wc, acc[v]);
    }
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < NV; v++) {
    const double s = warp_sum(acc[v]);
    if (lane == 0) sh[wp][v] = s;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k][threadIdx.x];
    partial[(size_t)(kGsB + v0 + threadIdx.x) * gridDim.x + blockIdx.x] = s;
  }
}
#define CGS_DOTS(NV)                                                                                            \
  __global__ void __launch_bounds__(256) k_cgs_dots##NV(size_t n, int v0, const double *const *Q,               \
                                                        const double *w, double *partial) {                     \
    cgs_dots_body<NV>(n, v0, Q, w, partial);                                                                   \
  }
CGS_DOTS(1)
CGS_DOTS(2)
CGS_DOTS(3)
CGS_DOTS(4)
CGS_DOTS(5)
CGS_DOTS(6)
CGS_DOTS(7)
CGS_DOTS(8)
#undef CGS_DOTS

// One block per basis vector v: d = Q_v.w summed in a fixed order, then
// h_v = d / ||Q_v|| (the Hessenberg entry, red[v]) and the update
// coefficient h_v / ||Q_v|| (red[kGsB + v]); dsv[2v+1] = 1 / ||Q_v||.
__global__ void k_cgs_reduce(const double *__restrict__ partial, int nb, const double *__restrict__ dsv,
                             double *red) {
  const int v = blockIdx.x;
  double s = 0.;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) s += partial[(size_t)(kGsB + v) * nb + q];
  s = block_sum(s);
  if (threadIdx.x == 0) {
    const double sinv = dsv[2 * v + 1], hv = s * sinv;
    red[v] = hv;
    red[kGsB + v] = hv * sinv;
  }
}

// w -= sum_v red[kGsB + v] Q_v; block partials of ||w||^2.
__global__ void __launch_bounds__(256) k_cgs_update(size_t n, int nv, const double *const *__restrict__ Q,
                                                    const double *__restrict__ red, double *__restrict__ w,
                                                    double *partial) {
  const size_t base = (size_t)blockIdx.x * blockDim.x * kGsTile + threadIdx.x;
  double aw[kGsTile];
#pragma unroll
  for (int t = 0; t < kGsTile; t++) {
    const size_t c = base + (size_t)t * blockDim.x;
    aw[t] = c < n ? w[c] : 0.;
  }
  for (int v = 0; v < nv; v++) {
    const double *p = Q[v];
    const double cb = -red[kGsB + v];
#pragma unroll
    for (int t = 0; t < kGsTile; t++) {
      const size_t c = base + (size_t)t * blockDim.x;
      if (c < n) aw[t] = fma(cb, __ldcs(&p[c]), aw[t]);
    }
  }
  double ss = 0.;
#pragma unroll
  for (int t = 0; t < kGsTile; t++) {
    const size_t c = base + (size_t)t * blockDim.x;
    if (c < n) {
      w[c] = aw[t];
      ss = fma(aw[t], aw[t], ss);
    }
  }
  ss = block_sum(ss);
  if (threadIdx.x == 0) partial[blockIdx.x] = ss;
}

#define GS_DOTS(NV)                                                                                            \
  __global__ void __launch_bounds__(256) k_gs_dots##NV(size_t n, int v0, const double *const *Q,               \
                                                       const double *u, const double *w, int first,            \
                                                       double *partial) {                                      \
    gs_dots_body<NV>(n, v0, Q, u, w, first, partial);                                                         \
  }
GS_DOTS(0)
GS_DOTS(1)
GS_DOTS(2)
GS_DOTS(3)
GS_DOTS(4)
GS_DOTS(5)
GS_DOTS(6)
GS_DOTS(7)
GS_DOTS(8)
#undef GS_DOTS

// Sums the used partial rows (one block per row: Q.u rows 0..nv-1, Q.w rows
// kGsB.., then u.u and u.w) in a fixed order into red at the same row index.
__global__ void k_gs_reduce(const double *__restrict__ partial, int nb, int nv, double *red) {
  const int r = blockIdx.x;
  const int row = r < nv ? r : r < 2 * nv ? kGsB + r - nv : kGsUU + r - 2 * nv;
  double s = 0.;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) s += partial[(size_t)row * nb + q];
  s = block_sum(s);
  if (threadIdx.x == 0) red[row] = s;
}

// Step coefficients from the reduced dots: r = ||u - Q a|| by Pythagoras
// (the reorthogonalisation coefficients a = Q.u are small next to ||u||),
// h = Q_j.w for the finished Q_j = (u - Q a) / r.  red[kGsR] = r,
// red[kGsR + 1] = h, red[kGsR + 2] = 1 / r (0 when r is 0).
__global__ void k_gs_coef(int nv, double *red) {
  if (threadIdx.x != 0) return;
  double aa = 0., ab = 0.;
  for (int v = 0; v < nv; v++) {
    aa = fma(red[v], red[v], aa);
    ab = fma(red[v], red[kGsB + v], ab);
  }
  const double r2 = red[kGsUU] - aa;
  const double r = r2 > 0. ? sqrt(r2) : 0.;
  const double rinv = r > 0. ? 1. / r : 0.;
  red[kGsR] = r;
  red[kGsR + 1] = (red[kGsUU + 1] - ab) * rinv;
  red[kGsR + 2] = rinv;
}

// Q_j = (u - sum_v a_v Q_v) / r written over u; w -= sum_v b_v Q_v + h Q_j;
// block partials of ||w||^2.  Each basis vector streams once; the u and w
// tiles stay in registers.
__global__ void __launch_bounds__(256) k_gs_update(size_t n, int nv, const double *const *__restrict__ Q,
                                                   const double *__restrict__ red, double *__restrict__ u,
                                                   double *__restrict__ w, double *partial) {
  const size_t base = (size_t)blockIdx.x * blockDim.x * kGsTile + threadIdx.x;
  double au[kGsTile], aw[kGsTile];
#pragma unroll
  for (int t = 0; t < kGsTile; t++) {
    const size_t c = base + (size_t)t * blockDim.x;
    au[t] = c < n ? u[c] : 0.;
    aw[t] = c < n ? w[c] : 0.;
  }
  for (int v = 0; v < nv; v++) {
    const double *p = Q[v];
    const double ca = -red[v], cb = -red[kGsB + v];
#pragma unroll
    for (int t = 0; t < kGsTile; t++) {
      const size_t c = base + (size_t)t * blockDim.x;
      if (c < n) {
        const double qv = __ldcs(&p[c]);
        au[t] = fma(ca, qv, au[t]);
        aw[t] = fma(cb, qv, aw[t]);
      }
    }
  }
  const double rinv = red[kGsR + 2], hj = -red[kGsR + 1];
  double ss = 0.;
#pragma unroll
  for (int t = 0; t < kGsTile; t++) {
    const size_t c = base + (size_t)t * blockDim.x;
    if (c < n) {
      const double qj = au[t] * rinv;
      const double wn = fma(hj, qj, aw[t]);
      u[c] = qj;
      w[c] = wn;
      ss = fma(wn, wn, ss);
    }
  }
  ss = block_sum(ss);
  if (threadIdx.x == 0) partial[blockIdx.x] = ss;
}

// x += sum_v coef[v] Z_v
__global__ void __launch_bounds__(256) k_axpy_multi(size_t n, int nv, const double *const *__restrict__ Z,
                                                    const double *__restrict__ coef, double *__restrict__ x) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    double acc = x[c];
    for (int v = 0; v < nv; v++) acc = fma(coef[v], __ldcs(&Z[v][c]), acc);
    x[c] = acc;
  }
}

// out = (s v) * scale in FP64: the aj row scaling that turns the FP64
// Krylov vector into the FP64 V-cycle's right-hand side; with sinv set, s is
// multiplied by sinv[0] (the inverse norm of v, formed on the device).
__global__ void k_scale_to(size_t n, const double *__restrict__ v, double s, const double *__restrict__ sinv,
                           const double *__restrict__ scale, double *__restrict__ out) {
  if (sinv) s *= sinv[0];
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    out[c] = s * v[c] * scale[c];
}
// The same into the FP32 V-cycle's right-hand side, with the products in
// FP32 (the result is rounded to FP32 anyway and FP64 arithmetic is the
// scarce pipe), one element per thread.
// split_nx > 0: out is in the parity-split row layout of rows of split_nx
// cells (the finest FP32 level's right-hand side under the checkerboard
// smoother).
__global__ void __launch_bounds__(256) k_scale_to32(size_t n, const double *__restrict__ v, float s,
                                                    const float *__restrict__ sinv, const float *__restrict__ scale,
                                                    float *__restrict__ out, int split_nx) {
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  size_t o = c;
  if (split_nx > 0) {
    const uint32_t i = (uint32_t)(c % (uint32_t)split_nx);
    o = c - i + split_pos((int)i, split_nx);
  }
  out[o] = (float)v[c] * ((sinv ? s * sinv[0] : s) * scale[c]);
}
// ||V||^2 from the block partials into out[0], 1/||V|| into out[1] and
// out32[0] (0 for a zero vector); one block
__global__ void k_reduce_norm(const double *partial, int nb, double *out, float *out32) {
  double s = 0.;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) s += partial[q];
  s = block_sum(s);
  if (threadIdx.x == 0) {
    const double inv = s > 0. ? 1. / sqrt(s) : 0.;
    out[0] = s;
    out[1] = inv;
    out32[0] = (float)inv;
  }
}
// out = x (the V-cycle's result in FP32 or FP64, widened), one element per thread
// split_nx > 0: x32 is in the parity-split row layout (rows of split_nx)
__global__ void __launch_bounds__(256) k_to64(size_t n, const float *__restrict__ x32,
                                              const double *__restrict__ x64, double *__restrict__ out,
                                              int split_nx) {
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  size_t o = c;
  if (x32 && split_nx > 0) {
    const uint32_t i = (uint32_t)(c % (uint32_t)split_nx);
    o = c - i + split_pos((int)i, split_nx);
  }
  out[c] = x32 ? (double)x32[o] : x64[c];
}
__global__ void k_sumsq(size_t n, const double *__restrict__ x, double *partial) {
  double s = 0.;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    s = fma(x[c], x[c], s);
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// ---- history projection of the initial guess ----
// Block partials (grid-stride, fixed block count: deterministic) of the dot
// products v . Y_j for j < K and of v . v: row j of `partial` holds v . Y_j,
// row K holds v . v.  K is a template argument, so that no FMA of an
// unused slot is issued on the FP64 pipe.
template <int K>
__device__ __forceinline__ void hist_dots_body(size_t n, const HistPtrs &Y, const double *__restrict__ v,
                                               double *partial) {
  double s[K + 1];
#pragma unroll
  for (int j = 0; j <= K; j++) s[j] = 0.;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const double vc = v[c];
#pragma unroll
    for (int j = 0; j < K; j++) s[j] = fma(vc, __ldg(&Y.p[j][c]), s[j]);
    s[K] = fma(vc, vc, s[K]);
  }
#pragma unroll
  for (int j = 0; j <= K; j++) {
    const double t = block_sum(s[j]);
    if (threadIdx.x == 0) partial[(size_t)j * gridDim.x + blockIdx.x] = t;
  }
}
// one kernel per basis size: up to 7 vectors the accumulators fit the 32
// registers of 8 resident blocks; larger sizes get 64 (4 blocks) instead of
// spilling
template <int K>
__global__ void __launch_bounds__(256, K <= 7 ? 8 : 4) k_hist_dots(size_t n, HistPtrs Y,
                                                                  const double *__restrict__ v, double *partial) {
  hist_dots_body<K>(n, Y, v, partial);
}

// x = sum_j c_j X_j and r = b - sum_j c_j Y_j (Y_j = A X_j), with the block
// partials of ||r||^2.  coefficients in `c` (device, k values).
template <int K>
__device__ __forceinline__ void hist_combine_body(size_t n, const HistPtrs &X, const HistPtrs &Y,
                                                  const double *__restrict__ c, const double *__restrict__ b,
                                                  double *__restrict__ x, double *__restrict__ r, double *partial) {
  double cj[K];
#pragma unroll
  for (int j = 0; j < K; j++) cj[j] = c[j];
  double s = 0.;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    double xv = 0., yv = 0.;
#pragma unroll
    for (int j = 0; j < K; j++) {
      xv = fma(cj[j], __ldg(&X.p[j][q]), xv);
      yv = fma(cj[j], __ldg(&Y.p[j][q]), yv);
    }
    const double rv = b[q] - yv;
    x[q] = xv;
    r[q] = rv;
    s = fma(rv, rv, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}
template <int K>
__global__ void __launch_bounds__(256, K <= 8 ? 8 : 4) k_hist_combine(size_t n, HistPtrs X, HistPtrs Y,
                                                                     const double *__restrict__ c,
                                                                     const double *__restrict__ b,
                                                                     double *__restrict__ x, double *__restrict__ r,
                                                                     double *partial) {
  hist_combine_body<K>(n, X, Y, c, b, x, r, partial);
}

// Moments over the fluid cells of z, for the estimated error of a guess
// (z = one V-cycle of its residual): pass 0 writes the block partials of
// sum z (row 0) and of the cell count (row 1); pass 1 those of
// sum (z - mean)^2 (row 0).
__global__ void __launch_bounds__(256) k_fluid_moments(size_t n, const uint8_t *__restrict__ fluid,
                                                       const double *__restrict__ z, double mean, int pass,
                                                       double *partial) {
  double s = 0., cnt = 0.;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    if (!fluid[q]) continue;
    const double v = z[q];
    if (pass == 0) {
      s += v;
      cnt += 1.;
    } else {
      const double d = v - mean;
      s = fma(d, d, s);
    }
  }
  s = block_sum(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (pass == 0) {
    cnt = block_sum(cnt);
    if (threadIdx.x == 0) partial[gridDim.x + blockIdx.x] = cnt;
  }
}

// A converged solve into the history: its iterate x and image y = b - r
// (r = b - A x, the solve's final FP64 residual).  FIRST: x and y become
// the newest solution Xn, Yn, and row 0 of `partial` gets the block
// partials of y . y.  Otherwise the differences from the previous newest,
// dx = x - Xn and e = y - Yn, go to a difference slot (dX, dY), x and y
// replace Xn and Yn, and the rows get e . E_j for the M other differences
// E_j of the window (rows 0..M-1), e . e (row M), Yn_old . e (row M + 1)
// and y . y (row M + 2).  The differences are formed per cell before any
// product, so that their Gram entries carry rounding relative to their own
// size, not to the size of the nearly parallel solutions.
template <int M, bool FIRST>
__device__ __forceinline__ void hist_push_body(size_t n, const double *__restrict__ x, const double *__restrict__ b,
                                               const double *__restrict__ r, double *Xn, double *Yn,
                                               double *__restrict__ dX, double *__restrict__ dY, const HistPtrs &E,
                                               double *partial) {
  constexpr int R = FIRST ? 1 : M + 3;
  double s[R];
#pragma unroll
  for (int j = 0; j < R; j++) s[j] = 0.;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const double xv = x[q], y = b[q] - r[q];
    if (FIRST) {
      Xn[q] = xv;
      Yn[q] = y;
      s[0] = fma(y, y, s[0]);
      continue;
    }
    const double xo = Xn[q], yo = Yn[q], e = y - yo;
    dX[q] = xv - xo;
    dY[q] = e;
    Xn[q] = xv;
    Yn[q] = y;
#pragma unroll
    for (int j = 0; j < M; j++) s[j] = fma(e, __ldg(&E.p[j][q]), s[j]);
    s[M] = fma(e, e, s[M]);
    s[M + 1] = fma(yo, e, s[M + 1]);
    s[M + 2] = fma(y, y, s[M + 2]);
  }
#pragma unroll
  for (int j = 0; j < R; j++) {
    const double t = block_sum(s[j]);
    if (threadIdx.x == 0) partial[(size_t)j * gridDim.x + blockIdx.x] = t;
  }
}
template <int M, bool FIRST>
__global__ void __launch_bounds__(256, FIRST || M <= 1 ? 8 : 4) k_hist_push(size_t n, const double *__restrict__ x,
                                                                         const double *__restrict__ b,
                                                                         const double *__restrict__ r, double *Xn,
                                                                         double *Yn, double *dX, double *dY,
                                                                         HistPtrs E, double *partial) {
  hist_push_body<M, FIRST>(n, x, b, r, Xn, Yn, dX, dY, E, partial);
}

// Host launches of the history kernels for a basis of k vectors (push: m
// other differences in the window); sizes outside 1..kHistMax (0..kHistMax-2
// for m) launch nothing.
void launch_hist_dots(cudaStream_t st, int blocks, size_t n, const HistPtrs &Y, int k, const double *v,
                      double *partial) {
  switch (k) {
#define VFS_K(K) \
  case K: k_hist_dots<K><<<blocks, 256, 0, st>>>(n, Y, v, partial); break;
    VFS_K(1) VFS_K(2) VFS_K(3) VFS_K(4) VFS_K(5) VFS_K(6) VFS_K(7) VFS_K(8) VFS_K(9) VFS_K(10) VFS_K(11) VFS_K(12)
#undef VFS_K
    default: break;
  }
}
void launch_hist_combine(cudaStream_t st, int blocks, size_t n, const HistPtrs &X, const HistPtrs &Y, int k,
                         const double *c, const double *b, double *x, double *r, double *partial) {
  switch (k) {
#define VFS_K(K) \
  case K: k_hist_combine<K><<<blocks, 256, 0, st>>>(n, X, Y, c, b, x, r, partial); break;
    VFS_K(1) VFS_K(2) VFS_K(3) VFS_K(4) VFS_K(5) VFS_K(6) VFS_K(7) VFS_K(8) VFS_K(9) VFS_K(10) VFS_K(11) VFS_K(12)
#undef VFS_K
    default: break;
  }
}
void launch_hist_push(cudaStream_t st, int blocks, size_t n, const double *x, const double *b, const double *r,
                      double *Xn, double *Yn, double *dX, double *dY, const HistPtrs &E, int m, bool first,
                      double *partial) {
  if (first) {
    k_hist_push<0, true><<<blocks, 256, 0, st>>>(n, x, b, r, Xn, Yn, dX, dY, E, partial);
    return;
  }
  switch (m) {
#define VFS_M(M) \
  case M: k_hist_push<M, false><<<blocks, 256, 0, st>>>(n, x, b, r, Xn, Yn, dX, dY, E, partial); break;
    VFS_M(0) VFS_M(1) VFS_M(2) VFS_M(3) VFS_M(4) VFS_M(5) VFS_M(6) VFS_M(7) VFS_M(8) VFS_M(9) VFS_M(10)
#undef VFS_M
    default: break;
  }
}

#define TYPED(T, S, TRI_THREADS, TRI_MINB)                                                                         \
  __global__ void __launch_bounds__(256) k_residual_##S(Box b, const T *A, const T *x, const T *rhs, T *r,  \
                                                        int color) {                                       \
    residual_body<T>(b, A, x, rhs, r, color);                                                              \
  }                                                                                                        \
  __global__ void k_line_lu_##S(Box b, const double *A64, T *inv, T *cp, const uint8_t *colflag) {            \
    line_lu_body<T>(b, A64, inv, cp, colflag);                                                            \
  }                                                                                                        \
  __global__ void __launch_bounds__(768, 1) k_line_sweep_##S(Box b, const T *A, const T *inv, const T *cp,      \
                                                           const T *x, const T *rhs, T *xo, T omega, int zg) { \
    line_sweep_body<T, kLineChunk>(b, A, inv, cp, x, rhs, xo, omega, zg);                                   \
  }                                                                                                        \
  __global__ void __launch_bounds__(TRI_THREADS, TRI_MINB) k_line_tri_##S(Box b, const T *r, const T *Asp, const T *inv,  \
                                                       const T *cp, T *x, T omega, int zg, int color) {        \
    line_tri_body<T, kLineChunk>(b, r, Asp, inv, cp, x, omega, zg, color);                                    \
  }                                                                                                        \
  __global__ void __launch_bounds__(256) k_coarsest_##S(int nd, const int *dmap, const int *didx,             \
                                                        const double *dinv, const T *rhs, T *x, int n) {     \
    coarsest_body<T>(nd, dmap, didx, dinv, rhs, x, n);                                                     \
  }                                                                                                        \
  __global__ void k_cast_planes_##S(const double *src, T *dst, size_t n) { cast_body<T>(src, dst, n); }
// the line kernel keeps a whole chunk in registers: at most 384 threads per
// block (16 columns of up to 24 chunks in FP32, 4 columns in FP64) so that
// neither precision spills
TYPED(float, f32, kLineMaxThreads, 1)
TYPED(double, f64, kLineMaxThreads, 1)
#undef TYPED
// the finest FP32 level with x and the right-hand side in the split layout
__global__ void __launch_bounds__(kLineMaxThreads, 1) k_line_tri_f32_split(Box b, const float *r, const float *Asp,
                                                                          const float *inv, const float *cp, float *x,
                                                                          float omega, int zg, int color) {
  line_tri_body<float, kLineChunk, true>(b, r, Asp, inv, cp, x, omega, zg, color);
}

}  // namespace vfs
