// unet.cu -- the learned initial guess: a 3-level 3-D U-Net (16/32/64
// channels, 3x3x3 convolutions, ReLU, average-pool down, nearest up, skip
// concatenation, 1x1 head) with BF16 weights and activations on the tensor
// cores and FP32 accumulation, trained by its own forward, backward and
// Adam kernels.  No counterpart in the reference.
//
// Activations are channels-last BF16 tensors [z][y][x][C] over the interior
// box of a level (C a multiple of 16); gradients of activations are FP32.
// Convolutions are implicit GEMMs on mma.sync m16n8k16 (A = 16 voxels along
// x by 16 input channels of one tap, B = 16 input by 8 output channels):
//   * k_conv: a CTA computes a 16x8x4 voxel tile for CT output channels; the
//     input tile with its one-voxel halo (18x10x6 voxels x 16 channels) is
//     staged in shared memory one 16-channel group at a time, rows padded to
//     48 bytes so that ldmatrix rows fall in distinct banks; weights are
//     pre-packed in mma fragment order and read through L1.  The loader
//     fuses the skip concatenation (two sources) and the nearest-neighbour
//     upsampling (a half-resolution source); zero padding at the box edges.
//     The same kernel computes data gradients with flipped, transposed
//     weights and an FP32 epilogue.
//   * k_wgrad: weight gradients, A = input tile transposed (ldmatrix.trans),
//     B = pre-activation gradient tile; a warp owns one tap of a dz plane,
//     a CTA loops over voxel tiles and flushes with one atomic per weight.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "vfs_poisson.h"

namespace vfs {
void set_last_error(const std::string &msg);  // poisson.cu
}

namespace {

typedef __nv_bfloat16 bf16;

constexpr int TX = 16, TY = 8, TZ = 4;                       // output tile
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;         // with halo
constexpr int HVOX = HX * HY * HZ;                           // 1080
constexpr int ROWB = 48;                                     // 16 ch + pad, bytes
constexpr int CONV_SMEM = HVOX * ROWB;                       // 51840
constexpr int CONV_THREADS = 256;                            // 8 warps x 4 rows

struct Src {
  const bf16 *p;  // channels-last tensor
  int c;          // its channel count
  int up;         // 1: half resolution, read at (x/2, y/2, z/2)
};

struct ConvGeom {
  int nx, ny, nz;  // output (and full-resolution input) dims
  Src s0, s1;      // concatenated input: s0 channels first
  int groups;      // (s0.c + s1.c) / 16
  int nt_tot;      // output channels / 8
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4(uint32_t *r, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t *r, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::);
}

// Stage channel group g of the concatenated input around the output tile
// origin (x0, y0, z0) into `tile` ([HVOX][ROWB bytes]); zeros outside.
__device__ void load_group(const ConvGeom &G, int g, int x0, int y0, int z0, unsigned char *tile) {
  const int g0 = G.s0.c / 16;
  const Src &S = g < g0 ? G.s0 : G.s1;
  const int coff = (g < g0 ? g : g - g0) * 16;
  const int sx = S.up ? G.nx / 2 : G.nx, sy = S.up ? G.ny / 2 : G.ny;
  for (int q = threadIdx.x; q < HVOX * 2; q += blockDim.x) {
    const int v = q >> 1, half = q & 1;
    const int hx = v % HX, hy = (v / HX) % HY, hz = v / (HX * HY);
    const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
    unsigned char *dst = tile + v * ROWB + half * 16;
    if (gx < 0 || gy < 0 || gz < 0 || gx >= G.nx || gy >= G.ny || gz >= G.nz) {
      *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
    } else {
      size_t vox = S.up ? ((size_t)(gz >> 1) * sy + (gy >> 1)) * sx + (gx >> 1) : ((size_t)gz * sy + gy) * sx + gx;
      cp_async16(smem_u32(dst), S.p + vox * S.c + coff + half * 8);
    }
  }
  cp_async_wait_all();
}

// Forward (FWD: + bias, ReLU, BF16 out) or data-gradient (FP32 out split
// into two destinations at channel `split`) 3x3x3 convolution.
template <int CT, bool FWD>
__global__ void __launch_bounds__(CONV_THREADS) k_conv(ConvGeom G, const uint2 *__restrict__ wpk,
                                                       const float *__restrict__ bias, int relu, bf16 *out_b,
                                                       float *out0, float *out1, int split) {
  extern __shared__ __align__(16) unsigned char tile[];
  constexpr int NT = CT / 8, MT = 4;
  const int tiles_x = (G.nx + TX - 1) / TX;
  const int x0 = (blockIdx.x % tiles_x) * TX, y0 = (blockIdx.x / tiles_x) * TY, z0 = blockIdx.y * TZ;
  const int slice = blockIdx.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float acc[MT][NT][4];
#pragma unroll
  for (int m = 0; m < MT; m++)
#pragma unroll
    for (int n = 0; n < NT; n++) acc[m][n][0] = acc[m][n][1] = acc[m][n][2] = acc[m][n][3] = 0.f;
  const uint32_t tbase = smem_u32(tile);
  for (int g = 0; g < G.groups; g++) {
    __syncthreads();
    load_group(G, g, x0, y0, z0, tile);
    __syncthreads();
    for (int tap = 0; tap < 27; tap++) {
      const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // halo offsets 0..2
      uint2 b[NT];
      const uint2 *wp = wpk + ((size_t)(tap * G.groups + g) * G.nt_tot + slice * NT) * 32 + lane;
#pragma unroll
      for (int n = 0; n < NT; n++) b[n] = __ldg(wp + n * 32);
#pragma unroll
      for (int m = 0; m < MT; m++) {
        const int r = warp * MT + m, yy = r % TY, zz = r / TY;
        const int hv = ((zz + dz) * HY + (yy + dy)) * HX + (lane & 15) + dx;
        uint32_t a[4];
        ldsm_x4(a, tbase + hv * ROWB + (lane >> 4) * 16);
#pragma unroll
        for (int n = 0; n < NT; n++) mma_bf16(acc[m][n], a, b[n].x, b[n].y);
      }
    }
  }
  // epilogue: rows lane/4 and lane/4 + 8 of each m-tile, channels pairs
  const int cout = G.nt_tot * 8;
#pragma unroll
  for (int m = 0; m < MT; m++) {
    const int r = warp * MT + m, y = y0 + r % TY, z = z0 + r / TY;
    if (y >= G.ny || z >= G.nz) continue;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int x = x0 + (lane >> 2) + h * 8;
      if (x >= G.nx) continue;
      const size_t v = ((size_t)z * G.ny + y) * G.nx + x;
#pragma unroll
      for (int n = 0; n < NT; n++) {
        const int co = slice * CT + n * 8 + (lane & 3) * 2;
        float c0 = acc[m][n][2 * h], c1 = acc[m][n][2 * h + 1];
        if (FWD) {
          c0 += bias[co];
          c1 += bias[co + 1];
          if (relu) { c0 = fmaxf(c0, 0.f); c1 = fmaxf(c1, 0.f); }
          *reinterpret_cast<__nv_bfloat162 *>(out_b + v * cout + co) = __floats2bfloat162_rn(c0, c1);
        } else if (co < split) {
          *reinterpret_cast<float2 *>(out0 + v * split + co) = make_float2(c0, c1);
        } else {
          *reinterpret_cast<float2 *>(out1 + v * (cout - split) + co - split) = make_float2(c0, c1);
        }
      }
    }
  }
}

// Weight gradient dW[tap][ci][co] += sum_v X[v + off(tap)][ci] * Gp[v][co]
// for input channel group blockIdx.y and the 9 taps of plane dz =
// blockIdx.z - 1 (warp w: dy = w / 3 - 1, dx = w % 3 - 1).
template <int COUT>
__global__ void __launch_bounds__(288) k_wgrad(ConvGeom G, const bf16 *__restrict__ gpre, float *dW) {
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned char *xt = smem;
  unsigned char *gt = smem + CONV_SMEM;
  constexpr int GROW = COUT * 2 + 16;  // bytes per voxel row of the gradient tile
  constexpr int NT = COUT / 8;
  const int g = blockIdx.y, dzi = blockIdx.z;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int dyi = warp / 3, dxi = warp % 3;
  const int tiles_x = (G.nx + TX - 1) / TX, tiles_y = (G.ny + TY - 1) / TY, tiles_z = (G.nz + TZ - 1) / TZ;
  const int ntiles = tiles_x * tiles_y * tiles_z;
  float acc[NT][4];
#pragma unroll
  for (int n = 0; n < NT; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
  const uint32_t xb = smem_u32(xt), gb = smem_u32(gt);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int x0 = (t % tiles_x) * TX, y0 = ((t / tiles_x) % tiles_y) * TY, z0 = (t / (tiles_x * tiles_y)) * TZ;
    __syncthreads();
    // gradient tile (TX x TY x TZ voxels, COUT channels), zeros outside
    for (int q = threadIdx.x; q < TX * TY * TZ * (COUT / 8); q += blockDim.x) {
      const int v = q / (COUT / 8), part = q % (COUT / 8);
      const int x = x0 + v % TX, y = y0 + (v / TX) % TY, z = z0 + v / (TX * TY);
      unsigned char *dst = gt + v * GROW + part * 16;
      if (x >= G.nx || y >= G.ny || z >= G.nz)
        *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
      else
        cp_async16(smem_u32(dst), gpre + (((size_t)z * G.ny + y) * G.nx + x) * COUT + part * 8);
    }
    load_group(G, g, x0, y0, z0, xt);  // waits for both tiles' copies
    __syncthreads();
    for (int r = 0; r < TY * TZ; r++) {
      const int yy = r % TY, zz = r / TY;
      // A = X^T: rows ci, columns voxels; matrix i = lane / 8 holds
      // (ci half i & 1, voxel half i >> 1)
      const int vox = ((lane >> 4) << 3) + (lane & 7);
      const int hv = ((zz + dzi) * HY + (yy + dyi)) * HX + vox + dxi;
      uint32_t a[4];
      ldsm_x4_t(a, xb + hv * ROWB + ((lane >> 3) & 1) * 16);
#pragma unroll
      for (int n = 0; n < NT; n += 2) {
        // B = gradient rows (voxels) x 8 output channels; x4.trans covers
        // (voxel half i & 1, n-tile n + (i >> 1))
        const int gv = (r * TX) + (((lane >> 3) & 1) << 3) + (lane & 7);
        uint32_t b[4];
        ldsm_x4_t(b, gb + gv * GROW + (n + (lane >> 4)) * 16);
        mma_bf16(acc[n], a, b[0], b[1]);
        mma_bf16(acc[n + 1], a, b[2], b[3]);
      }
    }
  }
  const int tap = dzi * 9 + dyi * 3 + dxi;
  const int cin = G.groups * 16;
#pragma unroll
  for (int n = 0; n < NT; n++) {
    const int ci = g * 16 + (lane >> 2), co = n * 8 + (lane & 3) * 2;
    float *w = dW + ((size_t)tap * cin + ci) * COUT + co;
    atomicAdd(w, acc[n][0]);
    atomicAdd(w + 1, acc[n][1]);
    atomicAdd(w + 8 * COUT, acc[n][2]);
    atomicAdd(w + 8 * COUT + 1, acc[n][3]);
  }
}

// Pack FP32 weights W[tap][ci][co] into mma B fragments: forward
// (k = ci, n = co) and data-gradient (tap flipped, k = co, n = ci).
__global__ void k_pack(const float *W, int cin, int cout, uint2 *fwd, uint2 *bwd) {
  const int total = 27 * (cin / 16) * (cout / 8) * 32;
  const int total_t = 27 * (cout / 16) * (cin / 8) * 32;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total + total_t; e += gridDim.x * blockDim.x) {
    const bool tr = e >= total;
    const int q = tr ? e - total : e;
    const int lane = q & 31, rest = q >> 5;
    const int NTt = tr ? cin / 8 : cout / 8, Gt = tr ? cout / 16 : cin / 16;
    const int nt = rest % NTt, g = (rest / NTt) % Gt, tap = rest / (NTt * Gt);
    const int k0 = g * 16 + (lane & 3) * 2, n = nt * 8 + (lane >> 2);
    float w[4];
    for (int s = 0; s < 4; s++) {
      const int k = k0 + (s & 1) + (s >> 1) * 8;
      w[s] = tr ? W[((size_t)(26 - tap) * cin + n) * cout + k] : W[((size_t)tap * cin + k) * cout + n];
    }
    __nv_bfloat162 lo = __floats2bfloat162_rn(w[0], w[1]), hi = __floats2bfloat162_rn(w[2], w[3]);
    uint2 v;
    v.x = *reinterpret_cast<uint32_t *>(&lo);
    v.y = *reinterpret_cast<uint32_t *>(&hi);
    (tr ? bwd : fwd)[q] = v;
  }
}

// Network input: 4 FP32 feature planes (a sub-box of planes of dims
// (fx, fy, fz) starting at (ox, oy, oz)) -> BF16 [v][16], channels 4..15 zero.
__global__ void k_input(const float *feat, int fx, int fy, int fz, int ox, int oy, int oz, int nx, int ny, int nz,
                        bf16 *xin) {
  const size_t n = (size_t)nx * ny * nz;
  const size_t plane = (size_t)fx * fy * fz;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const uint32_t vr = (uint32_t)v / (uint32_t)nx;  // < 2^32 voxels
    const int x = (int)((uint32_t)v - vr * (uint32_t)nx), y = (int)(vr % (uint32_t)ny), z = (int)(vr / (uint32_t)ny);
    const size_t s = ((size_t)(z + oz) * fy + (y + oy)) * fx + (x + ox);
    __align__(16) bf16 row[16];
    for (int c = 0; c < 16; c++) row[c] = __float2bfloat16_rn(c < 4 ? feat[c * plane + s] : 0.f);
    uint4 *d = reinterpret_cast<uint4 *>(xin + v * 16);
    d[0] = reinterpret_cast<uint4 *>(row)[0];
    d[1] = reinterpret_cast<uint4 *>(row)[1];
  }
}

// 2x2x2 average pool of a BF16 tensor (fine dims nx, ny, nz).
__global__ void k_pool(const bf16 *in, int nx, int ny, int nz, int C, bf16 *out) {
  const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
  const size_t n = (size_t)cx * cy * cz * C;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % C);
    const size_t v = e / C;
    const int x = (int)(v % cx), y = (int)((v / cx) % cy), z = (int)(v / ((size_t)cx * cy));
    float s = 0.f;
    for (int q = 0; q < 8; q++) {
      const size_t f = ((size_t)(2 * z + (q >> 2)) * ny + 2 * y + ((q >> 1) & 1)) * nx + 2 * x + (q & 1);
      s += __bfloat162float(in[f * C + c]);
    }
    out[e] = __float2bfloat16_rn(0.125f * s);
  }
}

// Gradient of the pool: fine[v][c] += 0.125 * coarse[parent][c].
__global__ void k_pool_bwd(const float *gc, int nx, int ny, int nz, int C, float *gf) {
  const size_t n = (size_t)nx * ny * nz * C;
  const int cx = nx / 2, cy = ny / 2;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % C);
    const size_t v = e / C;
    const uint32_t vr = (uint32_t)v / (uint32_t)nx;  // < 2^32 voxels
    const int x = (int)((uint32_t)v - vr * (uint32_t)nx), y = (int)(vr % (uint32_t)ny), z = (int)(vr / (uint32_t)ny);
    gf[e] += 0.125f * gc[(((size_t)(z >> 1) * cy + (y >> 1)) * cx + (x >> 1)) * C + c];
  }
}

// Gradient of the nearest upsampling: coarse[v][c] = sum of the 8 children.
__global__ void k_up_bwd(const float *gf, int nx, int ny, int nz, int C, float *gc) {
  const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
  const size_t n = (size_t)cx * cy * cz * C;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % C);
    const size_t v = e / C;
    const int x = (int)(v % cx), y = (int)((v / cx) % cy), z = (int)(v / ((size_t)cx * cy));
    float s = 0.f;
    for (int q = 0; q < 8; q++) {
      const size_t f = ((size_t)(2 * z + (q >> 2)) * ny + 2 * y + ((q >> 1) & 1)) * nx + 2 * x + (q & 1);
      s += gf[f * C + c];
    }
    gc[e] = s;
  }
}

// ReLU backward + bias gradient: gp = bf16(g * (y > 0)); db[c] += sum gp.
// The grid stride is a multiple of C, so a thread keeps one channel.
__global__ void k_relu_bwd(const float *g, const bf16 *y, size_t n, int C, bf16 *gp, float *db) {
  __shared__ float red[256];
  float s = 0.f;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const float v = __bfloat162float(y[e]) > 0.f ? g[e] : 0.f;
    gp[e] = __float2bfloat16_rn(v);
    s += v;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  if ((int)threadIdx.x < C) {
    float t = 0.f;
    for (int q = threadIdx.x; q < (int)blockDim.x; q += C) t += red[q];
    atomicAdd(&db[threadIdx.x], t);
  }
}

__device__ __forceinline__ float block_sum(float v, float *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  float t = 0.f;
  if (threadIdx.x < 32) {
    t = l < (int)(blockDim.x >> 5) ? sh[l] : 0.f;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

// Sum of the loss weights of a sub-box (for the mean).
__global__ void k_weight_sum(const float *wt, int fx, int fy, int ox, int oy, int oz, int nx, int ny, int nz,
                             float *out) {
  __shared__ float sh[32];
  const size_t n = (size_t)nx * ny * nz;
  float s = 0.f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const uint32_t vr = (uint32_t)v / (uint32_t)nx;  // < 2^32 voxels
    const int x = (int)((uint32_t)v - vr * (uint32_t)nx), y = (int)(vr % (uint32_t)ny), z = (int)(vr / (uint32_t)ny);
    s += wt[((size_t)(z + oz) * fy + (y + oy)) * fx + (x + ox)];
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) atomicAdd(out, s);
}

// 1x1 head: out = sum_c d[v][c] * wh[c] + bh.  With a target: the weighted
// mean squared error (weights / their sum), its gradient into gd (FP32
// [v][16]) and the head's parameter gradients.
__global__ void k_head(const bf16 *d, size_t n, const float *wh, float *out, const float *tgt, const float *wt,
                       int fx, int fy, int ox, int oy, int oz, int nx, int ny, const float *wsum, float *gd,
                       float *gwh, float *loss) {
  __shared__ float sh[32];
  float lw[17];
  for (int c = 0; c < 17; c++) lw[c] = 0.f;
  float ls = 0.f;
  const float inv = tgt ? 1.f / fmaxf(*wsum, 1.f) : 0.f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    float dv[16];
    const uint4 *src = reinterpret_cast<const uint4 *>(d + v * 16);
    uint4 q0 = src[0], q1 = src[1];
    const bf16 *h0 = reinterpret_cast<const bf16 *>(&q0), *h1 = reinterpret_cast<const bf16 *>(&q1);
    float o = wh[16];
    for (int c = 0; c < 8; c++) {
      dv[c] = __bfloat162float(h0[c]);
      dv[c + 8] = __bfloat162float(h1[c]);
    }
    for (int c = 0; c < 16; c++) o += dv[c] * wh[c];
    if (out) out[v] = o;
    if (tgt) {
      const uint32_t vr = (uint32_t)v / (uint32_t)nx;  // < 2^32 voxels
      const int x = (int)((uint32_t)v - vr * (uint32_t)nx), y = (int)(vr % (uint32_t)ny), z = (int)(vr / (uint32_t)ny);
      const size_t s = ((size_t)(z + oz) * fy + (y + oy)) * fx + (x + ox);
      const float w = wt[s] * inv, e = o - tgt[s];
      ls += w * e * e;
      const float go = 2.f * w * e;
      float4 *gdst = reinterpret_cast<float4 *>(gd + v * 16);
      for (int c = 0; c < 4; c++)
        gdst[c] = make_float4(go * wh[4 * c], go * wh[4 * c + 1], go * wh[4 * c + 2], go * wh[4 * c + 3]);
      for (int c = 0; c < 16; c++) lw[c] += go * dv[c];
      lw[16] += go;
    }
  }
  if (!tgt) return;
  for (int c = 0; c < 17; c++) {
    const float t = block_sum(lw[c], sh);
    if (threadIdx.x == 0) atomicAdd(&gwh[c], t);
  }
  const float t = block_sum(ls, sh);
  if (threadIdx.x == 0) atomicAdd(loss, t);
}

// Stencil offsets of the 19-point operator planes (slot order of the
// reference's PoissonLHSNew: C E W N S T B NE SE NW SW TN BN TS BS TE BE TW BW).
__constant__ int8_t c_off[19][3] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                    {0, 0, 1},   {0, 0, -1},  {1, 1, 0},  {1, -1, 0}, {-1, 1, 0},
                                    {-1, -1, 0}, {0, 1, 1},   {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
                                    {1, 0, 1},   {1, 0, -1},  {-1, 0, 1}, {-1, 0, -1}};

struct Crop {
  int fx, fy, fz, ox, oy, oz, nx, ny, nz;
  __device__ size_t glob(int x, int y, int z) const {
    return ((size_t)(z + oz) * fy + (y + oy)) * fx + (x + ox);
  }
  __device__ bool inner(int x, int y, int z) const {
    return x >= 1 && y >= 1 && z >= 1 && x < nx - 1 && y < ny - 1 && z < nz - 1;
  }
};

// Residual of the learned correction on the crop's inner cells (all 19
// neighbours inside the crop): res = f2 - s * (A out), A the row-scaled
// operator (19 planes over the feature grid), q = w res; acc[0] += w,
// acc[1] += w res^2.
__global__ void k_res_fwd(Crop cr, const float *__restrict__ op, const float *__restrict__ f2,
                          const float *__restrict__ wt, const float *__restrict__ out, float s, float *q,
                          float *acc) {
  __shared__ float sh[32];
  const size_t n = (size_t)cr.nx * cr.ny * cr.nz, plane = (size_t)cr.fx * cr.fy * cr.fz;
  float sw = 0.f, sr = 0.f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(v % cr.nx), y = (int)((v / cr.nx) % cr.ny), z = (int)(v / ((size_t)cr.nx * cr.ny));
    float qv = 0.f;
    if (cr.inner(x, y, z)) {
      const size_t gv = cr.glob(x, y, z);
      const float w = wt[gv];
      if (w > 0.f) {
        float a = 0.f;
        for (int t = 0; t < 19; t++)
          a += op[t * plane + gv] * out[((size_t)(z + c_off[t][2]) * cr.ny + (y + c_off[t][1])) * cr.nx + x + c_off[t][0]];
        const float res = f2[gv] - s * a;
        qv = w * res;
        sw += w;
        sr += w * res * res;
      }
    }
    q[v] = qv;
  }
  sw = block_sum(sw, sh);
  if (threadIdx.x == 0) atomicAdd(acc, sw);
  sr = block_sum(sr, sh);
  if (threadIdx.x == 0) atomicAdd(acc + 1, sr);
}

// dLoss/dout = alpha * 2 w (out - t) / sum(w)  -  beta * 2 s A^T q / acc[0];
// the MSE part is added to the loss.
__global__ void k_res_bwd(Crop cr, const float *__restrict__ op, const float *__restrict__ q, const float *acc,
                          float s, float beta, const float *__restrict__ out, const float *__restrict__ tgt,
                          const float *__restrict__ wt, const float *wsum, float alpha, float *gout, float *loss) {
  __shared__ float sh[32];
  const size_t n = (size_t)cr.nx * cr.ny * cr.nz, plane = (size_t)cr.fx * cr.fy * cr.fz;
  const float ir = acc[0] > 0.f ? 2.f * s * beta / acc[0] : 0.f;
  const float im = alpha / fmaxf(*wsum, 1.f);
  float lm = 0.f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(v % cr.nx), y = (int)((v / cr.nx) % cr.ny), z = (int)(v / ((size_t)cr.nx * cr.ny));
    const size_t gv = cr.glob(x, y, z);
    float g = 0.f;
    if (alpha > 0.f) {
      const float w = wt[gv] * im, e = out[v] - tgt[gv];
      g += 2.f * w * e;
      lm += w * e * e;
    }
    float at = 0.f;
    for (int t = 0; t < 19; t++) {
      const int xi = x - c_off[t][0], yi = y - c_off[t][1], zi = z - c_off[t][2];
      if (!cr.inner(xi, yi, zi)) continue;
      at += op[t * plane + cr.glob(xi, yi, zi)] * q[((size_t)zi * cr.ny + yi) * cr.nx + xi];
    }
    gout[v] = g - ir * at;
  }
  lm = block_sum(lm, sh);
  if (threadIdx.x == 0) atomicAdd(loss, lm);
}

// Head backward from dLoss/dout: gd[v][c] = gout wh[c]; head gradients.
__global__ void k_head_bwd(const bf16 *d, size_t n, const float *wh, const float *gout, float *gd, float *gwh) {
  __shared__ float sh[32];
  float lw[17];
  for (int c = 0; c < 17; c++) lw[c] = 0.f;
  for (size_t v = blockIdx.x * (size_t)blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
    const uint4 *src = reinterpret_cast<const uint4 *>(d + v * 16);
    uint4 q0 = src[0], q1 = src[1];
    const bf16 *h0 = reinterpret_cast<const bf16 *>(&q0), *h1 = reinterpret_cast<const bf16 *>(&q1);
    const float go = gout[v];
    float4 *gdst = reinterpret_cast<float4 *>(gd + v * 16);
    for (int c = 0; c < 4; c++)
      gdst[c] = make_float4(go * wh[4 * c], go * wh[4 * c + 1], go * wh[4 * c + 2], go * wh[4 * c + 3]);
    for (int c = 0; c < 8; c++) {
      lw[c] += go * __bfloat162float(h0[c]);
      lw[c + 8] += go * __bfloat162float(h1[c]);
    }
    lw[16] += go;
  }
  for (int c = 0; c < 17; c++) {
    const float t = block_sum(lw[c], sh);
    if (threadIdx.x == 0) atomicAdd(&gwh[c], t);
  }
}

// Adam (bias-corrected; c1 = 1 - beta1^t, c2 = 1 - beta2^t).
__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float c1,
                       float c2, float eps) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

int grid_for(size_t n, int threads = 256) {
  size_t b = (n + threads - 1) / threads;
  return (int)(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}

int fail(int code, const std::string &m) {
  vfs::set_last_error(m);
  return code;
}

struct Conv {
  int cin, cout;     // cin = concatenated input channels
  int c0, c1, up0;   // concat split and upsampling of the first source
  size_t w, b;       // offsets of weights [27][cin][cout] and bias in params
  size_t pk, pkt;    // offsets of the packed fragments (uint2)
};

}  // namespace

// Layer table of the network (indices into the activation list below).
struct vfs_unet {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<Conv> conv;
  size_t nparams = 0, npk = 0, head = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  uint2 *pk = nullptr;
  int64_t t = 0;
  bool packed = false;
  // activations for the current dims
  int nx = 0, ny = 0, nz = 0;
  bool train_bufs = false;
  std::vector<void *> bufs;
  bf16 *xin, *e0a, *e0b, *p0, *e1a, *e1b, *p1, *e2a, *e2b, *d1a, *d1b, *d0a, *d0b, *gpre;
  float *g_d0b, *g_d0a, *g_upd1b, *g_e0b, *g_d1b, *g_d1a, *g_upe2b, *g_e1b, *g_e2b, *g_e2a, *g_p1, *g_e1a, *g_p0,
      *g_e0a, *scal, *obuf, *qbuf, *gobuf;
  int64_t launches = 0;
};

namespace {

int setup_layers(vfs_unet *u) {
  // (cin, cout, c0, c1, up0): e0a e0b e1a e1b e2a e2b d1a d1b d0a d0b
  const int tab[10][5] = {{16, 16, 16, 0, 0}, {16, 16, 16, 0, 0}, {16, 32, 16, 0, 0}, {32, 32, 32, 0, 0},
                          {32, 64, 32, 0, 0}, {64, 64, 64, 0, 0}, {96, 32, 64, 32, 1}, {32, 32, 32, 0, 0},
                          {48, 16, 32, 16, 1}, {16, 16, 16, 0, 0}};
  size_t off = 0, pk = 0;
  for (auto &r : tab) {
    Conv c{r[0], r[1], r[2], r[3], r[4], 0, 0, 0, 0};
    c.w = off;
    off += (size_t)27 * c.cin * c.cout;
    c.b = off;
    off += c.cout;
    c.pk = pk;
    pk += (size_t)27 * (c.cin / 16) * (c.cout / 8) * 32;
    c.pkt = pk;
    pk += (size_t)27 * (c.cout / 16) * (c.cin / 8) * 32;
    u->conv.push_back(c);
  }
  u->head = off;
  off += 17;
  u->nparams = off;
  u->npk = pk;
  return 0;
}

void free_bufs(vfs_unet *u) {
  for (void *p : u->bufs) cudaFree(p);
  u->bufs.clear();
  u->nx = u->ny = u->nz = 0;
}

template <typename T>
int balloc(vfs_unet *u, T **p, size_t count) {
  if (cudaMalloc((void **)p, count * sizeof(T) + 16) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return fail(VFS_ENOMEM, "U-Net activation allocation failed");
  }
  u->bufs.push_back(*p);
  return VFS_OK;
}

int ensure_bufs(vfs_unet *u, int nx, int ny, int nz, bool train) {
  if (u->nx == nx && u->ny == ny && u->nz == nz && (u->train_bufs || !train)) return VFS_OK;
  free_bufs(u);
  const size_t n0 = (size_t)nx * ny * nz, n1 = n0 / 8, n2 = n0 / 64;
  int rc = VFS_OK;
#define A(p, n) \
  if ((rc = balloc(u, &u->p, n)) != VFS_OK) return rc;
  A(xin, n0 * 16) A(e0a, n0 * 16) A(e0b, n0 * 16) A(p0, n1 * 16) A(e1a, n1 * 32) A(e1b, n1 * 32) A(p1, n2 * 32)
  A(e2a, n2 * 64) A(e2b, n2 * 64) A(d1a, n1 * 32) A(d1b, n1 * 32) A(d0a, n0 * 16) A(d0b, n0 * 16) A(scal, 64)
  if (train) {
    A(gpre, n0 * 16) A(g_d0b, n0 * 16) A(g_d0a, n0 * 16) A(g_upd1b, n0 * 32) A(g_e0b, n0 * 16) A(g_d1b, n1 * 32)
    A(g_d1a, n1 * 32) A(g_upe2b, n1 * 64) A(g_e1b, n1 * 32) A(g_e2b, n2 * 64) A(g_e2a, n2 * 64) A(g_p1, n2 * 32)
    A(g_e1a, n1 * 32) A(g_p0, n1 * 16) A(g_e0a, n0 * 16) A(obuf, n0) A(qbuf, n0) A(gobuf, n0)
  }
#undef A
  u->nx = nx;
  u->ny = ny;
  u->nz = nz;
  u->train_bufs = train;
  return VFS_OK;
}

bool kernels_configured = false;
std::mutex cfg_mu;

template <typename K>
bool smem_attr(K kernel, int bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess;
}

int configure_kernels() {
  std::lock_guard<std::mutex> lk(cfg_mu);
  if (kernels_configured) return VFS_OK;
  const int wg = CONV_SMEM + TX * TY * TZ * 16;  // + gradient tile rows of (2 COUT + 16) bytes
  bool ok = smem_attr(k_conv<16, true>, CONV_SMEM) && smem_attr(k_conv<32, true>, CONV_SMEM) &&
            smem_attr(k_conv<16, false>, CONV_SMEM) && smem_attr(k_conv<32, false>, CONV_SMEM) &&
            smem_attr(k_wgrad<16>, wg + TX * TY * TZ * 32) && smem_attr(k_wgrad<32>, wg + TX * TY * TZ * 64) &&
            smem_attr(k_wgrad<64>, wg + TX * TY * TZ * 128);
  if (!ok) {
    cudaGetLastError();
    return fail(VFS_ECUDA, "cudaFuncSetAttribute failed for the U-Net kernels");
  }
  kernels_configured = true;
  return VFS_OK;
}

ConvGeom geom(const Conv &c, int nx, int ny, int nz, const bf16 *s0, const bf16 *s1) {
  ConvGeom G;
  G.nx = nx; G.ny = ny; G.nz = nz;
  G.s0 = Src{s0, c.c0, c.up0};
  G.s1 = Src{s1, c.c1, 0};
  G.groups = c.cin / 16;
  G.nt_tot = c.cout / 8;
  return G;
}

dim3 conv_grid(int nx, int ny, int nz, int slices) {
  return dim3(((nx + TX - 1) / TX) * ((ny + TY - 1) / TY), (nz + TZ - 1) / TZ, slices);
}

void conv_fwd(vfs_unet *u, int li, int nx, int ny, int nz, const bf16 *s0, const bf16 *s1, bf16 *out) {
  const Conv &c = u->conv[li];
  ConvGeom G = geom(c, nx, ny, nz, s0, s1);
  const uint2 *w = u->pk + c.pk;
  const float *b = u->params + c.b;
  if (c.cout % 32 == 0)
    k_conv<32, true><<<conv_grid(nx, ny, nz, c.cout / 32), CONV_THREADS, CONV_SMEM, u->stream>>>(
        G, w, b, 1, out, nullptr, nullptr, 0);
  else
    k_conv<16, true><<<conv_grid(nx, ny, nz, c.cout / 16), CONV_THREADS, CONV_SMEM, u->stream>>>(
        G, w, b, 1, out, nullptr, nullptr, 0);
  u->launches++;
}

// data gradient of conv li: input gradient (gp, cout channels) -> FP32
// gradients of its sources (first c0 channels to d0, the rest to d1).
void conv_dgrad(vfs_unet *u, int li, int nx, int ny, int nz, const bf16 *gp, float *d0, float *d1) {
  const Conv &c = u->conv[li];
  Conv t{c.cout, c.cin, c.cout, 0, 0, 0, 0, 0, 0};
  ConvGeom G = geom(t, nx, ny, nz, gp, nullptr);
  const uint2 *w = u->pk + c.pkt;
  if (c.cin % 32 == 0)
    k_conv<32, false><<<conv_grid(nx, ny, nz, c.cin / 32), CONV_THREADS, CONV_SMEM, u->stream>>>(
        G, w, nullptr, 0, nullptr, d0, d1, c.c0);
  else
    k_conv<16, false><<<conv_grid(nx, ny, nz, c.cin / 16), CONV_THREADS, CONV_SMEM, u->stream>>>(
        G, w, nullptr, 0, nullptr, d0, d1, c.c0);
  u->launches++;
}

void conv_wgrad(vfs_unet *u, int li, int nx, int ny, int nz, const bf16 *s0, const bf16 *s1, const bf16 *gp) {
  const Conv &c = u->conv[li];
  ConvGeom G = geom(c, nx, ny, nz, s0, s1);
  const int ntiles = ((nx + TX - 1) / TX) * ((ny + TY - 1) / TY) * ((nz + TZ - 1) / TZ);
  const int per = 152 * 2 / (G.groups * 3);
  dim3 grid(ntiles < per ? ntiles : (per < 1 ? 1 : per), G.groups, 3);
  float *dW = u->grads + c.w;
  const int smem = CONV_SMEM + TX * TY * TZ * (c.cout * 2 + 16);
  if (c.cout == 16) k_wgrad<16><<<grid, 288, smem, u->stream>>>(G, gp, dW);
  else if (c.cout == 32) k_wgrad<32><<<grid, 288, smem, u->stream>>>(G, gp, dW);
  else k_wgrad<64><<<grid, 288, smem, u->stream>>>(G, gp, dW);
  u->launches++;
}

void relu_bwd(vfs_unet *u, int li, const float *g, const bf16 *y, size_t nvox) {
  const Conv &c = u->conv[li];
  const size_t n = nvox * c.cout;
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_relu_bwd<<<(int)blocks, 256, 0, u->stream>>>(g, y, n, c.cout, u->gpre, u->grads + c.b);
  u->launches++;
}

int pack(vfs_unet *u) {
  for (const Conv &c : u->conv) {
    size_t tot = (size_t)27 * (c.cin / 16) * (c.cout / 8) * 32 * 2;
    k_pack<<<grid_for(tot), 256, 0, u->stream>>>(u->params + c.w, c.cin, c.cout, u->pk + c.pk, u->pk + c.pkt);
    u->launches++;
  }
  u->packed = true;
  return VFS_OK;
}

struct Box3 {
  const float *feat, *tgt, *wt;
  int fx, fy, fz, ox, oy, oz;
};

void forward(vfs_unet *u, const Box3 &b) {
  const int nx = u->nx, ny = u->ny, nz = u->nz;
  const int x1 = nx / 2, y1 = ny / 2, z1 = nz / 2, x2 = nx / 4, y2 = ny / 4, z2 = nz / 4;
  const size_t n0 = (size_t)nx * ny * nz, n1 = n0 / 8, n2 = n0 / 64;
  cudaStream_t s = u->stream;
  k_input<<<grid_for(n0), 256, 0, s>>>(b.feat, b.fx, b.fy, b.fz, b.ox, b.oy, b.oz, nx, ny, nz, u->xin);
  conv_fwd(u, 0, nx, ny, nz, u->xin, nullptr, u->e0a);
  conv_fwd(u, 1, nx, ny, nz, u->e0a, nullptr, u->e0b);
  k_pool<<<grid_for(n1 * 16), 256, 0, s>>>(u->e0b, nx, ny, nz, 16, u->p0);
  conv_fwd(u, 2, x1, y1, z1, u->p0, nullptr, u->e1a);
  conv_fwd(u, 3, x1, y1, z1, u->e1a, nullptr, u->e1b);
  k_pool<<<grid_for(n2 * 32), 256, 0, s>>>(u->e1b, x1, y1, z1, 32, u->p1);
  conv_fwd(u, 4, x2, y2, z2, u->p1, nullptr, u->e2a);
  conv_fwd(u, 5, x2, y2, z2, u->e2a, nullptr, u->e2b);
  conv_fwd(u, 6, x1, y1, z1, u->e2b, u->e1b, u->d1a);
  conv_fwd(u, 7, x1, y1, z1, u->d1a, nullptr, u->d1b);
  conv_fwd(u, 8, nx, ny, nz, u->d1b, u->e0b, u->d0a);
  conv_fwd(u, 9, nx, ny, nz, u->d0a, nullptr, u->d0b);
  u->launches += 3;
  (void)n1;
}

void backward(vfs_unet *u) {
  const int nx = u->nx, ny = u->ny, nz = u->nz;
  const int x1 = nx / 2, y1 = ny / 2, z1 = nz / 2, x2 = nx / 4, y2 = ny / 4, z2 = nz / 4;
  const size_t n0 = (size_t)nx * ny * nz, n1 = n0 / 8, n2 = n0 / 64;
  cudaStream_t s = u->stream;
  // d0b = relu(conv9(d0a))
  relu_bwd(u, 9, u->g_d0b, u->d0b, n0);
  conv_wgrad(u, 9, nx, ny, nz, u->d0a, nullptr, u->gpre);
  conv_dgrad(u, 9, nx, ny, nz, u->gpre, u->g_d0a, nullptr);
  // d0a = relu(conv8(cat(up(d1b), e0b)))
  relu_bwd(u, 8, u->g_d0a, u->d0a, n0);
  conv_wgrad(u, 8, nx, ny, nz, u->d1b, u->e0b, u->gpre);
  conv_dgrad(u, 8, nx, ny, nz, u->gpre, u->g_upd1b, u->g_e0b);
  k_up_bwd<<<grid_for(n1 * 32), 256, 0, s>>>(u->g_upd1b, nx, ny, nz, 32, u->g_d1b);
  // d1b = relu(conv7(d1a))
  relu_bwd(u, 7, u->g_d1b, u->d1b, n1);
  conv_wgrad(u, 7, x1, y1, z1, u->d1a, nullptr, u->gpre);
  conv_dgrad(u, 7, x1, y1, z1, u->gpre, u->g_d1a, nullptr);
  // d1a = relu(conv6(cat(up(e2b), e1b)))
  relu_bwd(u, 6, u->g_d1a, u->d1a, n1);
  conv_wgrad(u, 6, x1, y1, z1, u->e2b, u->e1b, u->gpre);
  conv_dgrad(u, 6, x1, y1, z1, u->gpre, u->g_upe2b, u->g_e1b);
  k_up_bwd<<<grid_for(n2 * 64), 256, 0, s>>>(u->g_upe2b, x1, y1, z1, 64, u->g_e2b);
  // e2b = relu(conv5(e2a)), e2a = relu(conv4(p1))
  relu_bwd(u, 5, u->g_e2b, u->e2b, n2);
  conv_wgrad(u, 5, x2, y2, z2, u->e2a, nullptr, u->gpre);
  conv_dgrad(u, 5, x2, y2, z2, u->gpre, u->g_e2a, nullptr);
  relu_bwd(u, 4, u->g_e2a, u->e2a, n2);
  conv_wgrad(u, 4, x2, y2, z2, u->p1, nullptr, u->gpre);
  conv_dgrad(u, 4, x2, y2, z2, u->gpre, u->g_p1, nullptr);
  k_pool_bwd<<<grid_for(n1 * 32), 256, 0, s>>>(u->g_p1, x1, y1, z1, 32, u->g_e1b);
  // e1b = relu(conv3(e1a)), e1a = relu(conv2(p0))
  relu_bwd(u, 3, u->g_e1b, u->e1b, n1);
  conv_wgrad(u, 3, x1, y1, z1, u->e1a, nullptr, u->gpre);
  conv_dgrad(u, 3, x1, y1, z1, u->gpre, u->g_e1a, nullptr);
  relu_bwd(u, 2, u->g_e1a, u->e1a, n1);
  conv_wgrad(u, 2, x1, y1, z1, u->p0, nullptr, u->gpre);
  conv_dgrad(u, 2, x1, y1, z1, u->gpre, u->g_p0, nullptr);
  k_pool_bwd<<<grid_for(n0 * 16), 256, 0, s>>>(u->g_p0, nx, ny, nz, 16, u->g_e0b);
  // e0b = relu(conv1(e0a)), e0a = relu(conv0(xin))
  relu_bwd(u, 1, u->g_e0b, u->e0b, n0);
  conv_wgrad(u, 1, nx, ny, nz, u->e0a, nullptr, u->gpre);
  conv_dgrad(u, 1, nx, ny, nz, u->gpre, u->g_e0a, nullptr);
  relu_bwd(u, 0, u->g_e0a, u->e0a, n0);
  conv_wgrad(u, 0, nx, ny, nz, u->xin, nullptr, u->gpre);
  u->launches += 4;
}

int check_dims(int nx, int ny, int nz) {
  if (nx < 4 || ny < 4 || nz < 4 || nx % 4 || ny % 4 || nz % 4)
    return fail(VFS_EINVAL, "U-Net box dims must be multiples of 4 (two 2x pooling levels)");
  return VFS_OK;
}

int cuda_status(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VFS_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return VFS_OK;
}

// Loss and gradient of one sub-box; grads are accumulated (zeroed by the caller).
int loss_grad(vfs_unet *u, const vfs_unet_batch *bt, double *loss) {
  int rc = check_dims(bt->nx, bt->ny, bt->nz);
  if (rc) return rc;
  if (bt->ox < 0 || bt->oy < 0 || bt->oz < 0 || bt->ox + bt->nx > bt->fx || bt->oy + bt->ny > bt->fy ||
      bt->oz + bt->nz > bt->fz)
    return fail(VFS_EINVAL, "sub-box outside the feature planes");
  if (bt->op && (bt->nx < 3 || bt->ny < 3 || bt->nz < 3)) return fail(VFS_EINVAL, "residual loss needs inner cells");
  if ((rc = ensure_bufs(u, bt->nx, bt->ny, bt->nz, true))) return rc;
  if (!u->packed) pack(u);
  Box3 b{bt->features, bt->target, bt->weight, bt->fx, bt->fy, bt->fz, bt->ox, bt->oy, bt->oz};
  const size_t n0 = (size_t)bt->nx * bt->ny * bt->nz;
  forward(u, b);
  cudaMemsetAsync(u->scal, 0, 64 * sizeof(float), u->stream);
  k_weight_sum<<<grid_for(n0), 256, 0, u->stream>>>(b.wt, b.fx, b.fy, b.ox, b.oy, b.oz, bt->nx, bt->ny, bt->nz,
                                                   u->scal);
  if (!bt->op) {
    k_head<<<grid_for(n0), 256, 0, u->stream>>>(u->d0b, n0, u->params + u->head, nullptr, b.tgt, b.wt, b.fx, b.fy,
                                               b.ox, b.oy, b.oz, bt->nx, bt->ny, u->scal, u->g_d0b,
                                               u->grads + u->head, u->scal + 1);
    u->launches += 2;
  } else {
    // residual loss (+ optional MSE) through the row-scaled operator
    Crop cr{b.fx, b.fy, b.fz, b.ox, b.oy, b.oz, bt->nx, bt->ny, bt->nz};
    const size_t plane = (size_t)b.fx * b.fy * b.fz;
    k_head<<<grid_for(n0), 256, 0, u->stream>>>(u->d0b, n0, u->params + u->head, u->obuf, nullptr, nullptr, 0, 0,
                                               0, 0, 0, bt->nx, bt->ny, nullptr, nullptr, nullptr, nullptr);
    k_res_fwd<<<grid_for(n0), 256, 0, u->stream>>>(cr, bt->op, b.feat + 2 * plane, b.wt, u->obuf, bt->op_scale,
                                                  u->qbuf, u->scal + 2);
    k_res_bwd<<<grid_for(n0), 256, 0, u->stream>>>(cr, bt->op, u->qbuf, u->scal + 2, bt->op_scale, bt->res_weight,
                                                  u->obuf, b.tgt, b.wt, u->scal, bt->mse_weight, u->gobuf,
                                                  u->scal + 1);
    k_head_bwd<<<grid_for(n0), 256, 0, u->stream>>>(u->d0b, n0, u->params + u->head, u->gobuf, u->g_d0b,
                                                   u->grads + u->head);
    u->launches += 5;
  }
  backward(u);
  float l[4] = {0.f, 0.f, 0.f, 0.f};
  cudaMemcpyAsync(l, u->scal, 4 * sizeof(float), cudaMemcpyDeviceToHost, u->stream);
  cudaError_t e = cudaStreamSynchronize(u->stream);
  if (e != cudaSuccess) return fail(VFS_ECUDA, std::string("U-Net step: ") + cudaGetErrorString(e));
  if (loss) *loss = l[1] + (bt->op && l[2] > 0.f ? bt->res_weight * l[3] / l[2] : 0.f);
  return cuda_status("U-Net step");
}

}  // namespace

extern "C" {

int vfs_unet_create(unsigned int seed, vfs_unet **out) {
  if (!out) return fail(VFS_EINVAL, "null argument");
  *out = nullptr;
  int rc = configure_kernels();
  if (rc) return rc;
  vfs_unet *u = new vfs_unet();
  cudaGetDevice(&u->device);
  setup_layers(u);
  auto al = [&](void **p, size_t bytes) {
    if (cudaMalloc(p, bytes) != cudaSuccess) { cudaGetLastError(); return false; }
    return true;
  };
  if (!al((void **)&u->params, u->nparams * 4) || !al((void **)&u->grads, u->nparams * 4) ||
      !al((void **)&u->m, u->nparams * 4) || !al((void **)&u->v, u->nparams * 4) ||
      !al((void **)&u->pk, u->npk * sizeof(uint2))) {
    vfs_unet_destroy(u);
    return fail(VFS_ENOMEM, "U-Net parameter allocation failed");
  }
  // He-uniform initialisation from a seeded generator; biases zero; the
  // head starts at zero so that the untrained network predicts no change.
  std::vector<float> p(u->nparams, 0.f);
  std::mt19937 gen(seed);
  for (const Conv &c : u->conv) {
    const float lim = std::sqrt(6.f / (27.f * c.cin));
    std::uniform_real_distribution<float> dist(-lim, lim);
    for (size_t i = 0; i < (size_t)27 * c.cin * c.cout; i++) p[c.w + i] = dist(gen);
  }
  cudaMemcpy(u->params, p.data(), u->nparams * 4, cudaMemcpyHostToDevice);
  cudaMemset(u->grads, 0, u->nparams * 4);
  cudaMemset(u->m, 0, u->nparams * 4);
  cudaMemset(u->v, 0, u->nparams * 4);
  rc = cuda_status("U-Net create");
  if (rc) {
    vfs_unet_destroy(u);
    return rc;
  }
  *out = u;
  return VFS_OK;
}

void vfs_unet_destroy(vfs_unet *u) {
  if (!u) return;
  free_bufs(u);
  cudaFree(u->params);
  cudaFree(u->grads);
  cudaFree(u->m);
  cudaFree(u->v);
  cudaFree(u->pk);
  delete u;
}

int vfs_unet_set_stream(vfs_unet *u, void *stream) {
  if (!u) return fail(VFS_EINVAL, "null argument");
  u->stream = (cudaStream_t)stream;
  return VFS_OK;
}

int64_t vfs_unet_num_params(vfs_unet *u) { return u ? (int64_t)u->nparams : 0; }

int vfs_unet_get_params(vfs_unet *u, float *out) {
  if (!u || !out) return fail(VFS_EINVAL, "null argument");
  cudaMemcpyAsync(out, u->params, u->nparams * 4, cudaMemcpyDefault, u->stream);
  if (cudaStreamSynchronize(u->stream) != cudaSuccess) return cuda_status("get_params");
  return VFS_OK;
}

int vfs_unet_set_params(vfs_unet *u, const float *in) {
  if (!u || !in) return fail(VFS_EINVAL, "null argument");
  cudaMemcpyAsync(u->params, in, u->nparams * 4, cudaMemcpyDefault, u->stream);
  u->packed = false;
  if (cudaStreamSynchronize(u->stream) != cudaSuccess) return cuda_status("set_params");
  return VFS_OK;
}

int vfs_unet_forward(vfs_unet *u, const vfs_unet_batch *bt, float *out) {
  if (!u || !bt || !bt->features || !out) return fail(VFS_EINVAL, "null argument");
  int rc = check_dims(bt->nx, bt->ny, bt->nz);
  if (rc) return rc;
  if (bt->ox < 0 || bt->oy < 0 || bt->oz < 0 || bt->ox + bt->nx > bt->fx || bt->oy + bt->ny > bt->fy ||
      bt->oz + bt->nz > bt->fz)
    return fail(VFS_EINVAL, "sub-box outside the feature planes");
  if ((rc = ensure_bufs(u, bt->nx, bt->ny, bt->nz, false))) return rc;
  if (!u->packed) pack(u);
  Box3 b{bt->features, nullptr, nullptr, bt->fx, bt->fy, bt->fz, bt->ox, bt->oy, bt->oz};
  forward(u, b);
  const size_t n0 = (size_t)bt->nx * bt->ny * bt->nz;
  k_head<<<grid_for(n0), 256, 0, u->stream>>>(u->d0b, n0, u->params + u->head, out, nullptr, nullptr, 0, 0, 0, 0,
                                             0, bt->nx, bt->ny, nullptr, nullptr, nullptr, nullptr);
  u->launches++;
  return cuda_status("U-Net forward");
}

int vfs_unet_gradient(vfs_unet *u, const vfs_unet_batch *bt, float *grad, double *loss) {
  if (!u || !bt || !bt->features || !bt->target || !bt->weight) return fail(VFS_EINVAL, "null argument");
  cudaMemsetAsync(u->grads, 0, u->nparams * 4, u->stream);
  int rc = loss_grad(u, bt, loss);
  if (rc) return rc;
  if (grad) {
    cudaMemcpyAsync(grad, u->grads, u->nparams * 4, cudaMemcpyDefault, u->stream);
    if (cudaStreamSynchronize(u->stream) != cudaSuccess) return cuda_status("gradient");
  }
  return VFS_OK;
}

int vfs_unet_train_step(vfs_unet *u, const vfs_unet_batch *bt, double lr, double *loss) {
  if (!u || !bt || !bt->features || !bt->target || !bt->weight) return fail(VFS_EINVAL, "null argument");
  if (!(lr > 0)) return fail(VFS_EINVAL, "learning rate must be positive");
  cudaMemsetAsync(u->grads, 0, u->nparams * 4, u->stream);
  int rc = loss_grad(u, bt, loss);
  if (rc) return rc;
  return vfs_unet_adam(u, lr, 0.9, 0.999, 1e-8);
}

int vfs_unet_adam(vfs_unet *u, double lr, double beta1, double beta2, double eps) {
  if (!u) return fail(VFS_EINVAL, "null argument");
  u->t++;
  const float c1 = (float)(1.0 - std::pow(beta1, (double)u->t)), c2 = (float)(1.0 - std::pow(beta2, (double)u->t));
  k_adam<<<grid_for(u->nparams), 256, 0, u->stream>>>(u->params, u->grads, u->m, u->v, u->nparams, (float)lr,
                                                      (float)beta1, (float)beta2, c1, c2, (float)eps);
  u->launches++;
  pack(u);
  return cuda_status("U-Net Adam step");
}

int vfs_unet_set_grads(vfs_unet *u, const float *grad) {
  if (!u || !grad) return fail(VFS_EINVAL, "null argument");
  cudaMemcpyAsync(u->grads, grad, u->nparams * 4, cudaMemcpyDefault, u->stream);
  if (cudaStreamSynchronize(u->stream) != cudaSuccess) return cuda_status("set_grads");
  return VFS_OK;
}

int64_t vfs_unet_kernel_launches(vfs_unet *u) { return u ? u->launches : 0; }

}  // extern "C"
