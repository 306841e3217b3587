// ibm.cu -- immersed-boundary node classification on the GPU: the blanking
// flags nvert of one body from its triangulated surface (ibm_search_advanced,
// Source/ibm.c:92-594, point_cell_advanced :1075-1200, randomdirection
// :59-91, intsect_triangle Source/compgeom.c:25-60).
//
// Compiled with -fmad=false (and host code with -ffp-contract=off) so that
// every ray-triangle test rounds exactly like the reference's C.
//
// Layout of the search structure: the reference hashes the triangles into a
// 40x40x40 grid over the body box and, for a cell centre in hash cell
// (ic,jc,kc), tests every triangle listed in the hash cells (ic,jc,k>=kc),
// each once.  Here each hash column (ic,jc) keeps one deduplicated list of
// its triangles sorted by the top hash cell they reach, so that the search
// of a cell is the prefix of its column list with top cell >= kc: the same
// triangle set without a per-thread "already searched" bitmap.
#include <climits>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "vfs_poisson.h"

namespace vfs {
void set_last_error(const std::string &msg);  // poisson.cu

int ibm_context(vfs_poisson *h, IbmContext *c);
}  // namespace vfs

using namespace vfs;

namespace {

constexpr int kHash = 40;       // ncx = ncy = ncz (ibm.c:111)
constexpr int kMaxTries = 64;   // rays per cell before giving up
constexpr int kMaxHits = 64;    // intersections kept per ray

// First glibc rand() value after srand(seed) (TYPE_3 additive feedback
// generator r[i] = r[i-31] + r[i-3] mod 2^32, seeded by Park-Miller
// r[i] = 16807 r[i-1] mod 2^31-1, r[31..33] = r[0..2], 310 outputs dropped).
unsigned glibc_rand_first(unsigned seed) {
  int32_t r[345];
  r[0] = (int32_t)(seed == 0 ? 1 : seed);
  for (int i = 1; i < 31; i++) {
    long long hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
    long long word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = (int32_t)word;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 34; i < 345; i++) r[i] = (int32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
  return ((uint32_t)r[344]) >> 1;
}

struct HashBox {
  double xmin, ymin, zmin, xmax, ymax, zmax, dcx, dcy, dcz;
};

// One cell centre: 4 if a ray from it crosses the surface an odd number of
// times, 0 if even, -1 if every ray met a singular (double) intersection or
// too many intersections.
__device__ int point_cell(const double p[3], int ip, int jp, int kp, const HashBox &H, const int *col_start,
                          const int *col_tri, const int *col_kmax, const double *tv, const double *nf,
                          const double *s_tab) {
  const int col = jp * kHash + ip;
  const int e0 = col_start[col], e1 = col_start[col + 1];
  for (int tries = 1; tries <= kMaxTries; tries++) {
    const double xpc = H.dcx * (ip + 0.5) + H.xmin, ypc = H.dcy * (jp + 0.5) + H.ymin;
    const double s = s_tab[tries];
    double dir[3] = {xpc + s * H.dcx - p[0], ypc + s * H.dcy - p[1], H.zmax + 0.2 - p[2]};
    const double nrm = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    dir[0] /= nrm; dir[1] /= nrm; dir[2] /= nrm;
    double dt[kMaxHits];
    int dn[kMaxHits];
    int nintp = 0;
    bool singular = false, overflow = false;
    for (int q = e0; q < e1 && !singular; q++) {
      if (col_kmax[q] - 1 < kp) break;  // list sorted by top hash cell, descending
      const int e = col_tri[q];
      const double *v = &tv[(size_t)e * 9];
      // intsect_triangle, compgeom.c:25-60
      const double EPS = 0.00000001;
      double e1v[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
      double e2v[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
      double pv[3] = {dir[1] * e2v[2] - dir[2] * e2v[1], dir[2] * e2v[0] - dir[0] * e2v[2],
                      dir[0] * e2v[1] - dir[1] * e2v[0]};
      double det = e1v[0] * pv[0] + e1v[1] * pv[1] + e1v[2] * pv[2];
      if (det > -EPS && det < EPS) continue;
      double inv = 1.0 / det;
      double tvv[3] = {p[0] - v[0], p[1] - v[1], p[2] - v[2]};
      double u = (tvv[0] * pv[0] + tvv[1] * pv[1] + tvv[2] * pv[2]) * inv;
      if (u < 0.0 || u > 1.0) continue;
      double qv[3] = {tvv[1] * e1v[2] - tvv[2] * e1v[1], tvv[2] * e1v[0] - tvv[0] * e1v[2],
                      tvv[0] * e1v[1] - tvv[1] * e1v[0]};
      double w = (dir[0] * qv[0] + dir[1] * qv[1] + dir[2] * qv[2]) * inv;
      if (w < 0.0 || u + w > 1.0) continue;
      double t = (e2v[0] * qv[0] + e2v[1] * qv[1] + e2v[2] * qv[2]) * inv;
      if (!(t > 0)) continue;
      if (nintp == kMaxHits) { overflow = true; break; }
      dt[nintp] = t;
      dn[nintp] = e;
      nintp++;
      for (int m = 0; m < nintp - 1; m++) {
        const double *a = &nf[(size_t)dn[m] * 3], *b = &nf[(size_t)e * 3];
        double ndotn = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
        if (fabs(t - dt[m]) < 1.e-8 && ndotn > -0.97) singular = true;
      }
    }
    if (overflow) return -1;
    if (!singular) return (nintp % 2) ? 4 : 0;
  }
  return -1;
}

// Classification of one body (ibm_search_advanced, ibm.c:92-325) as a
// copying pass over every DA point: boundary points take src unchanged,
// interior points whose centre lies in the body's hash box the larger of
// their value and the ray-parity test (4 inside), body 0 first clearing
// every value below 5 (src may be dst: each point reads and writes only
// itself).
__global__ void k_ibm_classify_from(Grid g, const double *__restrict__ cent, int ibi, HashBox H,
                                    const int *__restrict__ col_start, const int *__restrict__ col_tri,
                                    const int *__restrict__ col_kmax, const double *__restrict__ tv,
                                    const double *__restrict__ nf, const double *__restrict__ s_tab, const double *src,
                                    double *dst, uint8_t *is4, int *failed, int3 lo, int3 hi) {
  const int i = lo.x + blockIdx.x * blockDim.x + threadIdx.x, j = lo.y + blockIdx.y, k = lo.z + blockIdx.z;
  if (i >= hi.x) return;
  const size_t t = g.at(i, j, k);
  double nv = src[t];
  if (i >= 1 && i < g.mx - 1 && j >= 1 && j < g.my - 1 && k >= 1 && k < g.mz - 1) {
    if (ibi == 0 && nv < 5.) nv = 0;
    const double p[3] = {cent[t * 3], cent[t * 3 + 1], cent[t * 3 + 2]};
    if (p[0] > H.xmin && p[0] < H.xmax && p[1] > H.ymin && p[1] < H.ymax && p[2] > H.zmin && p[2] < H.zmax) {
      const int ic = (int)floor((p[0] - H.xmin) / H.dcx);
      const int jc = (int)floor((p[1] - H.ymin) / H.dcy);
      const int kc = (int)floor((p[2] - H.zmin) / H.dcz);
      int val = point_cell(p, ic, jc, kc, H, col_start, col_tri, col_kmax, tv, nf, s_tab);
      if (val < 0) {
        atomicAdd(failed, 1);
        val = 0;
      }
      nv = nv > val ? nv : (double)val;
      if (nv < 0) nv = 0;
    }
  }
  dst[t] = nv;
  // the dilation's test of this point as a neighbour, (int)(max(v, 0) + 0.5)
  // == 4, once here instead of in each of its 27 neighbours (integer loads
  // there; FP64 arithmetic is the scarce pipe)
  if (is4) is4[t] = (int)((nv < 0 ? 0. : nv) + 0.5) == 4;
}

// The search of a body after the first needs the index box of the interior
// cells whose centre lies strictly inside its hash box.  The centres are
// bounded per block of 8x8x8 interior cells once per grid (k_cent_blocks);
// a block whose bounds miss the hash box holds no such cell, so only the
// cells of the other blocks are tested, with the same strict comparisons.
constexpr int kCentBlock = 8;
__global__ void __launch_bounds__(512) k_cent_blocks(Grid g, const double *__restrict__ cent, int nbx, int nby,
                                                     double *bbox) {
  const int b = blockIdx.x;
  const int bi = b % nbx, bj = (b / nbx) % nby, bk = b / (nbx * nby);
  const int i = 1 + bi * kCentBlock + (threadIdx.x & 7), j = 1 + bj * kCentBlock + ((threadIdx.x >> 3) & 7),
            k = 1 + bk * kCentBlock + (threadIdx.x >> 6);
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  if (i < g.mx - 1 && j < g.my - 1 && k < g.mz - 1) {
    const size_t t = g.at(i, j, k);
    for (int q = 0; q < 3; q++) lo[q] = hi[q] = cent[t * 3 + q];
  }
  for (int q = 0; q < 3; q++)
    for (int o = 16; o > 0; o >>= 1) {
      lo[q] = fmin(lo[q], __shfl_xor_sync(0xffffffffu, lo[q], o));
      hi[q] = fmax(hi[q], __shfl_xor_sync(0xffffffffu, hi[q], o));
    }
  __shared__ double sh[16][6];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int q = 0; q < 3; q++) { sh[w][q] = lo[q]; sh[w][3 + q] = hi[q]; }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = sh[0][threadIdx.x];
    for (int u = 1; u < 16; u++) v = threadIdx.x < 3 ? fmin(v, sh[u][threadIdx.x]) : fmax(v, sh[u][threadIdx.x]);
    bbox[(size_t)b * 6 + threadIdx.x] = v;
  }
}

// One thread tests one block's bounds and lists the block when they meet
// the hash box (box[6]: the count); then every thread block of a fixed grid
// takes listed blocks in turn and tests their cells, two per thread (box[0..5]:
// atomic min/max of i, j, k), so that a large box's blocks spread over the
// whole GPU.
__global__ void __launch_bounds__(256) k_ibm_box_hits(const double *__restrict__ bbox, int nblocks, HashBox H,
                                                      int *box, int *hits) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  const double *q = bbox + (size_t)b * 6;
  if (q[3] > H.xmin && q[0] < H.xmax && q[4] > H.ymin && q[1] < H.ymax && q[5] > H.zmin && q[2] < H.zmax)
    hits[atomicAdd(&box[6], 1)] = b;
}
__global__ void __launch_bounds__(256) k_ibm_box_cells(Grid g, const double *__restrict__ cent, int nbx, int nby,
                                                       HashBox H, const int *__restrict__ hits, int *box) {
  const int nh = *(volatile int *)&box[6];
  for (int w = blockIdx.x; w < nh; w += gridDim.x) {
    const int bb = hits[w];
    const int bi = bb % nbx, bj = (bb / nbx) % nby, bk = bb / (nbx * nby);
    for (int c = threadIdx.x; c < kCentBlock * kCentBlock * kCentBlock; c += blockDim.x) {
      const int i = 1 + bi * kCentBlock + (c & 7), j = 1 + bj * kCentBlock + ((c >> 3) & 7),
                k = 1 + bk * kCentBlock + (c >> 6);
      if (i >= g.mx - 1 || j >= g.my - 1 || k >= g.mz - 1) continue;
      const size_t t = g.at(i, j, k);
      const double p0 = cent[t * 3], p1 = cent[t * 3 + 1], p2 = cent[t * 3 + 2];
      if (p0 > H.xmin && p0 < H.xmax && p1 > H.ymin && p1 < H.ymax && p2 > H.zmin && p2 < H.zmax) {
        atomicMin(&box[0], i); atomicMin(&box[1], j); atomicMin(&box[2], k);
        atomicMax(&box[3], i); atomicMax(&box[4], j); atomicMax(&box[5], k);
      }
    }
  }
}

// near-boundary dilation over every DA point (ibm.c:326-348); a parallel pass
// over a snapshot equals the in-place loop because it only writes 2 and
// reads only the 4s.
__global__ void k_ibm_dilate(Grid g, const double *src, double *dst) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  const size_t t = g.at(i, j, k);
  double v = src[t];
  if (v < 0) v = 0;
  if ((int)(v + 0.5) != 4) {
    const int ip = i < g.mx - 1 ? i + 1 : i, im = i > 0 ? i - 1 : i;
    const int jp = j < g.my - 1 ? j + 1 : j, jm = j > 0 ? j - 1 : j;
    const int kp = k < g.mz - 1 ? k + 1 : k, km = k > 0 ? k - 1 : k;
    for (int kk = km; kk <= kp; kk++)
      for (int jj = jm; jj <= jp; jj++)
        for (int ii = im; ii <= ip; ii++) {
          double w = src[g.at(ii, jj, kk)];
          if (w < 0) w = 0;
          if ((int)(w + 0.5) == 4) v = v > 2 ? v : 2;
        }
  }
  dst[t] = v;
}

// back to 3 / 1 and the wall rows of bctype -1 / -2 (ibm.c:514-543)
__device__ __forceinline__ double ibm_finish_value(const Grid &g, int b0, int b1, int b2, int b3, int b4, int b5,
                                                   int i, int j, int k, double v) {
  if ((int)(v + 0.5) == 2) v = 1;
  if ((int)(v + 0.5) == 4) v = 3;
  for (int q = -1; q >= -2; q--) {
    if (b0 == q && i == 1) v = 1;
    if (b1 == q && i == g.mx - 2) v = 1;
    if (b2 == q && j == 1) v = 1;
    if (b3 == q && j == g.my - 2) v = 1;
    if (b4 == q && k == 1) v = 1;
    if (b5 == q && k == g.mz - 2) v = 1;
  }
  return v;
}
__global__ void k_ibm_finish(Grid g, int b0, int b1, int b2, int b3, int b4, int b5, double *nvert) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
  if (i >= g.mx - 1) return;
  const size_t t = g.at(i, j, k);
  nvert[t] = ibm_finish_value(g, b0, b1, b2, b3, b4, b5, i, j, k, nvert[t]);
}
// the dilation and the finishing pass in one (the search without IB node
// records, where nothing reads the dilated marks in between): every DA
// point of dst gets the dilation of src, the interior points then their
// finished value
__global__ void k_ibm_dilate_finish(Grid g, int b0, int b1, int b2, int b3, int b4, int b5,
                                    const double *__restrict__ src, const uint8_t *__restrict__ is4,
                                    double *__restrict__ dst, int3 lo, int3 hi) {
  int i = lo.x + blockIdx.x * blockDim.x + threadIdx.x, j = lo.y + blockIdx.y, k = lo.z + blockIdx.z;
  if (i >= hi.x) return;
  const size_t t = g.at(i, j, k);
  double v = src[t];
  if (v < 0) v = 0;
  if (!is4[t]) {
    const int ip = i < g.mx - 1 ? i + 1 : i, im = i > 0 ? i - 1 : i;
    const int jp = j < g.my - 1 ? j + 1 : j, jm = j > 0 ? j - 1 : j;
    const int kp = k < g.mz - 1 ? k + 1 : k, km = k > 0 ? k - 1 : k;
    bool near = false;
    for (int kk = km; kk <= kp; kk++)
      for (int jj = jm; jj <= jp; jj++)
        for (int ii = im; ii <= ip; ii++) near |= is4[g.at(ii, jj, kk)] != 0;
    if (near) v = v > 2 ? v : 2;
  }
  if (i >= 1 && i < g.mx - 1 && j >= 1 && j < g.my - 1 && k >= 1 && k < g.mz - 1)
    v = ibm_finish_value(g, b0, b1, b2, b3, b4, b5, i, j, k, v);
  dst[t] = v;
}

// ---- IB interpolation records (ibm.c:373-508) ----
// One thread per IB node: the nearest surface element (nearestcell1,
// :1373-1518), the interception of the normal ray with the 3x3 patches of
// neighbouring cell centres (InterceptionPoint, :1766-2258, ICP :1666-1764)
// and the boundary fallback (:423-505), in the reference's operation order
// (compiled without FMA contraction).
struct V3 {
  double x, y, z;
};
struct V2 {
  double x, y;
};
__device__ inline V3 vload(const double *a, size_t t) { return V3{a[3 * t], a[3 * t + 1], a[3 * t + 2]}; }
__device__ inline double vdist(V3 a, V3 b) {
  return sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (a.z - b.z) * (a.z - b.z));
}
// ISSameSide2D (compgeom.c:62-114)
__device__ inline int same_side(V2 p, V2 p1, V2 p2, V2 p3) {
  const double t1 = (p.x - p1.x) * (p2.y - p1.y) - (p.y - p1.y) * (p2.x - p1.x);
  const double t2 = (p3.x - p1.x) * (p2.y - p1.y) - (p3.y - p1.y) * (p2.x - p1.x);
  const double lt = sqrt((p1.x - p2.x) * (p1.x - p2.x) + (p1.y - p2.y) * (p1.y - p2.y));
  if (fabs(t1 / lt) < 1.e-10) return 1;
  if (t1 > 0) return t2 > 0 ? 1 : -1;
  return t2 < 0 ? 1 : -1;
}
// ISInsideTriangle2D / ISPointInTriangle (compgeom.c:116-166)
__device__ inline int point_in_triangle(V3 p, V3 p1, V3 p2, V3 p3, double nx, double ny, double nz) {
  V2 a, b, c, e;
  if (fabs(nz) >= fabs(nx) && fabs(nz) >= fabs(ny)) {
    a = {p.x, p.y}; b = {p1.x, p1.y}; c = {p2.x, p2.y}; e = {p3.x, p3.y};
  } else if (fabs(nx) >= fabs(ny) && fabs(nx) >= fabs(nz)) {
    a = {p.z, p.y}; b = {p1.z, p1.y}; c = {p2.z, p2.y}; e = {p3.z, p3.y};
  } else {
    a = {p.x, p.z}; b = {p1.x, p1.z}; c = {p2.x, p2.z}; e = {p3.x, p3.z};
  }
  int ls = same_side(a, b, c, e);
  if (ls < 0) return ls;
  ls = same_side(a, c, e, b);
  if (ls < 0) return ls;
  return same_side(a, e, b, c);
}
// Dis_P_Line (compgeom.c:168-194)
__device__ inline void dist_point_line(V3 p, V3 p1, V3 p2, V3 &po, double &d) {
  const double dx21 = p2.x - p1.x, dy21 = p2.y - p1.y, dz21 = p2.z - p1.z;
  const double dx31 = p.x - p1.x, dy31 = p.y - p1.y, dz31 = p.z - p1.z;
  const double t = (dx31 * dx21 + dy31 * dy21 + dz31 * dz21) / (dx21 * dx21 + dy21 * dy21 + dz21 * dz21);
  if (t < 0) {
    po = p1;
    d = sqrt(dx31 * dx31 + dy31 * dy31 + dz31 * dz31);
  } else if (t > 1) {
    po = p2;
    d = sqrt((p.x - po.x) * (p.x - po.x) + (p.y - po.y) * (p.y - po.y) + (p.z - po.z) * (p.z - po.z));
  } else {
    po = V3{p1.x + t * dx21, p1.y + t * dy21, p1.z + t * dz21};
    d = sqrt((p.x - po.x) * (p.x - po.x) + (p.y - po.y) * (p.y - po.y) + (p.z - po.z) * (p.z - po.z));
  }
}
// triangle_intp / triangle_intp2 (compgeom.c:196-230) on the plane the
// dominant normal component picks
__device__ inline void project_bary(V3 p, V3 p1, V3 p2, V3 p3, double nx, double ny, double nz, double w[3]) {
  V2 a, b, c, e;
  if (fabs(nx) >= fabs(ny) && fabs(nx) >= fabs(nz)) {
    a = {p.y, p.z}; b = {p1.y, p1.z}; c = {p2.y, p2.z}; e = {p3.y, p3.z};
  } else if (fabs(ny) >= fabs(nx) && fabs(ny) >= fabs(nz)) {
    a = {p.x, p.z}; b = {p1.x, p1.z}; c = {p2.x, p2.z}; e = {p3.x, p3.z};
  } else if (fabs(nz) >= fabs(ny) && fabs(nz) >= fabs(nx)) {
    a = {p.y, p.x}; b = {p1.y, p1.x}; c = {p2.y, p2.x}; e = {p3.y, p3.x};
  } else {
    return;
  }
  const double x13 = b.x - e.x, y13 = b.y - e.y, x23 = c.x - e.x, y23 = c.y - e.y;
  const double xp3 = a.x - e.x, yp3 = a.y - e.y;
  const double det = x13 * y23 - x23 * y13;
  w[0] = (y23 * xp3 - x23 * yp3) / det;
  w[1] = (-y13 * xp3 + x13 * yp3) / det;
  w[2] = 1. - w[0] - w[1];
}
__constant__ int kPatchTri[8][3] = {{0, 1, 4}, {1, 2, 4}, {2, 4, 5}, {4, 5, 8}, {4, 7, 8}, {4, 6, 7}, {3, 4, 6}, {3, 4, 0}};

// the cells of one body marked 2 (IB node) after the dilation, interior
// only: per 256-cell block, their count ...
__global__ void k_ibm_mark_count(Grid g, const double *nvert, int *bcount) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool mark = false;
  if (t < g.n()) {
    const int i = (int)(t % g.mx), j = (int)((t / g.mx) % g.my), k = (int)(t / ((size_t)g.mx * g.my));
    mark = i >= 1 && i < g.mx - 1 && j >= 1 && j < g.my - 1 && k >= 1 && k < g.mz - 1 &&
           (int)(nvert[t] + 0.5) == 2;
  }
  const int c = __syncthreads_count(mark);
  if (threadIdx.x == 0) bcount[blockIdx.x] = c;
}
// ... and their DA indices in order, from the blocks' exclusive offsets
__global__ void k_ibm_mark_scatter(Grid g, const double *nvert, const int *boff, int *list) {
  __shared__ int wsum[8];
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool mark = false;
  if (t < g.n()) {
    const int i = (int)(t % g.mx), j = (int)((t / g.mx) % g.my), k = (int)(t / ((size_t)g.mx * g.my));
    mark = i >= 1 && i < g.mx - 1 && j >= 1 && j < g.my - 1 && k >= 1 && k < g.mz - 1 &&
           (int)(nvert[t] + 0.5) == 2;
  }
  const unsigned ball = __ballot_sync(0xffffffffu, mark);
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  if (lane == 0) wsum[wp] = __popc(ball);
  __syncthreads();
  int base = boff[blockIdx.x];
  for (int q = 0; q < wp; q++) base += wsum[q];
  if (mark) list[base + __popc(ball & ((1u << lane) - 1u))] = (int)t;
}

__global__ void k_ibm_nodes(Grid g, const double *__restrict__ cent, const int *__restrict__ list, int n_nodes,
                            int n_elmt, const double *__restrict__ tv, const double *__restrict__ nf,
                            const double *__restrict__ qv, const double *__restrict__ rad, vfs_ibm_node *out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const size_t t = (size_t)list[n];
  const int i = (int)(t % g.mx), j = (int)((t / g.mx) % g.my), k = (int)(t / ((size_t)g.mx * g.my));
  vfs_ibm_node nd;
  nd.i = i; nd.j = j; nd.k = k;
  const V3 p = vload(cent, t);
  // nearestcell1
  double dmin = 1.e20;
  int cell_min = -100;
  V3 pmin{0., 0., 0.};
  for (int e = 0; e < n_elmt; e++) {
    const V3 qe{qv[3 * e], qv[3 * e + 1], qv[3 * e + 2]};
    const double d_center = vdist(p, qe);
    if (!(d_center - rad[e] < dmin)) continue;
    const double *v = &tv[(size_t)e * 9];
    const V3 p1{v[0], v[1], v[2]}, p2{v[3], v[4], v[5]}, p3{v[6], v[7], v[8]};
    const double nfx = nf[3 * e], nfy = nf[3 * e + 1], nfz = nf[3 * e + 2];
    double tf = (p.x - p1.x) * nfx + (p.y - p1.y) * nfy + (p.z - p1.z) * nfz;
    if (fabs(tf) < 1.e-10) tf = 1.e-10;
    if (!(tf >= 0)) continue;
    const V3 pj{p.x - tf * nfx, p.y - tf * nfy, p.z - tf * nfz};
    if (point_in_triangle(pj, p1, p2, p3, nfx, nfy, nfz) == 1) {
      if (tf < dmin) { dmin = tf; pmin = pj; cell_min = e; }
    } else {
      V3 po;
      double d;
      dist_point_line(p, p1, p2, po, d);
      if (d < dmin) { dmin = d; pmin = po; cell_min = e; }
      dist_point_line(p, p2, p3, po, d);
      if (d < dmin) { dmin = d; pmin = po; cell_min = e; }
      dist_point_line(p, p3, p1, po, d);
      if (d < dmin) { dmin = d; pmin = po; cell_min = e; }
    }
  }
  nd.cell = cell_min;
  nd.pmin[0] = pmin.x; nd.pmin[1] = pmin.y; nd.pmin[2] = pmin.z;
  nd.d_s = dmin;
  nd.cs[0] = nd.cs[1] = nd.cs[2] = 0.;
  if (cell_min >= 0) {
    const double *v = &tv[(size_t)cell_min * 9];
    project_bary(pmin, V3{v[0], v[1], v[2]}, V3{v[3], v[4], v[5]}, V3{v[6], v[7], v[8]}, nf[3 * cell_min],
                 nf[3 * cell_min + 1], nf[3 * cell_min + 2], nd.cs);
  }
  // InterceptionPoint: the patches at i-1, i+1, j-1, j+1, k-1, k+1
  double nfx = p.x - pmin.x, nfy = p.y - pmin.y, nfz = p.z - pmin.z;
  const double dr = sqrt(nfx * nfx + nfy * nfy + nfz * nfz);
  nfx /= dr; nfy /= dr; nfz /= dr;
  nd.imode = -100;
  for (int s = 0; s < 3; s++) { nd.ip[s] = i; nd.jp[s] = j; nd.kp[s] = k; nd.cr[s] = 0.; }
  nd.d_i = 0.;
  for (int face = 0; face < 6 && nd.imode < 0; face++) {
    int ip[9], jp[9], kp[9];
    V3 pc[9];
    for (int s = 0; s < 9; s++) {
      const int a = s % 3 - 1, b = s / 3 - 1;
      switch (face) {
        case 0: ip[s] = i - 1; jp[s] = j + a; kp[s] = k + b; break;
        case 1: ip[s] = i + 1; jp[s] = j + a; kp[s] = k + b; break;
        case 2: ip[s] = i + a; jp[s] = j - 1; kp[s] = k + b; break;
        case 3: ip[s] = i + a; jp[s] = j + 1; kp[s] = k + b; break;
        case 4: ip[s] = i + a; jp[s] = j + b; kp[s] = k - 1; break;
        default: ip[s] = i + a; jp[s] = j + b; kp[s] = k + 1; break;
      }
      pc[s] = vload(cent, g.at(ip[s], jp[s], kp[s]));
    }
    for (int tr = 0; tr < 8; tr++) {  // ICP
      const V3 p1 = pc[kPatchTri[tr][0]], p2 = pc[kPatchTri[tr][1]], p3 = pc[kPatchTri[tr][2]];
      const double dx1 = p.x - p1.x, dy1 = p.y - p1.y, dz1 = p.z - p1.z;
      const double dx2 = p2.x - p1.x, dy2 = p2.y - p1.y, dz2 = p2.z - p1.z;
      const double dx3 = p3.x - p1.x, dy3 = p3.y - p1.y, dz3 = p3.z - p1.z;
      double d = (nfx * (dy2 * dz3 - dz2 * dy3) - nfy * (dx2 * dz3 - dz2 * dx3) + nfz * (dx2 * dy3 - dy2 * dx3));
      if (!(fabs(d) > 1.e-10)) continue;
      d = -(dx1 * (dy2 * dz3 - dz2 * dy3) - dy1 * (dx2 * dz3 - dz2 * dx3) + dz1 * (dx2 * dy3 - dy2 * dx3)) / d;
      if (!(d > 0)) continue;
      const V3 pint{p.x + d * nfx, p.y + d * nfy, p.z + d * nfz};
      const double rx1 = p2.x - p1.x, ry1 = p2.y - p1.y, rz1 = p2.z - p1.z;
      const double rx2 = p3.x - p1.x, ry2 = p3.y - p1.y, rz2 = p3.z - p1.z;
      const double nfxt = ry1 * rz2 - rz1 * ry2, nfyt = -rx1 * rz2 + rz1 * rx2, nfzt = rx1 * ry2 - ry1 * rx2;
      if (point_in_triangle(pint, p1, p2, p3, nfxt, nfyt, nfzt) >= 0) {
        double w[3] = {0., 0., 0.};
        project_bary(pint, p1, p2, p3, nfxt, nfyt, nfzt, w);
        nd.d_i = sqrt((pint.x - p.x) * (pint.x - p.x) + (pint.y - p.y) * (pint.y - p.y) +
                      (pint.z - p.z) * (pint.z - p.z));
        nd.imode = tr;
        for (int q = 0; q < 3; q++) {
          const int s = kPatchTri[tr][q];
          nd.ip[q] = ip[s]; nd.jp[q] = jp[s]; nd.kp[q] = kp[s];
          nd.cr[q] = w[q];
        }
        break;
      }
    }
  }
  nd.status = 0;
  if (nd.imode < 0) {
    int di = 0, dj = 0, dk = 0;
    if (i == 1 || i == g.mx - 2 || j == 1 || j == g.my - 2) {
      dk = (cell_min >= 0 && nf[3 * cell_min + 2] > 0) ? 1 : -1;
      nd.status = 1;
    } else if (k == 1 || k == g.mz - 2) {
      dj = 1;
      nd.status = 1;
    } else {
      nd.status = 2;
    }
    if (nd.status == 1) {
      const V3 c0 = p, c1 = vload(cent, g.at(i + di, j + dj, k + dk));
      nd.d_i = sqrt((c0.x - c1.x) * (c0.x - c1.x) + (c0.y - c1.y) * (c0.y - c1.y) + (c0.z - c1.z) * (c0.z - c1.z));
      nd.cr[0] = 1.; nd.cr[1] = 0.; nd.cr[2] = 0.;
      for (int q = 0; q < 3; q++) { nd.ip[q] = i + di; nd.jp[q] = j + dj; nd.kp[q] = k + dk; }
    }
  }
  out[n] = nd;
}

int fail(int code, const std::string &m) {
  set_last_error(m);
  return code;
}

bool on_device(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

namespace {

// BoundingSphere (ibm.c:1282-1370): per element, a sphere through the
// longest edge's end points centred on the circumcentre side
void bounding_sphere(int n_elmt, const int32_t *tri, const std::vector<double> &x, const std::vector<double> &y,
                     const std::vector<double> &z, std::vector<double> &q, std::vector<double> &rad) {
  struct P { double x, y, z; };
  auto dist = [](P a, P b) {
    return std::sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (a.z - b.z) * (a.z - b.z));
  };
  const P p0{0., 0., 0.};
  q.assign((size_t)n_elmt * 3, 0.);
  rad.assign(n_elmt, 0.);
  for (int e = 0; e < n_elmt; e++) {
    const int n1 = tri[3 * e], n2 = tri[3 * e + 1], n3 = tri[3 * e + 2];
    const P p1{x[n1], y[n1], z[n1]}, p2{x[n2], y[n2], z[n2]}, p3{x[n3], y[n3], z[n3]};
    const double l12 = dist(p1, p2), l23 = dist(p2, p3), l31 = dist(p3, p1);
    P pa, pb, pc;
    if (l12 > l23) {
      if (l12 > l31) { pa = p1; pb = p2; pc = p3; } else { pa = p3; pb = p1; pc = p2; }
    } else {
      if (l31 < l23) { pa = p2; pb = p3; pc = p1; } else { pa = p3; pb = p1; pc = p2; }
    }
    const P pf{0.5 * (pa.x + pb.x), 0.5 * (pa.y + pb.y), 0.5 * (pa.z + pb.z)};
    const P pu{pa.x - pf.x, pa.y - pf.y, pa.z - pf.z}, pv{pc.x - pf.x, pc.y - pf.y, pc.z - pf.z};
    const P pt{pu.y * pv.z - pu.z * pv.y, pu.z * pv.x - pu.x * pv.z, pu.x * pv.y - pu.y * pv.x};
    const P pd{pt.y * pu.z - pt.z * pu.y, pt.z * pu.x - pt.x * pu.z, pt.x * pu.y - pt.y * pu.x};
    double gama = -(dist(pu, p0) * dist(pu, p0) - dist(pv, p0) * dist(pv, p0));
    const P pw{pv.x - pu.x, pv.y - pu.y, pv.z - pu.z};
    double lamda = 2 * (pd.x * pw.x + pd.y * pw.y + pd.z * pw.z);
    gama /= lamda;
    lamda = gama < 0 ? 0 : gama;
    const P qq{pf.x + lamda * pd.x, pf.y + lamda * pd.y, pf.z + lamda * pd.z};
    q[3 * e] = qq.x; q[3 * e + 1] = qq.y; q[3 * e + 2] = qq.z;
    rad[e] = dist(qq, pa);
  }
}

int ibm_search_impl(vfs_poisson *h, int ibi, int n_v, const double *xyz, int n_elmt, const int32_t *tri,
                    const int *bctype, double *nvert, int *n_failed, bool want_nodes, int *n_nodes) {
  if (!h || !xyz || !tri || !nvert || n_v < 3 || n_elmt < 1) return fail(VFS_EINVAL, "bad surface arguments");
  if (want_nodes && (ibi < 0 || ibi > 1023)) return fail(VFS_EINVAL, "body index out of range");
  IbmContext cx;
  int rc = ibm_context(h, &cx);
  if (rc != VFS_OK) return rc;
  const Grid g = cx.g;
  // the surface is small: it is prepared on the host (exact same double
  // operations as the reference's set-up loops)
  std::vector<double> x(n_v), y(n_v), z(n_v);
  for (int q = 0; q < n_v; q++) { x[q] = xyz[3 * q]; y[q] = xyz[3 * q + 1]; z[q] = xyz[3 * q + 2]; }
  for (int e = 0; e < 3 * n_elmt; e++)
    if (tri[e] < 0 || tri[e] >= n_v) return fail(VFS_EINVAL, "triangle vertex index out of range");
  HashBox H{1.e23, 1.e23, 1.e23, -1.e23, -1.e23, -1.e23, 0, 0, 0};
  for (int q = 0; q < n_v; q++) {
    H.xmin = std::min(H.xmin, x[q]); H.xmax = std::max(H.xmax, x[q]);
    H.ymin = std::min(H.ymin, y[q]); H.ymax = std::max(H.ymax, y[q]);
    H.zmin = std::min(H.zmin, z[q]); H.zmax = std::max(H.zmax, z[q]);
  }
  H.xmin -= 0.05; H.xmax += 0.05;
  H.ymin -= 0.05; H.ymax += 0.05;
  H.zmin -= 0.05; H.zmax += 0.05;
  H.dcx = (H.xmax - H.xmin) / (kHash - 1.);
  H.dcy = (H.ymax - H.ymin) / (kHash - 1.);
  H.dcz = (H.zmax - H.zmin) / (kHash - 1.);
  std::vector<std::vector<std::pair<int, int>>> cols(kHash * kHash);  // (kv_max, triangle)
  std::vector<double> tv((size_t)n_elmt * 9), nf((size_t)n_elmt * 3);
  for (int e = 0; e < n_elmt; e++) {
    const int a = tri[3 * e], b = tri[3 * e + 1], c = tri[3 * e + 2];
    const double xv_min = std::min(std::min(x[a], x[b]), x[c]), xv_max = std::max(std::max(x[a], x[b]), x[c]);
    const double yv_min = std::min(std::min(y[a], y[b]), y[c]), yv_max = std::max(std::max(y[a], y[b]), y[c]);
    const double zv_max = std::max(std::max(z[a], z[b]), z[c]);
    int iv_min = (int)std::floor((xv_min - H.xmin) / H.dcx), iv_max = (int)std::floor((xv_max - H.xmin) / H.dcx) + 1;
    int jv_min = (int)std::floor((yv_min - H.ymin) / H.dcy), jv_max = (int)std::floor((yv_max - H.ymin) / H.dcy) + 1;
    int kv_max = (int)std::floor((zv_max - H.zmin) / H.dcz) + 1;
    iv_min = std::max(iv_min, 0); iv_max = std::min(iv_max, kHash);
    jv_min = std::max(jv_min, 0); jv_max = jv_max > kHash ? kHash : jv_max;
    kv_max = std::min(kv_max, kHash);
    for (int jj = jv_min; jj < jv_max; jj++)
      for (int ii = iv_min; ii < iv_max; ii++) cols[jj * kHash + ii].push_back({kv_max, e});
    const double vv[9] = {x[a], y[a], z[a], x[b], y[b], z[b], x[c], y[c], z[c]};
    std::copy(vv, vv + 9, &tv[(size_t)e * 9]);
    // face normal as the UCD reader computes it (Source/ibm_io.c:997-1011)
    const double dx12 = x[b] - x[a], dy12 = y[b] - y[a], dz12 = z[b] - z[a];
    const double dx13 = x[c] - x[a], dy13 = y[c] - y[a], dz13 = z[c] - z[a];
    const double fx = dy12 * dz13 - dz12 * dy13, fy = -dx12 * dz13 + dz12 * dx13, fz = dx12 * dy13 - dy12 * dx13;
    const double dr = std::sqrt(fx * fx + fy * fy + fz * fz);
    nf[(size_t)e * 3] = fx / dr; nf[(size_t)e * 3 + 1] = fy / dr; nf[(size_t)e * 3 + 2] = fz / dr;
  }
  std::vector<int> col_start(kHash * kHash + 1, 0), col_tri, col_kmax;
  for (int q = 0; q < kHash * kHash; q++) {
    auto &L = cols[q];
    std::stable_sort(L.begin(), L.end(), [](const std::pair<int, int> &a, const std::pair<int, int> &b) {
      return a.first > b.first;
    });
    col_start[q] = (int)col_tri.size();
    for (auto &pr : L) { col_kmax.push_back(pr.first); col_tri.push_back(pr.second); }
  }
  col_start[kHash * kHash] = (int)col_tri.size();
  std::vector<double> s_tab(kMaxTries + 1, 0.);
  for (int q = 1; q <= kMaxTries; q++) s_tab[q] = glibc_rand_first((unsigned)q) / ((double)2147483647 + 1) - 0.5;

  // device copies in the handle's search buffers (grown on demand)
  const size_t N = g.n();
  void **buf = cx.scratch->buf;
  size_t sizes[11] = {col_start.size() * 4, std::max<size_t>(col_tri.size(), 1) * 4,
                      std::max<size_t>(col_kmax.size(), 1) * 4, tv.size() * 8, nf.size() * 8, s_tab.size() * 8,
                      N * 8, N * 8, 4, N, 7 * 4};
  cudaStream_t st = cx.stream;
  for (int q = 0; q < 11; q++)
    if (cx.scratch->cap[q] < sizes[q]) {
      if (buf[q]) {
        cudaStreamSynchronize(st);
        cudaFree(buf[q]);
      }
      buf[q] = nullptr;
      cx.scratch->cap[q] = 0;
      if (cudaMalloc(&buf[q], sizes[q]) != cudaSuccess) {
        cudaGetLastError();
        buf[q] = nullptr;
        return fail(VFS_ENOMEM, "device allocation for the surface search failed");
      }
      cx.scratch->cap[q] = sizes[q];
    }
  const void *host[6] = {col_start.data(), col_tri.data(), col_kmax.data(), tv.data(), nf.data(), s_tab.data()};
  size_t hsz[6] = {col_start.size() * 4, col_tri.size() * 4, col_kmax.size() * 4, tv.size() * 8, nf.size() * 8,
                   s_tab.size() * 8};
  for (int q = 0; q < 6; q++)
    if (hsz[q]) cudaMemcpyAsync(buf[q], host[q], hsz[q], cudaMemcpyHostToDevice, st);
  double *dnv = (double *)buf[6], *dtmp = (double *)buf[7];
  int *dfail = (int *)buf[8];
  const bool dev = on_device(nvert);
  int b[6] = {0, 0, 0, 0, 0, 0};
  if (bctype)
    for (int q = 0; q < 6; q++) b[q] = bctype[q];
  // the classification reads nvert where it lies (a host array is staged)
  const double *src = nvert;
  if (!dev) {
    cudaMemcpyAsync(dtmp, nvert, N * 8, cudaMemcpyHostToDevice, st);
    src = dtmp;
  }
  cudaMemsetAsync(dfail, 0, 4, st);
  dim3 gi((g.mx - 2 + 127) / 128, g.my - 2, g.mz - 2), gd((g.mx + 127) / 128, g.my, g.mz);
  uint8_t *dis4 = (uint8_t *)buf[9];
  const int3 all_lo = make_int3(0, 0, 0), all_hi = make_int3(g.mx, g.my, g.mz);
  if (!want_nodes && ibi > 0) {
    // A body after the first changes only the cells whose centre lies in its
    // hash box and, by the dilation, their neighbours: the earlier bodies'
    // marks are finished (no 2 or 4 is left) and the wall rows' rule gives
    // what it gave before.  So both passes run on that index box, grown by
    // one cell for the dilation and by one more for the copy it reads.
    int init[7] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, 0}, bx[6];
    int *dbox = (int *)buf[10];
    const int nbx = (g.mx - 2 + kCentBlock - 1) / kCentBlock, nby = (g.my - 2 + kCentBlock - 1) / kCentBlock,
              nbz = (g.mz - 2 + kCentBlock - 1) / kCentBlock, nblocks = nbx * nby * nbz;
    IbmScratch &sc = *cx.scratch;
    if (!sc.bbox_valid) {
      const size_t need = (size_t)nblocks * 6 * 8;
      if (sc.bbox_cap < need) {
        if (sc.bbox) {
          cudaStreamSynchronize(st);
          cudaFree(sc.bbox);
        }
        sc.bbox = nullptr;
        sc.bbox_cap = 0;
        if (cudaMalloc(&sc.bbox, need) != cudaSuccess) {
          cudaGetLastError();
          sc.bbox = nullptr;
          return fail(VFS_ENOMEM, "device allocation for the surface search failed");
        }
        sc.bbox_cap = need;
      }
      k_cent_blocks<<<nblocks, 512, 0, st>>>(g, cx.cent, nbx, nby, sc.bbox);
      *cx.launches += 1;
      sc.bbox_valid = true;
    }
    if (sc.hits_cap < (size_t)nblocks * 4) {
      if (sc.hits) {
        cudaStreamSynchronize(st);
        cudaFree(sc.hits);
      }
      sc.hits = nullptr;
      sc.hits_cap = 0;
      if (cudaMalloc(&sc.hits, (size_t)nblocks * 4) != cudaSuccess) {
        cudaGetLastError();
        sc.hits = nullptr;
        return fail(VFS_ENOMEM, "device allocation for the surface search failed");
      }
      sc.hits_cap = (size_t)nblocks * 4;
    }
    cudaMemcpyAsync(dbox, init, sizeof(init), cudaMemcpyHostToDevice, st);
    k_ibm_box_hits<<<(nblocks + 255) / 256, 256, 0, st>>>(sc.bbox, nblocks, H, dbox, sc.hits);
    k_ibm_box_cells<<<152 * 4, 256, 0, st>>>(g, cx.cent, nbx, nby, H, sc.hits, dbox);
    cudaMemcpyAsync(bx, dbox, sizeof(bx), cudaMemcpyDeviceToHost, st);
    *cx.launches += 2;
    cudaError_t eb = cudaStreamSynchronize(st);
    if (eb != cudaSuccess) {
      cudaGetLastError();
      return fail(VFS_ECUDA, std::string("surface search: ") + cudaGetErrorString(eb));
    }
    if (n_failed) *n_failed = 0;
    if (n_nodes) *n_nodes = 0;
    if (bx[0] > bx[3]) return VFS_OK;  // no cell centre in the body's box: nothing changes
    auto grow = [&](int m) {
      return std::make_pair(make_int3(std::max(bx[0] - m, 0), std::max(bx[1] - m, 0), std::max(bx[2] - m, 0)),
                            make_int3(std::min(bx[3] + m + 1, g.mx), std::min(bx[4] + m + 1, g.my),
                                      std::min(bx[5] + m + 1, g.mz)));
    };
    const auto r2 = grow(2), r1 = grow(1);
    auto grid_of = [](int3 lo, int3 hi) { return dim3((hi.x - lo.x + 127) / 128, hi.y - lo.y, hi.z - lo.z); };
    if (!dev) cudaMemcpyAsync(dtmp, nvert, N * 8, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(dfail, 0, 4, st);
    k_ibm_classify_from<<<grid_of(r2.first, r2.second), 128, 0, st>>>(
        g, cx.cent, ibi, H, (int *)buf[0], (int *)buf[1], (int *)buf[2], (double *)buf[3], (double *)buf[4],
        (double *)buf[5], dev ? nvert : dtmp, dnv, dis4, dfail, r2.first, r2.second);
    k_ibm_dilate_finish<<<grid_of(r1.first, r1.second), 128, 0, st>>>(g, b[0], b[1], b[2], b[3], b[4], b[5], dnv,
                                                                      dis4, dev ? nvert : dtmp, r1.first, r1.second);
    *cx.launches += 2;
    int nfail = 0;
    if (!dev) cudaMemcpyAsync(nvert, dtmp, N * 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&nfail, dfail, 4, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(VFS_ECUDA, std::string("surface search: ") + cudaGetErrorString(e));
    }
    if (n_failed) *n_failed = nfail;
    return VFS_OK;
  }
  k_ibm_classify_from<<<gd, 128, 0, st>>>(g, cx.cent, ibi, H, (int *)buf[0], (int *)buf[1], (int *)buf[2],
                                          (double *)buf[3], (double *)buf[4], (double *)buf[5], src, dnv,
                                          want_nodes ? nullptr : dis4, dfail, all_lo, all_hi);
  if (!want_nodes) {
    // dilation and finish in one pass, straight into a device nvert
    double *out = dev ? nvert : dtmp;
    k_ibm_dilate_finish<<<gd, 128, 0, st>>>(g, b[0], b[1], b[2], b[3], b[4], b[5], dnv, dis4, out, all_lo, all_hi);
    *cx.launches += 2;
    int nfail = 0;
    if (!dev) cudaMemcpyAsync(nvert, dtmp, N * 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&nfail, dfail, 4, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(VFS_ECUDA, std::string("surface search: ") + cudaGetErrorString(e));
    }
    if (n_failed) *n_failed = nfail;
    if (n_nodes) *n_nodes = 0;
    return VFS_OK;
  }
  k_ibm_dilate<<<gd, 128, 0, st>>>(g, dnv, dtmp);
  int nodes_found = 0;
  if (want_nodes) {  // the IB nodes (marked 2) and their interpolation records
    const int nb = (int)((N + 255) / 256);
    std::vector<double> q, rad;
    bounding_sphere(n_elmt, tri, x, y, z, q, rad);
    std::vector<int> bcount(nb), boff(nb + 1, 0);
    int *dcount = nullptr, *dlist = nullptr;
    double *dq = nullptr, *drad = nullptr;
    bool ok = cudaMalloc(&dcount, (size_t)nb * 4) == cudaSuccess;
    if (ok) {
      k_ibm_mark_count<<<nb, 256, 0, st>>>(g, dtmp, dcount);
      ok = cudaMemcpyAsync(bcount.data(), dcount, (size_t)nb * 4, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
           cudaStreamSynchronize(st) == cudaSuccess;
    }
    if (ok) {
      for (int q2 = 0; q2 < nb; q2++) boff[q2 + 1] = boff[q2] + bcount[q2];
      nodes_found = boff[nb];
      ok = cudaMemcpyAsync(dcount, boff.data(), (size_t)nb * 4, cudaMemcpyHostToDevice, st) == cudaSuccess &&
           cudaMalloc(&dlist, (size_t)std::max(nodes_found, 1) * 4) == cudaSuccess &&
           cudaMalloc(&dq, q.size() * 8) == cudaSuccess && cudaMalloc(&drad, rad.size() * 8) == cudaSuccess;
    }
    IbmBody body;
    body.n_nodes = nodes_found;
    body.n_elmt = n_elmt;
    body.n_v = n_v;
    if (ok)
      ok = cudaMalloc(&body.nodes, (size_t)std::max(nodes_found, 1) * sizeof(vfs_ibm_node)) == cudaSuccess &&
           cudaMalloc(&body.tri, (size_t)n_elmt * 3 * 4) == cudaSuccess;
    if (ok) {
      cudaMemcpyAsync(dq, q.data(), q.size() * 8, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(drad, rad.data(), rad.size() * 8, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(body.tri, tri, (size_t)n_elmt * 3 * 4, cudaMemcpyHostToDevice, st);
      k_ibm_mark_scatter<<<nb, 256, 0, st>>>(g, dtmp, dcount, dlist);
      if (nodes_found > 0)
        k_ibm_nodes<<<(nodes_found + 127) / 128, 128, 0, st>>>(g, cx.cent, dlist, nodes_found, n_elmt,
                                                               (const double *)buf[3], (const double *)buf[4], dq,
                                                               drad, body.nodes);
      *cx.launches += 3;
      ok = cudaStreamSynchronize(st) == cudaSuccess;
    }
    if (dcount) cudaFree(dcount);
    if (dlist) cudaFree(dlist);
    if (dq) cudaFree(dq);
    if (drad) cudaFree(drad);
    if (!ok) {
      cudaGetLastError();
      if (body.nodes) cudaFree(body.nodes);
      if (body.tri) cudaFree(body.tri);
      return fail(VFS_ECUDA, "IB node records: allocation or launch failed");
    }
    auto &B = *cx.bodies;
    if ((int)B.size() <= ibi) B.resize(ibi + 1);
    if (B[ibi].nodes) cudaFree(B[ibi].nodes);
    if (B[ibi].tri) cudaFree(B[ibi].tri);
    B[ibi] = body;
  }
  k_ibm_finish<<<gi, 128, 0, st>>>(g, b[0], b[1], b[2], b[3], b[4], b[5], dtmp);
  *cx.launches += 3;
  int nfail = 0;
  cudaMemcpyAsync(nvert, dtmp, N * 8, on_device(nvert) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&nfail, dfail, 4, cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(VFS_ECUDA, std::string("surface search: ") + cudaGetErrorString(e));
  }
  if (n_failed) *n_failed = nfail;
  if (n_nodes) *n_nodes = nodes_found;
  return VFS_OK;
}

}  // namespace

extern "C" int vfs_poisson_ibm_search(vfs_poisson *h, int ibi, int n_v, const double *xyz, int n_elmt,
                                      const int32_t *tri, const int *bctype, double *nvert, int *n_failed) {
  return ibm_search_impl(h, ibi, n_v, xyz, n_elmt, tri, bctype, nvert, n_failed, false, nullptr);
}

extern "C" int vfs_poisson_ibm_search_nodes(vfs_poisson *h, int ibi, int n_v, const double *xyz, int n_elmt,
                                            const int32_t *tri, const int *bctype, double *nvert, int *n_failed,
                                            int *n_nodes) {
  return ibm_search_impl(h, ibi, n_v, xyz, n_elmt, tri, bctype, nvert, n_failed, true, n_nodes);
}

extern "C" int vfs_poisson_ibm_nodes(vfs_poisson *h, int ibi, vfs_ibm_node *nodes, int max_nodes, int *n_nodes) {
  if (!h || max_nodes < 0 || (max_nodes > 0 && !nodes)) return fail(VFS_EINVAL, "bad arguments");
  IbmContext cx;
  int rc = ibm_context(h, &cx);
  if (rc != VFS_OK) return rc;
  const auto &B = *cx.bodies;
  if (ibi < 0 || ibi >= (int)B.size() || !B[ibi].nodes) return fail(VFS_ESTATE, "no IB nodes for this body");
  const int n = B[ibi].n_nodes;
  if (n_nodes) *n_nodes = n;
  const int c = std::min(n, max_nodes);
  if (c > 0 && cudaMemcpy(nodes, B[ibi].nodes, (size_t)c * sizeof(vfs_ibm_node), cudaMemcpyDeviceToHost) !=
                   cudaSuccess) {
    cudaGetLastError();
    return fail(VFS_ECUDA, "copy of the IB node records failed");
  }
  return VFS_OK;
}

// ---- ibm_interpolation_advanced and IB_BC (launched by poisson.cu) ----
namespace vfs {

// noslip velocity and interpolated pressure at every IB node of one body
// (ibm.c:3405-3560, wallfunction.c:140-156); lucat / lp are the inputs as
// read (the reference's local copies), ucat / p are written at the nodes.
__global__ void k_ibm_apply(Grid g, const vfs_ibm_node *nodes, int n_nodes, const int *tri, const double *u_surf,
                            const double *nvert, const double *lucat, const double *lp, double *ucat, double *p) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  const vfs_ibm_node nd = nodes[n];
  const size_t t = g.at(nd.i, nd.j, nd.k);
  const size_t t1 = g.at(nd.ip[0], nd.jp[0], nd.kp[0]), t2 = g.at(nd.ip[1], nd.jp[1], nd.kp[1]),
               t3 = g.at(nd.ip[2], nd.jp[2], nd.kp[2]);
  const double sb = nd.d_s, sc = sb + nd.d_i;
  const double sk1 = nd.cr[0], sk2 = nd.cr[1], sk3 = nd.cr[2];
  double ua[3] = {0., 0., 0.};
  if (nd.cell >= 0 && u_surf) {
    const int v1 = tri[3 * nd.cell], v2 = tri[3 * nd.cell + 1], v3 = tri[3 * nd.cell + 2];
    for (int q = 0; q < 3; q++)
      ua[q] = u_surf[3 * v1 + q] * nd.cs[0] + u_surf[3 * v2 + q] * nd.cs[1] + u_surf[3 * v3 + q] * nd.cs[2];
  }
  if (nvert[t1] + nvert[t2] + nvert[t3] > 0.1 || nvert[t] > 2.9) {
    for (int q = 0; q < 3; q++) ucat[t * 3 + q] = 0.;
  } else {
    for (int q = 0; q < 3; q++) {
      const double uc = (lucat[t1 * 3 + q] * sk1 + lucat[t2 * 3 + q] * sk2 + lucat[t3 * 3 + q] * sk3);
      const double uq = uc - ua[q];
      double v = sb / sc * uq;
      v += ua[q];
      ucat[t * 3 + q] = v;
    }
  }
  p[t] = (lp[t1] * sk1 + lp[t2] * sk2 + lp[t3] * sk3);
}

__device__ inline double face_flux(const double *lu, size_t a, size_t b, const double *m) {
  const double ucx = (lu[a * 3] + lu[b * 3]) * 0.5;
  const double ucy = (lu[a * 3 + 1] + lu[b * 3 + 1]) * 0.5;
  const double ucz = (lu[a * 3 + 2] + lu[b * 3 + 2]) * 0.5;
  return ucx * m[0] + ucy * m[1] + ucz * m[2];
}

// the face fluxes around the IB nodes (ibm.c:3577-3630): every interior
// cell writes only its own three faces, so cells are independent
__global__ void k_ibm_faces(Grid g, const double *nvert, const double *lu, const double *icsi, const double *jeta,
                            const double *kzet, double f, int b0, int b1, int b2, int b3, int b4, int b5,
                            double *ucont) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
  if (i >= g.mx - 1) return;
  const size_t t = g.at(i, j, k), te = g.at(i + 1, j, k), tn = g.at(i, j + 1, k), tt = g.at(i, j, k + 1);
  const bool wi0 = b0 == -1 || b0 == -2, wi1 = b1 == -1 || b1 == -2, wj0 = b2 == -1 || b2 == -2,
             wj1 = b3 == -1 || b3 == -2, wk0 = b4 == -1 || b4 == -2, wk1 = b5 == -1 || b5 == -2;
  if ((int)(nvert[t] + 0.5) == 1) {
    ucont[t * 3] = face_flux(lu, t, te, &icsi[t * 3]) * f;
    ucont[t * 3 + 1] = face_flux(lu, tn, t, &jeta[t * 3]) * f;
    ucont[t * 3 + 2] = face_flux(lu, tt, t, &kzet[t * 3]) * f;
    if (wi0 && i == 1) ucont[t * 3] = 0;
    if (wj0 && j == 1) ucont[t * 3 + 1] = 0;
    if (wk0 && k == 1) ucont[t * 3 + 2] = 0;
  }
  if ((int)(nvert[te] + 0.5) == 1) {
    ucont[t * 3] = face_flux(lu, t, te, &icsi[t * 3]) * f;
    if (wi1 && i == g.mx - 3) ucont[t * 3] = 0;
  }
  if ((int)(nvert[tn] + 0.5) == 1) {
    ucont[t * 3 + 1] = face_flux(lu, tn, t, &jeta[t * 3]) * f;
    if (wj1 && j == g.my - 3) ucont[t * 3 + 1] = 0;
  }
  if ((int)(nvert[tt] + 0.5) == 1) {
    ucont[t * 3 + 2] = face_flux(lu, tt, t, &kzet[t * 3]) * f;
    if (wk1 && k == g.mz - 3) ucont[t * 3 + 2] = 0;
  }
}

// IB_BC's interior loop (momentum.c:2114-2178): the IB faces from ucat
// ((int)nvert == 1), the immersed == 3 zeroing and the -1/-2 walls in i and
// j (the i == 1 / j == 1 rows write the face below them, which no other cell
// of this loop writes)
__global__ void k_ib_bc_faces(Grid g, const double *nvert, const double *lu, const double *icsi,
                              const double *jeta, const double *kzet, int immersed, int b0, int b1, int b2, int b3,
                              double *ucont) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
  if (i >= g.mx - 1) return;
  const size_t t = g.at(i, j, k), te = g.at(i + 1, j, k), tn = g.at(i, j + 1, k), tt = g.at(i, j, k + 1);
  if (immersed) {
    const double f = immersed == 3 ? 0. : 1.;
    if ((int)nvert[t] == 1) {
      ucont[t * 3] = face_flux(lu, t, te, &icsi[t * 3]) * f;
      ucont[t * 3 + 1] = face_flux(lu, tn, t, &jeta[t * 3]) * f;
      ucont[t * 3 + 2] = face_flux(lu, tt, t, &kzet[t * 3]) * f;
    }
    if ((int)(nvert[te]) == 1) ucont[t * 3] = face_flux(lu, t, te, &icsi[t * 3]) * f;
    if ((int)(nvert[tn]) == 1) ucont[t * 3 + 1] = face_flux(lu, tn, t, &jeta[t * 3]) * f;
    if ((int)(nvert[tt]) == 1) ucont[t * 3 + 2] = face_flux(lu, tt, t, &kzet[t * 3]) * f;
    if (immersed == 3) {
      if ((nvert[te] + nvert[t]) > 1.1) ucont[t * 3] = 0;
      if ((nvert[tn] + nvert[t]) > 1.1) ucont[t * 3 + 1] = 0;
      if ((nvert[tt] + nvert[t]) > 1.1) ucont[t * 3 + 2] = 0;
    }
  }
  const bool wi0 = b0 == -1 || b0 == -2, wi1 = b1 == -1 || b1 == -2, wj0 = b2 == -1 || b2 == -2,
             wj1 = b3 == -1 || b3 == -2;
  if ((wi0 && i == 1) || (wi1 && i == g.mx - 2)) {
    if (i == 1) ucont[g.at(i - 1, j, k) * 3] = 0;
    else ucont[t * 3] = 0;
  }
  if ((wj0 && j == 1) || (wj1 && j == g.my - 2)) {
    if (j == 1) ucont[g.at(i, j - 1, k) * 3 + 1] = 0;
    else ucont[t * 3 + 1] = 0;
  }
}

// IB_BC's closing loop over every DA point (momentum.c:2180-2210): the slip
// (10) walls and the periodic faces.  The reference runs it in place in
// k, j, i order; a periodic copy there reads its partner before a slip rule
// of the same row could zero it, so every value follows from the values
// before the loop (uold).
__global__ void k_ib_bc_edges(Grid g, const double *uold, int b0, int b1, int b2, int b3, int b4, int b5,
                              double *ucont) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  const size_t t = g.at(i, j, k);
  double vx = uold[t * 3], vy = uold[t * 3 + 1], vz = uold[t * 3 + 2];
  if (i == 0) {
    if (g.px) vx = uold[g.at(g.mx - 2, j, k) * 3];
    if (b0 == 10) vx = 0;
  } else if (i == g.mx - 1) {
    if (g.px) vx = uold[g.at(1, j, k) * 3];
  }
  if (i == g.mx - 2 && b1 == 10) vx = 0;
  if (j == 0) {
    if (g.py) vy = uold[g.at(i, g.my - 2, k) * 3 + 1];
    if (b2 == 10) vy = 0;
  } else if (j == g.my - 1) {
    if (g.py) vy = uold[g.at(i, 1, k) * 3 + 1];
  }
  if (j == g.my - 2 && b3 == 10) vy = 0;
  if (k == 0) {
    if (g.pz) vz = uold[g.at(i, j, g.mz - 2) * 3 + 2];
    if (b4 == 10) vz = 0;
  } else if (k == g.mz - 1) {
    if (g.pz) vz = uold[g.at(i, j, 1) * 3 + 2];
  }
  if (k == g.mz - 2 && b5 == 10) vz = 0;
  ucont[t * 3] = vx;
  ucont[t * 3 + 1] = vy;
  ucont[t * 3 + 2] = vz;
}

}  // namespace vfs
