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

__global__ void k_ibm_classify(Grid g, const double *__restrict__ cent, int ibi, HashBox H,
                               const int *__restrict__ col_start, const int *__restrict__ col_tri,
                               const int *__restrict__ col_kmax, const double *__restrict__ tv,
                               const double *__restrict__ nf, const double *__restrict__ s_tab, double *nvert,
                               int *failed) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
  if (i >= g.mx - 1) return;
  const size_t t = g.at(i, j, k);
  double nv = nvert[t];
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
  nvert[t] = nv;
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
__global__ void k_ibm_finish(Grid g, int b0, int b1, int b2, int b3, int b4, int b5, double *nvert) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
  if (i >= g.mx - 1) return;
  const size_t t = g.at(i, j, k);
  double v = nvert[t];
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
  nvert[t] = v;
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

extern "C" int vfs_poisson_ibm_search(vfs_poisson *h, int ibi, int n_v, const double *xyz, int n_elmt,
                                      const int32_t *tri, const int *bctype, double *nvert, int *n_failed) {
  if (!h || !xyz || !tri || !nvert || n_v < 3 || n_elmt < 1) return fail(VFS_EINVAL, "bad surface arguments");
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

  // device copies (freed before returning)
  const size_t N = g.n();
  void *buf[9] = {};
  auto cleanup = [&]() {
    for (void *p : buf)
      if (p) cudaFree(p);
  };
  size_t sizes[9] = {col_start.size() * 4, std::max<size_t>(col_tri.size(), 1) * 4,
                     std::max<size_t>(col_kmax.size(), 1) * 4, tv.size() * 8, nf.size() * 8, s_tab.size() * 8,
                     N * 8, N * 8, 4};
  for (int q = 0; q < 9; q++)
    if (cudaMalloc(&buf[q], sizes[q]) != cudaSuccess) {
      cudaGetLastError();
      cleanup();
      return fail(VFS_ENOMEM, "device allocation for the surface search failed");
    }
  cudaStream_t st = cx.stream;
  const void *host[6] = {col_start.data(), col_tri.data(), col_kmax.data(), tv.data(), nf.data(), s_tab.data()};
  size_t hsz[6] = {col_start.size() * 4, col_tri.size() * 4, col_kmax.size() * 4, tv.size() * 8, nf.size() * 8,
                   s_tab.size() * 8};
  for (int q = 0; q < 6; q++)
    if (hsz[q]) cudaMemcpyAsync(buf[q], host[q], hsz[q], cudaMemcpyHostToDevice, st);
  double *dnv = (double *)buf[6], *dtmp = (double *)buf[7];
  int *dfail = (int *)buf[8];
  cudaMemcpyAsync(dnv, nvert, N * 8, on_device(nvert) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(dfail, 0, 4, st);
  dim3 gi((g.mx - 2 + 127) / 128, g.my - 2, g.mz - 2), gd((g.mx + 127) / 128, g.my, g.mz);
  k_ibm_classify<<<gi, 128, 0, st>>>(g, cx.cent, ibi, H, (int *)buf[0], (int *)buf[1], (int *)buf[2],
                                     (double *)buf[3], (double *)buf[4], (double *)buf[5], dnv, dfail);
  k_ibm_dilate<<<gd, 128, 0, st>>>(g, dnv, dtmp);
  int b[6] = {0, 0, 0, 0, 0, 0};
  if (bctype)
    for (int q = 0; q < 6; q++) b[q] = bctype[q];
  k_ibm_finish<<<gi, 128, 0, st>>>(g, b[0], b[1], b[2], b[3], b[4], b[5], dtmp);
  *cx.launches += 3;
  int nfail = 0;
  cudaMemcpyAsync(nvert, dtmp, N * 8, on_device(nvert) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&nfail, dfail, 4, cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(VFS_ECUDA, std::string("surface search: ") + cudaGetErrorString(e));
  }
  if (n_failed) *n_failed = nfail;
  return VFS_OK;
}
