// setup.cu -- grid metrics, dof numbering, operator assembly, right-hand
// side, pressure update, projection, divergence and the multigrid transfer
// operators.
//
// This translation unit is compiled with -fmad=false: every floating-point
// expression is rounded in the reference's source order, so these kernels
// reproduce the reference's arithmetic (restated in the oracle) bit for bit.
// Each kernel names the reference lines it follows.
#include "common.cuh"
#include "kernels.cuh"

namespace vfs {

static constexpr double kThr = 0.1;  // poisson_threshold, Source/main.c:124

// --------------------------------------------------------------------------
// FormMetrics (Source/metrics.c:12-1355; metrics.c:10 defines NEWMETRIC)
// --------------------------------------------------------------------------
#define CO(i, j, k, c) coor[g.at(i, j, k) * 3 + (c)]

// cell centres (metrics.c:89-108) and, for every interior cell, aj = 1/J and
// the cell metrics csi/eta/zet from the 8-node differences
// (metrics.c:194-256, the NEWMETRIC branch)
__global__ void k_metrics_cell(Grid g, const double *__restrict__ coor, MetricPtrs m) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  size_t t = g.at(i, j, k);
  const int mx = g.mx, my = g.my, mz = g.mz;
  if (!(i >= 1 && i < mx - 1 && j >= 1 && j < my - 1 && k >= 1 && k < mz - 1)) return;
  for (int c = 0; c < 3; c++)
    m.cent[t * 3 + c] = 0.125 * (CO(i, j, k, c) + CO(i, j - 1, k, c) + CO(i, j, k - 1, c) + CO(i, j - 1, k - 1, c) +
                                 CO(i - 1, j, k, c) + CO(i - 1, j - 1, k, c) + CO(i - 1, j, k - 1, c) +
                                 CO(i - 1, j - 1, k - 1, c));
  double dc[3], de[3], dz[3];
  for (int c = 0; c < 3; c++) {
    dc[c] = 0.25 * (CO(i, j, k, c) + CO(i, j - 1, k, c) + CO(i, j, k - 1, c) + CO(i, j - 1, k - 1, c) -
                    CO(i - 1, j, k, c) - CO(i - 1, j - 1, k, c) - CO(i - 1, j, k - 1, c) - CO(i - 1, j - 1, k - 1, c));
    de[c] = 0.25 * (CO(i, j, k, c) + CO(i - 1, j, k, c) + CO(i, j, k - 1, c) + CO(i - 1, j, k - 1, c) -
                    CO(i, j - 1, k, c) - CO(i - 1, j - 1, k, c) - CO(i, j - 1, k - 1, c) - CO(i - 1, j - 1, k - 1, c));
    dz[c] = 0.25 * (CO(i, j, k, c) + CO(i, j - 1, k, c) + CO(i - 1, j, k, c) + CO(i - 1, j - 1, k, c) -
                    CO(i, j, k - 1, c) - CO(i, j - 1, k - 1, c) - CO(i - 1, j, k - 1, c) - CO(i - 1, j - 1, k - 1, c));
  }
  double det = dc[0] * (de[1] * dz[2] - de[2] * dz[1]) - dc[1] * (de[0] * dz[2] - de[2] * dz[0]) +
               dc[2] * (de[0] * dz[1] - de[1] * dz[0]);
  m.aj[t] = 1. / det;
  double *cs = &m.csi[t * 3], *et = &m.eta[t * 3], *ze = &m.zet[t * 3];
  cs[0] = de[1] * dz[2] - de[2] * dz[1];
  cs[1] = -de[0] * dz[2] + de[2] * dz[0];
  cs[2] = de[0] * dz[1] - de[1] * dz[0];
  et[0] = dz[1] * dc[2] - dz[2] * dc[1];
  et[1] = -dz[0] * dc[2] + dz[2] * dc[0];
  et[2] = dz[0] * dc[1] - dz[1] * dc[0];
  ze[0] = dc[1] * de[2] - dc[2] * de[1];
  ze[1] = -dc[0] * de[2] + dc[2] * de[0];
  ze[2] = dc[0] * de[1] - dc[1] * de[0];
}

// boundary mirror of csi, eta, zet and aj, one direction per launch, in the
// order x, y, z of metrics.c:262-342.
__global__ void k_metrics_mirror(Grid g, MetricPtrs m, int dir) {
  int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y;
  int nu = dir == 0 ? g.my : g.mx, nv = dir == 2 ? g.my : g.mz;
  if (u >= nu || v >= nv) return;
  for (int side = 0; side < 2; side++) {
    size_t t, s;
    if (dir == 0) { int i = side ? g.mx - 1 : 0; t = g.at(i, u, v); s = g.at(side ? i - 1 : 1, u, v); }
    else if (dir == 1) { int j = side ? g.my - 1 : 0; t = g.at(u, j, v); s = g.at(u, side ? j - 1 : 1, v); }
    else { int k = side ? g.mz - 1 : 0; t = g.at(u, v, k); s = g.at(u, v, side ? k - 1 : 1); }
    for (int c = 0; c < 3; c++) {
      m.csi[t * 3 + c] = m.csi[s * 3 + c];
      m.eta[t * 3 + c] = m.eta[s * 3 + c];
      m.zet[t * 3 + c] = m.zet[s * 3 + c];
    }
    m.aj[t] = m.aj[s];
  }
}

// periodic ghost copy: of the cell metrics before the face averages
// (metrics.c:360-397), of all sixteen arrays at the end (metrics.c:1227-1262).
// A source cell has every periodic coordinate inside 1..m-2, so it is never
// a target.
__global__ void k_metrics_periodic(Grid g, MetricPtrs m, int faces) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  int a, b, c, fi, fj, fk;
  if (!g.remap(i, j, k, a, b, c, fi, fj, fk)) return;
  size_t s = g.at(a, b, c), t = g.at(i, j, k);
  double *v3[12] = {m.csi, m.eta, m.zet, m.icsi, m.ieta, m.izet, m.jcsi, m.jeta, m.jzet, m.kcsi, m.keta, m.kzet};
  double *v1[4] = {m.aj, m.iaj, m.jaj, m.kaj};
  const int n3 = faces ? 12 : 3, n1 = faces ? 4 : 1;
  for (int q = 0; q < n3; q++)
    for (int e = 0; e < 3; e++) v3[q][t * 3 + e] = v3[q][s * 3 + e];
  for (int q = 0; q < n1; q++) v1[q][t] = v1[q][s];
}

// NEWMETRIC face metrics (metrics.c:588-592, :696-700, :804-808): the
// arithmetic mean of the two adjacent cells' csi/eta/zet (AxByC,
// Source/momentum.c:40-45) and the harmonic mean of their aj; i faces
// i = 0..mx-2 of the interior j, k; j faces j = 0..my-2; k faces k = 0..mz-2.
__global__ void k_metrics_face(Grid g, MetricPtrs m, int dir) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  const int mx = g.mx, my = g.my, mz = g.mz;
  bool in;
  if (dir == 0) in = i < mx - 1 && j >= 1 && j < my - 1 && k >= 1 && k < mz - 1;
  else if (dir == 1) in = i >= 1 && i < mx - 1 && j < my - 1 && k >= 1 && k < mz - 1;
  else in = i >= 1 && i < mx - 1 && j >= 1 && j < my - 1 && k < mz - 1;
  if (!in) return;
  const size_t t = g.at(i, j, k);
  const size_t u = dir == 0 ? g.at(i + 1, j, k) : dir == 1 ? g.at(i, j + 1, k) : g.at(i, j, k + 1);
  double *fc = dir == 0 ? m.icsi : dir == 1 ? m.jcsi : m.kcsi;
  double *fe = dir == 0 ? m.ieta : dir == 1 ? m.jeta : m.keta;
  double *fz = dir == 0 ? m.izet : dir == 1 ? m.jzet : m.kzet;
  double *fa = dir == 0 ? m.iaj : dir == 1 ? m.jaj : m.kaj;
  for (int c = 0; c < 3; c++) {
    fc[t * 3 + c] = 0.5 * m.csi[t * 3 + c] + 0.5 * m.csi[u * 3 + c];
    fe[t * 3 + c] = 0.5 * m.eta[t * 3 + c] + 0.5 * m.eta[u * 3 + c];
    fz[t * 3 + c] = 0.5 * m.zet[t * 3 + c] + 0.5 * m.zet[u * 3 + c];
  }
  fa[t] = 2. / (1. / m.aj[t] + 1. / m.aj[u]);
}
#undef CO

// --------------------------------------------------------------------------
// Dof numbering, setup_lidx2 (Source/poisson.c:188-335)
// --------------------------------------------------------------------------
__device__ inline bool is_dof_cell(const Grid &g, const double *nvert, int i, int j, int k) {
  // poisson.c:244-251: interior and (int)nvert <= poisson_threshold
  if (i <= 0 || i >= g.mx - 1 || j <= 0 || j >= g.my - 1 || k <= 0 || k >= g.mz - 1) return false;
  return !((int)nvert[g.at(i, j, k)] > kThr);
}
// dof test of a possibly-ghost point, with the periodic aliasing of
// poisson.c:299-332 (Gid of a periodic ghost is its partner's Gid).
__device__ inline bool has_dof(const Grid &g, const double *nvert, int i, int j, int k) {
  int a, b, c, fi, fj, fk;
  g.remap(i, j, k, a, b, c, fi, fj, fk);
  return is_dof_cell(g, nvert, a, b, c);
}

// per-block dof counts over the box order (k-j-i, the reference's loop order)
__global__ void k_count_dofs(Grid g, Box b, const double *nvert, int *block_count) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  if (c < b.n()) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    f = is_dof_cell(g, nvert, i + 1, j + 1, k + 1) ? 1 : 0;
  }
  int s = block_sum<int>(f);
  if (threadIdx.x == 0) block_count[blockIdx.x] = s;
}
// exclusive scan of the block counts by one block (sequential per thread
// chunk, then a scan over the 1024 chunk totals).
__global__ void k_scan_blocks(int *block_count, int nblocks, int *total) {
  __shared__ int part[1024];
  int per = (nblocks + blockDim.x - 1) / blockDim.x;
  int lo = threadIdx.x * per, hi = min(nblocks, lo + per);
  int s = 0;
  for (int q = lo; q < hi; q++) s += block_count[q];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int q = 0; q < (int)blockDim.x; q++) { int v = part[q]; part[q] = run; run += v; }
    *total = run;
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int q = lo; q < hi; q++) { int v = block_count[q]; block_count[q] = run; run += v; }
}
__global__ void k_number_dofs(Grid g, Box b, const double *nvert, const int *block_off, int *gid_box) {
  __shared__ int warp_tot[32];
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  if (c < b.n()) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    f = is_dof_cell(g, nvert, i + 1, j + 1, k + 1) ? 1 : 0;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned bal = __ballot_sync(0xffffffffu, f);
  int pre = __popc(bal & ((1u << lane) - 1u));
  if (lane == 0) warp_tot[w] = __popc(bal);
  __syncthreads();
  int off = 0;
  for (int q = 0; q < w; q++) off += warp_tot[q];
  if (c < b.n()) gid_box[c] = f ? block_off[blockIdx.x] + off + pre : -1;
}
// DA-layout Gid with periodic ghost aliasing.
__global__ void k_gid_da(Grid g, Box b, const int *gid_box, int *gid_da) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  int a, bb, c, fi, fj, fk;
  g.remap(i, j, k, a, bb, c, fi, fj, fk);
  int v = -1;
  if (a >= 1 && a < g.mx - 1 && bb >= 1 && bb < g.my - 1 && c >= 1 && c < g.mz - 1)
    v = gid_box[b.at(a - 1, bb - 1, c - 1)];
  gid_da[g.at(i, j, k)] = v;
}

// --------------------------------------------------------------------------
// PoissonLHSNew (Source/poisson.c:977-1688), level set off (r = 1)
// --------------------------------------------------------------------------
// g11..g33 at a face with the periodic source remap of poisson.c:1102-1138
__device__ inline double gface_at(const MetricPtrs &m, int q, size_t s) {
  const double *X, *Y, *AJ;
  switch (q) {
    case 0: X = m.icsi; Y = m.icsi; AJ = m.iaj; break;
    case 1: X = m.ieta; Y = m.icsi; AJ = m.iaj; break;
    case 2: X = m.izet; Y = m.icsi; AJ = m.iaj; break;
    case 3: X = m.jcsi; Y = m.jeta; AJ = m.jaj; break;
    case 4: X = m.jeta; Y = m.jeta; AJ = m.jaj; break;
    case 5: X = m.jzet; Y = m.jeta; AJ = m.jaj; break;
    case 6: X = m.kcsi; Y = m.kzet; AJ = m.kaj; break;
    case 7: X = m.keta; Y = m.kzet; AJ = m.kaj; break;
    default: X = m.kzet; Y = m.kzet; AJ = m.kaj; break;
  }
  return (X[s * 3] * Y[s * 3] + X[s * 3 + 1] * Y[s * 3 + 1] + X[s * 3 + 2] * Y[s * 3 + 2]) * AJ[s];
}
__device__ inline double gface(const Grid &g, const MetricPtrs &m, int q, int i, int j, int k) {
  int a, b, c, fi, fj, fk;
  g.remap(i, j, k, a, b, c, fi, fj, fk);
  const size_t s = g.at(a, b, c);
  return m.gface ? m.gface[(size_t)q * g.n() + s] : gface_at(m, q, s);
}
// the nine face coefficients of every DA point, as gface forms them (no FMA
// contraction in this unit: the same bits)
__global__ void k_face_coef(Grid g, MetricPtrs m, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  const size_t s = g.at(i, j, k), n = g.n();
#pragma unroll
  for (int q = 0; q < 9; q++) out[(size_t)q * n + s] = gface_at(m, q, s);
}

// mean (Source/level.c:2276-2280): the harmonic mean of two densities
__device__ inline double ls_mean(double A, double B) { return 2.0 * A * B / (A + B); }

// One row of the operator, accumulated in the reference's statement order.
// With a level set (ls.on) every face coefficient is divided by the face
// density and the Dirichlet top / bottom rows of poisson.c:1295-1554 apply.
template <bool LS>
__device__ void assemble_row_t(const Grid &g, const double *nvert, const MetricPtrs &m, int i, int j, int k,
                               double v[NSLOT], const LevelSet &ls) {
  // a face coefficient divided by the face density: without a level set
  // the density is exactly 1 and the division (exact there) is not issued
#define DR(x) (LS ? (x) / r : (x))
  const int mx = g.mx, my = g.my, mz = g.mz;
  const bool ip = g.px, jp = g.py, kp = g.pz;
  const double thr = kThr;
  double r = 1.0;
#define RHO(a, b, c) ls.rho[g.at(a, b, c)]
#define NV(a, b, c) nvert[g.at(a, b, c)]
#define G(q, a, b, c) gface(g, m, q, a, b, c)
  for (int s = 0; s < NSLOT; s++) v[s] = 0.;
  if (NV(i + 1, j, k) < thr && (i != mx - 2 || ip)) {  // poisson.c:1167-1230
    r = ls.on ? ls_mean(RHO(i + 1, j, k), RHO(i, j, k)) : 1.0;
    double g0 = G(0, i, j, k), g1 = G(1, i, j, k), g2 = G(2, i, j, k);
    v[CP] -= DR(g0); v[EP] += DR(g0);
    if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i + 1, j + 1, k) > thr) {
      if (NV(i, j - 1, k) + NV(i + 1, j - 1, k) < thr && j != 1) {
        v[CP] += DR(g1 * 0.5); v[EP] += DR(g1 * 0.5); v[SP] -= DR(g1 * 0.5); v[SE] -= DR(g1 * 0.5);
      }
    } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i + 1, j - 1, k) > thr) {
      if (NV(i, j + 1, k) + NV(i + 1, j + 1, k) < thr) {
        v[NP] += DR(g1 * 0.5); v[NE] += DR(g1 * 0.5); v[CP] -= DR(g1 * 0.5); v[EP] -= DR(g1 * 0.5);
      }
    } else {
      v[NP] += DR(g1 * 0.25); v[NE] += DR(g1 * 0.25); v[SP] -= DR(g1 * 0.25); v[SE] -= DR(g1 * 0.25);
    }
    if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i + 1, j, k + 1) > thr) {
      if (NV(i, j, k - 1) + NV(i + 1, j, k - 1) < thr && k != 1) {
        v[CP] += DR(g2 * 0.5); v[EP] += DR(g2 * 0.5); v[BP] -= DR(g2 * 0.5); v[BE] -= DR(g2 * 0.5);
      }
    } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i + 1, j, k - 1) > thr) {
      if (NV(i, j, k + 1) + NV(i + 1, j, k + 1) < thr) {
        v[TP] += DR(g2 * 0.5); v[TE] += DR(g2 * 0.5); v[CP] -= DR(g2 * 0.5); v[EP] -= DR(g2 * 0.5);
      }
    } else {
      v[TP] += DR(g2 * 0.25); v[TE] += DR(g2 * 0.25); v[BP] -= DR(g2 * 0.25); v[BE] -= DR(g2 * 0.25);
    }
  }
  if (NV(i - 1, j, k) < thr && (i != 1 || ip)) {  // poisson.c:1233-1293
    r = ls.on ? ls_mean(RHO(i - 1, j, k), RHO(i, j, k)) : 1.0;
    double g0 = G(0, i - 1, j, k), g1 = G(1, i - 1, j, k), g2 = G(2, i - 1, j, k);
    v[CP] -= DR(g0); v[WP] += DR(g0);
    if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i - 1, j + 1, k) > thr) {
      if (NV(i, j - 1, k) + NV(i - 1, j - 1, k) < thr && j != 1) {
        v[CP] -= DR(g1 * 0.5); v[WP] -= DR(g1 * 0.5); v[SP] += DR(g1 * 0.5); v[SW] += DR(g1 * 0.5);
      }
    } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i - 1, j - 1, k) > thr) {
      if (NV(i, j + 1, k) + NV(i - 1, j + 1, k) < thr) {
        v[NP] -= DR(g1 * 0.5); v[NW] -= DR(g1 * 0.5); v[CP] += DR(g1 * 0.5); v[WP] += DR(g1 * 0.5);
      }
    } else {
      v[NP] -= DR(g1 * 0.25); v[NW] -= DR(g1 * 0.25); v[SP] += DR(g1 * 0.25); v[SW] += DR(g1 * 0.25);
    }
    if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i - 1, j, k + 1) > thr) {
      if (NV(i, j, k - 1) + NV(i - 1, j, k - 1) < thr && k != 1) {
        v[CP] -= DR(g2 * 0.5); v[WP] -= DR(g2 * 0.5); v[BP] += DR(g2 * 0.5); v[BW] += DR(g2 * 0.5);
      }
    } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i - 1, j, k - 1) > thr) {
      if (NV(i, j, k + 1) + NV(i - 1, j, k + 1) < thr) {
        v[TP] -= DR(g2 * 0.5); v[TW] -= DR(g2 * 0.5); v[CP] += DR(g2 * 0.5); v[WP] += DR(g2 * 0.5);
      }
    } else {
      v[TP] -= DR(g2 * 0.25); v[TW] -= DR(g2 * 0.25); v[BP] += DR(g2 * 0.25); v[BW] += DR(g2 * 0.25);
    }
  }
  if (NV(i, j + 1, k) < thr && (j != my - 2 || jp || (ls.on && ls.bc3 == 4 && j == my - 2))) {  // poisson.c:1296-1361
    r = ls.on ? ls_mean(RHO(i, j + 1, k), RHO(i, j, k)) : 1.0;
    double g3 = G(3, i, j, k), g4 = G(4, i, j, k), g5 = G(5, i, j, k);
    if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j + 1, k) > thr) {
      if (NV(i - 1, j, k) + NV(i - 1, j + 1, k) < thr && i != 1) {
        v[CP] += DR(g3 * 0.5); v[NP] += DR(g3 * 0.5); v[WP] -= DR(g3 * 0.5); v[NW] -= DR(g3 * 0.5);
      }
    } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j + 1, k) > thr) {
      if (NV(i + 1, j, k) + NV(i + 1, j + 1, k) < thr) {
        v[EP] += DR(g3 * 0.5); v[NE] += DR(g3 * 0.5); v[CP] -= DR(g3 * 0.5); v[NP] -= DR(g3 * 0.5);
      }
    } else {
      v[EP] += DR(g3 * 0.25); v[NE] += DR(g3 * 0.25); v[WP] -= DR(g3 * 0.25); v[NW] -= DR(g3 * 0.25);
    }
    if (ls.on && ls.bc3 == 4 && j == my - 2) v[CP] -= DR(g4 / 0.5);  // zero Dirichlet pressure, :1328
    else { v[CP] -= DR(g4); v[NP] += DR(g4); }
    if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j + 1, k + 1) > thr) {
      if (NV(i, j, k - 1) + NV(i, j + 1, k - 1) < thr && k != 1) {
        v[CP] += DR(g5 * 0.5); v[NP] += DR(g5 * 0.5); v[BP] -= DR(g5 * 0.5); v[BN] -= DR(g5 * 0.5);
      }
    } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j + 1, k - 1) > thr) {
      if (NV(i, j, k + 1) + NV(i, j + 1, k + 1) < thr) {
        v[TP] += DR(g5 * 0.5); v[TN] += DR(g5 * 0.5); v[CP] -= DR(g5 * 0.5); v[NP] -= DR(g5 * 0.5);
      }
    } else {
      v[TP] += DR(g5 * 0.25); v[TN] += DR(g5 * 0.25); v[BP] -= DR(g5 * 0.25); v[BN] -= DR(g5 * 0.25);
    }
  }
  if (NV(i, j - 1, k) < thr && (j != 1 || jp)) {  // poisson.c:1364-1422
    r = ls.on ? ls_mean(RHO(i, j - 1, k), RHO(i, j, k)) : 1.0;
    double g3 = G(3, i, j - 1, k), g4 = G(4, i, j - 1, k), g5 = G(5, i, j - 1, k);
    if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j - 1, k) > thr) {
      if (NV(i - 1, j, k) + NV(i - 1, j - 1, k) < thr && i != 1) {
        v[CP] -= DR(g3 * 0.5); v[SP] -= DR(g3 * 0.5); v[WP] += DR(g3 * 0.5); v[SW] += DR(g3 * 0.5);
      }
    } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j - 1, k) > thr) {
      if (NV(i + 1, j, k) + NV(i + 1, j - 1, k) < thr) {
        v[EP] -= DR(g3 * 0.5); v[SE] -= DR(g3 * 0.5); v[CP] += DR(g3 * 0.5); v[SP] += DR(g3 * 0.5);
      }
    } else {
      v[EP] -= DR(g3 * 0.25); v[SE] -= DR(g3 * 0.25); v[WP] += DR(g3 * 0.25); v[SW] += DR(g3 * 0.25);
    }
    v[CP] -= DR(g4); v[SP] += DR(g4);
    if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j - 1, k + 1) > thr) {
      if (NV(i, j, k - 1) + NV(i, j - 1, k - 1) < thr && k != 1) {
        v[CP] -= DR(g5 * 0.5); v[SP] -= DR(g5 * 0.5); v[BP] += DR(g5 * 0.5); v[BS] += DR(g5 * 0.5);
      }
    } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j - 1, k - 1) > thr) {
      if (NV(i, j, k + 1) + NV(i, j - 1, k + 1) < thr) {
        v[TP] -= DR(g5 * 0.5); v[TS] -= DR(g5 * 0.5); v[CP] += DR(g5 * 0.5); v[SP] += DR(g5 * 0.5);
      }
    } else {
      v[TP] -= DR(g5 * 0.25); v[TS] -= DR(g5 * 0.25); v[BP] += DR(g5 * 0.25); v[BS] += DR(g5 * 0.25);
    }
  }
  if (NV(i, j, k + 1) < thr && (k != mz - 2 || kp || (ls.on && ls.bc5 == 4 && k == mz - 2))) {  // poisson.c:1425-1491
    r = ls.on ? ls_mean(RHO(i, j, k + 1), RHO(i, j, k)) : 1.0;
    double g6 = G(6, i, j, k), g7 = G(7, i, j, k), g8 = G(8, i, j, k);
    if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k + 1) > thr) {
      if (NV(i - 1, j, k) + NV(i - 1, j, k + 1) < thr && i != 1) {
        v[CP] += DR(g6 * 0.5); v[TP] += DR(g6 * 0.5); v[WP] -= DR(g6 * 0.5); v[TW] -= DR(g6 * 0.5);
      }
    } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k + 1) > thr) {
      if (NV(i + 1, j, k) + NV(i + 1, j, k + 1) < thr) {
        v[EP] += DR(g6 * 0.5); v[TE] += DR(g6 * 0.5); v[CP] -= DR(g6 * 0.5); v[TP] -= DR(g6 * 0.5);
      }
    } else {
      v[EP] += DR(g6 * 0.25); v[TE] += DR(g6 * 0.25); v[WP] -= DR(g6 * 0.25); v[TW] -= DR(g6 * 0.25);
    }
    if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k + 1) > thr) {
      if (NV(i, j - 1, k) + NV(i, j - 1, k + 1) < thr && j != 1) {
        v[CP] += DR(g7 * 0.5); v[TP] += DR(g7 * 0.5); v[SP] -= DR(g7 * 0.5); v[TS] -= DR(g7 * 0.5);
      }
    } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k + 1) > thr) {
      if (NV(i, j + 1, k) + NV(i, j + 1, k + 1) < thr) {
        v[NP] += DR(g7 * 0.5); v[TN] += DR(g7 * 0.5); v[CP] -= DR(g7 * 0.5); v[TP] -= DR(g7 * 0.5);
      }
    } else {
      v[NP] += DR(g7 * 0.25); v[TN] += DR(g7 * 0.25); v[SP] -= DR(g7 * 0.25); v[TS] -= DR(g7 * 0.25);
    }
    if (ls.on && ls.bc5 == 4 && k == mz - 2) v[CP] -= DR(g8 / 0.5);  // :1482-1484
    else { v[CP] -= DR(g8); v[TP] += DR(g8); }
  }
  if (NV(i, j, k - 1) < thr &&
      (k != 1 || kp || (ls.on && ls.bc4 == 5000 && k == 1 && ls.level[g.at(i, j, k)] < 0))) {  // poisson.c:1494-1561
    r = ls.on ? (k == 1 ? RHO(i, j, k) : ls_mean(RHO(i, j, k - 1), RHO(i, j, k))) : 1.0;
    double g6 = G(6, i, j, k - 1), g7 = G(7, i, j, k - 1), g8 = G(8, i, j, k - 1);
    if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k - 1) > thr) {
      if (NV(i - 1, j, k) + NV(i - 1, j, k - 1) < thr && i != 1) {
        v[CP] -= DR(g6 * 0.5); v[BP] -= DR(g6 * 0.5); v[WP] += DR(g6 * 0.5); v[BW] += DR(g6 * 0.5);
      }
    } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k - 1) > thr) {
      if (NV(i + 1, j, k) + NV(i + 1, j, k - 1) < thr) {
        v[EP] -= DR(g6 * 0.5); v[BE] -= DR(g6 * 0.5); v[CP] += DR(g6 * 0.5); v[BP] += DR(g6 * 0.5);
      }
    } else {
      v[EP] -= DR(g6 * 0.25); v[BE] -= DR(g6 * 0.25); v[WP] += DR(g6 * 0.25); v[BW] += DR(g6 * 0.25);
    }
    if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k - 1) > thr) {
      if (NV(i, j - 1, k) + NV(i, j - 1, k - 1) < thr && j != 1) {
        v[CP] -= DR(g7 * 0.5); v[BP] -= DR(g7 * 0.5); v[SP] += DR(g7 * 0.5); v[BS] += DR(g7 * 0.5);
      }
    } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k - 1) > thr) {
      if (NV(i, j + 1, k) + NV(i, j + 1, k - 1) < thr) {
        v[NP] -= DR(g7 * 0.5); v[BN] -= DR(g7 * 0.5); v[CP] += DR(g7 * 0.5); v[BP] += DR(g7 * 0.5);
      }
    } else {
      v[NP] -= DR(g7 * 0.25); v[BN] -= DR(g7 * 0.25); v[SP] += DR(g7 * 0.25); v[BS] += DR(g7 * 0.25);
    }
    if (ls.on && ls.bc4 == 5 && k == 1) v[CP] -= DR(g8 / 0.5);  // :1552-1554
    else { v[CP] -= DR(g8); v[BP] += DR(g8); }
  }
#undef RHO
#undef NV
#undef G
#undef DR
}
__device__ void assemble_row(const Grid &g, const double *nvert, const MetricPtrs &m, int i, int j, int k,
                             double v[NSLOT], const LevelSet &ls) {
  if (ls.on) assemble_row_t<true>(g, nvert, m, i, j, k, v, ls);
  else assemble_row_t<false>(g, nvert, m, i, j, k, v, ls);
}

// Assemble one level's operator into 19 box-layout planes.  filter: the
// reference's insertion test |v| > 1e-10 (poisson.c:1610-1614); scale: the
// aj row scaling of the poisson == -1 path (poisson.c:1563), used for the
// multigrid levels; split: store rows in the parity-split row layout of the
// multigrid levels (rowtype stays natural).  Slots whose column has no dof
// are zero (idx < 0).
__device__ __forceinline__ void assemble_cell(const Grid &g, const Box &b, const double *__restrict__ nvert,
                                              const MetricPtrs &m, int scale, int filter, int split, double *A,
                                              uint8_t *rowtype, const LevelSet &ls, int i, int j, int k) {
  const size_t n = b.n(), c = split ? b.at(split_pos(i, b.nx), j, k) : b.at(i, j, k);
  const size_t cr = b.at(i, j, k);
  const int I = i + 1, J = j + 1, K = k + 1;
  const size_t t = g.at(I, J, K);
  const bool dof = is_dof_cell(g, nvert, I, J, K);
  if (nvert[t] > 0.1 && dof) {  // identity row, poisson.c:1158-1160
    for (int s = 0; s < NSLOT; s++) A[s * n + c] = s == CP ? 1.0 : 0.0;
    rowtype[cr] = 2;
    return;
  }
  if (nvert[t] > kThr) {
    for (int s = 0; s < NSLOT; s++) A[s * n + c] = 0.0;
    rowtype[cr] = 0;
    return;
  }
  double v[NSLOT];
  assemble_row(g, nvert, m, I, J, K, v, ls);
  if (scale) {
    double a = m.aj[t];
    for (int s = 0; s < NSLOT; s++) v[s] *= a;
  }
  for (int s = 0; s < NSLOT; s++) {
    int di, dj, dk;
    slot_offset(s, di, dj, dk);
    bool keep = s == CP || (has_dof(g, nvert, I + di, J + dj, K + dk) && (!filter || fabs(v[s]) > 1.e-10));
    A[s * n + c] = keep ? v[s] : 0.0;
  }
  rowtype[cr] = 1;
}
__global__ void k_assemble(Grid g, Box b, const double *__restrict__ nvert, MetricPtrs m, int scale,
                           int filter, int split, double *A, uint8_t *rowtype, LevelSet ls) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= b.nx) return;
  assemble_cell(g, b, nvert, m, scale, filter, split, A, rowtype, ls, i, j, k);
}
// the same rows, only those listed (natural box indices rows[0 .. *nrows))
__global__ void k_assemble_rows(Grid g, Box b, const double *__restrict__ nvert, MetricPtrs m, int scale,
                                int filter, int split, double *A, uint8_t *rowtype, LevelSet ls,
                                const int *__restrict__ rows, const int *__restrict__ nrows) {
  const int nr = *nrows;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nr; w += gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, (size_t)rows[w], i, j, k);
    assemble_cell(g, b, nvert, m, scale, filter, split, A, rowtype, ls, i, j, k);
  }
}

// The fine level's two assemblies from one evaluation of each row: the
// unscaled operator with the reference's insertion filter in the natural
// layout (A0, the FGMRES operator: k_assemble scale 0, filter 1, split 0)
// and the aj-scaled one without the filter in the parity-split layout (A1,
// the finest multigrid level: scale 1, filter 0, split 1); the same values
// as the two k_assemble passes.
__device__ __forceinline__ void assemble_fine_cell(const Grid &g, const Box &b, const double *__restrict__ nvert,
                                                   const MetricPtrs &m, double *A0, uint8_t *rowtype0, double *A1,
                                                   uint8_t *rowtype1, const LevelSet &ls, int i, int j, int k) {
  const size_t n = b.n(), c0 = b.at(i, j, k), c1 = b.at(split_pos(i, b.nx), j, k);
  const int I = i + 1, J = j + 1, K = k + 1;
  const size_t t = g.at(I, J, K);
  const bool dof = is_dof_cell(g, nvert, I, J, K);
  if ((nvert[t] > 0.1 && dof) || nvert[t] > kThr) {  // identity row (poisson.c:1158-1160) or no row
    const bool ident = nvert[t] > 0.1 && dof;
    for (int s = 0; s < NSLOT; s++) {
      const double v = ident && s == CP ? 1.0 : 0.0;
      A0[s * n + c0] = v;
      A1[s * n + c1] = v;
    }
    rowtype0[c0] = rowtype1[c0] = ident ? 2 : 0;
    return;
  }
  double v[NSLOT];
  assemble_row(g, nvert, m, I, J, K, v, ls);
  const double a = m.aj[t];
  for (int s = 0; s < NSLOT; s++) {
    int di, dj, dk;
    slot_offset(s, di, dj, dk);
    const bool col = s == CP || has_dof(g, nvert, I + di, J + dj, K + dk);
    A0[s * n + c0] = col && (s == CP || fabs(v[s]) > 1.e-10) ? v[s] : 0.0;
    A1[s * n + c1] = col ? v[s] * a : 0.0;
  }
  rowtype0[c0] = rowtype1[c0] = 1;
}
__global__ void k_assemble_fine(Grid g, Box b, const double *__restrict__ nvert, MetricPtrs m, double *A0,
                                uint8_t *rowtype0, double *A1, uint8_t *rowtype1, LevelSet ls) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= b.nx) return;
  assemble_fine_cell(g, b, nvert, m, A0, rowtype0, A1, rowtype1, ls, i, j, k);
}
// the same rows, only those listed (natural box indices rows[0 .. *nrows))
__global__ void k_assemble_fine_rows(Grid g, Box b, const double *__restrict__ nvert, MetricPtrs m, double *A0,
                                     uint8_t *rowtype0, double *A1, uint8_t *rowtype1, LevelSet ls,
                                     const int *__restrict__ rows, const int *__restrict__ nrows) {
  const int nr = *nrows;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nr; w += gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, (size_t)rows[w], i, j, k);
    assemble_fine_cell(g, b, nvert, m, A0, rowtype0, A1, rowtype1, ls, i, j, k);
  }
}

// ---- incremental refill of the finest level on a new mask ----
// A row of the operator reads nvert within one point of its own (the
// one-sided differences and the neighbours' dof tests), where a periodic
// ghost neighbour's dof test reads its interior partner.  The rows to refill
// are those within two points of a point whose value changed, the periodic
// partners of ghost points included; every other row is the same as before.
__global__ void k_mask_changed(size_t N, const double *__restrict__ a, const double *__restrict__ b,
                               uint8_t *__restrict__ chg) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (size_t)gridDim.x * blockDim.x)
    chg[t] = a[t] != b[t] ? 1 : 0;
}
// dilation by R points along one axis (0: i, 1: j, 2: k) of the DA points,
// a ghost point of a periodic axis also standing for its interior partner
// (one thread per DA point of a (mx, my, mz) launch: no index divisions)
__global__ void k_dilate_axis(Grid g, int axis, int R, const uint8_t *__restrict__ src, uint8_t *__restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  const int x = axis == 0 ? i : axis == 1 ? j : k, m = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
  const bool per = axis == 0 ? g.px : axis == 1 ? g.py : g.pz;
  uint8_t f = 0;
  for (int d = -R; d <= R && !f; d++) {
    const int q = min(max(x + d, 0), m - 1);
    const int qa = per && q == 0 ? m - 2 : per && q == m - 1 ? 1 : q;
    for (int u = 0; u < 2; u++) {
      const int qq = u ? qa : q;
      const size_t s = axis == 0 ? g.at(qq, j, k) : axis == 1 ? g.at(i, qq, k) : g.at(i, j, qq);
      f |= src[s];
    }
  }
  dst[g.at(i, j, k)] = f;
}
// the interior rows at flagged points (natural box indices, in no order)
// and the j-columns that hold one
__global__ void k_list_rows(Grid g, Box b, const uint8_t *__restrict__ flag, int *rows, int *nrows,
                            uint8_t *colflag) {
  const size_t n = b.n();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    if (!flag[g.at(i + 1, j + 1, k + 1)]) continue;
    rows[atomicAdd(nrows, 1)] = (int)c;
    colflag[(size_t)k * b.nx + i] = 1;
  }
}

// Per-face dot products S = a.b of the projection and the face aj, so that
// Projection can form (dpdc*S)*aj exactly as poisson.c:2828-2950 does.
__global__ void k_projection_coef(Grid g, Box b, MetricPtrs m, double *pc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= b.nx) return;
  size_t c = b.at(i, j, k), n = b.n(), s = g.at(i + 1, j + 1, k + 1);
#define DOT(A, B) (m.A[s * 3] * m.B[s * 3] + m.A[s * 3 + 1] * m.B[s * 3 + 1] + m.A[s * 3 + 2] * m.B[s * 3 + 2])
  pc[0 * n + c] = DOT(icsi, icsi); pc[1 * n + c] = DOT(ieta, icsi); pc[2 * n + c] = DOT(izet, icsi);
  pc[3 * n + c] = m.iaj[s];
  pc[4 * n + c] = DOT(jcsi, jeta); pc[5 * n + c] = DOT(jeta, jeta); pc[6 * n + c] = DOT(jzet, jeta);
  pc[7 * n + c] = m.jaj[s];
  pc[8 * n + c] = DOT(kcsi, kzet); pc[9 * n + c] = DOT(keta, kzet); pc[10 * n + c] = DOT(kzet, kzet);
  pc[11 * n + c] = m.kaj[s];
#undef DOT
}

// Box-layout masks of a level: row-active flag from the assembly, blanking
// (nvert > 0.1) and the restriction weight max(0, 1 - nvert)
// (MyRestriction, poisson.c:433-441), in both precisions.
__global__ void k_level_masks(Grid g, Box b, const double *nvert, uint8_t *blank, double *w64, float *w32,
                              double *aj_box, const double *aj_da) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= b.n()) return;
  int i, j, k;
  box_ijk(b, c, i, j, k);
  double nv = nvert[g.at(i + 1, j + 1, k + 1)];
  double w = 1 - nv > 0. ? 1 - nv : 0.;
  if (blank) blank[c] = nv > 0.1 ? 1 : 0;  // (null outputs are skipped)
  if (w64) w64[c] = w;
  if (w32) w32[c] = (float)w;
  if (aj_box) aj_box[c] = aj_da[g.at(i + 1, j + 1, k + 1)];
}

// --------------------------------------------------------------------------
// Right-hand side: PoissonRHS2_hypre (Source/poisson_hypre.c:265-407) and
// Remove_Nullspace_Scale (:118-200)
// --------------------------------------------------------------------------
__global__ void k_rhs(Grid g, Box b, const double *__restrict__ nvert, const double *__restrict__ ucont,
                      const double *__restrict__ aj, double dt, double st, double coeff, double *rhs,
                      double *partial) {
  double sb = 0, sa = 0;
  const size_t n = b.n();
  const double f = -1.0 / dt * st * coeff;  // the reference's factor, formed once
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    size_t t = g.at(i, j, k);
    double val = 0.;
    if (nvert[t] < 0.1) {
#define U(a, bb, cc, q) ucont[g.at(a, bb, cc) * 3 + (q)]
      val -= U(i, j, k, 0);
      if (i == 1 && g.px) val += U(g.mx - 2, j, k, 0);
      else val += U(i - 1, j, k, 0);
      val -= U(i, j, k, 1);
      if (j == 1 && g.py) val += U(i, g.my - 2, k, 1);
      else val += U(i, j - 1, k, 1);
      val -= U(i, j, k, 2);
      if (k == 1 && g.pz) val += U(i, j, g.mz - 2, 2);
      else val += U(i, j, k - 1, 2);
#undef U
      val *= f;
      sb += val;
      sa += aj[t];
    }
    rhs[c] = val;
  }
  double tb = block_sum(sb);
  double ta = block_sum(sa);
  if (threadIdx.x == 0) { partial[blockIdx.x] = tb; partial[gridDim.x + blockIdx.x] = ta; }
}

// PoissonRHS2 (Source/poisson.c:1780-1906), the -poisson 0 / -1 variant:
// the same divergence on fluid cells, 0 on identity-row dofs, the aj row
// scaling for poisson == -1; block partials of the sum over every dof entry
// and of the fluid count for the unweighted mean removal.
__global__ void k_rhs2(Grid g, Box b, const double *__restrict__ nvert, const uint8_t *__restrict__ rowtype,
                       const double *__restrict__ ucont, const double *__restrict__ aj, double dt, double st,
                       double coeff, int poisson, double *rhs, double *partial) {
  double sb = 0, cnt = 0;
  const size_t n = b.n();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    size_t t = g.at(i, j, k);
    double val = 0.;
    if (nvert[t] < 0.1) {
#define U(a, bb, cc, q) ucont[g.at(a, bb, cc) * 3 + (q)]
      val -= U(i, j, k, 0);
      if (i == 1 && g.px) val += U(g.mx - 2, j, k, 0);
      else val += U(i - 1, j, k, 0);
      val -= U(i, j, k, 1);
      if (j == 1 && g.py) val += U(i, g.my - 2, k, 1);
      else val += U(i, j - 1, k, 1);
      val -= U(i, j, k, 2);
      if (k == 1 && g.pz) val += U(i, j, g.mz - 2, 2);
      else val += U(i, j, k - 1, 2);
#undef U
      val *= -1.0 / dt * st * coeff;
      if (poisson == -1) val *= aj[t];
      cnt += 1.;
    }
    if (rowtype[c]) sb += val;
    rhs[c] = val;
  }
  double tb = block_sum(sb);
  double tc = block_sum(cnt);
  if (threadIdx.x == 0) { partial[blockIdx.x] = tb; partial[gridDim.x + blockIdx.x] = tc; }
}
// the unweighted shift of PoissonRHS2 on fluid cells; for poisson == -1 the
// solver's (unscaled) right-hand side is B / aj on those rows
__global__ void k_rhs2_shift(Grid g, Box b, const double *__restrict__ nvert, const double *__restrict__ aj,
                             const double *sums, int poisson, double *rhs) {
  const double val = -sums[0] / (sums[1] > 0. ? sums[1] : 1.);
  const size_t n = b.n();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    size_t t = g.at(i, j, k);
    if (nvert[t] < 0.1) {
      rhs[c] += val;
      if (poisson == -1) rhs[c] = rhs[c] / aj[t];
    }
  }
}

// sums row blockIdx.x of `nb` block partials in a fixed tree order (launch
// one block per row)
__global__ void k_reduce_rows(const double *partial, int nb, int nrow, double *out) {
  const int r = blockIdx.x;
  if (r >= nrow) return;
  double s = 0;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) s += partial[(size_t)r * nb + q];
  s = block_sum(s);
  if (threadIdx.x == 0) out[r] = s;
}

// The reference's per-cell quotient (-sum aj) / sum_aj, correctly rounded
// (the bits of the division) in five FP64 operations instead of a division
// per cell: y = RN(1 / sum_aj) once, q = RN(a y), then two of Markstein's
// corrections q <- RN(q + RN(a - q sum_aj) y) with the exact FMA remainder
// (P. Markstein, IBM J. Res. Dev. 34 (1990) 111-119; a start within 1 ulp
// and y correctly rounded give the correctly rounded quotient, and the
// first correction brings RN(a y) within 1 ulp).  A sum_aj without a finite
// reciprocal takes the division.
__device__ __forceinline__ double div_rn(double a, double d, double y) {
  if (!isfinite(y)) return a / d;
  double q = a * y;
  double r = fma(-q, d, a);
  q = fma(r, y, q);
  r = fma(-q, d, a);
  return fma(r, y, q);
}

__global__ void k_rhs_nullspace(Grid g, Box b, const double *__restrict__ nvert, const double *__restrict__ aj,
                                const double *sums, double *rhs) {
  const double sum = sums[0], sum_aj = sums[1], y = 1.0 / sum_aj;
  const size_t n = b.n();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    size_t t = g.at(i, j, k);
    if (nvert[t] < 0.1) {
      const double val = div_rn(-sum * aj[t], sum_aj, y);
      rhs[c] += val;
    }
  }
}

// FullyBlocked (Source/poisson.c:1909-1993): per interior (i, j) column the
// first k (boundary layers included) with nvert > 0.1 into ksk[j mx + i]
// (-1 for none and on the boundary columns), and the count of interior
// columns without one (the multiple-null-space flag is that count == 0).
__global__ void k_fully_blocked(Grid g, const double *__restrict__ nvert, int *ksk, int *unblocked) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= g.mx) return;
  int first = -1;
  if (i >= 1 && i < g.mx - 1 && j >= 1 && j < g.my - 1) {
    for (int k = 0; k < g.mz; k++)
      if (nvert[g.at(i, j, k)] > 0.1) { first = k; break; }
    if (first < 0) atomicAdd(unblocked, 1);
  }
  ksk[(size_t)j * g.mx + i] = first;
}

// PoissonNullSpaceFunction_original (Source/poisson.c:757-943), first pass:
// block partials over the interior cells with nvert < 0.1 of the sum of x
// and the count, one pair of rows per region (multi: k below the column's
// first blocked k, then k at or above it; else the whole interior).
__global__ void k_nullspace_sums(Grid g, const double *__restrict__ nvert, const int *__restrict__ ksk, int multi,
                                 const double *__restrict__ x, double *partial) {
  double s[2] = {0., 0.}, c[2] = {0., 0.};
  const size_t n = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2);
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(q % (size_t)(g.mx - 2));
    const size_t r = q / (size_t)(g.mx - 2);
    const int j = 1 + (int)(r % (size_t)(g.my - 2)), k = 1 + (int)(r / (size_t)(g.my - 2));
    const size_t t = g.at(i, j, k);
    if (!(nvert[t] < 0.1)) continue;
    const int reg = multi && k >= ksk[(size_t)j * g.mx + i] ? 1 : 0;
    s[reg] += x[t];
    c[reg] += 1.;
  }
  for (int q = 0; q < 4; q++) {
    const double v = block_sum(q == 0 ? s[0] : q == 1 ? c[0] : q == 2 ? s[1] : c[1]);
    if (threadIdx.x == 0) partial[(size_t)q * gridDim.x + blockIdx.x] = v;
  }
}
// second pass: x += shift of its region on the interior cells with nvert <
// 0.1; the boundary layers and the cells with nvert > 0.1 become 0
__global__ void k_nullspace_apply(Grid g, const double *__restrict__ nvert, const int *__restrict__ ksk, int multi,
                                  double shift0, double shift1, double *x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  const size_t t = g.at(i, j, k);
  const bool bnd = i == 0 || i == g.mx - 1 || j == 0 || j == g.my - 1 || k == 0 || k == g.mz - 1;
  const double nv = nvert[t];
  if (!bnd && nv < 0.1) x[t] += multi && k >= ksk[(size_t)j * g.mx + i] ? shift1 : shift0;
  if (bnd || nv > 0.1) x[t] = 0.;
}

// Remove_Nullspace (Source/poisson_hypre.c:202-263) on a box vector: sum and
// count over nvert < 0.1
__global__ void k_mean_partial(Box b, const uint8_t *fluid, const double *x, double *partial) {
  double s = 0, cnt = 0;
  const size_t n = b.n();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    if (fluid[c]) { s += x[c]; cnt += 1.0; }
  double ts = block_sum(s);
  double tc = block_sum(cnt);
  if (threadIdx.x == 0) { partial[blockIdx.x] = ts; partial[gridDim.x + blockIdx.x] = tc; }
}
__global__ void k_fluid_mask(Grid g, Box b, const double *nvert, uint8_t *fluid) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= b.n()) return;
  int i, j, k;
  box_ijk(b, c, i, j, k);
  i++; j++; k++;
  fluid[c] = nvert[g.at(i, j, k)] < 0.1 ? 1 : 0;
}

// Remove_Nullspace's shift from the fluid sum and count (sums[0], sums[1]):
// sums[2] = -sum / count, as k_shift_fluid forms it
__global__ void k_mean_shift(double *sums) {
  if (threadIdx.x == 0 && blockIdx.x == 0) sums[2] = -sums[0] / sums[1];
}

// Convert_Phi2_Phi (Source/poisson.c:98-186): box phi -> DA phi, zero on
// non-dof cells and non-periodic ghosts, partner values on periodic ghosts.
// With `shift` (device, one value), Remove_Nullspace's x += shift on the
// fluid cells (nvert < 0.1) is applied on the way (x itself is left as is).
__global__ void k_box_to_da_phi(Grid g, Box b, const double *nvert, const double *x, double *phi,
                                const double *shift) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  int a, bb, c, fi, fj, fk;
  g.remap(i, j, k, a, bb, c, fi, fj, fk);
  double v = 0.;
  if (a >= 1 && a < g.mx - 1 && bb >= 1 && bb < g.my - 1 && c >= 1 && c < g.mz - 1) {
    const double nv = nvert[g.at(a, bb, c)];
    if (!((int)nv > kThr)) {
      v = x[b.at(a - 1, bb - 1, c - 1)];
      if (shift && nv < 0.1) v += shift[0];
    }
  }
  phi[g.at(i, j, k)] = v;
}
// DA -> box copy of the interior (warm start / inspection input)
__global__ void k_da_to_box(Grid g, Box b, const double *da, double *x) {
  size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= b.n()) return;
  int i, j, k;
  box_ijk(b, c, i, j, k);
  i++; j++; k++;
  x[c] = da[g.at(i, j, k)];
}
__global__ void k_box_to_da(Grid g, Box b, const double *x, double *da) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  double v = 0.;
  if (i >= 1 && i < g.mx - 1 && j >= 1 && j < g.my - 1 && k >= 1 && k < g.mz - 1)
    v = x[b.at(i - 1, j - 1, k - 1)];
  da[g.at(i, j, k)] = v;
}

// UpdatePressure (Source/poisson.c:3137-3297): interior update, then the
// periodic ghost copies of p and phi in a second launch.
__global__ void k_update_pressure(Grid g, const double *nvert, const double *phi, double *p) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i < 1 || i >= g.mx - 1 || j < 1 || j >= g.my - 1 || k < 1 || k >= g.mz - 1) return;
  size_t t = g.at(i, j, k);
  if (nvert[t] < 0.1) p[t] += phi[t];
  if (nvert[t] > 1.1) p[t] = 0;
}
__global__ void k_periodic_copy2(Grid g, double *p, double *phi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  int a, b, c, fi, fj, fk;
  if (!g.remap(i, j, k, a, b, c, fi, fj, fk)) return;
  size_t s = g.at(a, b, c), t = g.at(i, j, k);
  p[t] = p[s];
  if (phi) phi[t] = phi[s];
}

// Projection (Source/poisson.c:2700-3066), level set off.
// v * dt * st / coeff / r in the reference's left-to-right order.  A
// division by exactly 1 returns its dividend unchanged in IEEE arithmetic,
// so the divisions by coeff == 1 (time_coeff() without level set or RANS)
// and r == 1 (no density weighting) are skipped: the same bits, without the
// FP64 division sequence that dominates this kernel's FP64 pipe.
__device__ __forceinline__ double proj_scale(double v, double dt, double st, double coeff, double r) {
  v = v * dt * st;
  if (coeff != 1.0) v = v / coeff;
  if (r != 1.0) v = v / r;
  return v;
}

__global__ void k_projection(Grid g, Box b, const double *__restrict__ nvert, const double *__restrict__ phi,
                             const double *__restrict__ pc, double dt, double st, double coeff, double *ucont,
                             MetricPtrs m, LevelSet ls) {
  int ii = blockIdx.x * blockDim.x + threadIdx.x, jj = blockIdx.y, kk = blockIdx.z;
  if (ii >= b.nx) return;
  const int i = ii + 1, j = jj + 1, k = kk + 1;
  const int mx = g.mx, my = g.my, mz = g.mz;
  const bool ip = g.px, jp = g.py, kp = g.pz;
  const double thr = kThr;
  const size_t t = g.at(i, j, k), c = b.at(ii, jj, kk), n = b.n();
  double r1 = 1.0, r2 = 1.0, r3 = 1.0;
  if (ls.on) {  // poisson.c:2738-2749
    const double *rho = ls.rho;
    r1 = i == mx - 2 ? rho[t] : ls_mean(rho[t], rho[g.at(i + 1, j, k)]);
    r2 = j == my - 2 ? rho[t] : ls_mean(rho[t], rho[g.at(i, j + 1, k)]);
    r3 = k == mz - 2 ? rho[t] : ls_mean(rho[t], rho[g.at(i, j, k + 1)]);
  }
#define NV(a, bb, cc) nvert[g.at(a, bb, cc)]
#define PH(a, bb, cc) phi[g.at(a, bb, cc)]
  double dpdc, dpde, dpdz;
  if (i < mx - 2 || (ip && i == mx - 2)) {
    dpdc = PH(i + 1, j, k) - PH(i, j, k);
    if (i == mx - 2 && ip) dpdc = PH(1, j, k) - PH(i, j, k);
    dpde = 0.; dpdz = 0.;
    if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i + 1, j + 1, k) > thr) {
      if (NV(i, j - 1, k) + NV(i + 1, j - 1, k) < thr && (j != 1))
        dpde = (PH(i, j, k) + PH(i + 1, j, k) - PH(i, j - 1, k) - PH(i + 1, j - 1, k)) * 0.5;
    } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i + 1, j - 1, k) > thr) {
      if (NV(i, j + 1, k) + NV(i + 1, j + 1, k) < thr)
        dpde = (PH(i, j + 1, k) + PH(i + 1, j + 1, k) - PH(i, j, k) - PH(i + 1, j, k)) * 0.5;
    } else {
      dpde = (PH(i, j + 1, k) + PH(i + 1, j + 1, k) - PH(i, j - 1, k) - PH(i + 1, j - 1, k)) * 0.25;
    }
    if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i + 1, j, k + 1) > thr) {
      if (NV(i, j, k - 1) + NV(i + 1, j, k - 1) < thr && (k != 1))
        dpdz = (PH(i, j, k) + PH(i + 1, j, k) - PH(i, j, k - 1) - PH(i + 1, j, k - 1)) * 0.5;
    } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i + 1, j, k - 1) > thr) {
      if (NV(i, j, k + 1) + NV(i + 1, j, k + 1) < thr)
        dpdz = (PH(i, j, k + 1) + PH(i + 1, j, k + 1) - PH(i, j, k) - PH(i + 1, j, k)) * 0.5;
    } else {
      dpdz = (PH(i, j, k + 1) + PH(i + 1, j, k + 1) - PH(i, j, k - 1) - PH(i + 1, j, k - 1)) * 0.25;
    }
    if ((NV(i, j, k) + NV(i + 1, j, k)) < thr) {
      const double aj = pc[3 * n + c];
      ucont[t * 3 + 0] -= proj_scale(dpdc * pc[0 * n + c] * aj + dpde * pc[1 * n + c] * aj + dpdz * pc[2 * n + c] * aj, dt, st, coeff, r1);
    }
  }
  if (j < my - 2 || (jp && j == my - 2) || (ls.on && ls.bc3 == 4 && j == my - 2)) {
    dpdc = 0.; dpdz = 0.;
    if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j + 1, k) > thr) {
      if (NV(i - 1, j, k) + NV(i - 1, j + 1, k) < thr && (i != 1))
        dpdc = (PH(i, j, k) + PH(i, j + 1, k) - PH(i - 1, j, k) - PH(i - 1, j + 1, k)) * 0.5;
    } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j + 1, k) > thr) {
      if (NV(i + 1, j, k) + NV(i + 1, j + 1, k) < thr)
        dpdc = (PH(i + 1, j, k) + PH(i + 1, j + 1, k) - PH(i, j, k) - PH(i, j + 1, k)) * 0.5;
    } else {
      dpdc = (PH(i + 1, j, k) + PH(i + 1, j + 1, k) - PH(i - 1, j, k) - PH(i - 1, j + 1, k)) * 0.25;
    }
    if (ls.on && ls.bc3 == 4 && j == my - 2) dpde = PH(i, j, k) - PH(i, j - 1, k);
    else if (j == my - 2 && jp) dpde = PH(i, 1, k) - PH(i, j, k);
    else dpde = PH(i, j + 1, k) - PH(i, j, k);
    if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j + 1, k + 1) > thr) {
      if (NV(i, j, k - 1) + NV(i, j + 1, k - 1) < thr && (k != 1))
        dpdz = (PH(i, j, k) + PH(i, j + 1, k) - PH(i, j, k - 1) - PH(i, j + 1, k - 1)) * 0.5;
    } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j + 1, k - 1) > thr) {
      if (NV(i, j, k + 1) + NV(i, j + 1, k + 1) < thr)
        dpdz = (PH(i, j, k + 1) + PH(i, j + 1, k + 1) - PH(i, j, k) - PH(i, j + 1, k)) * 0.5;
    } else {
      dpdz = (PH(i, j, k + 1) + PH(i, j + 1, k + 1) - PH(i, j, k - 1) - PH(i, j + 1, k - 1)) * 0.25;
    }
    if ((NV(i, j, k) + NV(i, j + 1, k)) < thr || (int)(NV(i, j, k) + NV(i, j + 1, k)) == 5) {
      const double aj = pc[7 * n + c];
      ucont[t * 3 + 1] -= proj_scale(dpdc * pc[4 * n + c] * aj + dpde * pc[5 * n + c] * aj + dpdz * pc[6 * n + c] * aj, dt, st, coeff, r2);
    }
  }
  if (k < mz - 2 || (kp && k == mz - 2) || (ls.on && ls.bc5 == 4 && k == mz - 2)) {
    dpdc = 0.; dpde = 0.;
    if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k + 1) > thr) {
      if (NV(i - 1, j, k) + NV(i - 1, j, k + 1) < thr && (i != 1))
        dpdc = (PH(i, j, k) + PH(i, j, k + 1) - PH(i - 1, j, k) - PH(i - 1, j, k + 1)) * 0.5;
    } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k + 1) > thr) {
      if (NV(i + 1, j, k) + NV(i + 1, j, k + 1) < thr)
        dpdc = (PH(i + 1, j, k) + PH(i + 1, j, k + 1) - PH(i, j, k) - PH(i, j, k + 1)) * 0.5;
    } else {
      dpdc = (PH(i + 1, j, k) + PH(i + 1, j, k + 1) - PH(i - 1, j, k) - PH(i - 1, j, k + 1)) * 0.25;
    }
    if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k + 1) > thr) {
      if (NV(i, j - 1, k) + NV(i, j - 1, k + 1) < thr && (j != 1))
        dpde = (PH(i, j, k) + PH(i, j, k + 1) - PH(i, j - 1, k) - PH(i, j - 1, k + 1)) * 0.5;
    } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k + 1) > thr) {
      if (NV(i, j + 1, k) + NV(i, j + 1, k + 1) < thr)
        dpde = (PH(i, j + 1, k) + PH(i, j + 1, k + 1) - PH(i, j, k) - PH(i, j, k + 1)) * 0.5;
    } else {
      dpde = (PH(i, j + 1, k) + PH(i, j + 1, k + 1) - PH(i, j - 1, k) - PH(i, j - 1, k + 1)) * 0.25;
    }
    if (k == mz - 2 && kp) dpdz = PH(i, j, 1) - PH(i, j, k);
    else if (k == mz - 2 && ls.on && ls.bc5 == 4) dpdz = PH(i, j, k) - PH(i, j, k - 1);
    else dpdz = PH(i, j, k + 1) - PH(i, j, k);
    if ((NV(i, j, k) + NV(i, j, k + 1)) < thr) {
      const double aj = pc[11 * n + c];
      ucont[t * 3 + 2] -= proj_scale(dpdc * pc[8 * n + c] * aj + dpde * pc[9 * n + c] * aj + dpdz * pc[10 * n + c] * aj, dt, st, coeff, r3);
      if (ls.on && k == 1 && ls.bc4 == 5000 && ls.level[t] < 0) {  // poisson.c:2951-2956
        const size_t t0 = g.at(i, j, 0);
        const double *kz = &m.kzet[t0 * 3];
        const double r0 = ls.rho[t];
        ucont[t0 * 3 + 2] -= proj_scale(dpdz * (kz[0] * kz[0] + kz[1] * kz[1] + kz[2] * kz[2]) * m.kaj[t0], dt, st, coeff, r0);
      }
    }
  }
#undef NV
#undef PH
}
// periodic face copy of Ucont (poisson.c:2996-3036)
__global__ void k_periodic_faces(Grid g, double *ucont) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  int a, b, c, fi, fj, fk;
  if (!g.remap(i, j, k, a, b, c, fi, fj, fk)) return;
  size_t s = g.at(a, b, c), t = g.at(i, j, k);
  if (fi) ucont[t * 3 + 0] = ucont[s * 3 + 0];
  if (fj) ucont[t * 3 + 1] = ucont[s * 3 + 1];
  if (fk) ucont[t * 3 + 2] = ucont[s * 3 + 2];
}

// Divergence (Source/main.c:936-1074): block maxima of |div(Ucont) aj|.
__global__ void k_divergence(Grid g, Box b, const double *__restrict__ nvert, const double *__restrict__ ucont,
                             const double *__restrict__ aj, double *partial) {
  double best = 0.;
  const size_t n = b.n();
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_ijk(b, c, i, j, k);
    i++; j++; k++;
    const double v = divergence_cell(g, nvert, ucont, aj, i, j, k);
    best = v > best ? v : best;
  }
  double m = block_max(best);
  if (threadIdx.x == 0) partial[blockIdx.x] = m;
}
__global__ void k_reduce_max(const double *partial, int nb, double *out) {
  double m = 0.;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) m = partial[q] > m ? partial[q] : m;
  m = block_max(m);
  if (threadIdx.x == 0) *out = m;
}

// --------------------------------------------------------------------------
// Multigrid hierarchy set-up and transfer operators
// --------------------------------------------------------------------------
// coarse nodes are every other fine node (Source/init.c:402-455 with
// GridRestriction, poisson.c:337-363)
__global__ void k_coarse_nodes(Grid gf, Grid gc, int cx, int cy, int cz, const double *cf, double *cc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= gc.mx) return;
  size_t t = gc.at(i, j, k);
  if (i > gc.mx - 2 || j > gc.my - 2 || k > gc.mz - 2) {
    cc[t * 3] = cc[t * 3 + 1] = cc[t * 3 + 2] = 0.;
    return;
  }
  size_t s = gf.at(cx ? 2 * i : i, cy ? 2 * j : j, cz ? 2 * k : k);
  cc[t * 3] = cf[s * 3]; cc[t * 3 + 1] = cf[s * 3 + 1]; cc[t * 3 + 2] = cf[s * 3 + 2];
}

// MyNvertRestriction (poisson.c:1995-2083), first pass: a coarse cell is
// blanked when the product of its children's nvert exceeds 0.1.
__global__ void k_nvert_restrict(Grid gh, Grid gc, int cx, int cy, int cz, const double *nh, double *nc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= gc.mx) return;
  size_t t = gc.at(i, j, k);
  double v = 0.;
  if (i >= 1 && i < gc.mx - 1 && j >= 1 && j < gc.my - 1 && k >= 1 && k < gc.mz - 1) {
    const int ia = cx, ja = cy, ka = cz;
    int ih = cx ? 2 * i : i, jh = cy ? 2 * j : j, kh = cz ? 2 * k : k;
#define NH(a, b, c) nh[gh.at(a, b, c)]
    if (NH(ih, jh, kh) * NH(ih - ia, jh, kh) * NH(ih, jh - ja, kh) * NH(ih, jh, kh - ka) * NH(ih - ia, jh - ja, kh) *
            NH(ih - ia, jh, kh - ka) * NH(ih, jh - ja, kh - ka) * NH(ih - ia, jh - ja, kh - ka) >
        0.1)
      v = 1.;
#undef NH
  }
  nc[t] = v;
}
// second pass, isolated-cell fill.  The reference updates in place in k-j-i
// order; a cell is filled only when all six face neighbours are already
// blanked, so no fluid neighbour can change its decision and a parallel
// pass over a snapshot gives the same result.
__global__ void k_nvert_fill(Grid gc, const double *src, double *dst) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= gc.mx) return;
  size_t t = gc.at(i, j, k);
  double v = src[t];
  if (i >= 1 && i < gc.mx - 1 && j >= 1 && j < gc.my - 1 && k >= 1 && k < gc.mz - 1 && v < 0.1) {
    if (src[gc.at(i + 1, j, k)] + src[gc.at(i - 1, j, k)] > 1.1 && src[gc.at(i, j + 1, k)] + src[gc.at(i, j - 1, k)] > 1.1 &&
        src[gc.at(i, j, k + 1)] + src[gc.at(i, j, k - 1)] > 1.1)
      v = 1.;
  }
  dst[t] = v;
}

// MyRestriction (poisson.c:365-472) on box vectors: the eight weighted
// children in the reference's order, times 1/8; zero on blanked coarse cells.
template <typename T>
__device__ __forceinline__ void restrict_body(Box bf, Box bc, int cx, int cy, int cz, const T *__restrict__ rf,
                                              const T *__restrict__ wf, const uint8_t *__restrict__ blank_c,
                                              T *bc_out) {
  pdl_trigger();
  pdl_wait();
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= bc.nx) return;
  size_t cc = bc.at(i, j, k);
  if (blank_c[cc]) { bc_out[cc] = (T)0; return; }
  int i1 = cx ? 2 * i + 1 : i, j1 = cy ? 2 * j + 1 : j, k1 = cz ? 2 * k + 1 : k;
  int i0 = i1 - cx, j0 = j1 - cy, k0 = k1 - cz;
#define X(a, b, c) (rf[bf.at(a, b, c)] * wf[bf.at(a, b, c)])
  T s = X(i1, j1, k1) + X(i0, j1, k1) + X(i1, j0, k1) + X(i1, j1, k0) + X(i0, j0, k1) + X(i1, j0, k0) +
        X(i0, j1, k0) + X(i0, j0, k0);
#undef X
  bc_out[cc] = (T)0.125 * s;
}

// MyInterpolation (poisson.c:527-670, GridInterpolation macro :474-507),
// added onto the fine vector (the V-cycle correction).  add = 0 writes.
// FSPLIT: the fine vector is in the parity-split row layout (the finest
// FP32 level under the checkerboard smoother); blank flags stay natural.
template <typename T, bool FSPLIT = false>
__device__ __forceinline__ void prolong_body(Box bf, Box bc, int cx, int cy, int cz, const T *__restrict__ xc,
                                             const uint8_t *__restrict__ blank_c, const uint8_t *__restrict__ blank_f,
                                             T *xf, int add) {
  pdl_trigger();
  pdl_wait();
  // a thread takes rows j = blockIdx.y and blockIdx.y + gridDim.y of column
  // i (when inside the box): all the loads of both cells first, then both
  // results
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.z;
  if (i >= bf.nx) return;
  const int mx = bf.nx + 2, my = bf.ny + 2, mz = bf.nz + 2;
  const int I = i + 1, K = k + 1;
  int ic, kc, ia, ka;
  if (!cx) { ic = I; ia = 0; } else { ic = (I + 1) / 2; ia = (I - 2 * ic) == 0 ? 1 : -1; if (I == 1 || I == mx - 2) ia = 0; }
  if (!cz) { kc = K; ka = 0; } else { kc = (K + 1) / 2; ka = (K - 2 * kc) == 0 ? 1 : -1; if (K == 1 || K == mz - 2) ka = 0; }
  size_t c[2], cf[2];
  bool valid[2];
  int ja[2];
  uint8_t bf0[2], ni[2], nj[2], nk[2];
  T X[2][2][2][2], xold[2];  // [row][i side][j side][k side]
#pragma unroll
  for (int r = 0; r < 2; r++) {
    const int j = blockIdx.y + r * gridDim.y;
    valid[r] = j < bf.ny;
    if (!valid[r]) continue;
    c[r] = bf.at(i, j, k);
    cf[r] = FSPLIT ? c[r] - i + split_pos(i, bf.nx) : c[r];
    const int J = j + 1;
    int jc;
    if (!cy) { jc = J; ja[r] = 0; } else { jc = (J + 1) / 2; ja[r] = (J - 2 * jc) == 0 ? 1 : -1; if (J == 1 || J == my - 2) ja[r] = 0; }
    // every load in one round trip: the fine blank flag, the three coarse
    // neighbours' blank flags and the 8 coarse values at the unblanked
    // offsets (all inside the coarse box); a blanked neighbour then
    // selects the centre-side value, exactly the stencil the offsets
    // would give; 32-bit offsets into the coarse box (fewer than 2^31 cells)
    const int base = ((kc - 1) * bc.ny + (jc - 1)) * bc.nx + (ic - 1);
    const int oi = ia, oj = ja[r] * bc.nx, ok = ka * bc.nx * bc.ny;
    bf0[r] = blank_f[c[r]];
    nk[r] = blank_c[base + ok];
    nj[r] = blank_c[base + oj];
    ni[r] = blank_c[base + oi];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int a = q & 1, bb = (q >> 1) & 1, cc = q >> 2;
      X[r][a][bb][cc] = xc[base + a * oi + bb * oj + cc * ok];
    }
    xold[r] = add ? xf[cf[r]] : (T)0;
  }
#pragma unroll
  for (int r = 0; r < 2; r++) {
    if (!valid[r]) continue;
    if (bf0[r]) { if (!add) xf[cf[r]] = (T)0; continue; }
    // the reference zeroes an offset whose coarse neighbour is blank; an
    // offset already 0 reads the centre (its test reads the centre cell,
    // which an unblanked fine cell's parent is not).  Collapse the zeroed
    // offsets one axis after the other (constant indices keep X in
    // registers).
    const bool zk = ka != 0 && nk[r], zj = ja[r] != 0 && nj[r], zi = ia != 0 && ni[r];
#pragma unroll
    for (int q = 0; q < 4; q++) X[r][1][q & 1][q >> 1] = zi ? X[r][0][q & 1][q >> 1] : X[r][1][q & 1][q >> 1];
#pragma unroll
    for (int q = 0; q < 4; q++) X[r][q & 1][1][q >> 1] = zj ? X[r][q & 1][0][q >> 1] : X[r][q & 1][1][q >> 1];
#pragma unroll
    for (int q = 0; q < 4; q++) X[r][q & 1][q >> 1][1] = zk ? X[r][q & 1][q >> 1][0] : X[r][q & 1][q >> 1][1];
    T v = (X[r][0][0][0] * (T)9 + X[r][0][1][0] * (T)3 + X[r][1][0][0] * (T)3 + X[r][1][1][0]) * (T)3. / (T)64. +
          (X[r][0][0][1] * (T)9 + X[r][0][1][1] * (T)3 + X[r][1][0][1] * (T)3 + X[r][1][1][1]) / (T)64.;
    if (add) xf[cf[r]] = xold[r] + v;
    else xf[cf[r]] = v;
  }
}

__global__ void k_restrict_f32(Box bf, Box bc, int cx, int cy, int cz, const float *rf, const float *wf,
                               const uint8_t *blank_c, float *out) {
  restrict_body<float>(bf, bc, cx, cy, cz, rf, wf, blank_c, out);
}
__global__ void k_restrict_f64(Box bf, Box bc, int cx, int cy, int cz, const double *rf, const double *wf,
                               const uint8_t *blank_c, double *out) {
  restrict_body<double>(bf, bc, cx, cy, cz, rf, wf, blank_c, out);
}
__global__ void k_prolong_f32(Box bf, Box bc, int cx, int cy, int cz, const float *xc, const uint8_t *blank_c,
                              const uint8_t *blank_f, float *xf, int add) {
  prolong_body<float>(bf, bc, cx, cy, cz, xc, blank_c, blank_f, xf, add);
}
__global__ void k_prolong_f32_split(Box bf, Box bc, int cx, int cy, int cz, const float *xc, const uint8_t *blank_c,
                                    const uint8_t *blank_f, float *xf, int add) {
  prolong_body<float, true>(bf, bc, cx, cy, cz, xc, blank_c, blank_f, xf, add);
}
__global__ void k_prolong_f64(Box bf, Box bc, int cx, int cy, int cz, const double *xc, const uint8_t *blank_c,
                              const uint8_t *blank_f, double *xf, int add) {
  prolong_body<double>(bf, bc, cx, cy, cz, xc, blank_c, blank_f, xf, add);
}

}  // namespace vfs

namespace vfs {

// ---- VolumeFlux (Source/poisson.c:3563-3903, immersed == 1) ----
// Faces between a fluid cell and an IB cell (0.1 < nvert < 1.1), visited
// once each from the cell below them in i, j or k: s = 0 the cell is fluid
// and the face's neighbour IB, s = 1 the reverse.
struct VfluxFace {
  double *u;
  double a;
  int s;
};
__device__ inline int vflux_faces(Grid g, const double *nvert, MetricPtrs m, double *ucont, int i, int j, int k,
                                  VfluxFace f[6]) {
  const size_t t = g.at(i, j, k);
  const size_t nb[3] = {g.at(i + 1, j, k), g.at(i, j + 1, k), g.at(i, j, k + 1)};
  const bool in[3] = {i < g.mx - 2, j < g.my - 2, k < g.mz - 2};
  const double *met[3] = {m.csi, m.eta, m.zet};
  int nf = 0;
  for (int s = 0; s < 2; s++) {
    if (s == 0 && !(nvert[t] < 0.1)) continue;
    if (s == 1 && !(nvert[t] > 0.1 && nvert[t] < 1.1)) continue;
    for (int q = 0; q < 3; q++) {
      const double nn = nvert[nb[q]];
      const bool face = s == 0 ? (nn > 0.1 && nn < 1.1) : (nn < 0.1);
      if (!face || !in[q]) continue;
      const double *mm = &met[q][t * 3];
      f[nf].u = &ucont[t * 3 + q];
      f[nf].a = sqrt(mm[0] * mm[0] + mm[1] * mm[1] + mm[2] * mm[2]);
      f[nf].s = s;
      nf++;
    }
  }
  return nf;
}

// pass 0: zero |U| <= 1e-8 and sum flux, |U| (or |U| / area for flg 3)
// and area; pass 2: sum flux and area after the correction
__global__ void k_vflux_sum(Grid g, const double *__restrict__ nvert, MetricPtrs m, double *ucont, int flg, int pass,
                            double *partial) {
  double sf = 0, sab = 0, sa = 0;
  const size_t n = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = c % (g.mx - 2) + 1, j = (c / (g.mx - 2)) % (g.my - 2) + 1, k = c / ((size_t)(g.mx - 2) * (g.my - 2)) + 1;
    VfluxFace f[6];
    const int nf = vflux_faces(g, nvert, m, ucont, i, j, k, f);
    for (int q = 0; q < nf; q++) {
      const double u = *f[q].u;
      if (pass == 0) {
        if (fabs(u) > 1.e-8) {
          sf += f[q].s == 0 ? u : -u;
          sab += flg == 3 ? fabs(u) / f[q].a : fabs(u);
          sa += f[q].a;
        } else {
          *f[q].u = 0.;
        }
      } else {
        sf += f[q].s == 0 ? u : -u;
        sa += f[q].a;
      }
    }
  }
  const double t0 = block_sum(sf), t1 = block_sum(sab), t2 = block_sum(sa);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = t0;
    partial[gridDim.x + blockIdx.x] = t1;
    partial[2 * gridDim.x + blockIdx.x] = t2;
  }
}

__global__ void k_vflux_apply(Grid g, const double *__restrict__ nvert, MetricPtrs m, double *ucont, int flg,
                              double corr) {
  const size_t n = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = c % (g.mx - 2) + 1, j = (c / (g.mx - 2)) % (g.my - 2) + 1, k = c / ((size_t)(g.mx - 2) * (g.my - 2)) + 1;
    VfluxFace f[6];
    const int nf = vflux_faces(g, nvert, m, ucont, i, j, k, f);
    for (int q = 0; q < nf; q++) {
      const double u = *f[q].u;
      if (!(fabs(u) > 1.e-8)) continue;
      double dlt;
      if (flg == 3) dlt = corr * fabs(u) / f[q].a;
      else if (flg == 2) dlt = corr * fabs(u);
      else dlt = f[q].a * corr;
      *f[q].u = f[q].s == 0 ? u - dlt : u + dlt;
    }
  }
}

// ---- VolumeFlux, the overload for immersed != 1, 2 (Source/poisson.c:3299-3493) ----
// Faces between a fluid cell (nvert < 0.1) and a blanked one (nvert > 0.1),
// visited from the cell below them; the area term is the cell metric's norm.
__device__ inline int vflux0_faces(Grid g, const double *nvert, MetricPtrs m, double *ucont, int i, int j, int k,
                                   VfluxFace f[6]) {
  const size_t t = g.at(i, j, k);
  const size_t nb[3] = {g.at(i + 1, j, k), g.at(i, j + 1, k), g.at(i, j, k + 1)};
  const double *met[3] = {m.csi, m.eta, m.zet};
  int nf = 0;
  for (int s = 0; s < 2; s++) {
    if (s == 0 && !(nvert[t] < 0.1)) continue;
    if (s == 1 && !(nvert[t] > 0.1)) continue;
    for (int q = 0; q < 3; q++) {
      const double nn = nvert[nb[q]];
      if (s == 0 ? !(nn > 0.1) : !(nn < 0.1)) continue;
      const double *mm = &met[q][t * 3];
      f[nf].u = &ucont[t * 3 + q];
      f[nf].a = sqrt(mm[0] * mm[0] + mm[1] * mm[1] + mm[2] * mm[2]);
      f[nf].s = s;
      nf++;
    }
  }
  return nf;
}

// block partials of the flux (+U on the fluid side, -U on the blanked side)
// and of the area
__global__ void k_vflux0_sum(Grid g, const double *__restrict__ nvert, MetricPtrs m, double *ucont,
                             double *partial) {
  double sf = 0, sa = 0;
  const size_t n = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = c % (g.mx - 2) + 1, j = (c / (g.mx - 2)) % (g.my - 2) + 1, k = c / ((size_t)(g.mx - 2) * (g.my - 2)) + 1;
    VfluxFace f[6];
    const int nf = vflux0_faces(g, nvert, m, ucont, i, j, k, f);
    for (int q = 0; q < nf; q++) {
      const double u = *f[q].u;
      sf += f[q].s == 0 ? u : -u;
      sa += f[q].a;
    }
  }
  const double t0 = block_sum(sf), t1 = block_sum(sa);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = t0;
    partial[gridDim.x + blockIdx.x] = t1;
  }
}

// the correction: off the fluid side, onto the blanked side; then the face
// is zeroed when `zero` (immersed 0 or 3)
__global__ void k_vflux0_apply(Grid g, const double *__restrict__ nvert, MetricPtrs m, double *ucont, double corr,
                               int zero) {
  const size_t n = (size_t)(g.mx - 2) * (g.my - 2) * (g.mz - 2);
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = c % (g.mx - 2) + 1, j = (c / (g.mx - 2)) % (g.my - 2) + 1, k = c / ((size_t)(g.mx - 2) * (g.my - 2)) + 1;
    VfluxFace f[6];
    const int nf = vflux0_faces(g, nvert, m, ucont, i, j, k, f);
    for (int q = 0; q < nf; q++) {
      const double u = *f[q].u;
      const double dlt = f[q].a * corr;
      *f[q].u = zero ? 0. : (f[q].s == 0 ? u - dlt : u + dlt);
    }
  }
}

// ---- Contra2Cart (Source/rhs.c:35-749), its change of basis ----
// periodic ghosts of a Cmpnts DA array take their partners' values
__global__ void k_periodic_cmpnts(Grid g, const double *src, double *dst) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= g.mx) return;
  int a, b, c, fi, fj, fk;
  const size_t t = g.at(i, j, k);
  const size_t s = g.remap(i, j, k, a, b, c, fi, fj, fk) ? g.at(a, b, c) : t;
  for (int q = 0; q < 3; q++) dst[t * 3 + q] = src[s * 3 + q];
}
__global__ void k_contra2cart(Grid g, const double *__restrict__ nvert, MetricPtrs m, const double *__restrict__ lu,
                              double *ucat) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1, j = blockIdx.y + 1, k = blockIdx.z + 1;
  if (i >= g.mx - 1) return;
  const size_t t = g.at(i, j, k);
  if (!(nvert[t] < 0.1)) return;
  const double *c0 = &m.csi[t * 3], *e0 = &m.eta[t * 3], *z0 = &m.zet[t * 3];
  const double m00 = c0[0], m01 = c0[1], m02 = c0[2], m10 = e0[0], m11 = e0[1], m12 = e0[2], m20 = z0[0],
               m21 = z0[1], m22 = z0[2];
  const double q0 = 0.5 * (lu[g.at(i - 1, j, k) * 3 + 0] + lu[t * 3 + 0]);
  const double q1 = 0.5 * (lu[g.at(i, j - 1, k) * 3 + 1] + lu[t * 3 + 1]);
  const double q2 = 0.5 * (lu[g.at(i, j, k - 1) * 3 + 2] + lu[t * 3 + 2]);
  const double det = m00 * (m11 * m22 - m12 * m21) - m01 * (m10 * m22 - m12 * m20) + m02 * (m10 * m21 - m11 * m20);
  const double det0 = q0 * (m11 * m22 - m12 * m21) - q1 * (m01 * m22 - m02 * m21) + q2 * (m01 * m12 - m02 * m11);
  const double det1 = -q0 * (m10 * m22 - m12 * m20) + q1 * (m00 * m22 - m02 * m20) - q2 * (m00 * m12 - m02 * m10);
  const double det2 = q0 * (m10 * m21 - m11 * m20) - q1 * (m00 * m21 - m01 * m20) + q2 * (m00 * m11 - m01 * m10);
  ucat[t * 3 + 0] = det0 / det;
  ucat[t * 3 + 1] = det1 / det;
  ucat[t * 3 + 2] = det2 / det;
}
__global__ void k_zero_solid(Grid g, const double *nvert, double *ucat) {
  const size_t n = g.n();
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    if ((int)(nvert[t] + 0.1) == 3) ucat[t * 3] = ucat[t * 3 + 1] = ucat[t * 3 + 2] = 0.;
}

}  // namespace vfs

namespace vfs {

// A cell field (density, level set) on a coarse level: the average of the
// fine cells it covers (the children of MyNvertRestriction's mapping); a
// boundary-layer point takes the fine boundary-layer values it faces.
__global__ void k_cellfield_restrict(Grid gh, Grid gc, int cx, int cy, int cz, const double *fh, double *fc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
  if (i >= gc.mx) return;
  int ia[2], ja[2], ka[2];
  auto kids = [](int c, int m, int mh, int coarsened, int o[2]) {
    if (c == 0) { o[0] = o[1] = 0; return; }
    if (c == m - 1) { o[0] = o[1] = mh - 1; return; }
    const int h = coarsened ? 2 * c : c;
    o[0] = h;
    o[1] = h - coarsened;
  };
  kids(i, gc.mx, gh.mx, cx, ia);
  kids(j, gc.my, gh.my, cy, ja);
  kids(k, gc.mz, gh.mz, cz, ka);
  double s = 0.;
  for (int q = 0; q < 8; q++) s += fh[gh.at(ia[q & 1], ja[(q >> 1) & 1], ka[q >> 2])];
  fc[gc.at(i, j, k)] = 0.125 * s;
}

}  // namespace vfs
