/*
 * vfs_oracle.c -- CPU restatement of VFS-Wind's pressure-Poisson hot path.
 *
 * TEST INFRASTRUCTURE ONLY (checker + timed CPU baseline).  Parity unpinned:
 * the reference cannot be built here (it needs PETSc 3.1 / HYPRE / MPI) and
 * ships no golden vectors for this path.  Every function cites the reference
 * file:line it restates.  Compile with -ffp-contract=off so that every
 * floating-point expression is evaluated in the reference's source order on
 * both x86-64 and aarch64 hosts.
 */
#include "vfs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IX(d, i, j, k) ((size_t)(((size_t)(k) * (size_t)(d)->my + (size_t)(j)) * (size_t)(d)->mx + (size_t)(i)))

static const double POISSON_THRESHOLD = 0.1; /* Source/main.c:124 */

static inline int per_i(const or_dims *d) { return d->i_periodic || d->ii_periodic; }
static inline int per_j(const or_dims *d) { return d->j_periodic || d->jj_periodic; }
static inline int per_k(const or_dims *d) { return d->k_periodic || d->kk_periodic; }

/* Ghost remap repeated throughout the reference (e.g. Source/poisson.c:1143-1161,
 * :154-174, :3258-3276; Source/metrics.c:365-383).  Index 0 / m-1 of a periodic
 * direction take the value of cell m-2 / 1.  The ii/jj/kk variants address the
 * periodic DA's ghost index -2 / m+1, which hold exactly those cells. */
static inline int remap(const or_dims *d, int i, int j, int k, int *a, int *b, int *c,
                        int *fi, int *fj, int *fk)
{
  int ia = i, jb = j, kc = k, f1 = 0, f2 = 0, f3 = 0;
  if (per_i(d)) {
    if (i == 0) ia = d->mx - 2, f1 = 1;
    else if (i == d->mx - 1) ia = 1, f1 = 1;
  }
  if (per_j(d)) {
    if (j == 0) jb = d->my - 2, f2 = 1;
    else if (j == d->my - 1) jb = 1, f2 = 1;
  }
  if (per_k(d)) {
    if (k == 0) kc = d->mz - 2, f3 = 1;
    else if (k == d->mz - 1) kc = 1, f3 = 1;
  }
  *a = ia; *b = jb; *c = kc;
  if (fi) *fi = f1;
  if (fj) *fj = f2;
  if (fk) *fk = f3;
  return f1 | f2 | f3;
}

/* ------------------------------------------------------------------------ */
/* FormMetrics (Source/metrics.c:12-1355; metrics.c:10 defines NEWMETRIC).   */
/* ------------------------------------------------------------------------ */
/* Cell metrics csi/eta/zet and aj = 1/J of every interior cell come from the
 * 8-node differences (metrics.c:194-256); the boundary layer mirrors its
 * neighbour, i planes first, then j, then k (metrics.c:262-342); periodic
 * directions take their partner cells (metrics.c:360-397).  The face metrics
 * are NEWMETRIC averages of the two adjacent cells: arithmetic for the
 * vectors (AxByC, Source/momentum.c:40-45) and harmonic for aj
 * (metrics.c:588-592, :696-700, :804-808), over i faces i = 0..mx-2 of the
 * interior j, k; j faces j = 0..my-2; k faces k = 0..mz-2.  Faces outside
 * those ranges stay 0, and the periodic boundary layers finally take their
 * partners' values for every array (metrics.c:1227-1262). */
static void avg_face(const double *a, const double *b, double *o)
{
  for (int c = 0; c < 3; c++) o[c] = 0.5 * a[c] + 0.5 * b[c];
}

static void periodic_copy16(const or_dims *d, or_metrics *m, int faces)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  double *v3[12] = {m->csi, m->eta, m->zet, m->icsi, m->ieta, m->izet,
                    m->jcsi, m->jeta, m->jzet, m->kcsi, m->keta, m->kzet};
  double *v1[4] = {m->aj, m->iaj, m->jaj, m->kaj};
  const int n3 = faces ? 12 : 3, n1 = faces ? 4 : 1;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a, b, c;
        if (!remap(d, i, j, k, &a, &b, &c, 0, 0, 0)) continue;
        size_t s = IX(d, a, b, c), t = IX(d, i, j, k);
        for (int q = 0; q < n3; q++)
          for (int e = 0; e < 3; e++) v3[q][t * 3 + e] = v3[q][s * 3 + e];
        for (int q = 0; q < n1; q++) v1[q][t] = v1[q][s];
      }
}

void or_form_metrics(const or_dims *d, const double *coor, or_metrics *m)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t n = (size_t)mx * my * mz;
#define CO(i, j, k, c) coor[IX(d, i, j, k) * 3 + (c)]
  if (m->cent) memset(m->cent, 0, n * 3 * sizeof(double));
  memset(m->csi, 0, n * 3 * sizeof(double));
  memset(m->eta, 0, n * 3 * sizeof(double));
  memset(m->zet, 0, n * 3 * sizeof(double));
  memset(m->aj, 0, n * sizeof(double));
  memset(m->icsi, 0, n * 3 * sizeof(double)); memset(m->ieta, 0, n * 3 * sizeof(double));
  memset(m->izet, 0, n * 3 * sizeof(double)); memset(m->iaj, 0, n * sizeof(double));
  memset(m->jcsi, 0, n * 3 * sizeof(double)); memset(m->jeta, 0, n * 3 * sizeof(double));
  memset(m->jzet, 0, n * 3 * sizeof(double)); memset(m->jaj, 0, n * sizeof(double));
  memset(m->kcsi, 0, n * 3 * sizeof(double)); memset(m->keta, 0, n * 3 * sizeof(double));
  memset(m->kzet, 0, n * 3 * sizeof(double)); memset(m->kaj, 0, n * sizeof(double));

  /* cell centres: metrics.c:89-108 */
  if (m->cent) {
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          for (int c = 0; c < 3; c++)
            m->cent[IX(d, i, j, k) * 3 + c] =
                0.125 * (CO(i, j, k, c) + CO(i, j - 1, k, c) + CO(i, j, k - 1, c) +
                         CO(i, j - 1, k - 1, c) + CO(i - 1, j, k, c) + CO(i - 1, j - 1, k, c) +
                         CO(i - 1, j, k - 1, c) + CO(i - 1, j - 1, k - 1, c));
  }

  /* aj and the cell metrics of interior cells: metrics.c:194-256 */
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        double dc[3], de[3], dz[3];
        for (int c = 0; c < 3; c++) {
          dc[c] = 0.25 * (CO(i, j, k, c) + CO(i, j - 1, k, c) + CO(i, j, k - 1, c) + CO(i, j - 1, k - 1, c) -
                          CO(i - 1, j, k, c) - CO(i - 1, j - 1, k, c) - CO(i - 1, j, k - 1, c) -
                          CO(i - 1, j - 1, k - 1, c));
          de[c] = 0.25 * (CO(i, j, k, c) + CO(i - 1, j, k, c) + CO(i, j, k - 1, c) + CO(i - 1, j, k - 1, c) -
                          CO(i, j - 1, k, c) - CO(i - 1, j - 1, k, c) - CO(i, j - 1, k - 1, c) -
                          CO(i - 1, j - 1, k - 1, c));
          dz[c] = 0.25 * (CO(i, j, k, c) + CO(i, j - 1, k, c) + CO(i - 1, j, k, c) + CO(i - 1, j - 1, k, c) -
                          CO(i, j, k - 1, c) - CO(i, j - 1, k - 1, c) - CO(i - 1, j, k - 1, c) -
                          CO(i - 1, j - 1, k - 1, c));
        }
        const size_t t = IX(d, i, j, k);
        double det = dc[0] * (de[1] * dz[2] - de[2] * dz[1]) - dc[1] * (de[0] * dz[2] - de[2] * dz[0]) +
                     dc[2] * (de[0] * dz[1] - de[1] * dz[0]);
        m->aj[t] = 1. / det;
        double *cs = &m->csi[t * 3], *et = &m->eta[t * 3], *ze = &m->zet[t * 3];
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

  /* boundary mirror of all four cell arrays: metrics.c:262-342 */
  {
    double *v3[3] = {m->csi, m->eta, m->zet};
    for (int dir = 0; dir < 3; dir++) {
      const int nu = dir == 0 ? my : mx, nv = dir == 2 ? my : mz;
      for (int side = 0; side < 2; side++)
        for (int v = 0; v < nv; v++)
          for (int u = 0; u < nu; u++) {
            size_t t, s;
            if (dir == 0) { int i = side ? mx - 1 : 0; t = IX(d, i, u, v); s = IX(d, side ? i - 1 : 1, u, v); }
            else if (dir == 1) { int j = side ? my - 1 : 0; t = IX(d, u, j, v); s = IX(d, u, side ? j - 1 : 1, v); }
            else { int k = side ? mz - 1 : 0; t = IX(d, u, v, k); s = IX(d, u, v, side ? k - 1 : 1); }
            for (int q = 0; q < 3; q++)
              for (int c = 0; c < 3; c++) v3[q][t * 3 + c] = v3[q][s * 3 + c];
            m->aj[t] = m->aj[s];
          }
    }
  }
  /* periodic ghost copy of the cell metrics: metrics.c:360-397 */
  periodic_copy16(d, m, 0);

  /* face metrics, NEWMETRIC averages: metrics.c:588-592, :696-700, :804-808 */
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 0; i < mx - 1; i++) {
        const size_t t = IX(d, i, j, k), u = IX(d, i + 1, j, k);
        avg_face(&m->csi[t * 3], &m->csi[u * 3], &m->icsi[t * 3]);
        avg_face(&m->eta[t * 3], &m->eta[u * 3], &m->ieta[t * 3]);
        avg_face(&m->zet[t * 3], &m->zet[u * 3], &m->izet[t * 3]);
        m->iaj[t] = 2. / (1. / m->aj[t] + 1. / m->aj[u]);
      }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 0; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t t = IX(d, i, j, k), u = IX(d, i, j + 1, k);
        avg_face(&m->csi[t * 3], &m->csi[u * 3], &m->jcsi[t * 3]);
        avg_face(&m->eta[t * 3], &m->eta[u * 3], &m->jeta[t * 3]);
        avg_face(&m->zet[t * 3], &m->zet[u * 3], &m->jzet[t * 3]);
        m->jaj[t] = 2. / (1. / m->aj[t] + 1. / m->aj[u]);
      }
  for (int k = 0; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t t = IX(d, i, j, k), u = IX(d, i, j, k + 1);
        avg_face(&m->csi[t * 3], &m->csi[u * 3], &m->kcsi[t * 3]);
        avg_face(&m->eta[t * 3], &m->eta[u * 3], &m->keta[t * 3]);
        avg_face(&m->zet[t * 3], &m->zet[u * 3], &m->kzet[t * 3]);
        m->kaj[t] = 2. / (1. / m->aj[t] + 1. / m->aj[u]);
      }
  /* periodic boundary layers of every array: metrics.c:1227-1262 */
  periodic_copy16(d, m, 1);
#undef CO
}

/* ------------------------------------------------------------------------ */
/* setup_lidx2 (Source/poisson.c:188-335), poisson != -1 branch.            */
/* Returns the number of pressure dofs; gid is -1 where there is no dof.    */
/* ------------------------------------------------------------------------ */
int or_setup_lidx2(const or_dims *d, const double *nvert, int *gid)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  int n = 0;
  for (size_t q = 0; q < (size_t)mx * my * mz; q++) gid[q] = -1;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1) continue;
        if ((int)nvert[IX(d, i, j, k)] > POISSON_THRESHOLD) continue; /* poisson.c:246 */
        gid[IX(d, i, j, k)] = n++;
      }
  /* periodic aliasing of ghost ids: poisson.c:299-332 */
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a, b, c;
        if (remap(d, i, j, k, &a, &b, &c, 0, 0, 0)) gid[IX(d, i, j, k)] = gid[IX(d, a, b, c)];
      }
  return n;
}

/* ------------------------------------------------------------------------ */
/* PoissonLHSNew (Source/poisson.c:977-1688) without level set (r = 1).    */
/* Writes, per DA cell, the row class, the 19 stencil values in the order  */
/* of poisson.c:957-975 and the column (dof id) of each slot; slots that   */
/* MatSetValues would skip (poisson.c:1610-1614) get col = -1, vol = 0.    */
/* scale_by_aj reproduces the poisson == -1 row scaling (poisson.c:1563).  */
/* apply_filter = 0 keeps entries with |v| <= 1e-10 (used by the V-cycle).  */
/* ------------------------------------------------------------------------ */
/* Level-set context of PoissonLHSNew and Projection (poisson.c:1171-1561,
 * :2738-2950): density rho and level-set field at the cells (DA layout),
 * on = levelset, bc3 / bc4 / bc5 = user->bctype[3], [4], [5]. */
static struct {
  const double *rho, *level;
  int on, bc3, bc4, bc5;
} g_ls = {0, 0, 0, 0, 0, 0};

void or_set_levelset(const double *rho, const double *level, int on, int bc3, int bc4, int bc5)
{
  g_ls.rho = rho; g_ls.level = level; g_ls.on = on; g_ls.bc3 = bc3; g_ls.bc4 = bc4; g_ls.bc5 = bc5;
}

/* mean (level.c:2276-2280), the harmonic mean of two densities */
static double ls_mean(double A, double B) { return 2.0 * A * B / (A + B); }

int or_poisson_lhs(const or_dims *d, const double *nvert, const or_metrics *m, int scale_by_aj,
                   int apply_filter, int *gid, int *rowtype, double *vol, int *col)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t n = (size_t)mx * my * mz;
  const int ip = per_i(d), jp = per_j(d), kp = per_k(d);
  const double thr = POISSON_THRESHOLD;
  int ndof = or_setup_lidx2(d, nvert, gid);
  double *g = (double *)malloc(n * 9 * sizeof(double));
  /* g11..g33 with periodic source remap: poisson.c:1102-1138 */
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a, b, c;
        remap(d, i, j, k, &a, &b, &c, 0, 0, 0);
        size_t s = IX(d, a, b, c), t = IX(d, i, j, k);
        const double *ic = &m->icsi[s * 3], *ie = &m->ieta[s * 3], *iz = &m->izet[s * 3];
        const double *jc = &m->jcsi[s * 3], *je = &m->jeta[s * 3], *jz = &m->jzet[s * 3];
        const double *kc = &m->kcsi[s * 3], *ke = &m->keta[s * 3], *kz = &m->kzet[s * 3];
        double *gg = &g[t * 9];
        gg[0] = (ic[0] * ic[0] + ic[1] * ic[1] + ic[2] * ic[2]) * m->iaj[s];
        gg[1] = (ie[0] * ic[0] + ie[1] * ic[1] + ie[2] * ic[2]) * m->iaj[s];
        gg[2] = (iz[0] * ic[0] + iz[1] * ic[1] + iz[2] * ic[2]) * m->iaj[s];
        gg[3] = (jc[0] * je[0] + jc[1] * je[1] + jc[2] * je[2]) * m->jaj[s];
        gg[4] = (je[0] * je[0] + je[1] * je[1] + je[2] * je[2]) * m->jaj[s];
        gg[5] = (jz[0] * je[0] + jz[1] * je[1] + jz[2] * je[2]) * m->jaj[s];
        gg[6] = (kc[0] * kz[0] + kc[1] * kz[1] + kc[2] * kz[2]) * m->kaj[s];
        gg[7] = (ke[0] * kz[0] + ke[1] * kz[1] + ke[2] * kz[2]) * m->kaj[s];
        gg[8] = (kz[0] * kz[0] + kz[1] * kz[1] + kz[2] * kz[2]) * m->kaj[s];
      }
#define NV(i, j, k) nvert[IX(d, i, j, k)]
#define G(q, i, j, k) g[IX(d, i, j, k) * 9 + (q)]
#define RHO(i, j, k) g_ls.rho[IX(d, i, j, k)]
#define LEV(i, j, k) g_ls.level[IX(d, i, j, k)]
  for (size_t q = 0; q < n; q++) {
    rowtype[q] = OR_ROW_NONE;
    for (int s = 0; s < 19; s++) { vol[q * 19 + s] = 0.; col[q * 19 + s] = -1; }
  }
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t t = IX(d, i, j, k);
        int row = gid[t];
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1) continue;
        if (NV(i, j, k) > 0.1 && row >= 0) { /* poisson.c:1158-1160 */
          rowtype[t] = OR_ROW_IDENTITY;
          vol[t * 19 + OR_CP] = 1.0;
          col[t * 19 + OR_CP] = row;
          continue;
        }
        if (NV(i, j, k) > thr) continue;
        double v[19];
        for (int s = 0; s < 19; s++) v[s] = 0.;
        double r = 1.0;
        /* i+1 - i: poisson.c:1167-1230 */
        if (NV(i + 1, j, k) < thr && (i != mx - 2 || ip)) {
          r = g_ls.on ? ls_mean(RHO(i + 1, j, k), RHO(i, j, k)) : 1.0;
          v[OR_CP] -= G(0, i, j, k) / r;
          v[OR_EP] += G(0, i, j, k) / r;
          if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i + 1, j + 1, k) > thr) {
            if (NV(i, j - 1, k) + NV(i + 1, j - 1, k) < thr && j != 1) {
              v[OR_CP] += G(1, i, j, k) * 0.5 / r; v[OR_EP] += G(1, i, j, k) * 0.5 / r;
              v[OR_SP] -= G(1, i, j, k) * 0.5 / r; v[OR_SE] -= G(1, i, j, k) * 0.5 / r;
            }
          } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i + 1, j - 1, k) > thr) {
            if (NV(i, j + 1, k) + NV(i + 1, j + 1, k) < thr) {
              v[OR_NP] += G(1, i, j, k) * 0.5 / r; v[OR_NE] += G(1, i, j, k) * 0.5 / r;
              v[OR_CP] -= G(1, i, j, k) * 0.5 / r; v[OR_EP] -= G(1, i, j, k) * 0.5 / r;
            }
          } else {
            v[OR_NP] += G(1, i, j, k) * 0.25 / r; v[OR_NE] += G(1, i, j, k) * 0.25 / r;
            v[OR_SP] -= G(1, i, j, k) * 0.25 / r; v[OR_SE] -= G(1, i, j, k) * 0.25 / r;
          }
          if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i + 1, j, k + 1) > thr) {
            if (NV(i, j, k - 1) + NV(i + 1, j, k - 1) < thr && k != 1) {
              v[OR_CP] += G(2, i, j, k) * 0.5 / r; v[OR_EP] += G(2, i, j, k) * 0.5 / r;
              v[OR_BP] -= G(2, i, j, k) * 0.5 / r; v[OR_BE] -= G(2, i, j, k) * 0.5 / r;
            }
          } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i + 1, j, k - 1) > thr) {
            if (NV(i, j, k + 1) + NV(i + 1, j, k + 1) < thr) {
              v[OR_TP] += G(2, i, j, k) * 0.5 / r; v[OR_TE] += G(2, i, j, k) * 0.5 / r;
              v[OR_CP] -= G(2, i, j, k) * 0.5 / r; v[OR_EP] -= G(2, i, j, k) * 0.5 / r;
            }
          } else {
            v[OR_TP] += G(2, i, j, k) * 0.25 / r; v[OR_TE] += G(2, i, j, k) * 0.25 / r;
            v[OR_BP] -= G(2, i, j, k) * 0.25 / r; v[OR_BE] -= G(2, i, j, k) * 0.25 / r;
          }
        }
        /* i - i-1: poisson.c:1233-1293 */
        if (NV(i - 1, j, k) < thr && (i != 1 || ip)) {
          r = g_ls.on ? ls_mean(RHO(i - 1, j, k), RHO(i, j, k)) : 1.0;
          v[OR_CP] -= G(0, i - 1, j, k) / r;
          v[OR_WP] += G(0, i - 1, j, k) / r;
          if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i - 1, j + 1, k) > thr) {
            if (NV(i, j - 1, k) + NV(i - 1, j - 1, k) < thr && j != 1) {
              v[OR_CP] -= G(1, i - 1, j, k) * 0.5 / r; v[OR_WP] -= G(1, i - 1, j, k) * 0.5 / r;
              v[OR_SP] += G(1, i - 1, j, k) * 0.5 / r; v[OR_SW] += G(1, i - 1, j, k) * 0.5 / r;
            }
          } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i - 1, j - 1, k) > thr) {
            if (NV(i, j + 1, k) + NV(i - 1, j + 1, k) < thr) {
              v[OR_NP] -= G(1, i - 1, j, k) * 0.5 / r; v[OR_NW] -= G(1, i - 1, j, k) * 0.5 / r;
              v[OR_CP] += G(1, i - 1, j, k) * 0.5 / r; v[OR_WP] += G(1, i - 1, j, k) * 0.5 / r;
            }
          } else {
            v[OR_NP] -= G(1, i - 1, j, k) * 0.25 / r; v[OR_NW] -= G(1, i - 1, j, k) * 0.25 / r;
            v[OR_SP] += G(1, i - 1, j, k) * 0.25 / r; v[OR_SW] += G(1, i - 1, j, k) * 0.25 / r;
          }
          if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i - 1, j, k + 1) > thr) {
            if (NV(i, j, k - 1) + NV(i - 1, j, k - 1) < thr && k != 1) {
              v[OR_CP] -= G(2, i - 1, j, k) * 0.5 / r; v[OR_WP] -= G(2, i - 1, j, k) * 0.5 / r;
              v[OR_BP] += G(2, i - 1, j, k) * 0.5 / r; v[OR_BW] += G(2, i - 1, j, k) * 0.5 / r;
            }
          } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i - 1, j, k - 1) > thr) {
            if (NV(i, j, k + 1) + NV(i - 1, j, k + 1) < thr) {
              v[OR_TP] -= G(2, i - 1, j, k) * 0.5 / r; v[OR_TW] -= G(2, i - 1, j, k) * 0.5 / r;
              v[OR_CP] += G(2, i - 1, j, k) * 0.5 / r; v[OR_WP] += G(2, i - 1, j, k) * 0.5 / r;
            }
          } else {
            v[OR_TP] -= G(2, i - 1, j, k) * 0.25 / r; v[OR_TW] -= G(2, i - 1, j, k) * 0.25 / r;
            v[OR_BP] += G(2, i - 1, j, k) * 0.25 / r; v[OR_BW] += G(2, i - 1, j, k) * 0.25 / r;
          }
        }
        /* j+1 - j: poisson.c:1296-1361 */
        if (NV(i, j + 1, k) < thr && (j != my - 2 || jp || (g_ls.on && g_ls.bc3 == 4 && j == my - 2))) {
          r = g_ls.on ? ls_mean(RHO(i, j + 1, k), RHO(i, j, k)) : 1.0;
          if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j + 1, k) > thr) {
            if (NV(i - 1, j, k) + NV(i - 1, j + 1, k) < thr && i != 1) {
              v[OR_CP] += G(3, i, j, k) * 0.5 / r; v[OR_NP] += G(3, i, j, k) * 0.5 / r;
              v[OR_WP] -= G(3, i, j, k) * 0.5 / r; v[OR_NW] -= G(3, i, j, k) * 0.5 / r;
            }
          } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j + 1, k) > thr) {
            if (NV(i + 1, j, k) + NV(i + 1, j + 1, k) < thr) {
              v[OR_EP] += G(3, i, j, k) * 0.5 / r; v[OR_NE] += G(3, i, j, k) * 0.5 / r;
              v[OR_CP] -= G(3, i, j, k) * 0.5 / r; v[OR_NP] -= G(3, i, j, k) * 0.5 / r;
            }
          } else {
            v[OR_EP] += G(3, i, j, k) * 0.25 / r; v[OR_NE] += G(3, i, j, k) * 0.25 / r;
            v[OR_WP] -= G(3, i, j, k) * 0.25 / r; v[OR_NW] -= G(3, i, j, k) * 0.25 / r;
          }
          if (g_ls.on && g_ls.bc3 == 4 && j == my - 2) { /* zero Dirichlet pressure, poisson.c:1328 */
            v[OR_CP] -= G(4, i, j, k) / 0.5 / r;
          } else {
            v[OR_CP] -= G(4, i, j, k) / r;
            v[OR_NP] += G(4, i, j, k) / r;
          }
          if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j + 1, k + 1) > thr) {
            if (NV(i, j, k - 1) + NV(i, j + 1, k - 1) < thr && k != 1) {
              v[OR_CP] += G(5, i, j, k) * 0.5 / r; v[OR_NP] += G(5, i, j, k) * 0.5 / r;
              v[OR_BP] -= G(5, i, j, k) * 0.5 / r; v[OR_BN] -= G(5, i, j, k) * 0.5 / r;
            }
          } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j + 1, k - 1) > thr) {
            if (NV(i, j, k + 1) + NV(i, j + 1, k + 1) < thr) {
              v[OR_TP] += G(5, i, j, k) * 0.5 / r; v[OR_TN] += G(5, i, j, k) * 0.5 / r;
              v[OR_CP] -= G(5, i, j, k) * 0.5 / r; v[OR_NP] -= G(5, i, j, k) * 0.5 / r;
            }
          } else {
            v[OR_TP] += G(5, i, j, k) * 0.25 / r; v[OR_TN] += G(5, i, j, k) * 0.25 / r;
            v[OR_BP] -= G(5, i, j, k) * 0.25 / r; v[OR_BN] -= G(5, i, j, k) * 0.25 / r;
          }
        }
        /* j - j-1: poisson.c:1364-1422 */
        if (NV(i, j - 1, k) < thr && (j != 1 || jp)) {
          r = g_ls.on ? ls_mean(RHO(i, j - 1, k), RHO(i, j, k)) : 1.0;
          if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j - 1, k) > thr) {
            if (NV(i - 1, j, k) + NV(i - 1, j - 1, k) < thr && i != 1) {
              v[OR_CP] -= G(3, i, j - 1, k) * 0.5 / r; v[OR_SP] -= G(3, i, j - 1, k) * 0.5 / r;
              v[OR_WP] += G(3, i, j - 1, k) * 0.5 / r; v[OR_SW] += G(3, i, j - 1, k) * 0.5 / r;
            }
          } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j - 1, k) > thr) {
            if (NV(i + 1, j, k) + NV(i + 1, j - 1, k) < thr) {
              v[OR_EP] -= G(3, i, j - 1, k) * 0.5 / r; v[OR_SE] -= G(3, i, j - 1, k) * 0.5 / r;
              v[OR_CP] += G(3, i, j - 1, k) * 0.5 / r; v[OR_SP] += G(3, i, j - 1, k) * 0.5 / r;
            }
          } else {
            v[OR_EP] -= G(3, i, j - 1, k) * 0.25 / r; v[OR_SE] -= G(3, i, j - 1, k) * 0.25 / r;
            v[OR_WP] += G(3, i, j - 1, k) * 0.25 / r; v[OR_SW] += G(3, i, j - 1, k) * 0.25 / r;
          }
          v[OR_CP] -= G(4, i, j - 1, k) / r;
          v[OR_SP] += G(4, i, j - 1, k) / r;
          if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j - 1, k + 1) > thr) {
            if (NV(i, j, k - 1) + NV(i, j - 1, k - 1) < thr && k != 1) {
              v[OR_CP] -= G(5, i, j - 1, k) * 0.5 / r; v[OR_SP] -= G(5, i, j - 1, k) * 0.5 / r;
              v[OR_BP] += G(5, i, j - 1, k) * 0.5 / r; v[OR_BS] += G(5, i, j - 1, k) * 0.5 / r;
            }
          } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j - 1, k - 1) > thr) {
            if (NV(i, j, k + 1) + NV(i, j - 1, k + 1) < thr) {
              v[OR_TP] -= G(5, i, j - 1, k) * 0.5 / r; v[OR_TS] -= G(5, i, j - 1, k) * 0.5 / r;
              v[OR_CP] += G(5, i, j - 1, k) * 0.5 / r; v[OR_SP] += G(5, i, j - 1, k) * 0.5 / r;
            }
          } else {
            v[OR_TP] -= G(5, i, j - 1, k) * 0.25 / r; v[OR_TS] -= G(5, i, j - 1, k) * 0.25 / r;
            v[OR_BP] += G(5, i, j - 1, k) * 0.25 / r; v[OR_BS] += G(5, i, j - 1, k) * 0.25 / r;
          }
        }
        /* k+1 - k: poisson.c:1425-1491 */
        if (NV(i, j, k + 1) < thr && (k != mz - 2 || kp || (g_ls.on && g_ls.bc5 == 4 && k == mz - 2))) {
          r = g_ls.on ? ls_mean(RHO(i, j, k + 1), RHO(i, j, k)) : 1.0;
          if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k + 1) > thr) {
            if (NV(i - 1, j, k) + NV(i - 1, j, k + 1) < thr && i != 1) {
              v[OR_CP] += G(6, i, j, k) * 0.5 / r; v[OR_TP] += G(6, i, j, k) * 0.5 / r;
              v[OR_WP] -= G(6, i, j, k) * 0.5 / r; v[OR_TW] -= G(6, i, j, k) * 0.5 / r;
            }
          } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k + 1) > thr) {
            if (NV(i + 1, j, k) + NV(i + 1, j, k + 1) < thr) {
              v[OR_EP] += G(6, i, j, k) * 0.5 / r; v[OR_TE] += G(6, i, j, k) * 0.5 / r;
              v[OR_CP] -= G(6, i, j, k) * 0.5 / r; v[OR_TP] -= G(6, i, j, k) * 0.5 / r;
            }
          } else {
            v[OR_EP] += G(6, i, j, k) * 0.25 / r; v[OR_TE] += G(6, i, j, k) * 0.25 / r;
            v[OR_WP] -= G(6, i, j, k) * 0.25 / r; v[OR_TW] -= G(6, i, j, k) * 0.25 / r;
          }
          if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k + 1) > thr) {
            if (NV(i, j - 1, k) + NV(i, j - 1, k + 1) < thr && j != 1) {
              v[OR_CP] += G(7, i, j, k) * 0.5 / r; v[OR_TP] += G(7, i, j, k) * 0.5 / r;
              v[OR_SP] -= G(7, i, j, k) * 0.5 / r; v[OR_TS] -= G(7, i, j, k) * 0.5 / r;
            }
          } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k + 1) > thr) {
            if (NV(i, j + 1, k) + NV(i, j + 1, k + 1) < thr) {
              v[OR_NP] += G(7, i, j, k) * 0.5 / r; v[OR_TN] += G(7, i, j, k) * 0.5 / r;
              v[OR_CP] -= G(7, i, j, k) * 0.5 / r; v[OR_TP] -= G(7, i, j, k) * 0.5 / r;
            }
          } else {
            v[OR_NP] += G(7, i, j, k) * 0.25 / r; v[OR_TN] += G(7, i, j, k) * 0.25 / r;
            v[OR_SP] -= G(7, i, j, k) * 0.25 / r; v[OR_TS] -= G(7, i, j, k) * 0.25 / r;
          }
          if (g_ls.on && g_ls.bc5 == 4 && k == mz - 2) { /* poisson.c:1482-1484 */
            v[OR_CP] -= G(8, i, j, k) / 0.5 / r;
          } else {
            v[OR_CP] -= G(8, i, j, k) / r;
            v[OR_TP] += G(8, i, j, k) / r;
          }
        }
        /* k - k-1: poisson.c:1494-1561 */
        if (NV(i, j, k - 1) < thr && (k != 1 || kp || (g_ls.on && g_ls.bc4 == 5000 && k == 1 && LEV(i, j, k) < 0))) {
          r = g_ls.on ? (k == 1 ? RHO(i, j, k) : ls_mean(RHO(i, j, k - 1), RHO(i, j, k))) : 1.0;
          if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k - 1) > thr) {
            if (NV(i - 1, j, k) + NV(i - 1, j, k - 1) < thr && i != 1) {
              v[OR_CP] -= G(6, i, j, k - 1) * 0.5 / r; v[OR_BP] -= G(6, i, j, k - 1) * 0.5 / r;
              v[OR_WP] += G(6, i, j, k - 1) * 0.5 / r; v[OR_BW] += G(6, i, j, k - 1) * 0.5 / r;
            }
          } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k - 1) > thr) {
            if (NV(i + 1, j, k) + NV(i + 1, j, k - 1) < thr) {
              v[OR_EP] -= G(6, i, j, k - 1) * 0.5 / r; v[OR_BE] -= G(6, i, j, k - 1) * 0.5 / r;
              v[OR_CP] += G(6, i, j, k - 1) * 0.5 / r; v[OR_BP] += G(6, i, j, k - 1) * 0.5 / r;
            }
          } else {
            v[OR_EP] -= G(6, i, j, k - 1) * 0.25 / r; v[OR_BE] -= G(6, i, j, k - 1) * 0.25 / r;
            v[OR_WP] += G(6, i, j, k - 1) * 0.25 / r; v[OR_BW] += G(6, i, j, k - 1) * 0.25 / r;
          }
          if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k - 1) > thr) {
            if (NV(i, j - 1, k) + NV(i, j - 1, k - 1) < thr && j != 1) {
              v[OR_CP] -= G(7, i, j, k - 1) * 0.5 / r; v[OR_BP] -= G(7, i, j, k - 1) * 0.5 / r;
              v[OR_SP] += G(7, i, j, k - 1) * 0.5 / r; v[OR_BS] += G(7, i, j, k - 1) * 0.5 / r;
            }
          } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k - 1) > thr) {
            if (NV(i, j + 1, k) + NV(i, j + 1, k - 1) < thr) {
              v[OR_NP] -= G(7, i, j, k - 1) * 0.5 / r; v[OR_BN] -= G(7, i, j, k - 1) * 0.5 / r;
              v[OR_CP] += G(7, i, j, k - 1) * 0.5 / r; v[OR_BP] += G(7, i, j, k - 1) * 0.5 / r;
            }
          } else {
            v[OR_NP] -= G(7, i, j, k - 1) * 0.25 / r; v[OR_BN] -= G(7, i, j, k - 1) * 0.25 / r;
            v[OR_SP] += G(7, i, j, k - 1) * 0.25 / r; v[OR_BS] += G(7, i, j, k - 1) * 0.25 / r;
          }
          if (g_ls.on && g_ls.bc4 == 5 && k == 1) { /* poisson.c:1552-1554 */
            v[OR_CP] -= G(8, i, j, k - 1) / 0.5 / r;
          } else {
            v[OR_CP] -= G(8, i, j, k - 1) / r;
            v[OR_BP] += G(8, i, j, k - 1) / r;
          }
        }
        if (scale_by_aj)
          for (int s = 0; s < 19; s++) v[s] *= m->aj[t];
        /* column ids: poisson.c:1584-1603; entry filter: poisson.c:1610-1614 */
        static const int off[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                       {0, 0, 1},  {0, 0, -1}, {1, 1, 0},  {1, -1, 0}, {-1, 1, 0},
                                       {-1, -1, 0}, {0, 1, 1},  {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
                                       {1, 0, 1},  {1, 0, -1}, {-1, 0, 1}, {-1, 0, -1}};
        rowtype[t] = OR_ROW_FLUID;
        for (int s = 0; s < 19; s++) {
          int id = gid[IX(d, i + off[s][0], j + off[s][1], k + off[s][2])];
          int keep = (s == OR_CP) || (id >= 0 && (!apply_filter || fabs(v[s]) > 1.e-10));
          if (keep) {
            vol[t * 19 + s] = v[s];
            col[t * 19 + s] = id;
          }
        }
      }
#undef NV
#undef G
#undef RHO
#undef LEV
  free(g);
  return ndof;
}

/* ------------------------------------------------------------------------ */
/* PoissonRHS2_hypre (Source/poisson_hypre.c:265-407) without level set.   */
/* b has one entry per dof; entries of non-fluid dofs stay 0 (they are     */
/* never set, poisson_hypre.c:328-331).                                    */
/* ------------------------------------------------------------------------ */
void or_poisson_rhs2_hypre(const or_dims *d, const double *nvert, const int *gid,
                           const double *ucont, double dt, double st, double coeff, double *b)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const int ip = per_i(d), jp = per_j(d), kp = per_k(d);
#define U(i, j, k, c) ucont[IX(d, i, j, k) * 3 + (c)]
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (gid[t] >= 0) b[gid[t]] = 0.;
      }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] >= 0.1) continue;
        double val = 0;
        val -= U(i, j, k, 0);
        if (i == 1 && ip) val += U(mx - 2, j, k, 0);
        else val += U(i - 1, j, k, 0);
        val -= U(i, j, k, 1);
        if (j == 1 && jp) val += U(i, my - 2, k, 1);
        else val += U(i, j - 1, k, 1);
        val -= U(i, j, k, 2);
        if (k == 1 && kp) val += U(i, j, mz - 2, 2);
        else val += U(i, j, k - 1, 2);
        val *= -1.0 / dt * st * coeff;
        b[gid[t]] = val;
      }
#undef U
}

/* PoissonRHS2 (Source/poisson.c:1780-1906), the -poisson 0 / -1 right-hand
 * side: the PoissonRHS2_hypre divergence on fluid cells (nvert < 0.1), 0 on
 * identity-row dofs (nvert >= 0.1 with a dof, :1816-1819), the aj row
 * scaling when poisson == -1 (:1856), then the unweighted mean over the
 * fluid cells removed from the fluid entries (:1873-1889; VecSum runs over
 * every entry of B, the count over the fluid cells).  b has one entry per
 * dof. */
void or_poisson_rhs2(const or_dims *d, const double *nvert, const int *gid, const double *ucont,
                     const double *aj, double dt, double st, double coeff, int poisson, double *b)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const int ip = per_i(d), jp = per_j(d), kp = per_k(d);
  int count = 0;
#define U(i, j, k, c) ucont[IX(d, i, j, k) * 3 + (c)]
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        double val;
        if (nvert[t] >= 0.1) {
          if (gid[t] >= 0) val = 0;
          else continue;
        } else {
          val = 0;
          val -= U(i, j, k, 0);
          if (i == 1 && ip) val += U(mx - 2, j, k, 0);
          else val += U(i - 1, j, k, 0);
          val -= U(i, j, k, 1);
          if (j == 1 && jp) val += U(i, my - 2, k, 1);
          else val += U(i, j - 1, k, 1);
          val -= U(i, j, k, 2);
          if (k == 1 && kp) val += U(i, j, mz - 2, 2);
          else val += U(i, j, k - 1, 2);
          val *= -1.0 / dt * st * coeff;
          if (poisson == -1) val *= aj[t];
          count++;
        }
        b[gid[t]] = val;
      }
#undef U
  double sum = 0; /* every dof entry, in the grid order */
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (gid[t] >= 0) sum += b[gid[t]];
      }
  const double val = -sum / (double)(count > 0 ? count : 1);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] < 0.1) b[gid[t]] += val;
      }
}

/* Remove_Nullspace_Scale (Source/poisson_hypre.c:118-200). */
void or_remove_nullspace_scale(const or_dims *d, const double *nvert, const int *gid,
                               const double *aj, double *b, int bctype3)
{
  if (bctype3 == -10) return;
  const int mx = d->mx, my = d->my, mz = d->mz;
  double sum = 0, sum_aj = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] < 0.1) { sum += b[gid[t]]; sum_aj += aj[t]; }
      }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] < 0.1) {
          double val = -sum * aj[t] / sum_aj;
          b[gid[t]] += val;
        }
      }
}

/* FullyBlocked (Source/poisson.c:1909-1993): for every interior (i, j)
 * column the first k (boundary layers included) whose nvert exceeds 0.1, in
 * ksk[j * mx + i] (-1 for a column with none, and on the boundary columns);
 * returns the multiple-null-space flag: every interior column is blocked. */
int or_fully_blocked(const or_dims *d, const double *nvert, int *ksk)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  int multi = 1;
  for (int q = 0; q < mx * my; q++) ksk[q] = -1;
  for (int j = 1; j < my - 1; j++)
    for (int i = 1; i < mx - 1; i++) {
      for (int k = 0; k < mz; k++)
        if (nvert[IX(d, i, j, k)] > 0.1) { ksk[j * mx + i] = k; break; }
      if (ksk[j * mx + i] < 0) multi = 0;
    }
  return multi;
}

/* PoissonNullSpaceFunction_original (Source/poisson.c:757-943) on a
 * DA-layout vector x: the mean over the interior cells with nvert < 0.1 is
 * removed (with multi, separately below and above each column's first
 * blocked k, ksk from or_fully_blocked, summed in the reference's j-i-k
 * order); then the boundary layers and the cells with nvert > 0.1 are set
 * to 0. */
void or_nullspace_original(const or_dims *d, const double *nvert, const int *ksk, int multi, double *x)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  if (!multi) {
    double sum = 0, num = 0;
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          if (nvert[IX(d, i, j, k)] < 0.1) { sum += x[IX(d, i, j, k)]; num++; }
    sum = sum / (-1.0 * num);
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          if (nvert[IX(d, i, j, k)] < 0.1) x[IX(d, i, j, k)] += sum;
  } else {
    for (int above = 0; above < 2; above++) {
      double sum = 0, num = 0;
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          for (int k = 1; k < mz - 1; k++) {
            const int in = above ? k >= ksk[j * mx + i] : k < ksk[j * mx + i];
            if (in && nvert[IX(d, i, j, k)] < 0.1) { sum += x[IX(d, i, j, k)]; num++; }
          }
      sum /= -num;
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++)
          for (int k = 1; k < mz - 1; k++) {
            const int in = above ? k >= ksk[j * mx + i] : k < ksk[j * mx + i];
            if (in && nvert[IX(d, i, j, k)] < 0.1) x[IX(d, i, j, k)] += sum;
          }
    }
  }
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        const int bnd = i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1;
        if (bnd || nvert[IX(d, i, j, k)] > 0.1) x[IX(d, i, j, k)] = 0.;
      }
}

/* Remove_Nullspace (Source/poisson_hypre.c:202-263). */
void or_remove_nullspace(const or_dims *d, const double *nvert, const int *gid, double *phi2,
                         int bctype3)
{
  if (bctype3 == -10) return;
  const int mx = d->mx, my = d->my, mz = d->mz;
  double sum = 0;
  int count = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] < 0.1) { sum += phi2[gid[t]]; count++; }
      }
  double val = -sum / (double)count;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] < 0.1) phi2[gid[t]] += val;
      }
}

/* Convert_Phi2_Phi (Source/poisson.c:98-186). */
void or_convert_phi2_phi(const or_dims *d, const double *nvert, const double *phi2, double *phi)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  memset(phi, 0, sizeof(double) * (size_t)mx * my * mz);
  int pos = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if ((int)nvert[t] > POISSON_THRESHOLD) phi[t] = 0;
        else phi[t] = phi2[pos++];
      }
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a, b, c;
        if (remap(d, i, j, k, &a, &b, &c, 0, 0, 0)) phi[IX(d, i, j, k)] = phi[IX(d, a, b, c)];
      }
}

/* UpdatePressure (Source/poisson.c:3137-3297), non-PRIMITIVE_PRESSURE path. */
void or_update_pressure(const or_dims *d, const double *nvert, double *p, double *phi)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] < 0.1) p[t] += phi[t];
        if (nvert[t] > 1.1) p[t] = 0;
      }
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a, b, c;
        if (remap(d, i, j, k, &a, &b, &c, 0, 0, 0)) {
          p[IX(d, i, j, k)] = p[IX(d, a, b, c)];
          phi[IX(d, i, j, k)] = phi[IX(d, a, b, c)];
        }
      }
}

/* Projection (Source/poisson.c:2700-3066) without level set; Contra2Cart
 * (poisson.c:3060) is not part of this restatement. */
void or_projection(const or_dims *d, const double *nvert, const double *phi, const or_metrics *m,
                   double dt, double st, double coeff, double *ucont)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const int ip = per_i(d), jp = per_j(d), kp = per_k(d);
  const double thr = POISSON_THRESHOLD;
#define NV(i, j, k) nvert[IX(d, i, j, k)]
#define PH(i, j, k) phi[IX(d, i, j, k)]
#define M3(arr, i, j, k, c) m->arr[IX(d, i, j, k) * 3 + (c)]
#define DOT(A, B, i, j, k) (M3(A, i, j, k, 0) * M3(B, i, j, k, 0) + M3(A, i, j, k, 1) * M3(B, i, j, k, 1) + M3(A, i, j, k, 2) * M3(B, i, j, k, 2))
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        double r1 = 1.0, r2 = 1.0, r3 = 1.0;
        if (g_ls.on) { /* poisson.c:2738-2749 */
          const double *rho = g_ls.rho;
          r1 = i == mx - 2 ? rho[IX(d, i, j, k)] : ls_mean(rho[IX(d, i, j, k)], rho[IX(d, i + 1, j, k)]);
          r2 = j == my - 2 ? rho[IX(d, i, j, k)] : ls_mean(rho[IX(d, i, j, k)], rho[IX(d, i, j + 1, k)]);
          r3 = k == mz - 2 ? rho[IX(d, i, j, k)] : ls_mean(rho[IX(d, i, j, k)], rho[IX(d, i, j, k + 1)]);
        }
        double dpdc, dpde, dpdz;
        size_t t = IX(d, i, j, k);
        if (i < mx - 2 || (ip && i == mx - 2)) { /* poisson.c:2791-2834 */
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
            ucont[t * 3 + 0] -= (dpdc * DOT(icsi, icsi, i, j, k) * m->iaj[t] +
                                 dpde * DOT(ieta, icsi, i, j, k) * m->iaj[t] +
                                 dpdz * DOT(izet, icsi, i, j, k) * m->iaj[t]) *
                                dt * st / coeff / r1;
          }
        }
        if (j < my - 2 || (jp && j == my - 2) || (g_ls.on && g_ls.bc3 == 4 && j == my - 2)) { /* poisson.c:2837-2883 */
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
          if (g_ls.on && g_ls.bc3 == 4 && j == my - 2) dpde = PH(i, j, k) - PH(i, j - 1, k);
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
            ucont[t * 3 + 1] -= (dpdc * DOT(jcsi, jeta, i, j, k) * m->jaj[t] +
                                 dpde * DOT(jeta, jeta, i, j, k) * m->jaj[t] +
                                 dpdz * DOT(jzet, jeta, i, j, k) * m->jaj[t]) *
                                dt * st / coeff / r2;
          }
        }
        if (k < mz - 2 || (kp && k == mz - 2) || (g_ls.on && g_ls.bc5 == 4 && k == mz - 2)) { /* poisson.c:2886-2958 */
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
          else if (k == mz - 2 && g_ls.on && g_ls.bc5 == 4) dpdz = PH(i, j, k) - PH(i, j, k - 1);
          else dpdz = PH(i, j, k + 1) - PH(i, j, k);
          if ((NV(i, j, k) + NV(i, j, k + 1)) < thr) {
            ucont[t * 3 + 2] -= (dpdc * DOT(kcsi, kzet, i, j, k) * m->kaj[t] +
                                 dpde * DOT(keta, kzet, i, j, k) * m->kaj[t] +
                                 dpdz * DOT(kzet, kzet, i, j, k) * m->kaj[t]) *
                                dt * st / coeff / r3;
            if (g_ls.on && k == 1 && g_ls.bc4 == 5000 && g_ls.level[IX(d, i, j, k)] < 0) { /* poisson.c:2951-2956 */
              const size_t t0 = IX(d, i, j, 0);
              const double r0 = g_ls.rho[IX(d, i, j, k)];
              ucont[t0 * 3 + 2] -= (dpdz * DOT(kzet, kzet, i, j, 0) * m->kaj[t0]) * dt * st / coeff / r0;
            }
          }
        }
      }
  /* periodic face copy: poisson.c:2996-3036 */
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a, b, c, fi, fj, fk;
        if (!remap(d, i, j, k, &a, &b, &c, &fi, &fj, &fk)) continue;
        size_t s = IX(d, a, b, c), t = IX(d, i, j, k);
        if (fi) ucont[t * 3 + 0] = ucont[s * 3 + 0];
        if (fj) ucont[t * 3 + 1] = ucont[s * 3 + 1];
        if (fk) ucont[t * 3 + 2] = ucont[s * 3 + 2];
      }
#undef NV
#undef PH
#undef M3
#undef DOT
}

/* Divergence (Source/main.c:936-1074): max over interior cells of
 * |div(Ucont) * aj|, zero next to any blanked cell. */
double or_divergence(const or_dims *d, const double *nvert, const double *ucont, const double *aj)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  double best = 0.;
#define U(i, j, k, c) ucont[IX(d, i, j, k) * 3 + (c)]
#define NV(i, j, k) nvert[IX(d, i, j, k)]
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        double v = fabs((U(i, j, k, 0) - U(i - 1, j, k, 0) + U(i, j, k, 1) - U(i, j - 1, k, 1) +
                         U(i, j, k, 2) - U(i, j, k - 1, 2)) *
                        aj[IX(d, i, j, k)]);
        if (NV(i, j, k) + NV(i, j, k + 1) + NV(i, j, k - 1) + NV(i, j + 1, k) + NV(i, j - 1, k) +
                NV(i + 1, j, k) + NV(i - 1, j, k) >
            0.1)
          v = 0.;
        if (v > best) best = v;
      }
#undef U
#undef NV
  return best;
}

/* ------------------------------------------------------------------------ */
/* Multigrid transfer operators.                                            */
/* ------------------------------------------------------------------------ */
/* MyNvertRestriction (Source/poisson.c:1995-2083). */
void or_my_nvert_restriction(const or_dims *dh, const or_dims *dc, int isc, int jsc, int ksc,
                             const double *nvert_h, double *nvert_c)
{
  const int mx = dc->mx, my = dc->my, mz = dc->mz;
  const int ia = isc ? 0 : 1, ja = jsc ? 0 : 1, ka = ksc ? 0 : 1;
  memset(nvert_c, 0, sizeof(double) * (size_t)mx * my * mz);
#define NH(i, j, k) nvert_h[IX(dh, i, j, k)]
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        int ih = isc ? i : 2 * i, jh = jsc ? j : 2 * j, kh = ksc ? k : 2 * k;
        if (NH(ih, jh, kh) * NH(ih - ia, jh, kh) * NH(ih, jh - ja, kh) * NH(ih, jh, kh - ka) *
                NH(ih - ia, jh - ja, kh) * NH(ih - ia, jh, kh - ka) * NH(ih, jh - ja, kh - ka) *
                NH(ih - ia, jh - ja, kh - ka) >
            0.1) {
          double *o = &nvert_c[IX(dc, i, j, k)];
          *o = (1. > *o) ? 1. : *o;
        }
      }
#undef NH
  /* isolated-cell fill, done in place in k-j-i order as the reference does;
   * the boundary layer of the coarse array stays 0 (VecSet above) */
  double *l = (double *)malloc(sizeof(double) * (size_t)mx * my * mz);
  memcpy(l, nvert_c, sizeof(double) * (size_t)mx * my * mz);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(dc, i, j, k);
        if (l[t] < 0.1) {
          if (l[IX(dc, i + 1, j, k)] + l[IX(dc, i - 1, j, k)] > 1.1 &&
              l[IX(dc, i, j + 1, k)] + l[IX(dc, i, j - 1, k)] > 1.1 &&
              l[IX(dc, i, j, k + 1)] + l[IX(dc, i, j, k - 1)] > 1.1)
            l[t] = 1.;
        }
      }
  memcpy(nvert_c, l, sizeof(double) * (size_t)mx * my * mz);
  free(l);
}

/* MyRestriction (Source/poisson.c:365-472): f_c = 1/8 * sum over the
 * children of x_f * max(0, 1 - nvert_f); zero on blanked coarse cells. */
void or_my_restriction(const or_dims *dc, const or_dims *df, int isc, int jsc, int ksc,
                       const double *nvert_c, const double *nvert_f, const double *xf, double *fc)
{
  const int mx = dc->mx, my = dc->my, mz = dc->mz;
  const int ia = isc ? 0 : 1, ja = jsc ? 0 : 1, ka = ksc ? 0 : 1;
#define X(i, j, k) xf[IX(df, i, j, k)]
#define W(i, j, k) (1 - nvert_f[IX(df, i, j, k)] > 0. ? 1 - nvert_f[IX(df, i, j, k)] : 0.)
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t t = IX(dc, i, j, k);
        if (k == 0 || k == mz - 1 || j == 0 || j == my - 1 || i == 0 || i == mx - 1) {
          fc[t] = 0.;
          continue;
        }
        int ih = isc ? i : 2 * i, jh = jsc ? j : 2 * j, kh = ksc ? k : 2 * k;
        fc[t] = 0.125 * (X(ih, jh, kh) * W(ih, jh, kh) + X(ih - ia, jh, kh) * W(ih - ia, jh, kh) +
                         X(ih, jh - ja, kh) * W(ih, jh - ja, kh) + X(ih, jh, kh - ka) * W(ih, jh, kh - ka) +
                         X(ih - ia, jh - ja, kh) * W(ih - ia, jh - ja, kh) +
                         X(ih, jh - ja, kh - ka) * W(ih, jh - ja, kh - ka) +
                         X(ih - ia, jh, kh - ka) * W(ih - ia, jh, kh - ka) +
                         X(ih - ia, jh - ja, kh - ka) * W(ih - ia, jh - ja, kh - ka));
        if (nvert_c[t] > 0.1) fc[t] = 0.;
      }
#undef X
#undef W
}

/* MyInterpolation (Source/poisson.c:527-670) with the GridInterpolation
 * macro (poisson.c:474-507): trilinear (3/4, 1/4) weights, one-sided next
 * to boundaries and blanked coarse neighbours. */
void or_my_interpolation(const or_dims *df, const or_dims *dc, int isc, int jsc, int ksc,
                         const double *nvert_f, const double *nvert_c, const double *xc, double *ff)
{
  const int mx = df->mx, my = df->my, mz = df->mz;
#define XC(i, j, k) xc[IX(dc, i, j, k)]
#define NC(i, j, k) nvert_c[IX(dc, i, j, k)]
  memset(ff, 0, sizeof(double) * (size_t)mx * my * mz);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        int ic, jc, kc, ia, ja, ka;
        if (isc) { ic = i; ia = 0; }
        else { ic = (i + 1) / 2; ia = (i - 2 * ic) == 0 ? 1 : -1; if (i == 1 || i == mx - 2) ia = 0; }
        if (jsc) { jc = j; ja = 0; }
        else { jc = (j + 1) / 2; ja = (j - 2 * jc) == 0 ? 1 : -1; if (j == 1 || j == my - 2) ja = 0; }
        if (ksc) { kc = k; ka = 0; }
        else { kc = (k + 1) / 2; ka = (k - 2 * kc) == 0 ? 1 : -1; if (k == 1 || k == mz - 2) ka = 0; }
        if (ka == -1 && NC(ic, jc, kc - 1) > 0.1) ka = 0;
        else if (ka == 1 && NC(ic, jc, kc + 1) > 0.1) ka = 0;
        if (ja == -1 && NC(ic, jc - 1, kc) > 0.1) ja = 0;
        else if (ja == 1 && NC(ic, jc + 1, kc) > 0.1) ja = 0;
        if (ia == -1 && NC(ic - 1, jc, kc) > 0.1) ia = 0;
        else if (ia == 1 && NC(ic + 1, jc, kc) > 0.1) ia = 0;
        ff[IX(df, i, j, k)] = (XC(ic, jc, kc) * 9 + XC(ic, jc + ja, kc) * 3 + XC(ic + ia, jc, kc) * 3 +
                               XC(ic + ia, jc + ja, kc)) * 3. / 64. +
                              (XC(ic, jc, kc + ka) * 9 + XC(ic, jc + ja, kc + ka) * 3 +
                               XC(ic + ia, jc, kc + ka) * 3 + XC(ic + ia, jc + ja, kc + ka)) / 64.;
      }
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t t = IX(df, i, j, k);
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1) ff[t] = 0.;
        if (nvert_f[t] > 0.1) ff[t] = 0.;
      }
#undef XC
#undef NC
}

void or_stencil_apply(const or_dims *d, const int *rowtype, const double *vol, const double *x,
                      double *y)
{
  /* y = A x on the DA layout; x must carry its periodic ghost copies. */
  static const int off[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                 {0, 0, 1},  {0, 0, -1}, {1, 1, 0},  {1, -1, 0}, {-1, 1, 0},
                                 {-1, -1, 0}, {0, 1, 1},  {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
                                 {1, 0, 1},  {1, 0, -1}, {-1, 0, 1}, {-1, 0, -1}};
  const int mx = d->mx, my = d->my, mz = d->mz;
  memset(y, 0, sizeof(double) * (size_t)mx * my * mz);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (rowtype[t] == OR_ROW_NONE) continue;
        double s = 0;
        for (int q = 0; q < 19; q++)
          s += vol[t * 19 + q] * x[IX(d, i + off[q][0], j + off[q][1], k + off[q][2])];
        y[t] = s;
      }
}

/* VolumeFlux, the immersed == 1 variant (Source/poisson.c:3563-3903): the
 * net flux through the faces between fluid cells and IB cells (0.1 < nvert
 * < 1.1) is removed.  Faces with |U| <= 1e-8 are zeroed; the correction is
 * (flux + flux_intp_sum) / sum|U|(/|metric|) for flg 2 / 3, (flux +
 * flux_intp_sum) / area for flg 1 and flux / area for flg 0, spread by the
 * face area (flg 0, 1), |U| (flg 2) or |U| / area (flg 3); fluid-side
 * faces lose it, IB-side faces gain it.  out[0..1]: the flux and area
 * after the correction (the reference's ibm_Flux, ibm_Area). */
void or_volume_flux(const or_dims *d, const double *nvert, const double *csi, const double *eta, const double *zet,
                    double *ucont, int flg, double flux_intp_sum, double *out)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const double eps = 1.e-8, ibmval = 1.1;
  const double *met[3] = {csi, eta, zet};
  double flux = 0, flux_abs = 0, area = 0;
  for (int pass = 0; pass < 3; pass++) {
    double corr = 0;
    if (pass == 1) {
      if (area > 1.e-15) {
        if (flg > 1) corr = (flux + flux_intp_sum) / flux_abs;
        else if (flg) corr = (flux + flux_intp_sum) / area;
        else corr = flux / area;
      }
    }
    if (pass == 2) { flux = 0; area = 0; }
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++) {
          const size_t t = IX(d, i, j, k);
          const size_t nb[3] = {IX(d, i + 1, j, k), IX(d, i, j + 1, k), IX(d, i, j, k + 1)};
          const int inside[3] = {i < mx - 2, j < my - 2, k < mz - 2};
          for (int s = 0; s < 2; s++) {   /* s 0: fluid cell, s 1: IB cell */
            if (s == 0 && !(nvert[t] < 0.1)) continue;
            if (s == 1 && !(nvert[t] > 0.1 && nvert[t] < ibmval)) continue;
            for (int q = 0; q < 3; q++) {
              const double nn = nvert[nb[q]];
              const int face = s == 0 ? (nn > 0.1 && nn < ibmval) : (nn < 0.1);
              if (!face || !inside[q]) continue;
              double *u = &ucont[t * 3 + q];
              const double *m = &met[q][t * 3];
              const double a = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
              if (pass == 0) {
                if (fabs(*u) > eps) {
                  flux += s == 0 ? *u : -*u;
                  flux_abs += flg == 3 ? fabs(*u) / a : fabs(*u);
                  area += a;
                } else {
                  *u = 0.;
                }
              } else if (pass == 1) {
                if (fabs(*u) > eps) {
                  double dlt;
                  if (flg == 3) dlt = corr * fabs(*u) / a;
                  else if (flg == 2) dlt = corr * fabs(*u);
                  else dlt = a * corr;
                  if (s == 0) *u -= dlt;
                  else *u += dlt;
                }
              } else {
                flux += s == 0 ? *u : -*u;
                area += a;
              }
            }
          }
        }
  }
  out[0] = flux;
  out[1] = area;
}

/* VolumeFlux, the overload PoissonSolver_Hypre calls when immersed is not 1
 * or 2 (Source/poisson.c:3299-3493, called at poisson_hypre.c:561 with the
 * global Ucont): over the interior cells in k, j, i order, the faces between
 * a fluid cell (nvert < 0.1) and a blanked one (nvert > 0.1), in either
 * order, add +-U to the flux and |csi|, |eta| or |zet| of the cell (the
 * cell metric) to the area; the correction flux / area (0 if the area is at
 * most 1e-15) is taken off the fluid side and added to the blanked side,
 * and with immersed 0 or 3 those faces are then zeroed; immersed 2 applies
 * nothing.  out[0..1]: the sums formed again afterwards. */
void or_volume_flux0(const or_dims *d, const double *nvert, const double *csi, const double *eta,
                     const double *zet, double *ucont, int immersed, double *out)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const double thr = 0.1;
  const double *met[3] = {csi, eta, zet};
  double flux = 0, area = 0;
  for (int pass = 0; pass < 3; pass++) {
    double corr = 0;
    if (pass == 1) {
      if (area > 1.e-15) corr = flux / area;
      if (immersed == 2) continue;
    }
    if (pass == 2) { flux = 0; area = 0; }
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++) {
          const size_t t = IX(d, i, j, k);
          const size_t nb[3] = {IX(d, i + 1, j, k), IX(d, i, j + 1, k), IX(d, i, j, k + 1)};
          for (int s = 0; s < 2; s++) {  /* s 0: fluid cell, s 1: blanked cell */
            if (s == 0 && !(nvert[t] < thr)) continue;
            if (s == 1 && !(nvert[t] > thr)) continue;
            for (int q = 0; q < 3; q++) {
              const double nn = nvert[nb[q]];
              if (s == 0 ? !(nn > thr) : !(nn < thr)) continue;
              double *u = &ucont[t * 3 + q];
              const double *m = &met[q][t * 3];
              const double a = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
              if (pass == 1) {
                if (s == 0) *u -= a * corr;
                else *u += a * corr;
                if (immersed == 3 || !immersed) *u = 0;
              } else {
                if (s == 0) flux += *u;
                else flux -= *u;
                area += a;
              }
            }
          }
        }
  }
  out[0] = flux;
  out[1] = area;
}

/* Contra2Cart (Source/rhs.c:35-749), its change of basis: periodic ghost
 * values of Ucont are taken from the partner cells (:122-155); on fluid
 * cells the centred face-flux averages q are turned into Cartesian
 * velocity by Cramer's rule with the cell metrics csi, eta, zet (:160-240);
 * the periodic ghosts of Ucat take their partners' values (:256-283); with
 * zero_solid, cells with (int)(nvert + 0.1) == 3 get 0 (:304-307).  The
 * wall-function and boundary-condition parts of the reference routine are
 * momentum-solver physics and are not restated.  ucat in/out. */
void or_contra2cart(const or_dims *d, const double *nvert, const double *csi, const double *eta, const double *zet,
                    const double *ucont, double *ucat, int zero_solid)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const int ip = per_i(d), jp = per_j(d), kp = per_k(d);
  const size_t N = (size_t)mx * my * mz;
  double *lu = (double *)malloc(sizeof(double) * 3 * N);
  memcpy(lu, ucont, sizeof(double) * 3 * N);
  if (ip || jp || kp)
    for (int k = 0; k < mz; k++)
      for (int j = 0; j < my; j++)
        for (int i = 0; i < mx; i++) {
          int a = i, b = j, c = k, flag = 0;
          if (ip && i == 0) a = mx - 2, flag = 1; else if (ip && i == mx - 1) a = 1, flag = 1;
          if (jp && j == 0) b = my - 2, flag = 1; else if (jp && j == my - 1) b = 1, flag = 1;
          if (kp && k == 0) c = mz - 2, flag = 1; else if (kp && k == mz - 1) c = 1, flag = 1;
          if (flag) for (int q = 0; q < 3; q++) lu[IX(d, i, j, k) * 3 + q] = lu[IX(d, a, b, c) * 3 + q];
        }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t t = IX(d, i, j, k);
        if (!(nvert[t] < 0.1)) continue;
        const double *c0 = &csi[t * 3], *e0 = &eta[t * 3], *z0 = &zet[t * 3];
        double m[3][3] = {{c0[0], c0[1], c0[2]}, {e0[0], e0[1], e0[2]}, {z0[0], z0[1], z0[2]}};
        double q0 = 0.5 * (lu[IX(d, i - 1, j, k) * 3 + 0] + lu[t * 3 + 0]);
        double q1 = 0.5 * (lu[IX(d, i, j - 1, k) * 3 + 1] + lu[t * 3 + 1]);
        double q2 = 0.5 * (lu[IX(d, i, j, k - 1) * 3 + 2] + lu[t * 3 + 2]);
        double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                     m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                     m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        double det0 = q0 * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                      q1 * (m[0][1] * m[2][2] - m[0][2] * m[2][1]) +
                      q2 * (m[0][1] * m[1][2] - m[0][2] * m[1][1]);
        double det1 = -q0 * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                      q1 * (m[0][0] * m[2][2] - m[0][2] * m[2][0]) -
                      q2 * (m[0][0] * m[1][2] - m[0][2] * m[1][0]);
        double det2 = q0 * (m[1][0] * m[2][1] - m[1][1] * m[2][0]) -
                      q1 * (m[0][0] * m[2][1] - m[0][1] * m[2][0]) +
                      q2 * (m[0][0] * m[1][1] - m[0][1] * m[1][0]);
        ucat[t * 3 + 0] = det0 / det;
        ucat[t * 3 + 1] = det1 / det;
        ucat[t * 3 + 2] = det2 / det;
      }
  if (ip || jp || kp)
    for (int k = 0; k < mz; k++)
      for (int j = 0; j < my; j++)
        for (int i = 0; i < mx; i++) {
          int a = i, b = j, c = k, flag = 0;
          if (ip && i == 0) a = mx - 2, flag = 1; else if (ip && i == mx - 1) a = 1, flag = 1;
          if (jp && j == 0) b = my - 2, flag = 1; else if (jp && j == my - 1) b = 1, flag = 1;
          if (kp && k == 0) c = mz - 2, flag = 1; else if (kp && k == mz - 1) c = 1, flag = 1;
          if (flag) for (int q = 0; q < 3; q++) ucat[IX(d, i, j, k) * 3 + q] = ucat[IX(d, a, b, c) * 3 + q];
        }
  if (zero_solid)
    for (size_t t = 0; t < N; t++)
      if ((int)(nvert[t] + 0.1) == 3) ucat[t * 3] = ucat[t * 3 + 1] = ucat[t * 3 + 2] = 0.;
  free(lu);
}
