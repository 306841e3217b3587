/*
 * ibm_interp_oracle.c -- CPU restatement of VFS-Wind's immersed-boundary
 * velocity reconstruction:
 *   - the interpolation records of the IB nodes, built by
 *     ibm_search_advanced (Source/ibm.c:373-508) from nearestcell1
 *     (:1373-1518, with BoundingSphere :1282-1370) and InterceptionPoint
 *     (:1766-2258, ICP :1666-1764), with compgeom.c's ISPointInTriangle,
 *     ISInsideTriangle2D, ISSameSide2D, Dis_P_Line, triangle_intp and
 *     triangle_intp2 (:62-240);
 *   - ibm_interpolation_advanced (Source/ibm.c:3301-3640) with noslip
 *     (Source/wallfunction.c:140-156): the velocity and pressure of every IB
 *     node from the wall and the fluid cells along the wall normal, the face
 *     fluxes around the IB nodes, then Contra2Cart (rhs.c:35);
 *   - IB_BC (Source/momentum.c:2016-2220): the same face fluxes from a
 *     given ucat plus the wall, slip and periodic face rules.
 *
 * TEST INFRASTRUCTURE ONLY (checker).  Parity unpinned like the rest of the
 * oracle: the reference ships no IB interpolation fixtures.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "vfs_oracle.h"

#define IX(d, i, j, k) ((size_t)(((size_t)(k) * (size_t)(d)->my + (size_t)(j)) * (size_t)(d)->mx + (size_t)(i)))

typedef struct { double x, y, z; } v3;
typedef struct { double x, y; } v2;

static v3 vat(const double *a, size_t t) { v3 r = {a[3 * t], a[3 * t + 1], a[3 * t + 2]}; return r; }
/* Dist (ibm.c:35) */
static double dist(v3 a, v3 b) { return sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (a.z - b.z) * (a.z - b.z)); }

/* BoundingSphere (ibm.c:1282-1370): per element, the circumcentre-based
 * sphere through the longest edge's end points. */
void or_bounding_sphere(int n_elmt, const int *nv, const double *x, const double *y, const double *z, double *q,
                        double *rad)
{
  v3 p0 = {0., 0., 0.};
  for (int e = 0; e < n_elmt; e++) {
    int n1 = nv[3 * e], n2 = nv[3 * e + 1], n3 = nv[3 * e + 2];
    v3 p1 = {x[n1], y[n1], z[n1]}, p2 = {x[n2], y[n2], z[n2]}, p3 = {x[n3], y[n3], z[n3]};
    double l12 = dist(p1, p2), l23 = dist(p2, p3), l31 = dist(p3, p1);
    v3 pa, pb, pc;
    if (l12 > l23) {
      if (l12 > l31) { pa = p1; pb = p2; pc = p3; }
      else { pa = p3; pb = p1; pc = p2; }
    } else {
      if (l31 < l23) { pa = p2; pb = p3; pc = p1; }
      else { pa = p3; pb = p1; pc = p2; }
    }
    v3 pf = {0.5 * (pa.x + pb.x), 0.5 * (pa.y + pb.y), 0.5 * (pa.z + pb.z)};
    v3 pu = {pa.x - pf.x, pa.y - pf.y, pa.z - pf.z};
    v3 pv = {pc.x - pf.x, pc.y - pf.y, pc.z - pf.z};
    v3 pt = {pu.y * pv.z - pu.z * pv.y, pu.z * pv.x - pu.x * pv.z, pu.x * pv.y - pu.y * pv.x};
    v3 pd = {pt.y * pu.z - pt.z * pu.y, pt.z * pu.x - pt.x * pu.z, pt.x * pu.y - pt.y * pu.x};
    double gama = -(dist(pu, p0) * dist(pu, p0) - dist(pv, p0) * dist(pv, p0));
    v3 pw = {pv.x - pu.x, pv.y - pu.y, pv.z - pu.z};
    double lamda = 2 * (pd.x * pw.x + pd.y * pw.y + pd.z * pw.z);
    gama /= lamda;
    lamda = gama < 0 ? 0 : gama;
    q[3 * e] = pf.x + lamda * pd.x;
    q[3 * e + 1] = pf.y + lamda * pd.y;
    q[3 * e + 2] = pf.z + lamda * pd.z;
    v3 qq = {q[3 * e], q[3 * e + 1], q[3 * e + 2]};
    rad[e] = dist(qq, pa);
  }
}

/* ISSameSide2D (compgeom.c:62-114; the t3 branch does not reach the result) */
static int same_side(v2 p, v2 p1, v2 p2, v2 p3)
{
  const double epsilon = 1.e-10;
  double t1 = (p.x - p1.x) * (p2.y - p1.y) - (p.y - p1.y) * (p2.x - p1.x);
  double t2 = (p3.x - p1.x) * (p2.y - p1.y) - (p3.y - p1.y) * (p2.x - p1.x);
  double lt = sqrt((p1.x - p2.x) * (p1.x - p2.x) + (p1.y - p2.y) * (p1.y - p2.y));
  if (fabs(t1 / lt) < epsilon) return 1;
  if (t1 > 0) return t2 > 0 ? 1 : -1;
  return t2 < 0 ? 1 : -1;
}
/* ISInsideTriangle2D (compgeom.c:116-137) */
static int inside_2d(v2 p, v2 pa, v2 pb, v2 pc)
{
  int ls = same_side(p, pa, pb, pc);
  if (ls < 0) return ls;
  ls = same_side(p, pb, pc, pa);
  if (ls < 0) return ls;
  return same_side(p, pc, pa, pb);
}
/* ISPointInTriangle (compgeom.c:139-166) */
static int point_in_triangle(v3 p, v3 p1, v3 p2, v3 p3, double nfx, double nfy, double nfz)
{
  v2 a, b, c, e;
  if (fabs(nfz) >= fabs(nfx) && fabs(nfz) >= fabs(nfy)) {
    a.x = p.x; a.y = p.y; b.x = p1.x; b.y = p1.y; c.x = p2.x; c.y = p2.y; e.x = p3.x; e.y = p3.y;
  } else if (fabs(nfx) >= fabs(nfy) && fabs(nfx) >= fabs(nfz)) {
    a.x = p.z; a.y = p.y; b.x = p1.z; b.y = p1.y; c.x = p2.z; c.y = p2.y; e.x = p3.z; e.y = p3.y;
  } else {
    a.x = p.x; a.y = p.z; b.x = p1.x; b.y = p1.z; c.x = p2.x; c.y = p2.z; e.x = p3.x; e.y = p3.z;
  }
  return inside_2d(a, b, c, e);
}
/* Dis_P_Line (compgeom.c:168-194) */
static void dist_point_line(v3 p, v3 p1, v3 p2, v3 *po, double *d)
{
  double dx21 = p2.x - p1.x, dy21 = p2.y - p1.y, dz21 = p2.z - p1.z;
  double dx31 = p.x - p1.x, dy31 = p.y - p1.y, dz31 = p.z - p1.z;
  double t = (dx31 * dx21 + dy31 * dy21 + dz31 * dz21) / (dx21 * dx21 + dy21 * dy21 + dz21 * dz21);
  if (t < 0) {
    *po = p1;
    *d = sqrt(dx31 * dx31 + dy31 * dy31 + dz31 * dz31);
  } else if (t > 1) {
    *po = p2;
    *d = sqrt((p.x - po->x) * (p.x - po->x) + (p.y - po->y) * (p.y - po->y) + (p.z - po->z) * (p.z - po->z));
  } else {
    po->x = p1.x + t * dx21; po->y = p1.y + t * dy21; po->z = p1.z + t * dz21;
    *d = sqrt((p.x - po->x) * (p.x - po->x) + (p.y - po->y) * (p.y - po->y) + (p.z - po->z) * (p.z - po->z));
  }
}
/* triangle_intp / triangle_intp2 (compgeom.c:196-230): barycentric weights */
static void bary(v2 p, v2 p1, v2 p2, v2 p3, double w[3])
{
  double x13 = p1.x - p3.x, y13 = p1.y - p3.y;
  double x23 = p2.x - p3.x, y23 = p2.y - p3.y;
  double xp3 = p.x - p3.x, yp3 = p.y - p3.y;
  double a = x13 * y23 - x23 * y13;
  w[0] = (y23 * xp3 - x23 * yp3) / a;
  w[1] = (-y13 * xp3 + x13 * yp3) / a;
  w[2] = 1. - w[0] - w[1];
}
/* the 2-D projection both barycentric callers use, by the dominant normal */
static void project_bary(v3 p, v3 p1, v3 p2, v3 p3, double nfx, double nfy, double nfz, double w[3])
{
  v2 a, b, c, e;
  if (fabs(nfx) >= fabs(nfy) && fabs(nfx) >= fabs(nfz)) {
    a.x = p.y; a.y = p.z; b.x = p1.y; b.y = p1.z; c.x = p2.y; c.y = p2.z; e.x = p3.y; e.y = p3.z;
  } else if (fabs(nfy) >= fabs(nfx) && fabs(nfy) >= fabs(nfz)) {
    a.x = p.x; a.y = p.z; b.x = p1.x; b.y = p1.z; c.x = p2.x; c.y = p2.z; e.x = p3.x; e.y = p3.z;
  } else if (fabs(nfz) >= fabs(nfy) && fabs(nfz) >= fabs(nfx)) {
    a.x = p.y; a.y = p.x; b.x = p1.y; b.y = p1.x; c.x = p2.y; c.y = p2.x; e.x = p3.y; e.y = p3.x;
  } else {
    return;  /* a NaN normal: the reference leaves the weights unchanged */
  }
  bary(a, b, c, e, w);
}

/* nearestcell1 (ibm.c:1373-1518) */
static void nearest_element(v3 p, int n_elmt, const int *nv, const double *x, const double *y, const double *z,
                            const double *nf, const double *q, const double *rad, or_ibm_node *nd)
{
  double dmin = 1.e20;
  int cell_min = -100;
  v3 pmin = {0., 0., 0.};
  for (int e = 0; e < n_elmt; e++) {
    v3 qe = {q[3 * e], q[3 * e + 1], q[3 * e + 2]};
    double d_center = dist(p, qe);
    if (!(d_center - rad[e] < dmin)) continue;
    int n1 = nv[3 * e], n2 = nv[3 * e + 1], n3 = nv[3 * e + 2];
    double nfx = nf[3 * e], nfy = nf[3 * e + 1], nfz = nf[3 * e + 2];
    v3 p1 = {x[n1], y[n1], z[n1]}, p2 = {x[n2], y[n2], z[n2]}, p3 = {x[n3], y[n3], z[n3]};
    double tf = (p.x - x[n1]) * nfx + (p.y - y[n1]) * nfy + (p.z - z[n1]) * nfz;
    if (fabs(tf) < 1.e-10) tf = 1.e-10;
    if (!(tf >= 0)) continue;
    v3 pj = {p.x - tf * nfx, p.y - tf * nfy, p.z - tf * nfz};
    if (point_in_triangle(pj, p1, p2, p3, nfx, nfy, nfz) == 1) {
      if (tf < dmin) { dmin = tf; pmin = pj; cell_min = e; }
    } else {
      v3 po;
      double d;
      dist_point_line(p, p1, p2, &po, &d);
      if (d < dmin) { dmin = d; pmin = po; cell_min = e; }
      dist_point_line(p, p2, p3, &po, &d);
      if (d < dmin) { dmin = d; pmin = po; cell_min = e; }
      dist_point_line(p, p3, p1, &po, &d);
      if (d < dmin) { dmin = d; pmin = po; cell_min = e; }
    }
  }
  nd->cell = cell_min;
  nd->pmin[0] = pmin.x; nd->pmin[1] = pmin.y; nd->pmin[2] = pmin.z;
  nd->d_s = dmin;
  nd->cs[0] = nd->cs[1] = nd->cs[2] = 0.;
  if (cell_min < 0) return;  /* the reference exits here ("Nearest Cell Searching Error") */
  int n1 = nv[3 * cell_min], n2 = nv[3 * cell_min + 1], n3 = nv[3 * cell_min + 2];
  v3 p1 = {x[n1], y[n1], z[n1]}, p2 = {x[n2], y[n2], z[n2]}, p3 = {x[n3], y[n3], z[n3]};
  project_bary(pmin, p1, p2, p3, nf[3 * cell_min], nf[3 * cell_min + 1], nf[3 * cell_min + 2], nd->cs);
}

/* ICP (ibm.c:1666-1764) on one 3x3 patch of cell centres; the triangle
 * index (0-7) or -100; *_w, *d_i set on success */
static const int kTri[8][3] = {{0, 1, 4}, {1, 2, 4}, {2, 4, 5}, {4, 5, 8}, {4, 7, 8}, {4, 6, 7}, {3, 4, 6}, {3, 4, 0}};
static int icp(v3 p, const v3 pc[9], double nfx, double nfy, double nfz, double w[3], double *d_i)
{
  for (int t = 0; t < 8; t++) {
    v3 p1 = pc[kTri[t][0]], p2 = pc[kTri[t][1]], p3 = pc[kTri[t][2]];
    double dx1 = p.x - p1.x, dy1 = p.y - p1.y, dz1 = p.z - p1.z;
    double dx2 = p2.x - p1.x, dy2 = p2.y - p1.y, dz2 = p2.z - p1.z;
    double dx3 = p3.x - p1.x, dy3 = p3.y - p1.y, dz3 = p3.z - p1.z;
    double d = (nfx * (dy2 * dz3 - dz2 * dy3) - nfy * (dx2 * dz3 - dz2 * dx3) + nfz * (dx2 * dy3 - dy2 * dx3));
    if (!(fabs(d) > 1.e-10)) continue;
    d = -(dx1 * (dy2 * dz3 - dz2 * dy3) - dy1 * (dx2 * dz3 - dz2 * dx3) + dz1 * (dx2 * dy3 - dy2 * dx3)) / d;
    if (!(d > 0)) continue;
    v3 pint = {p.x + d * nfx, p.y + d * nfy, p.z + d * nfz};
    double rx1 = p2.x - p1.x, ry1 = p2.y - p1.y, rz1 = p2.z - p1.z;
    double rx2 = p3.x - p1.x, ry2 = p3.y - p1.y, rz2 = p3.z - p1.z;
    double nfxt = ry1 * rz2 - rz1 * ry2;
    double nfyt = -rx1 * rz2 + rz1 * rx2;
    double nfzt = rx1 * ry2 - ry1 * rx2;
    if (point_in_triangle(pint, p1, p2, p3, nfxt, nfyt, nfzt) >= 0) {
      project_bary(pint, p1, p2, p3, nfxt, nfyt, nfzt, w);
      *d_i = sqrt((pint.x - p.x) * (pint.x - p.x) + (pint.y - p.y) * (pint.y - p.y) + (pint.z - p.z) * (pint.z - p.z));
      return t;
    }
  }
  return -100;
}

/* InterceptionPoint (ibm.c:1766-2258): the ray from the node away from the
 * surface's nearest point, against the patches of the neighbouring cell
 * centres at i-1, i+1, j-1, j+1, k-1, k+1 in turn */
static void interception(const or_dims *d, const double *cent, int i, int j, int k, or_ibm_node *nd)
{
  v3 p = vat(cent, IX(d, i, j, k));
  double nfx = p.x - nd->pmin[0], nfy = p.y - nd->pmin[1], nfz = p.z - nd->pmin[2];
  double dr = sqrt(nfx * nfx + nfy * nfy + nfz * nfz);
  nfx /= dr; nfy /= dr; nfz /= dr;
  nd->imode = -100;
  for (int face = 0; face < 6; face++) {
    int ip[9], jp[9], kp[9];
    for (int s = 0; s < 9; s++) {
      const int a = s % 3 - 1, b = s / 3 - 1;  /* in-patch offsets */
      switch (face) {
        case 0: ip[s] = i - 1; jp[s] = j + a; kp[s] = k + b; break;
        case 1: ip[s] = i + 1; jp[s] = j + a; kp[s] = k + b; break;
        case 2: ip[s] = i + a; jp[s] = j - 1; kp[s] = k + b; break;
        case 3: ip[s] = i + a; jp[s] = j + 1; kp[s] = k + b; break;
        case 4: ip[s] = i + a; jp[s] = j + b; kp[s] = k - 1; break;
        default: ip[s] = i + a; jp[s] = j + b; kp[s] = k + 1; break;
      }
    }
    v3 pc[9];
    for (int s = 0; s < 9; s++) pc[s] = vat(cent, IX(d, ip[s], jp[s], kp[s]));
    double w[3] = {0., 0., 0.}, di = 0.;
    const int t = icp(p, pc, nfx, nfy, nfz, w, &di);
    if (t >= 0) {
      nd->imode = t;
      for (int q = 0; q < 3; q++) {
        const int s = kTri[t][q];
        nd->ip[q] = ip[s]; nd->jp[q] = jp[s]; nd->kp[q] = kp[s];
        nd->cr[q] = w[q];
      }
      nd->d_i = di;
      return;
    }
  }
}

/* The IB nodes of one body -- the cells marked 2 (IB node) in nvert after
 * the dilation, in the reference's k, j, i order -- with their
 * interpolation records (ibm.c:373-508).  Returns the node count (at most
 * max_nodes are written). */
int or_ibm_nodes(const or_dims *d, const double *cent, const double *nvert_marked, int n_v, const double *x,
                 const double *y, const double *z, int n_elmt, const int *nv, or_ibm_node *nodes, int max_nodes)
{
  (void)n_v;
  const int mx = d->mx, my = d->my, mz = d->mz;
  double *nf = (double *)malloc(sizeof(double) * 3 * (n_elmt > 0 ? n_elmt : 1));
  double *q = (double *)malloc(sizeof(double) * 3 * (n_elmt > 0 ? n_elmt : 1));
  double *rad = (double *)malloc(sizeof(double) * (n_elmt > 0 ? n_elmt : 1));
  or_triangle_normals(n_elmt, nv, x, y, z, nf);
  or_bounding_sphere(n_elmt, nv, x, y, z, q, rad);
  int count = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        if ((int)(nvert_marked[IX(d, i, j, k)] + 0.5) != 2) continue;
        or_ibm_node nd;
        memset(&nd, 0, sizeof nd);
        nd.i = i; nd.j = j; nd.k = k;
        nearest_element(vat(cent, IX(d, i, j, k)), n_elmt, nv, x, y, z, nf, q, rad, &nd);
        interception(d, cent, i, j, k, &nd);
        if (nd.imode < 0) {
          /* next to an i or j boundary: the k neighbour on the normal's z
           * side; next to a k boundary: the j+1 neighbour (ibm.c:423-505) */
          int di = 0, dj = 0, dk = 0;
          if (i == 1 || i == mx - 2 || j == 1 || j == my - 2) {
            dk = (nd.cell >= 0 && nf[3 * nd.cell + 2] > 0) ? 1 : -1;
            nd.status = 1;
          } else if (k == 1 || k == mz - 2) {
            dj = 1;
            nd.status = 1;
          } else {
            nd.status = 2;  /* "IBM Searching Fail": the reference keeps the previous node's values */
          }
          if (nd.status == 1) {
            v3 c0 = vat(cent, IX(d, i, j, k)), c1 = vat(cent, IX(d, i + di, j + dj, k + dk));
            nd.d_i = sqrt((c0.x - c1.x) * (c0.x - c1.x) + (c0.y - c1.y) * (c0.y - c1.y) + (c0.z - c1.z) * (c0.z - c1.z));
            nd.cr[0] = 1.; nd.cr[1] = 0.; nd.cr[2] = 0.;
            for (int s = 0; s < 3; s++) { nd.ip[s] = i + di; nd.jp[s] = j + dj; nd.kp[s] = k + dk; }
          } else {
            for (int s = 0; s < 3; s++) { nd.ip[s] = i; nd.jp[s] = j; nd.kp[s] = k; nd.cr[s] = 0.; }
            nd.d_i = 0.;
          }
        }
        if (count < max_nodes) nodes[count] = nd;
        count++;
      }
  free(nf); free(q); free(rad);
  return count;
}

/* the periodic ghost planes of a DA Cmpnts field take their partners'
 * values (a DAGlobalToLocal of a periodic DA, as Contra2Cart's input) */
static void ghost_fill3(const or_dims *d, double *u)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const int ip = d->i_periodic || d->ii_periodic, jp = d->j_periodic || d->jj_periodic,
            kp = d->k_periodic || d->kk_periodic;
  if (!(ip || jp || kp)) return;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a = i, b = j, c = k, flag = 0;
        if (ip && i == 0) a = mx - 2, flag = 1; else if (ip && i == mx - 1) a = 1, flag = 1;
        if (jp && j == 0) b = my - 2, flag = 1; else if (jp && j == my - 1) b = 1, flag = 1;
        if (kp && k == 0) c = mz - 2, flag = 1; else if (kp && k == mz - 1) c = 1, flag = 1;
        if (flag) for (int q = 0; q < 3; q++) u[IX(d, i, j, k) * 3 + q] = u[IX(d, a, b, c) * 3 + q];
      }
}

/* face flux of the face between cells t and t + s (metric m of that face) */
static double face_flux(const double *lu, size_t t, size_t s, const double *m)
{
  double ucx = (lu[t * 3] + lu[s * 3]) * 0.5;
  double ucy = (lu[t * 3 + 1] + lu[s * 3 + 1]) * 0.5;
  double ucz = (lu[t * 3 + 2] + lu[s * 3 + 2]) * 0.5;
  return ucx * m[0] + ucy * m[1] + ucz * m[2];
}

/* ibm_interpolation_advanced (ibm.c:3301-3640) for one body without
 * averaging, level set, moving bodies, inviscid or wall-function options:
 * noslip velocity and interpolated pressure at every IB node, then the face
 * fluxes of the cells with (int)(nvert + 0.5) == 1 and of their +i/+j/+k
 * neighbours' faces (f = 0 with immersed == 3; the -1/-2 wall faces
 * zeroed), then Contra2Cart with the solid zeroing.  u_surf: the surface
 * vertex velocities (n_v x 3) or NULL for a resting body.  ucat, p, ucont:
 * DA arrays, in/out (ucat and p are read as the ghosted local copies). */
void or_ibm_interpolate(const or_dims *d, const double *nvert, const or_ibm_node *nodes, int n_nodes,
                        const int *nv, const double *u_surf, const double *icsi, const double *jeta,
                        const double *kzet, const double *csi, const double *eta, const double *zet,
                        const int *bctype, int immersed, double *ucat, double *p, double *ucont)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t N = (size_t)mx * my * mz;
  double *lu = (double *)malloc(sizeof(double) * 3 * N), *lp = (double *)malloc(sizeof(double) * N);
  memcpy(lu, ucat, sizeof(double) * 3 * N);
  memcpy(lp, p, sizeof(double) * N);
  for (int n = 0; n < n_nodes; n++) {
    const or_ibm_node *nd = &nodes[n];
    const size_t t = IX(d, nd->i, nd->j, nd->k);
    const size_t t1 = IX(d, nd->ip[0], nd->jp[0], nd->kp[0]), t2 = IX(d, nd->ip[1], nd->jp[1], nd->kp[1]),
                 t3 = IX(d, nd->ip[2], nd->jp[2], nd->kp[2]);
    const double sb = nd->d_s, sc = sb + nd->d_i;
    const double sk1 = nd->cr[0], sk2 = nd->cr[1], sk3 = nd->cr[2];
    const double cs1 = nd->cs[0], cs2 = nd->cs[1], cs3 = nd->cs[2];
    double ua[3] = {0., 0., 0.}, uc[3];
    const int ni = nd->cell;
    if (ni >= 0 && u_surf) {
      const int v1 = nv[3 * ni], v2 = nv[3 * ni + 1], v3 = nv[3 * ni + 2];
      for (int q = 0; q < 3; q++) ua[q] = u_surf[3 * v1 + q] * cs1 + u_surf[3 * v2 + q] * cs2 + u_surf[3 * v3 + q] * cs3;
    }
    for (int q = 0; q < 3; q++) uc[q] = (lu[t1 * 3 + q] * sk1 + lu[t2 * 3 + q] * sk2 + lu[t3 * 3 + q] * sk3);
    if (nvert[t1] + nvert[t2] + nvert[t3] > 0.1 || nvert[t] > 2.9) {
      for (int q = 0; q < 3; q++) ucat[t * 3 + q] = 0.;
    } else {  /* noslip (wallfunction.c:140-156) */
      for (int q = 0; q < 3; q++) {
        double uq = uc[q] - ua[q];
        ucat[t * 3 + q] = sb / sc * uq;
        ucat[t * 3 + q] += ua[q];
      }
    }
    p[t] = (lp[t1] * sk1 + lp[t2] * sk2 + lp[t3] * sk3);
  }
  memcpy(lu, ucat, sizeof(double) * 3 * N);
  ghost_fill3(d, lu);
  const double f = immersed == 3 ? 0. : 1.;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t t = IX(d, i, j, k);
        const size_t te = IX(d, i + 1, j, k), tn = IX(d, i, j + 1, k), tt = IX(d, i, j, k + 1);
        if ((int)(nvert[t] + 0.5) == 1) {
          ucont[t * 3] = face_flux(lu, t, te, &icsi[t * 3]) * f;
          ucont[t * 3 + 1] = face_flux(lu, tn, t, &jeta[t * 3]) * f;
          ucont[t * 3 + 2] = face_flux(lu, tt, t, &kzet[t * 3]) * f;
          if (bctype && (bctype[0] == -1 || bctype[0] == -2) && i == 1) ucont[t * 3] = 0;
          if (bctype && (bctype[2] == -1 || bctype[2] == -2) && j == 1) ucont[t * 3 + 1] = 0;
          if (bctype && (bctype[4] == -1 || bctype[4] == -2) && k == 1) ucont[t * 3 + 2] = 0;
        }
        if ((int)(nvert[te] + 0.5) == 1) {
          ucont[t * 3] = face_flux(lu, t, te, &icsi[t * 3]) * f;
          if (bctype && (bctype[1] == -1 || bctype[1] == -2) && i == mx - 3) ucont[t * 3] = 0;
        }
        if ((int)(nvert[tn] + 0.5) == 1) {
          ucont[t * 3 + 1] = face_flux(lu, tn, t, &jeta[t * 3]) * f;
          if (bctype && (bctype[3] == -1 || bctype[3] == -2) && j == my - 3) ucont[t * 3 + 1] = 0;
        }
        if ((int)(nvert[tt] + 0.5) == 1) {
          ucont[t * 3 + 2] = face_flux(lu, tt, t, &kzet[t * 3]) * f;
          if (bctype && (bctype[5] == -1 || bctype[5] == -2) && k == mz - 3) ucont[t * 3 + 2] = 0;
        }
      }
  free(lu); free(lp);
  or_contra2cart(d, nvert, csi, eta, zet, ucont, ucat, 1);
}

/* IB_BC (Source/momentum.c:2016-2220) with immersed set: periodic ghosts of
 * ucat from their partners (in place, as the reference writes them into
 * lUcat), the face fluxes of the cells with (int)nvert == 1 and of their
 * +i/+j/+k neighbours' faces (f = 0 with immersed == 3, and faces between
 * cells whose nvert sum exceeds 1.1 zeroed then), the -1/-2 wall faces, the
 * slip (10) faces and the periodic face copies.  ucat, ucont: DA arrays,
 * in/out.  The first-step wall marking of nvert (immersed == 0) and the
 * air-flow level-set faces are not restated. */
void or_ib_bc(const or_dims *d, const double *nvert, const double *icsi, const double *jeta, const double *kzet,
              const int *bctype, int immersed, double *ucat, double *ucont)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  ghost_fill3(d, ucat);
  const double f = immersed == 3 ? 0. : 1.;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        const size_t t = IX(d, i, j, k);
        const size_t te = IX(d, i + 1, j, k), tn = IX(d, i, j + 1, k), tt = IX(d, i, j, k + 1);
        if (immersed) {
          if ((int)nvert[t] == 1) {
            ucont[t * 3] = face_flux(ucat, t, te, &icsi[t * 3]) * f;
            ucont[t * 3 + 1] = face_flux(ucat, tn, t, &jeta[t * 3]) * f;
            ucont[t * 3 + 2] = face_flux(ucat, tt, t, &kzet[t * 3]) * f;
          }
          if ((int)(nvert[te]) == 1) ucont[t * 3] = face_flux(ucat, t, te, &icsi[t * 3]) * f;
          if ((int)(nvert[tn]) == 1) ucont[t * 3 + 1] = face_flux(ucat, tn, t, &jeta[t * 3]) * f;
          if ((int)(nvert[tt]) == 1) ucont[t * 3 + 2] = face_flux(ucat, tt, t, &kzet[t * 3]) * f;
          if (immersed == 3) {
            if ((nvert[te] + nvert[t]) > 1.1) ucont[t * 3] = 0;
            if ((nvert[tn] + nvert[t]) > 1.1) ucont[t * 3 + 1] = 0;
            if ((nvert[tt] + nvert[t]) > 1.1) ucont[t * 3 + 2] = 0;
          }
        }
        if (bctype) {
          for (int v = -2; v <= -1; v++) {
            if ((bctype[0] == v && i == 1) || (bctype[1] == v && i == mx - 2)) {
              if (i == 1) ucont[IX(d, i - 1, j, k) * 3] = 0;
              else ucont[t * 3] = 0;
            }
          }
          for (int v = -2; v <= -1; v++) {
            if ((bctype[2] == v && j == 1) || (bctype[3] == v && j == my - 2)) {
              if (j == 1) ucont[IX(d, i, j - 1, k) * 3 + 1] = 0;
              else ucont[t * 3 + 1] = 0;
            }
          }
        }
      }
  const int ip = d->i_periodic, jp = d->j_periodic, kp = d->k_periodic;
  const int iip = d->ii_periodic, jjp = d->jj_periodic, kkp = d->kk_periodic;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        if (bctype) {
          if (bctype[0] == 10 && i == 1) ucont[IX(d, 0, j, k) * 3] = 0;
          if (bctype[1] == 10 && i == mx - 2) ucont[IX(d, mx - 2, j, k) * 3] = 0;
          if (bctype[2] == 10 && j == 1) ucont[IX(d, i, 0, k) * 3 + 1] = 0;
          if (bctype[3] == 10 && j == my - 2) ucont[IX(d, i, my - 2, k) * 3 + 1] = 0;
          if (bctype[4] == 10 && k == 1) ucont[IX(d, i, j, 0) * 3 + 2] = 0;
          if (bctype[5] == 10 && k == mz - 2) ucont[IX(d, i, j, mz - 2) * 3 + 2] = 0;
        }
        /* i/j/k_periodic and the DA-periodic ii/jj/kk flags name the same
         * partner faces on the stored array */
        if ((ip || iip) && i == 0) ucont[IX(d, 0, j, k) * 3] = ucont[IX(d, mx - 2, j, k) * 3];
        if ((ip || iip) && i == mx - 1) ucont[IX(d, mx - 1, j, k) * 3] = ucont[IX(d, 1, j, k) * 3];
        if ((jp || jjp) && j == 0) ucont[IX(d, i, 0, k) * 3 + 1] = ucont[IX(d, i, my - 2, k) * 3 + 1];
        if ((jp || jjp) && j == my - 1) ucont[IX(d, i, my - 1, k) * 3 + 1] = ucont[IX(d, i, 1, k) * 3 + 1];
        if ((kp || kkp) && k == 0) ucont[IX(d, i, j, 0) * 3 + 2] = ucont[IX(d, i, j, mz - 2) * 3 + 2];
        if ((kp || kkp) && k == mz - 1) ucont[IX(d, i, j, mz - 1) * 3 + 2] = ucont[IX(d, i, j, 1) * 3 + 2];
      }
}
