/*
 * ibm_oracle.c -- CPU restatement of VFS-Wind's immersed-boundary node
 * classification (ibm_search_advanced, Source/ibm.c:92-594, with
 * point_cell_advanced :1075-1200, randomdirection :59-91 and
 * intsect_triangle, Source/compgeom.c:25-60).
 *
 * TEST INFRASTRUCTURE ONLY (checker).  Parity unpinned like the rest of the
 * oracle, except for the random numbers: the ray directions use glibc's
 * rand(), restated here from glibc's published algorithm and pinned in the
 * tests against the C library itself.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "vfs_oracle.h"

#define IX(d, i, j, k) ((size_t)(((size_t)(k) * (size_t)(d)->my + (size_t)(j)) * (size_t)(d)->mx + (size_t)(i)))

/* First value of glibc rand() after srand(seed): the TYPE_3 additive
 * feedback generator r[i] = r[i-31] + r[i-3] (mod 2^32), seeded by the
 * Park-Miller LCG r[i] = 16807 r[i-1] mod (2^31 - 1), with r[31..33] =
 * r[0..2] and the first 310 outputs discarded; the output is r[344] >> 1. */
unsigned int or_glibc_rand_first(unsigned int seed)
{
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

/* Face normals as the UCD reader computes them (Source/ibm_io.c:997-1011). */
void or_triangle_normals(int n_elmt, const int *nv, const double *x, const double *y, const double *z,
                         double *nf)
{
  for (int e = 0; e < n_elmt; e++) {
    int n1 = nv[3 * e], n2 = nv[3 * e + 1], n3 = nv[3 * e + 2];
    double dx12 = x[n2] - x[n1], dy12 = y[n2] - y[n1], dz12 = z[n2] - z[n1];
    double dx13 = x[n3] - x[n1], dy13 = y[n3] - y[n1], dz13 = z[n3] - z[n1];
    double fx = dy12 * dz13 - dz12 * dy13;
    double fy = -dx12 * dz13 + dz12 * dx13;
    double fz = dx12 * dy13 - dy12 * dx13;
    double dr = sqrt(fx * fx + fy * fy + fz * fz);
    nf[3 * e] = fx / dr; nf[3 * e + 1] = fy / dr; nf[3 * e + 2] = fz / dr;
  }
}

/* intsect_triangle (Source/compgeom.c:25-60). */
static int intsect(const double orig[3], const double dir[3], const double v0[3], const double v1[3],
                   const double v2[3], double *t, double *u, double *v)
{
  const double EPS = 0.00000001;
  double e1[3], e2[3], tv[3], pv[3], qv[3];
  for (int c = 0; c < 3; c++) { e1[c] = v1[c] - v0[c]; e2[c] = v2[c] - v0[c]; }
  pv[0] = dir[1] * e2[2] - dir[2] * e2[1];
  pv[1] = dir[2] * e2[0] - dir[0] * e2[2];
  pv[2] = dir[0] * e2[1] - dir[1] * e2[0];
  double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  if (det > -EPS && det < EPS) return 0;
  double inv = 1.0 / det;
  for (int c = 0; c < 3; c++) tv[c] = orig[c] - v0[c];
  *u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * inv;
  if (*u < 0.0 || *u > 1.0) return 0;
  qv[0] = tv[1] * e1[2] - tv[2] * e1[1];
  qv[1] = tv[2] * e1[0] - tv[0] * e1[2];
  qv[2] = tv[0] * e1[1] - tv[1] * e1[0];
  *v = (dir[0] * qv[0] + dir[1] * qv[1] + dir[2] * qv[2]) * inv;
  if (*v < 0.0 || *u + *v > 1.0) return 0;
  *t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
  return 1;
}

typedef struct {
  int ncx, ncy, ncz;
  double xmin, ymin, zmin, xmax, ymax, zmax, dcx, dcy, dcz;
  int *head, *next, *tri; /* linked lists per hash cell */
  int nent;
} hashgrid;

/* spatial hash of the triangles over the body box (ibm.c:138-218) */
static void build_hash(hashgrid *H, int n_v, const double *x, const double *y, const double *z, int n_elmt,
                       const int *nv)
{
  H->ncx = H->ncy = H->ncz = 40;
  H->xmin = H->ymin = H->zmin = 1.e23;
  H->xmax = H->ymax = H->zmax = -1.e23;
  for (int i = 0; i < n_v; i++) {
    H->xmin = H->xmin < x[i] ? H->xmin : x[i]; H->xmax = H->xmax > x[i] ? H->xmax : x[i];
    H->ymin = H->ymin < y[i] ? H->ymin : y[i]; H->ymax = H->ymax > y[i] ? H->ymax : y[i];
    H->zmin = H->zmin < z[i] ? H->zmin : z[i]; H->zmax = H->zmax > z[i] ? H->zmax : z[i];
  }
  H->xmin -= 0.05; H->xmax += 0.05;
  H->ymin -= 0.05; H->ymax += 0.05;
  H->zmin -= 0.05; H->zmax += 0.05;
  H->dcx = (H->xmax - H->xmin) / (H->ncx - 1.);
  H->dcy = (H->ymax - H->ymin) / (H->ncy - 1.);
  H->dcz = (H->zmax - H->zmin) / (H->ncz - 1.);
  int ncell = H->ncx * H->ncy * H->ncz;
  H->head = (int *)malloc(sizeof(int) * ncell);
  for (int q = 0; q < ncell; q++) H->head[q] = -1;
  int cap = 1024;
  H->next = (int *)malloc(sizeof(int) * cap);
  H->tri = (int *)malloc(sizeof(int) * cap);
  H->nent = 0;
  for (int e = 0; e < n_elmt; e++) {
    int a = nv[3 * e], b = nv[3 * e + 1], c = nv[3 * e + 2];
    double xv_min = fmin(fmin(x[a], x[b]), x[c]), xv_max = fmax(fmax(x[a], x[b]), x[c]);
    double yv_min = fmin(fmin(y[a], y[b]), y[c]), yv_max = fmax(fmax(y[a], y[b]), y[c]);
    double zv_min = fmin(fmin(z[a], z[b]), z[c]), zv_max = fmax(fmax(z[a], z[b]), z[c]);
    int iv_min = (int)floor((xv_min - H->xmin) / H->dcx), iv_max = (int)floor((xv_max - H->xmin) / H->dcx) + 1;
    int jv_min = (int)floor((yv_min - H->ymin) / H->dcy), jv_max = (int)floor((yv_max - H->ymin) / H->dcy) + 1;
    int kv_min = (int)floor((zv_min - H->zmin) / H->dcz), kv_max = (int)floor((zv_max - H->zmin) / H->dcz) + 1;
    iv_min = iv_min < 0 ? 0 : iv_min; iv_max = iv_max > H->ncx ? H->ncx : iv_max;
    jv_min = jv_min < 0 ? 0 : jv_min; jv_max = jv_max > H->ncx ? H->ncy : jv_max; /* ibm.c:204 */
    kv_min = kv_min < 0 ? 0 : kv_min; kv_max = kv_max > H->ncz ? H->ncz : kv_max;
    for (int k = kv_min; k < kv_max; k++)
      for (int j = jv_min; j < jv_max; j++)
        for (int i = iv_min; i < iv_max; i++) {
          if (H->nent == cap) {
            cap *= 2;
            H->next = (int *)realloc(H->next, sizeof(int) * cap);
            H->tri = (int *)realloc(H->tri, sizeof(int) * cap);
          }
          int q = (k * H->ncy + j) * H->ncx + i;
          H->tri[H->nent] = e;
          H->next[H->nent] = H->head[q];
          H->head[q] = H->nent++;
        }
  }
}

/* point_cell_advanced (ibm.c:1075-1200); returns 4 inside, 0 outside, or
 * -1 when more than `max_tries` rays met a singular intersection. */
static int point_cell(const double p[3], int ip, int jp, int kp, const hashgrid *H, int n_elmt, const int *nv,
                      const double *x, const double *y, const double *z, const double *nf, unsigned char *seen,
                      int max_tries)
{
  for (int searchtimes = 1; searchtimes <= max_tries; searchtimes++) {
    double xpc = H->dcx * (ip + 0.5) + H->xmin, ypc = H->dcy * (jp + 0.5) + H->ymin;
    double s = or_glibc_rand_first((unsigned)searchtimes) / ((double)2147483647 + 1) - 0.5;
    double dir[3] = {xpc + s * H->dcx - p[0], ypc + s * H->dcy - p[1], H->zmax + 0.2 - p[2]};
    double nrm = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    dir[0] /= nrm; dir[1] /= nrm; dir[2] /= nrm;
    memset(seen, 0, (size_t)n_elmt);
    int nintp = 0, singular = 0;
    double dt[1000], dn[1000][3];
    for (int k = kp; k < H->ncz && !singular; k++) {
      for (int q = H->head[(k * H->ncy + jp) * H->ncx + ip]; q >= 0 && !singular; q = H->next[q]) {
        int e = H->tri[q];
        if (seen[e]) continue;
        seen[e] = 1;
        int a = nv[3 * e], b = nv[3 * e + 1], c = nv[3 * e + 2];
        double v0[3] = {x[a], y[a], z[a]}, v1[3] = {x[b], y[b], z[b]}, v2[3] = {x[c], y[c], z[c]};
        double t, u, v;
        int hit = intsect(p, dir, v0, v1, v2, &t, &u, &v);
        if (hit > 0 && t > 0) {
          if (nintp >= 1000) return -1;
          dt[nintp] = t;
          dn[nintp][0] = nf[3 * e]; dn[nintp][1] = nf[3 * e + 1]; dn[nintp][2] = nf[3 * e + 2];
          nintp++;
          for (int m = 0; m < nintp - 1; m++) {
            double ndotn = dn[m][0] * nf[3 * e] + dn[m][1] * nf[3 * e + 1] + dn[m][2] * nf[3 * e + 2];
            if (fabs(t - dt[m]) < 1.e-8 && ndotn > -0.97) singular = 1;
          }
        }
      }
    }
    if (!singular) return (nintp % 2) ? 4 : 0;
  }
  return -1;
}

/* ibm_search_advanced for one body (ibm.c:92-594 without the thin-body and
 * interpolation-stencil parts).  cent: cell centres (DA layout, Cmpnts);
 * nvert: in/out; bctype: the six boundary codes.  Returns the number of
 * cells whose ray search gave up (0 normally). */
int or_ibm_mark(const or_dims *d, const double *cent, int ibi, int n_v, const double *x, const double *y,
                const double *z, int n_elmt, const int *nv, double *nvert, int max_tries)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  hashgrid H;
  build_hash(&H, n_v, x, y, z, n_elmt, nv);
  double *nf = (double *)malloc(sizeof(double) * 3 * (n_elmt > 0 ? n_elmt : 1));
  or_triangle_normals(n_elmt, nv, x, y, z, nf);
  unsigned char *seen = (unsigned char *)malloc((size_t)(n_elmt > 0 ? n_elmt : 1));
  int failed = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if (ibi == 0 && nvert[t] < 5.) nvert[t] = 0;
        const double *p = &cent[t * 3];
        if (p[0] > H.xmin && p[0] < H.xmax && p[1] > H.ymin && p[1] < H.ymax && p[2] > H.zmin && p[2] < H.zmax) {
          int ic = (int)floor((p[0] - H.xmin) / H.dcx);
          int jc = (int)floor((p[1] - H.ymin) / H.dcy);
          int kc = (int)floor((p[2] - H.zmin) / H.dcz);
          int val = point_cell(p, ic, jc, kc, &H, n_elmt, nv, x, y, z, nf, seen, max_tries);
          if (val < 0) { failed++; val = 0; }
          nvert[t] = nvert[t] > val ? nvert[t] : val;
          if (nvert[t] < 0) nvert[t] = 0;
        }
      }
  /* near-boundary dilation over every DA point (ibm.c:326-348) */
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t t = IX(d, i, j, k);
        if (nvert[t] < 0) nvert[t] = 0;
        int ip = i < mx - 1 ? i + 1 : i, im = i > 0 ? i - 1 : i;
        int jp = j < my - 1 ? j + 1 : j, jm = j > 0 ? j - 1 : j;
        int kp = k < mz - 1 ? k + 1 : k, km = k > 0 ? k - 1 : k;
        if ((int)(nvert[t] + 0.5) != 4) {
          for (int kk = km; kk < kp + 1; kk++)
            for (int jj = jm; jj < jp + 1; jj++)
              for (int ii = im; ii < ip + 1; ii++)
                if ((int)(nvert[IX(d, ii, jj, kk)] + 0.5) == 4) nvert[t] = nvert[t] > 2 ? nvert[t] : 2;
        }
      }
  free(H.head); free(H.next); free(H.tri); free(nf); free(seen);
  return failed;
}

/* back to 3 / 1 and the wall rows (ibm.c:514-543) */
void or_ibm_finish(const or_dims *d, const int *bctype, double *nvert)
{
  const int mx = d->mx, my = d->my, mz = d->mz;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t t = IX(d, i, j, k);
        if ((int)(nvert[t] + 0.5) == 2) nvert[t] = 1;
        if ((int)(nvert[t] + 0.5) == 4) nvert[t] = 3;
        if (bctype) {
          for (int q = 0; q < 2; q++) {
            int v = -1 - q;
            if (bctype[0] == v && i == 1) nvert[t] = 1;
            if (bctype[1] == v && i == mx - 2) nvert[t] = 1;
            if (bctype[2] == v && j == 1) nvert[t] = 1;
            if (bctype[3] == v && j == my - 2) nvert[t] = 1;
            if (bctype[4] == v && k == 1) nvert[t] = 1;
            if (bctype[5] == v && k == mz - 2) nvert[t] = 1;
          }
        }
      }
}

/* ibm_search_advanced for one body: the marking (classification and
 * dilation, 4 = inside, 2 = IB node) then the finish (3 / 1 and walls). */
int or_ibm_search(const or_dims *d, const double *cent, int ibi, int n_v, const double *x, const double *y,
                  const double *z, int n_elmt, const int *nv, const int *bctype, double *nvert, int max_tries)
{
  int failed = or_ibm_mark(d, cent, ibi, n_v, x, y, z, n_elmt, nv, nvert, max_tries);
  or_ibm_finish(d, bctype, nvert);
  return failed;
}
