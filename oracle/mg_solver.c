/*
 * mg_solver.c -- FP64 CPU solver used as the oracle's exact solve and as the
 * timed CPU baseline.  TEST INFRASTRUCTURE ONLY; parity unpinned (see
 * vfs_oracle.h).
 *
 * The reference's production solve is HYPRE GMRES(51) + BoomerAMG
 * (Source/poisson_hypre.c:34-97, :603); HYPRE is an external library that is
 * not available here.  This baseline follows the reference's own geometric
 * multigrid path instead (PoissonSolver_MG_original, Source/poisson.c:2325-2698):
 *   - FGMRES outer iteration on the unscaled operator of PoissonLHSNew;
 *   - a multiplicative V-cycle on aj-scaled, re-discretised level operators
 *     (poisson.c:1563, :2366-2375) whose coarse grids take every other node
 *     (Source/init.c:402-455), with semi-coarsening flags per level
 *     (GridRestriction, poisson.c:337-363);
 *   - restriction MyRestriction, prolongation MyInterpolation, coarse
 *     blanking MyNvertRestriction (poisson.c:365-670, :1995-2083);
 *   - damped j-line Jacobi smoothing (tridiagonal solves along j) in place of
 *     the reference's FGMRES+BJacobi/ILU smoothers (poisson.c:2473-2546), and
 *     a dense direct solve on the coarsest level.
 * The GPU solver runs the same algorithm, so this is a like-for-like CPU
 * port.  OpenMP parallelises every grid loop.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "vfs_oracle.h"

#define NS 19
static const int OFF[NS][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                               {0, 0, 1},  {0, 0, -1}, {1, 1, 0},  {1, -1, 0}, {-1, 1, 0},
                               {-1, -1, 0}, {0, 1, 1},  {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
                               {1, 0, 1},  {1, 0, -1}, {-1, 0, 1}, {-1, 0, -1}};

typedef struct {
  int nx, ny, nz, px, py, pz;
  int cx, cy, cz; /* coarsening applied to reach the next level */
  size_t n;
  or_dims d;
  double *coor, *nvert;
  double *A;           /* [NS][n] aj-scaled level operator */
  unsigned char *act;  /* 1 = dof row */
  double *inv, *cp;    /* j-line LU factors */
  double *x, *b, *r, *t;
  /* coarsest level dense inverse */
  int nd;
  int *didx;
  double *dinv;
} lvl_t;

typedef struct {
  int nl;
  lvl_t L[32];
  /* fine operator (unscaled, reference filter) for the outer iteration */
  double *A0;
  unsigned char *act0;
  double *scale; /* aj on fluid rows, 1 on identity rows, 0 elsewhere */
  double setup_ms;
} mg_t;

static double now_ms(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static inline long nbr(const lvl_t *l, int i, int j, int k, int s)
{
  int a = i + OFF[s][0], b = j + OFF[s][1], c = k + OFF[s][2];
  if (a < 0) { if (!l->px) return -1; a += l->nx; }
  if (a >= l->nx) { if (!l->px) return -1; a -= l->nx; }
  if (b < 0) { if (!l->py) return -1; b += l->ny; }
  if (b >= l->ny) { if (!l->py) return -1; b -= l->ny; }
  if (c < 0) { if (!l->pz) return -1; c += l->nz; }
  if (c >= l->nz) { if (!l->pz) return -1; c -= l->nz; }
  return ((long)c * l->ny + b) * l->nx + a;
}

static void alloc_metrics(or_metrics *m, size_t n)
{
  m->cent = (double *)calloc(n * 3, 8);
  m->csi = (double *)calloc(n * 3, 8); m->eta = (double *)calloc(n * 3, 8);
  m->zet = (double *)calloc(n * 3, 8); m->aj = (double *)calloc(n, 8);
  m->icsi = (double *)calloc(n * 3, 8); m->ieta = (double *)calloc(n * 3, 8);
  m->izet = (double *)calloc(n * 3, 8); m->iaj = (double *)calloc(n, 8);
  m->jcsi = (double *)calloc(n * 3, 8); m->jeta = (double *)calloc(n * 3, 8);
  m->jzet = (double *)calloc(n * 3, 8); m->jaj = (double *)calloc(n, 8);
  m->kcsi = (double *)calloc(n * 3, 8); m->keta = (double *)calloc(n * 3, 8);
  m->kzet = (double *)calloc(n * 3, 8); m->kaj = (double *)calloc(n, 8);
}
static void free_metrics(or_metrics *m)
{
  double **p = &m->cent;
  for (int q = 0; q < 17; q++) free(p[q]);
}

/* Largest cell extent per direction (distance between opposite face
 * centres), used to choose the coarsening directions of each level. */
static void max_spacing(const lvl_t *l, double H[3])
{
  const or_dims *d = &l->d;
  H[0] = H[1] = H[2] = 0;
#define CO(i, j, k, c) l->coor[(((size_t)(k) * d->my + (j)) * d->mx + (i)) * 3 + (c)]
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        double fp[3][3], fm[3][3];
        for (int c = 0; c < 3; c++) {
          fp[0][c] = 0.25 * (CO(i, j, k, c) + CO(i, j - 1, k, c) + CO(i, j, k - 1, c) + CO(i, j - 1, k - 1, c));
          fm[0][c] = 0.25 * (CO(i - 1, j, k, c) + CO(i - 1, j - 1, k, c) + CO(i - 1, j, k - 1, c) + CO(i - 1, j - 1, k - 1, c));
          fp[1][c] = 0.25 * (CO(i, j, k, c) + CO(i - 1, j, k, c) + CO(i, j, k - 1, c) + CO(i - 1, j, k - 1, c));
          fm[1][c] = 0.25 * (CO(i, j - 1, k, c) + CO(i - 1, j - 1, k, c) + CO(i, j - 1, k - 1, c) + CO(i - 1, j - 1, k - 1, c));
          fp[2][c] = 0.25 * (CO(i, j, k, c) + CO(i - 1, j, k, c) + CO(i, j - 1, k, c) + CO(i - 1, j - 1, k, c));
          fm[2][c] = 0.25 * (CO(i, j, k - 1, c) + CO(i - 1, j, k - 1, c) + CO(i, j - 1, k - 1, c) + CO(i - 1, j - 1, k - 1, c));
        }
        for (int q = 0; q < 3; q++) {
          double s = 0;
          for (int c = 0; c < 3; c++) s += (fp[q][c] - fm[q][c]) * (fp[q][c] - fm[q][c]);
          s = sqrt(s);
          if (s > H[q]) H[q] = s;
        }
      }
#undef CO
}

/* Coarsening choice: a direction is coarsened when it has an even cell
 * count >= 4 and its largest cell extent is at most twice the smallest of
 * the other directions' largest extents (anisotropy-aware semi-coarsening;
 * the j-line smoother covers strong j coupling). */
static int choose_coarsening(const lvl_t *l, int c[3])
{
  double H[3];
  int n[3] = {l->nx, l->ny, l->nz};
  max_spacing(l, H);
  int any = 0;
  for (int q = 0; q < 3; q++) {
    c[q] = 0;
    if (n[q] % 2 || n[q] < 4) continue;
    double mn = 1e300;
    for (int e = 0; e < 3; e++)
      if (e != q && n[e] >= 2 && H[e] < mn) mn = H[e];
    if (H[q] <= 2.0 * mn) { c[q] = 1; any = 1; }
  }
  if (!any) {
    int best = -1;
    for (int q = 0; q < 3; q++)
      if (n[q] % 2 == 0 && n[q] >= 4 && (best < 0 || H[q] < H[best])) best = q;
    if (best >= 0) { c[best] = 1; any = 1; }
  }
  return any;
}

static void build_level_operator(lvl_t *l, const or_metrics *given)
{
  size_t nda = (size_t)l->d.mx * l->d.my * l->d.mz;
  or_metrics m;
  int own = 0;
  if (given) m = *given;
  else {
    alloc_metrics(&m, nda);
    or_form_metrics(&l->d, l->coor, &m);
    own = 1;
  }
  int *gid = (int *)malloc(nda * sizeof(int));
  int *rt = (int *)malloc(nda * sizeof(int));
  double *vol = (double *)malloc(nda * NS * sizeof(double));
  int *col = (int *)malloc(nda * NS * sizeof(int));
  or_poisson_lhs(&l->d, l->nvert, &m, 1, 0, gid, rt, vol, col);
  l->A = (double *)calloc(l->n * NS, sizeof(double));
  l->act = (unsigned char *)calloc(l->n, 1);
  for (int k = 0; k < l->nz; k++)
    for (int j = 0; j < l->ny; j++)
      for (int i = 0; i < l->nx; i++) {
        size_t t = (((size_t)(k + 1) * l->d.my) + (j + 1)) * l->d.mx + (i + 1);
        size_t c = ((size_t)k * l->ny + j) * l->nx + i;
        if (rt[t] == OR_ROW_NONE) continue;
        l->act[c] = 1;
        for (int s = 0; s < NS; s++) l->A[s * l->n + c] = vol[t * NS + s];
      }
  free(gid); free(rt); free(vol); free(col);
  if (own) free_metrics(&m);
}

static void build_line_lu(lvl_t *l)
{
  l->inv = (double *)calloc(l->n, 8);
  l->cp = (double *)calloc(l->n, 8);
#pragma omp parallel for collapse(2)
  for (int k = 0; k < l->nz; k++)
    for (int i = 0; i < l->nx; i++) {
      double cprev = 0;
      for (int j = 0; j < l->ny; j++) {
        size_t c = ((size_t)k * l->ny + j) * l->nx + i;
        double a = 0, dd = 1, cc = 0;
        if (l->act[c]) {
          dd = l->A[0 * l->n + c];
          a = (j > 0) ? l->A[4 * l->n + c] : 0.;
          cc = (j < l->ny - 1) ? l->A[3 * l->n + c] : 0.;
        }
        double den = dd - a * cprev;
        l->inv[c] = 1.0 / den;
        l->cp[c] = cc * l->inv[c];
        cprev = l->cp[c];
      }
    }
}

/* Dense inverse of the coarsest operator; one pinned row per connected
 * component of the dof graph makes the singular (Neumann/periodic) system
 * regular. */
static void build_coarsest(lvl_t *l)
{
  int *map = (int *)malloc(l->n * sizeof(int));
  int nd = 0;
  for (size_t c = 0; c < l->n; c++) map[c] = l->act[c] ? nd++ : -1;
  l->nd = nd;
  l->didx = (int *)malloc((nd ? nd : 1) * sizeof(int));
  for (size_t c = 0; c < l->n; c++)
    if (map[c] >= 0) l->didx[map[c]] = (int)c;
  double *M = (double *)calloc((size_t)nd * nd, 8);
  for (int r = 0; r < nd; r++) {
    int c = l->didx[r];
    int i = c % l->nx, j = (c / l->nx) % l->ny, k = c / (l->nx * l->ny);
    for (int s = 0; s < NS; s++) {
      long q = nbr(l, i, j, k, s);
      if (q < 0 || map[q] < 0) continue;
      M[(size_t)r * nd + map[q]] += l->A[s * l->n + c];
    }
  }
  /* connected components (BFS over nonzero couplings) */
  int *comp = (int *)malloc((nd ? nd : 1) * sizeof(int));
  int *queue = (int *)malloc((nd ? nd : 1) * sizeof(int));
  for (int r = 0; r < nd; r++) comp[r] = -1;
  int ncomp = 0;
  for (int r0 = 0; r0 < nd; r0++) {
    if (comp[r0] >= 0) continue;
    int h = 0, tl = 0;
    queue[tl++] = r0; comp[r0] = ncomp;
    while (h < tl) {
      int r = queue[h++];
      for (int q = 0; q < nd; q++)
        if (comp[q] < 0 && (M[(size_t)r * nd + q] != 0. || M[(size_t)q * nd + r] != 0.)) {
          comp[q] = ncomp; queue[tl++] = q;
        }
    }
    /* pin the first row of the component */
    for (int q = 0; q < nd; q++) M[(size_t)r0 * nd + q] = 0.;
    M[(size_t)r0 * nd + r0] = 1.;
    ncomp++;
  }
  /* Gauss-Jordan with partial pivoting */
  double *I = (double *)calloc((size_t)nd * nd, 8);
  for (int r = 0; r < nd; r++) I[(size_t)r * nd + r] = 1.;
  for (int c = 0; c < nd; c++) {
    int p = c;
    for (int r = c + 1; r < nd; r++)
      if (fabs(M[(size_t)r * nd + c]) > fabs(M[(size_t)p * nd + c])) p = r;
    if (p != c)
      for (int q = 0; q < nd; q++) {
        double t1 = M[(size_t)c * nd + q]; M[(size_t)c * nd + q] = M[(size_t)p * nd + q]; M[(size_t)p * nd + q] = t1;
        double t2 = I[(size_t)c * nd + q]; I[(size_t)c * nd + q] = I[(size_t)p * nd + q]; I[(size_t)p * nd + q] = t2;
      }
    double piv = M[(size_t)c * nd + c];
    double ip = (piv != 0.) ? 1. / piv : 0.;
    for (int q = 0; q < nd; q++) { M[(size_t)c * nd + q] *= ip; I[(size_t)c * nd + q] *= ip; }
    for (int r = 0; r < nd; r++) {
      if (r == c) continue;
      double f = M[(size_t)r * nd + c];
      if (f == 0.) continue;
      for (int q = 0; q < nd; q++) { M[(size_t)r * nd + q] -= f * M[(size_t)c * nd + q]; I[(size_t)r * nd + q] -= f * I[(size_t)c * nd + q]; }
    }
  }
  /* the pinned rows' right-hand side is forced to zero at solve time:
   * fold that into the inverse by zeroing those columns */
  for (int r0 = 0, seen = 0; r0 < nd; r0++) {
    int first = 1;
    for (int q = 0; q < r0; q++) if (comp[q] == comp[r0]) { first = 0; break; }
    if (first) { for (int r = 0; r < nd; r++) I[(size_t)r * nd + r0] = 0.; seen++; }
  }
  l->dinv = I;
  free(M); free(map); free(comp); free(queue);
}

void *or_mg_create(const or_dims *d, const double *coor, const double *nvert,
                   const or_metrics *fine_metrics, const or_solve_opts *o)
{
  double t0 = now_ms();
  if (o && o->threads > 0) omp_set_num_threads(o->threads);
  mg_t *g = (mg_t *)calloc(1, sizeof(mg_t));
  int coarsest_max = (o && o->coarsest_max > 0) ? o->coarsest_max : 128;
  lvl_t *l = &g->L[0];
  l->d = *d;
  l->nx = d->mx - 2; l->ny = d->my - 2; l->nz = d->mz - 2;
  l->px = d->i_periodic || d->ii_periodic;
  l->py = d->j_periodic || d->jj_periodic;
  l->pz = d->k_periodic || d->kk_periodic;
  l->n = (size_t)l->nx * l->ny * l->nz;
  size_t nda = (size_t)d->mx * d->my * d->mz;
  l->coor = (double *)malloc(nda * 3 * 8); memcpy(l->coor, coor, nda * 3 * 8);
  l->nvert = (double *)malloc(nda * 8); memcpy(l->nvert, nvert, nda * 8);
  g->nl = 1;
  for (;;) {
    lvl_t *f = &g->L[g->nl - 1];
    int c[3];
    if (f->n <= (size_t)coarsest_max || g->nl >= 31 || !choose_coarsening(f, c)) break;
    f->cx = c[0]; f->cy = c[1]; f->cz = c[2];
    lvl_t *q = &g->L[g->nl];
    q->nx = c[0] ? f->nx / 2 : f->nx; q->ny = c[1] ? f->ny / 2 : f->ny; q->nz = c[2] ? f->nz / 2 : f->nz;
    q->px = f->px; q->py = f->py; q->pz = f->pz;
    q->n = (size_t)q->nx * q->ny * q->nz;
    q->d = f->d;
    q->d.mx = q->nx + 2; q->d.my = q->ny + 2; q->d.mz = q->nz + 2;
    size_t nq = (size_t)q->d.mx * q->d.my * q->d.mz;
    q->coor = (double *)calloc(nq * 3, 8);
    /* coarse nodes are every other fine node: Source/init.c:402-455 */
    for (int k = 0; k <= q->nz; k++)
      for (int j = 0; j <= q->ny; j++)
        for (int i = 0; i <= q->nx; i++) {
          int ih = c[0] ? 2 * i : i, jh = c[1] ? 2 * j : j, kh = c[2] ? 2 * k : k;
          for (int e = 0; e < 3; e++)
            q->coor[(((size_t)k * q->d.my + j) * q->d.mx + i) * 3 + e] =
                f->coor[(((size_t)kh * f->d.my + jh) * f->d.mx + ih) * 3 + e];
        }
    q->nvert = (double *)calloc(nq, 8);
    or_my_nvert_restriction(&f->d, &q->d, !c[0], !c[1], !c[2], f->nvert, q->nvert);
    g->nl++;
  }
  for (int li = 0; li < g->nl; li++) {
    lvl_t *q = &g->L[li];
    build_level_operator(q, li == 0 ? fine_metrics : NULL);
    build_line_lu(q);
    q->x = (double *)calloc(q->n, 8); q->b = (double *)calloc(q->n, 8);
    q->r = (double *)calloc(q->n, 8); q->t = (double *)calloc(q->n, 8);
  }
  build_coarsest(&g->L[g->nl - 1]);
  /* fine operator for the outer iteration: unscaled, reference entry filter */
  {
    lvl_t *f = &g->L[0];
    or_metrics m;
    int own = 0;
    if (fine_metrics) m = *fine_metrics;
    else { alloc_metrics(&m, nda); or_form_metrics(d, coor, &m); own = 1; }
    int *gid = (int *)malloc(nda * sizeof(int));
    int *rt = (int *)malloc(nda * sizeof(int));
    double *vol = (double *)malloc(nda * NS * 8);
    int *col = (int *)malloc(nda * NS * sizeof(int));
    or_poisson_lhs(d, nvert, &m, 0, 1, gid, rt, vol, col);
    g->A0 = (double *)calloc(f->n * NS, 8);
    g->act0 = (unsigned char *)calloc(f->n, 1);
    g->scale = (double *)calloc(f->n, 8);
    for (int k = 0; k < f->nz; k++)
      for (int j = 0; j < f->ny; j++)
        for (int i = 0; i < f->nx; i++) {
          size_t t = (((size_t)(k + 1) * d->my) + (j + 1)) * d->mx + (i + 1);
          size_t c = ((size_t)k * f->ny + j) * f->nx + i;
          if (rt[t] == OR_ROW_NONE) continue;
          g->act0[c] = 1;
          g->scale[c] = (rt[t] == OR_ROW_FLUID) ? m.aj[t] : 1.0;
          for (int s = 0; s < NS; s++) g->A0[s * f->n + c] = vol[t * NS + s];
        }
    free(gid); free(rt); free(vol); free(col);
    if (own) free_metrics(&m);
  }
  g->setup_ms = now_ms() - t0;
  return g;
}

static void apply(const lvl_t *l, const double *A, const unsigned char *act, const double *x, double *y)
{
#pragma omp parallel for collapse(2)
  for (int k = 0; k < l->nz; k++)
    for (int j = 0; j < l->ny; j++)
      for (int i = 0; i < l->nx; i++) {
        size_t c = ((size_t)k * l->ny + j) * l->nx + i;
        if (!act[c]) { y[c] = 0.; continue; }
        double s = 0;
        for (int q = 0; q < NS; q++) {
          long nb = nbr(l, i, j, k, q);
          if (nb >= 0) s += A[q * l->n + c] * x[nb];
        }
        y[c] = s;
      }
}

static void residual(const lvl_t *l, const double *A, const unsigned char *act, const double *x,
                     const double *b, double *r)
{
#pragma omp parallel for collapse(2)
  for (int k = 0; k < l->nz; k++)
    for (int j = 0; j < l->ny; j++)
      for (int i = 0; i < l->nx; i++) {
        size_t c = ((size_t)k * l->ny + j) * l->nx + i;
        if (!act[c]) { r[c] = 0.; continue; }
        double s = 0;
        for (int q = 0; q < NS; q++) {
          long nb = nbr(l, i, j, k, q);
          if (nb >= 0) s += A[q * l->n + c] * x[nb];
        }
        r[c] = b[c] - s;
      }
}

/* one damped j-line Jacobi sweep: x_out = x + w (L^-1 (b - (A - T) x) - x) */
static void line_sweep(const lvl_t *l, double omega, const double *x, const double *b, double *xo,
                       int zero_guess)
{
#pragma omp parallel for collapse(2)
  for (int k = 0; k < l->nz; k++)
    for (int i = 0; i < l->nx; i++) {
      double yprev = 0;
      for (int j = 0; j < l->ny; j++) {
        size_t c = ((size_t)k * l->ny + j) * l->nx + i;
        double rhs = 0;
        if (l->act[c]) {
          rhs = b[c];
          if (!zero_guess)
            for (int q = 1; q < NS; q++) {
              if ((q == 3 && j < l->ny - 1) || (q == 4 && j > 0)) continue;
              long nb = nbr(l, i, j, k, q);
              if (nb >= 0) rhs -= l->A[q * l->n + c] * x[nb];
            }
        }
        double a = (j > 0 && l->act[c]) ? l->A[4 * l->n + c] : 0.;
        double y = (rhs - a * yprev) * l->inv[c];
        xo[c] = y;
        yprev = y;
      }
      double xn = 0;
      for (int j = l->ny - 1; j >= 0; j--) {
        size_t c = ((size_t)k * l->ny + j) * l->nx + i;
        double v = xo[c] - ((j < l->ny - 1) ? l->cp[c] * xn : 0.);
        xn = v;
        double xold = zero_guess ? 0. : x[c];
        xo[c] = l->act[c] ? xold + omega * (v - xold) : 0.;
      }
    }
}

/* zebra j-line Gauss-Seidel: columns of colour (i + k) % 2 == 0, then 1;
 * each colour reads the other colour's newest values (x updated in place),
 * same-colour corner couplings see the values from before the sweep. */
static int g_zebra = 0;
static void zebra_sweep(const lvl_t *l, double omega, double *x, const double *b, double *tmp, int zero_guess)
{
  if (zero_guess) memset(x, 0, l->n * 8);
  for (int color = 0; color < 2; color++) {
    memcpy(tmp, x, l->n * 8);  /* snapshot: same-colour neighbours read old values */
#pragma omp parallel for collapse(2)
    for (int k = 0; k < l->nz; k++)
      for (int i = 0; i < l->nx; i++) {
        if ((g_zebra == 2 ? (k & 1) : ((i + k) & 1)) != color) continue;
        double yprev = 0;
        double ys[1024];
        for (int j = 0; j < l->ny; j++) {
          size_t c = ((size_t)k * l->ny + j) * l->nx + i;
          double rhs = 0;
          if (l->act[c]) {
            rhs = b[c];
            for (int q = 1; q < NS; q++) {
              if ((q == 3 && j < l->ny - 1) || (q == 4 && j > 0)) continue;
              long nb = nbr(l, i, j, k, q);
              if (nb >= 0) rhs -= l->A[q * l->n + c] * tmp[nb];
            }
          }
          double a = (j > 0 && l->act[c]) ? l->A[4 * l->n + c] : 0.;
          double y = (rhs - a * yprev) * l->inv[c];
          ys[j] = y;
          yprev = y;
        }
        double xn = 0;
        for (int j = l->ny - 1; j >= 0; j--) {
          size_t c = ((size_t)k * l->ny + j) * l->nx + i;
          double v = ys[j] - ((j < l->ny - 1) ? l->cp[c] * xn : 0.);
          xn = v;
          double xold = tmp[c];
          x[c] = l->act[c] ? xold + omega * (v - xold) : 0.;
        }
      }
  }
}

static void vcycle(mg_t *g, int li, int nu1, int nu2, double omega)
{
  lvl_t *l = &g->L[li];
  if (li == g->nl - 1) {
    for (size_t c = 0; c < l->n; c++) l->x[c] = 0.;
    for (int r = 0; r < l->nd; r++) {
      double s = 0;
      for (int q = 0; q < l->nd; q++) s += l->dinv[(size_t)r * l->nd + q] * l->b[l->didx[q]];
      l->x[l->didx[r]] = s;
    }
    return;
  }
  for (int s = 0; s < nu1; s++) {
    if (g_zebra) { zebra_sweep(l, omega, l->x, l->b, l->t, s == 0); continue; }
    line_sweep(l, omega, l->x, l->b, l->t, s == 0);
    double *tmp = l->x; l->x = l->t; l->t = tmp;
  }
  residual(l, l->A, l->act, l->x, l->b, l->r);
  lvl_t *q = &g->L[li + 1];
  /* restriction on DA-layout scratch, MyRestriction semantics */
  {
    const int ia = l->cx, ja = l->cy, ka = l->cz;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < q->nz; k++)
      for (int j = 0; j < q->ny; j++)
        for (int i = 0; i < q->nx; i++) {
          size_t cc = ((size_t)k * q->ny + j) * q->nx + i;
          if (q->nvert[(((size_t)(k + 1) * q->d.my) + j + 1) * q->d.mx + i + 1] > 0.1) {
            q->b[cc] = 0.;
            continue;
          }
          int i1 = ia ? 2 * i + 1 : i, j1 = ja ? 2 * j + 1 : j, k1 = ka ? 2 * k + 1 : k;
          int i0 = i1 - ia, j0 = j1 - ja, k0 = k1 - ka;
          int I[2] = {i1, i0}, J[2] = {j1, j0}, K[2] = {k1, k0};
          double s = 0;
          /* the eight terms in the order of poisson.c:433-441 */
          static const int ord[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                        {1, 1, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 1}};
          for (int e = 0; e < 8; e++) {
            int fi = I[ord[e][0]], fj = J[ord[e][1]], fk = K[ord[e][2]];
            size_t fc = ((size_t)fk * l->ny + fj) * l->nx + fi;
            double nv = l->nvert[(((size_t)(fk + 1) * l->d.my) + fj + 1) * l->d.mx + fi + 1];
            double w = 1 - nv > 0. ? 1 - nv : 0.;
            s += l->r[fc] * w;
          }
          q->b[cc] = 0.125 * s;
        }
  }
  vcycle(g, li + 1, nu1, nu2, omega);
  /* prolongation, MyInterpolation semantics, added to x */
  {
#pragma omp parallel for collapse(2)
    for (int k = 0; k < l->nz; k++)
      for (int j = 0; j < l->ny; j++)
        for (int i = 0; i < l->nx; i++) {
          size_t c = ((size_t)k * l->ny + j) * l->nx + i;
          if (!l->act[c]) continue;
          if (l->nvert[(((size_t)(k + 1) * l->d.my) + j + 1) * l->d.mx + i + 1] > 0.1) continue;
          int I = i + 1, J = j + 1, K = k + 1; /* DA indices */
          int ic, jc, kc, ia, ja, ka;
          if (!l->cx) { ic = I; ia = 0; }
          else { ic = (I + 1) / 2; ia = (I - 2 * ic) == 0 ? 1 : -1; if (I == 1 || I == l->d.mx - 2) ia = 0; }
          if (!l->cy) { jc = J; ja = 0; }
          else { jc = (J + 1) / 2; ja = (J - 2 * jc) == 0 ? 1 : -1; if (J == 1 || J == l->d.my - 2) ja = 0; }
          if (!l->cz) { kc = K; ka = 0; }
          else { kc = (K + 1) / 2; ka = (K - 2 * kc) == 0 ? 1 : -1; if (K == 1 || K == l->d.mz - 2) ka = 0; }
#define NC(a, b, c) q->nvert[(((size_t)(c)) * q->d.my + (b)) * q->d.mx + (a)]
#define XC(a, b, c) q->x[(((size_t)(c)-1) * q->ny + (b)-1) * q->nx + (a)-1]
          if (ka == -1 && NC(ic, jc, kc - 1) > 0.1) ka = 0;
          else if (ka == 1 && NC(ic, jc, kc + 1) > 0.1) ka = 0;
          if (ja == -1 && NC(ic, jc - 1, kc) > 0.1) ja = 0;
          else if (ja == 1 && NC(ic, jc + 1, kc) > 0.1) ja = 0;
          if (ia == -1 && NC(ic - 1, jc, kc) > 0.1) ia = 0;
          else if (ia == 1 && NC(ic + 1, jc, kc) > 0.1) ia = 0;
          double v = (XC(ic, jc, kc) * 9 + XC(ic, jc + ja, kc) * 3 + XC(ic + ia, jc, kc) * 3 +
                      XC(ic + ia, jc + ja, kc)) * 3. / 64. +
                     (XC(ic, jc, kc + ka) * 9 + XC(ic, jc + ja, kc + ka) * 3 + XC(ic + ia, jc, kc + ka) * 3 +
                      XC(ic + ia, jc + ja, kc + ka)) / 64.;
#undef NC
#undef XC
          l->x[c] += v;
        }
  }
  for (int s = 0; s < nu2; s++) {
    if (g_zebra) { zebra_sweep(l, omega, l->x, l->b, l->t, 0); continue; }
    line_sweep(l, omega, l->x, l->b, l->t, 0);
    double *tmp = l->x; l->x = l->t; l->t = tmp;
  }
}

/* 0: line Jacobi; 1: zebra j-line Gauss-Seidel over checkerboard-coloured
 * (i, k) columns; 2: zebra over k-planes (colour = k parity) */
void or_mg_set_smoother(int zebra) { g_zebra = zebra; }

static double dot(const double *a, const double *b, size_t n)
{
  double s = 0;
#pragma omp parallel for reduction(+ : s)
  for (size_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* z = M^-1 v with M^-1 = one V-cycle on the aj-scaled system */
static void precond(mg_t *g, const double *v, double *z, const or_solve_opts *o)
{
  lvl_t *l = &g->L[0];
#pragma omp parallel for
  for (size_t c = 0; c < l->n; c++) l->b[c] = g->scale[c] * v[c];
  vcycle(g, 0, o->nu1, o->nu2, o->omega);
  memcpy(z, l->x, l->n * 8);
}

static void da_to_int(const lvl_t *l, const double *da, double *v)
{
  for (int k = 0; k < l->nz; k++)
    for (int j = 0; j < l->ny; j++)
      for (int i = 0; i < l->nx; i++)
        v[((size_t)k * l->ny + j) * l->nx + i] = da[(((size_t)(k + 1) * l->d.my) + j + 1) * l->d.mx + i + 1];
}
static void int_to_da(const lvl_t *l, const double *v, double *da)
{
  for (int k = 0; k < l->nz; k++)
    for (int j = 0; j < l->ny; j++)
      for (int i = 0; i < l->nx; i++)
        da[(((size_t)(k + 1) * l->d.my) + j + 1) * l->d.mx + i + 1] = v[((size_t)k * l->ny + j) * l->nx + i];
}

int or_mg_vcycle(void *h, const double *r_da, double *z_da, int nu1, int nu2, double omega)
{
  mg_t *g = (mg_t *)h;
  lvl_t *l = &g->L[0];
  or_solve_opts o = {0};
  o.nu1 = nu1; o.nu2 = nu2; o.omega = omega;
  double *v = (double *)malloc(l->n * 8), *z = (double *)malloc(l->n * 8);
  da_to_int(l, r_da, v);
  precond(g, v, z, &o);
  int_to_da(l, z, z_da);
  free(v); free(z);
  return 0;
}

int or_mg_solve(void *h, const double *b_da, double *x_da, const or_solve_opts *o, or_solve_stats *st)
{
  mg_t *g = (mg_t *)h;
  lvl_t *l = &g->L[0];
  const size_t n = l->n;
  const int m = o->restart > 0 ? o->restart : 20;
  if (o->threads > 0) omp_set_num_threads(o->threads);
  double t0 = now_ms();
  double *b = (double *)calloc(n, 8), *x = (double *)calloc(n, 8), *r = (double *)calloc(n, 8);
  double *V = (double *)calloc(n * (m + 1), 8), *Z = (double *)calloc(n * m, 8);
  double *H = (double *)calloc((size_t)(m + 1) * m, 8), *cs = (double *)calloc(m, 8),
         *sn = (double *)calloc(m, 8), *gv = (double *)calloc(m + 1, 8), *y = (double *)calloc(m, 8);
  da_to_int(l, b_da, b);
  da_to_int(l, x_da, x);
  for (size_t c = 0; c < n; c++) if (!g->act0[c]) { b[c] = 0; x[c] = 0; }
  double bn = sqrt(dot(b, b, n));
  int it = 0;
  double rel = 0;
  if (bn == 0.) {
    memset(x, 0, n * 8);
  } else {
    residual(l, g->A0, g->act0, x, b, r);
    double beta = sqrt(dot(r, r, n));
    rel = beta / bn;
    while (rel > o->rtol && it < o->max_it) {
      for (size_t c = 0; c < n; c++) V[c] = r[c] / beta;
      memset(gv, 0, (m + 1) * 8);
      gv[0] = beta;
      int jj = 0;
      for (; jj < m && it < o->max_it; jj++) {
        double *vj = V + n * jj, *zj = Z + n * jj, *w = V + n * (jj + 1);
        precond(g, vj, zj, o);
        apply(l, g->A0, g->act0, zj, w);
        for (int i = 0; i <= jj; i++) { /* modified Gram-Schmidt */
          double hij = dot(w, V + n * i, n);
          H[(size_t)i * m + jj] = hij;
          const double *vi = V + n * i;
#pragma omp parallel for
          for (size_t c = 0; c < n; c++) w[c] -= hij * vi[c];
        }
        double hn = sqrt(dot(w, w, n));
        H[(size_t)(jj + 1) * m + jj] = hn;
        if (hn != 0.) {
#pragma omp parallel for
          for (size_t c = 0; c < n; c++) w[c] /= hn;
        }
        for (int i = 0; i < jj; i++) {
          double a = H[(size_t)i * m + jj], b2 = H[(size_t)(i + 1) * m + jj];
          H[(size_t)i * m + jj] = cs[i] * a + sn[i] * b2;
          H[(size_t)(i + 1) * m + jj] = -sn[i] * a + cs[i] * b2;
        }
        double a = H[(size_t)jj * m + jj], b2 = H[(size_t)(jj + 1) * m + jj];
        double den = sqrt(a * a + b2 * b2);
        cs[jj] = den != 0. ? a / den : 1.;
        sn[jj] = den != 0. ? b2 / den : 0.;
        H[(size_t)jj * m + jj] = den;
        H[(size_t)(jj + 1) * m + jj] = 0.;
        gv[jj + 1] = -sn[jj] * gv[jj];
        gv[jj] = cs[jj] * gv[jj];
        it++;
        if (fabs(gv[jj + 1]) / bn <= o->rtol) { jj++; break; }
      }
      for (int i = jj - 1; i >= 0; i--) {
        double s = gv[i];
        for (int q = i + 1; q < jj; q++) s -= H[(size_t)i * m + q] * y[q];
        y[i] = s / H[(size_t)i * m + i];
      }
      for (int i = 0; i < jj; i++) {
        const double *zi = Z + n * i;
        double yi = y[i];
#pragma omp parallel for
        for (size_t c = 0; c < n; c++) x[c] += yi * zi[c];
      }
      residual(l, g->A0, g->act0, x, b, r);
      beta = sqrt(dot(r, r, n));
      rel = beta / bn;
    }
  }
  int_to_da(l, x, x_da);
  if (st) {
    st->iterations = it;
    st->rel_residual = rel;
    st->setup_ms = g->setup_ms;
    st->solve_ms = now_ms() - t0;
    st->levels = g->nl;
  }
  free(b); free(x); free(r); free(V); free(Z); free(H); free(cs); free(sn); free(gv); free(y);
  return rel <= o->rtol ? 0 : 1;
}

int or_mg_level_info(void *h, int level, int *v)
{
  mg_t *g = (mg_t *)h;
  if (level < 0 || level >= g->nl) return g->nl;
  lvl_t *l = &g->L[level];
  v[0] = l->nx; v[1] = l->ny; v[2] = l->nz; v[3] = l->cx; v[4] = l->cy; v[5] = l->cz; v[6] = l->nd;
  return g->nl;
}

void or_mg_destroy(void *h)
{
  mg_t *g = (mg_t *)h;
  if (!g) return;
  for (int li = 0; li < g->nl; li++) {
    lvl_t *l = &g->L[li];
    free(l->coor); free(l->nvert); free(l->A); free(l->act); free(l->inv); free(l->cp);
    free(l->x); free(l->b); free(l->r); free(l->t); free(l->didx); free(l->dinv);
  }
  free(g->A0); free(g->act0); free(g->scale);
  free(g);
}
