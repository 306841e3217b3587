/*
 * vfs_oracle.h -- CPU restatement of VFS-Wind's pressure-Poisson path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation and the timed CPU baseline.  Nothing in the product
 * (vfs-wind_gb300/) links, loads or calls it; only tests/, bench.py's
 * cpu_baseline / reference arm and __graft_entry__.smoke() do.
 *
 * Parity status: the reference (the Source directory) needs PETSc 3.1, HYPRE and MPI,
 * which are external libraries that are not present, so it is treated as
 * unbuildable and the reference ships no golden vectors or fixtures for this
 * path.  This restatement is therefore "parity unpinned": it follows the
 * reference source line by line (citations on every function) and is
 * cross-checked only against itself (exact sparse solves, conservation and
 * null-space properties), not against outputs of the reference.
 *
 * Array conventions mirror the reference's PETSc DA layout on one rank:
 * scalars are double[mz][my][mx] (i fastest), vectors are Cmpnts AoS
 * double[mz][my][mx][3].  Index 0 and m-1 in each direction are the
 * boundary/ghost layer; interior cells are 1..m-2.  Node coordinates use the
 * same array shape, with node (i,j,k) for i < mx-1 (the last layer unused).
 */
#ifndef VFS_ORACLE_H
#define VFS_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Grid description; the six periodic flags carry the reference's globals
 * i/j/k_periodic (explicit copy) and ii/jj/kk_periodic (periodic DA). */
typedef struct {
  int mx, my, mz;
  int i_periodic, j_periodic, k_periodic;
  int ii_periodic, jj_periodic, kk_periodic;
} or_dims;

/* Metric arrays produced by FormMetrics (all double, DA layout). */
typedef struct {
  double *cent;                    /* cell centres (vec)            */
  double *csi, *eta, *zet, *aj;    /* cell metrics (vec, vec, vec, scalar) */
  double *icsi, *ieta, *izet, *iaj;
  double *jcsi, *jeta, *jzet, *jaj;
  double *kcsi, *keta, *kzet, *kaj;
} or_metrics;

/* Stencil slot order of the 19-point operator (Source/poisson.c:957-975). */
enum { OR_CP = 0, OR_EP, OR_WP, OR_NP, OR_SP, OR_TP, OR_BP, OR_NE, OR_SE, OR_NW,
       OR_SW, OR_TN, OR_BN, OR_TS, OR_BS, OR_TE, OR_BE, OR_TW, OR_BW };

/* Row classes written by or_poisson_lhs. */
enum { OR_ROW_NONE = 0, OR_ROW_FLUID = 1, OR_ROW_IDENTITY = 2 };

void or_form_metrics(const or_dims *d, const double *coor, or_metrics *m);

int or_setup_lidx2(const or_dims *d, const double *nvert, int *gid);

int or_poisson_lhs(const or_dims *d, const double *nvert, const or_metrics *m,
                   int scale_by_aj, int apply_filter, int *gid, int *rowtype,
                   double *vol, int *col);

void or_set_levelset(const double *rho, const double *level, int on, int bc3, int bc4, int bc5);
void or_volume_flux(const or_dims *d, const double *nvert, const double *csi, const double *eta, const double *zet,
                    double *ucont, int flg, double flux_intp_sum, double *out);
void or_volume_flux0(const or_dims *d, const double *nvert, const double *csi, const double *eta,
                     const double *zet, double *ucont, int immersed, double *out);
void or_contra2cart(const or_dims *d, const double *nvert, const double *csi, const double *eta, const double *zet,
                    const double *ucont, double *ucat, int zero_solid);
void or_poisson_rhs2(const or_dims *d, const double *nvert, const int *gid, const double *ucont,
                     const double *aj, double dt, double st, double coeff, int poisson, double *b);
void or_poisson_rhs2_hypre(const or_dims *d, const double *nvert, const int *gid,
                           const double *ucont, double dt, double st, double coeff,
                           double *b);
void or_remove_nullspace_scale(const or_dims *d, const double *nvert, const int *gid,
                               const double *aj, double *b, int bctype3);
int or_fully_blocked(const or_dims *d, const double *nvert, int *ksk);
void or_nullspace_original(const or_dims *d, const double *nvert, const int *ksk, int multi, double *x);
void or_remove_nullspace(const or_dims *d, const double *nvert, const int *gid,
                         double *phi2, int bctype3);
void or_convert_phi2_phi(const or_dims *d, const double *nvert, const double *phi2,
                         double *phi);
void or_update_pressure(const or_dims *d, const double *nvert, double *p, double *phi);
void or_projection(const or_dims *d, const double *nvert, const double *phi,
                   const or_metrics *m, double dt, double st, double coeff,
                   double *ucont);
double or_divergence(const or_dims *d, const double *nvert, const double *ucont,
                     const double *aj);

void or_my_nvert_restriction(const or_dims *dh, const or_dims *dc, int isc, int jsc,
                             int ksc, const double *nvert_h, double *nvert_c);
void or_my_restriction(const or_dims *dc, const or_dims *df, int isc, int jsc, int ksc,
                       const double *nvert_c, const double *nvert_f, const double *xf,
                       double *fc);
void or_my_interpolation(const or_dims *df, const or_dims *dc, int isc, int jsc, int ksc,
                         const double *nvert_f, const double *nvert_c, const double *xc,
                         double *ff);

/* y = A x over the DA layout using the stencil arrays from or_poisson_lhs. */
void or_stencil_apply(const or_dims *d, const int *rowtype, const double *vol,
                      const double *x, double *y);

/* Immersed-boundary classification (oracle/ibm_oracle.c). nv holds the
 * triangles' 0-based vertex ids, three per triangle. */
unsigned int or_glibc_rand_first(unsigned int seed);
void or_triangle_normals(int n_elmt, const int *nv, const double *x, const double *y, const double *z,
                         double *nf);
int or_ibm_search(const or_dims *d, const double *cent, int ibi, int n_v, const double *x, const double *y,
                  const double *z, int n_elmt, const int *nv, const int *bctype, double *nvert, int max_tries);
int or_ibm_mark(const or_dims *d, const double *cent, int ibi, int n_v, const double *x, const double *y,
                const double *z, int n_elmt, const int *nv, double *nvert, int max_tries);
void or_ibm_finish(const or_dims *d, const int *bctype, double *nvert);

/* One IB node's interpolation record (ibm_interp_oracle.c; the reference's
 * IBMInfo): the node, its nearest surface element and point, the distance
 * d_s and the point's weights on the element's vertices, the three cell
 * centres the normal ray meets with their weights and distance d_i, the
 * patch triangle (imode) and a status (0: found, 1: the reference's
 * boundary fallback, 2: the reference's search failure). */
typedef struct {
  int i, j, k;
  int cell;
  double pmin[3], d_s, cs[3];
  int ip[3], jp[3], kp[3];
  double cr[3], d_i;
  int imode, status;
} or_ibm_node;
void or_bounding_sphere(int n_elmt, const int *nv, const double *x, const double *y, const double *z, double *q,
                        double *rad);
int or_ibm_nodes(const or_dims *d, const double *cent, const double *nvert_marked, int n_v, const double *x,
                 const double *y, const double *z, int n_elmt, const int *nv, or_ibm_node *nodes, int max_nodes);
void or_ibm_interpolate(const or_dims *d, const double *nvert, const or_ibm_node *nodes, int n_nodes,
                        const int *nv, const double *u_surf, const double *icsi, const double *jeta,
                        const double *kzet, const double *csi, const double *eta, const double *zet,
                        const int *bctype, int immersed, double *ucat, double *p, double *ucont);
void or_ib_bc(const or_dims *d, const double *nvert, const double *icsi, const double *jeta, const double *kzet,
              const int *bctype, int immersed, double *ucat, double *ucont);

/* CPU baseline solver (oracle/mg_solver.c). */
typedef struct {
  int max_it;       /* outer FGMRES iterations          */
  int restart;      /* FGMRES restart length            */
  double rtol;      /* ||b-Ax||/||b|| target            */
  int nu1, nu2;     /* pre/post line-smoothing sweeps   */
  double omega;     /* line-Jacobi damping              */
  int threads;      /* OpenMP threads, 0 = default      */
  int coarsest_max; /* coarsest level cell budget       */
} or_solve_opts;

typedef struct {
  int iterations;
  double rel_residual;
  double setup_ms, solve_ms;
  int levels;
} or_solve_stats;

void *or_mg_create(const or_dims *d, const double *coor, const double *nvert,
                   const or_metrics *fine_metrics, const or_solve_opts *o);
int or_mg_solve(void *h, const double *b_da, double *x_da, const or_solve_opts *o,
                or_solve_stats *st);
int or_mg_vcycle(void *h, const double *r_da, double *z_da, int nu1, int nu2, double omega);
int or_mg_level_info(void *h, int level, int *dims7);
void or_mg_destroy(void *h);
/* 1: zebra j-line Gauss-Seidel smoothing (checkerboard columns), 0: damped
 * j-line Jacobi (default). */
void or_mg_set_smoother(int zebra);

#ifdef __cplusplus
}
#endif
#endif
