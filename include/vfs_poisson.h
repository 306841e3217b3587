/*
 * vfs_poisson.h -- C ABI of the GB300 pressure-Poisson projection for
 * VFS-Wind's fractional-step loop.
 *
 * One handle owns one block (one DA) on one GPU: its device buffers are
 * allocated at create / set-up time and reused across time steps.  All
 * array arguments use the reference's PETSc DA natural layout on a single
 * rank: scalars double[mz][my][mx] (i fastest), Cmpnts vectors
 * double[mz][my][mx][3], with index 0 and m-1 the boundary layer
 * (Source/init.c:157-161).  Every array pointer may be host memory or device
 * memory of the handle's GPU; the library detects which and copies host
 * arrays through the handle's stream.  Calls are synchronous on return and a
 * handle is not thread-safe.  The handle's private stream is a blocking
 * stream, so device inputs written on the legacy default stream are ready
 * when a call starts; inputs written on another stream must be complete (or
 * that stream passed to vfs_poisson_set_stream).
 *
 * Return codes: 0 on success, negative VFS_E* on failure; a failing call
 * leaves the handle usable.  vfs_last_error() gives a message.
 *
 * Reference interfaces replaced (all in Source/ of SAFL-CFD-Lab/VFS-Wind):
 *   FormMetrics               metrics.c:12         -> vfs_poisson_set_grid
 *   setup_lidx2, PoissonLHSNew poisson.c:188, :977 -> vfs_poisson_set_nvert
 *   PoissonRHS2_hypre + Remove_Nullspace_Scale
 *                             poisson_hypre.c:265, :118 -> vfs_poisson_rhs
 *   PoissonRHS2               poisson.c:1780       -> vfs_poisson_rhs2
 *   VolumeFlux (immersed)     poisson.c:3563       -> vfs_poisson_volume_flux
 *   VolumeFlux (immersed!=1)  poisson.c:3299       -> vfs_poisson_volume_flux0
 *   Contra2Cart               rhs.c:35             -> vfs_poisson_contra2cart
 *   levelset operator / projection poisson.c:1171, :2738 -> vfs_poisson_set_levelset
 *   PoissonSolver_Hypre       poisson_hypre.c:506  -> vfs_poisson_solve
 *   Remove_Nullspace          poisson_hypre.c:202  (inside vfs_poisson_solve)
 *   Convert_Phi2_Phi          poisson.c:98         (inside vfs_poisson_solve)
 *   UpdatePressure            poisson.c:3137       -> vfs_poisson_update_pressure
 *   Projection                poisson.c:2700       -> vfs_poisson_projection
 *   Divergence                main.c:936           -> vfs_poisson_divergence
 *   MyRestriction / MyInterpolation / MyNvertRestriction
 *                             poisson.c:365, :527, :1995 -> vfs_poisson_mg_*
 *   ibm_search_advanced       ibm.c:92             -> vfs_poisson_ibm_search
 *   IB interpolation records  ibm.c:373-508        -> vfs_poisson_ibm_search_nodes
 *   ibm_interpolation_advanced ibm.c:3301          -> vfs_poisson_ibm_interpolate
 *   IB_BC                     momentum.c:2016      -> vfs_poisson_ib_bc
 */
#ifndef VFS_POISSON_H
#define VFS_POISSON_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VFS_OK 0
#define VFS_EINVAL (-1)     /* bad argument or size                    */
#define VFS_ECUDA (-2)      /* CUDA runtime error                      */
#define VFS_ESTATE (-3)     /* call order (e.g. solve before set_nvert) */
#define VFS_ENOCONV (-4)    /* solver stopped above the tolerance      */
#define VFS_ENOMEM (-5)     /* device allocation failed                */
#define VFS_ETIMEOUT (-6)   /* a device-side watchdog gave up          */

/* Grid of one block.  mx/my/mz are the DA sizes (nodes + 1, i.e. interior
 * cells + 2).  The periodic flags are the reference's globals
 * i/j/k_periodic (explicit ghost copy) and ii/jj/kk_periodic (periodic DA);
 * either flag makes that direction periodic. */
typedef struct {
  int mx, my, mz;
  int i_periodic, j_periodic, k_periodic;
  int ii_periodic, jj_periodic, kk_periodic;
  int bctype3; /* user->bctype[3]; -10 disables both null-space removals */
} vfs_grid_desc;

/* Solver options (defaults from vfs_poisson_default_opts). */
typedef struct {
  double rtol;        /* ||b - A phi||_2 / ||b||_2 target (poisson_tol)   */
  int max_it;         /* outer iterations (poisson_it)                     */
  int restart;        /* FGMRES restart length                             */
  int precision;      /* 0: FP32 V-cycle in FP64 refinement, 1: all FP64   */
  int nu1, nu2;       /* pre / post j-line sweeps per level (default 1, 2) */
  double omega;       /* relaxation weight of the line sweeps; 0 picks the
                         smoother's own (1 for zebra, 0.8 for line Jacobi) */
  int use_graphs;     /* capture the V-cycle in a CUDA graph               */
  int coarsest_max;   /* coarsest level cell budget (default 256; the
                         hierarchy is built with the default at
                         vfs_poisson_set_nvert)                            */
  int warm_start;     /* 0: zero guess; 1: start from the phi passed in (Phi2
                         warm start; the last solution if phi is NULL);
                         2: start from the handle's iterate as left by the
                         last solve or by vfs_poisson_learned_guess */
  int smoother;       /* 0 fused line Jacobi, 1 line Jacobi in correction
                         form, 2 zebra line Gauss-Seidel over k-planes,
                         3 zebra line Gauss-Seidel over checkerboard
                         (i + k parity) columns, 4 (default) the same
                         sweep, bit-identical to 3, with each colour's
                         residual formed inside the line kernel on the
                         FP32 levels of at most 2^20 cells (3's kernels
                         elsewhere)                                        */
  int orth;           /* Arnoldi orthogonalisation: 0 (default) classical
                         Gram-Schmidt in one pass (PETSc GMRES's default
                         refinement "never"), 1 classical Gram-Schmidt
                         with delayed reorthogonalisation (DCGS2)          */
  int nu2_near;       /* post sweeps for a solve whose initial residual is
                         within 32x of rtol (default 0: nu2).  4 finishes
                         more such solves in one V-cycle; over a sequence
                         warm-started from the solution history it saved
                         no time (the history of solves that stop just
                         under rtol guesses less well)                     */
} vfs_solve_opts;

typedef struct {
  int iterations;
  double rel_residual;   /* true FP64 residual at exit */
  double initial_rel_residual;
  double ms_total;       /* device time of the whole solve */
  int levels;
  int status;            /* 0 converged, VFS_ENOCONV otherwise */
} vfs_solve_stats;

typedef struct vfs_poisson vfs_poisson;

const char *vfs_last_error(void);
void vfs_poisson_default_opts(vfs_solve_opts *o);

/* Create / destroy a handle on the current CUDA device. */
int vfs_poisson_create(const vfs_grid_desc *g, vfs_poisson **out);
void vfs_poisson_destroy(vfs_poisson *h);

/* Grid: node coordinates (Cmpnts DA layout, node (i,j,k) at i < mx-1).
 * Runs FormMetrics on the GPU.  If `face_metrics` is non-NULL it points to
 * 12 Cmpnts arrays followed by 4 scalar arrays in the order
 * icsi,ieta,izet, jcsi,jeta,jzet, kcsi,keta,kzet (Cmpnts) and iaj,jaj,kaj,aj
 * (scalars) that replace the computed fine-level metrics, as a drop-in for
 * an existing UserCtx. */
int vfs_poisson_set_grid(vfs_poisson *h, const double *coor, const double *const *face_metrics);

/* Immersed-boundary flags (0 fluid, 1 IB node, 3 solid; any value works
 * with the reference's thresholds).  Numbers the dofs (setup_lidx2),
 * assembles the FP64 operator (PoissonLHSNew) and builds the multigrid
 * hierarchy.  Call again whenever the mask moves. */
int vfs_poisson_set_nvert(vfs_poisson *h, const double *nvert);

/* Right-hand side from Ucont: PoissonRHS2_hypre + Remove_Nullspace_Scale.
 * coeff is time_coeff() (Source/poisson.c:23-31). */
int vfs_poisson_rhs(vfs_poisson *h, const double *ucont, double dt, double st, double coeff);

/* Level-set (two-phase) variant of the operator and the projection
 * (levelset in Source/poisson.c:1171-1561 and :2738-2956): every face
 * coefficient is divided by the harmonic mean of the two cells' densities
 * (mean(), Source/level.c:2276); bctype[3] == 4 / bctype[5] == 4 make the
 * top j / k face a zero-Dirichlet pressure face; bctype[4] == 5000 opens the
 * bottom k face of the cells with level < 0 (density of the cell there) and
 * bctype[4] == 5 makes it Dirichlet.  rho and level: DA-layout cell fields
 * (level may be NULL when bctype[4] != 5000).  The multigrid levels use
 * child averages of both fields.  With bctype[5] == 4 the right-hand side
 * and phi keep their means, as the reference skips both null-space
 * removals then.  Call before vfs_poisson_set_nvert (which assembles);
 * enable = 0 turns it off. */
int vfs_poisson_set_levelset(vfs_poisson *h, const double *rho, const double *level, const int *bctype, int enable);

/* PoissonRHS2 (Source/poisson.c:1780-1906), the right-hand side of the
 * -poisson 0 (poisson = 0) and -poisson -1 (poisson = -1) paths: the same
 * divergence as vfs_poisson_rhs on fluid cells, 0 on identity-row dofs,
 * rows times aj for -1, then the unweighted mean over the fluid cells
 * removed from the fluid entries (instead of Remove_Nullspace_Scale).  The
 * solve then uses this B (poisson = 0) or B / aj on the fluid rows
 * (poisson = -1: the same system without its row scaling; the reference's
 * aj-scaled rows with an unweighted mean removal are not consistent, so a
 * solve to a tight tolerance can stop at VFS_ENOCONV, as the reference's
 * own iteration stops at its iteration limit). */
int vfs_poisson_rhs2(vfs_poisson *h, const double *ucont, double dt, double st, double coeff, int poisson);

/* VolumeFlux, the immersed == 1 variant (Source/poisson.c:3563-3903): the
 * net flux through the faces between fluid and IB cells (0.1 < nvert <
 * 1.1) of ucont (DA Cmpnts, in/out) is removed before the right-hand side.
 * Faces with |U| <= 1e-8 are zeroed; flg selects the reference's
 * correction (0: flux / area spread by face area; 1: (flux +
 * flux_intp_sum) / area; 2: (flux + flux_intp_sum) / sum|U| spread by |U|;
 * 3: the same with |U| / area).  *ibm_flux and *ibm_area (may be NULL) get
 * the flux and area after the correction, as the reference returns them.
 * The per-face arithmetic is the reference's; the three sums are reduced in
 * a different order (their values agree to rounding). */
int vfs_poisson_volume_flux(vfs_poisson *h, double *ucont, int flg, double flux_intp_sum, double *ibm_flux,
                            double *ibm_area);

/* VolumeFlux, the overload PoissonSolver_Hypre calls when immersed is not
 * 1 or 2 (Source/poisson.c:3299-3493, called at poisson_hypre.c:561): the
 * faces between a fluid cell (nvert < 0.1) and a blanked one (nvert > 0.1)
 * of ucont (DA Cmpnts, in/out) carry the net flux; the correction flux /
 * area (area: the norms of the adjacent cell's metric) is taken off the
 * fluid side and added to the blanked side, and for immersed 0 or 3 those
 * faces are then zeroed (immersed 2 changes nothing).  *flux and *area (may
 * be NULL) get the sums formed afterwards, as the reference reports them.
 * Per-face arithmetic is the reference's; the two sums are reduced in a
 * different order (their values agree to rounding). */
int vfs_poisson_volume_flux0(vfs_poisson *h, double *ucont, int immersed, double *flux, double *area);

/* Contra2Cart (Source/rhs.c:35-749), the change of basis: Cartesian
 * velocity ucat (DA Cmpnts, in/out) at the fluid cells from the centred
 * averages of the face fluxes ucont (periodic ghosts taken from their
 * partners) by Cramer's rule with the cell metrics; periodic ghosts of ucat
 * then take their partners' values; with zero_solid, cells with
 * (int)(nvert + 0.1) == 3 are set to 0 (the reference does this when
 * neither movefsi nor rotatefsi is set).  Other cells keep their ucat.  The
 * reference routine's wall functions and boundary conditions belong to the
 * momentum solver and are not part of the library. */
int vfs_poisson_contra2cart(vfs_poisson *h, const double *ucont, double *ucat, int zero_solid);

/* Solve A phi = b to opts->rtol, remove the fluid mean of phi
 * (Remove_Nullspace) and write phi to `phi` in DA layout with periodic
 * ghost copies (Convert_Phi2_Phi).  With opts->warm_start == 1, `phi` is
 * read first as the initial guess; with 2 the solve starts from the
 * handle's iterate.  `phi` may be NULL to keep phi on the device. */
int vfs_poisson_solve(vfs_poisson *h, double *phi, const vfs_solve_opts *opts, vfs_solve_stats *stats);

/* PoissonSolver_Hypre in one call: rhs + solve. */
int vfs_poisson_solver_hypre(vfs_poisson *h, const double *ucont, double dt, double st, double coeff,
                             double *phi, const vfs_solve_opts *opts, vfs_solve_stats *stats);

/* UpdatePressure: p += phi on fluid cells, p = 0 where nvert > 1.1, then
 * periodic ghost copies of p and phi (both in/out, DA layout). */
int vfs_poisson_update_pressure(vfs_poisson *h, double *p, double *phi);

/* Projection: Ucont -= dt*st/coeff * (metric-weighted grad phi) using the
 * handle's current phi, then the periodic face copy.  ucont in/out. */
int vfs_poisson_projection(vfs_poisson *h, double *ucont, double dt, double st, double coeff);

/* Divergence: max |div(Ucont) aj| over interior cells not next to a
 * blanked cell (the "Maxdiv" diagnostic). */
int vfs_poisson_divergence(vfs_poisson *h, const double *ucont, double *maxdiv);

/* FullyBlocked (Source/poisson.c:1909-1993) on the nvert of the last
 * vfs_poisson_set_nvert: *multinullspace = 1 when every interior (i, j)
 * column has a cell with nvert > 0.1 somewhere in k (boundary layers
 * included), so that the operator of the -poisson -1 path has a null space
 * per side of the blocking; ksk[my][mx] (int32, host or device; may be NULL)
 * receives the first such k per column (KSKE[2 (j mx + i)]; -1 for none and
 * on the boundary columns, where the reference leaves the entry unset). */
int vfs_poisson_fully_blocked(vfs_poisson *h, int *multinullspace, int32_t *ksk);
/* PoissonNullSpaceFunction_original (Source/poisson.c:757-943), the null
 * space removal of the -poisson -1 multigrid solve, on a DA-layout array x
 * (host or device, in place): the mean over the interior cells with nvert
 * < 0.1 is removed (with multiple null spaces separately below and above
 * each column's first blocked k); then the boundary layers and the cells with
 * nvert > 0.1 are set to 0.  The sums are reduced in another order than the
 * reference's loops (agreement to rounding). */
int vfs_poisson_nullspace_original(vfs_poisson *h, double *x);

/* ---- inspection entry points (parity tests, drop-in diagnostics) ---- */

/* Number of pressure dofs (reduced_p_size) and, if gid != NULL, the dof id
 * per DA cell as int32 (-1 where none; periodic ghosts alias partners). */
int vfs_poisson_get_numbering(vfs_poisson *h, int *ndof, int32_t *gid);

/* The assembled FP64 operator: vol[mz][my][mx][19] in the slot order of
 * Source/poisson.c:957-975 (zero where MatSetValues would not insert) and
 * the row class per DA cell (0 none, 1 fluid, 2 identity). */
int vfs_poisson_get_operator(vfs_poisson *h, double *vol, int32_t *rowtype);

/* Metrics computed by vfs_poisson_set_grid; `which` indexes the order
 * icsi,ieta,izet,jcsi,jeta,jzet,kcsi,keta,kzet,csi,eta,zet,cent (Cmpnts)
 * = 0..12 and iaj,jaj,kaj,aj = 13..16 (scalars). */
int vfs_poisson_get_metric(vfs_poisson *h, int which, double *out);

/* The right-hand side b as a DA-layout array (zero where no dof). */
int vfs_poisson_get_rhs(vfs_poisson *h, double *b);

/* y = A x with the FP64 operator (x, y DA layout, interior cells used). */
int vfs_poisson_apply(vfs_poisson *h, const double *x, double *y);

/* Multigrid hierarchy: level count, then per level the interior sizes and
 * the coarsening flags towards the next level (dims6 = nx,ny,nz,cx,cy,cz). */
int vfs_poisson_mg_levels(vfs_poisson *h, int *nlevels);
int vfs_poisson_mg_level_info(vfs_poisson *h, int level, int *dims6);
/* nvert of a level (DA layout of that level), from MyNvertRestriction. */
int vfs_poisson_mg_get_nvert(vfs_poisson *h, int level, double *nvert);
/* MyRestriction from level `fine` to fine+1 and MyInterpolation from
 * fine+1 to `fine`, on DA-layout FP64 arrays of those levels. */
int vfs_poisson_mg_restrict(vfs_poisson *h, int fine, const double *xf, double *fc);
int vfs_poisson_mg_interpolate(vfs_poisson *h, int fine, const double *xc, double *ff);
/* One V-cycle z = M r of the chosen precision on DA-layout arrays. */
int vfs_poisson_mg_vcycle(vfs_poisson *h, int precision, const double *r, double *z);

/* Number of kernel launches issued by this library since the handle was
 * created (graph-launched kernels included). */
int64_t vfs_poisson_kernel_launches(vfs_poisson *h);

/* Run the handle's work on a caller's CUDA stream (cudaStream_t passed as
 * void*); NULL returns to a private (blocking) stream.  No reference counterpart: the
 * reference is CPU-only. */
int vfs_poisson_set_stream(vfs_poisson *h, void *stream);

/* Live timing of the dominant kernel (the finest-level j-line sweep): when
 * enabled, CUDA events bracket every such launch inside the solves and
 * vfs_poisson_profile_read returns their summed device time, their summed
 * algorithmic bytes and their count since enabling. */
int vfs_poisson_profile(vfs_poisson *h, int enable);
int vfs_poisson_profile_read(vfs_poisson *h, double *ms, double *bytes, int64_t *launches);

/* Divergence without a handle and without allocating: the same value as
 * vfs_poisson_divergence, for callers that may not allocate device memory
 * where they need it (inside a CUDA stream capture, or in codes whose device
 * memory is owned by their own pool allocator).  No counterpart in the
 * reference; it restates Divergence (Source/main.c:936-1074) like
 * vfs_poisson_divergence.  All five arrays must be device memory of the
 * current device (DA layout; ucont Cmpnts); the result is written to
 * *maxdiv (device memory) on `stream` (a cudaStream_t, NULL for the default
 * stream) and the call returns without waiting.  Its scratch is a fixed
 * device array of 4096 doubles (32 KiB) that every GPU loading the library
 * keeps until exit, which limits grids to 268,435,456 interior cells (larger
 * ones return VFS_EINVAL).  The first call on a device looks up that
 * array's address; make it before any stream capture.  Every call shares the
 * array, so calls that overlap on the GPU race. */
int vfs_divergence_noalloc(const vfs_grid_desc *g, const double *ucont, const double *nvert, const double *aj,
                           double *maxdiv, void *stream);

/* Immersed-boundary classification of one body (ibm_search_advanced,
 * Source/ibm.c:92-594; point_cell_advanced :1075-1200): marks the cells of
 * nvert (DA layout, in/out) whose centre lies inside the closed triangulated
 * surface (xyz: n_v vertices x/y/z; tri: n_elmt vertex triples, 0-based) as
 * 3 and the cells within one node of them as 1, on the cell centres of the
 * handle's grid (set_grid first).  ibi == 0 first clears every interior
 * value below 5 (the first body); later bodies keep the larger value.
 * bctype (six ints or NULL): the rows next to a -1 / -2 wall become 1.
 * Each cell casts up to 64 rays (the reference's glibc rand() directions)
 * until one meets no doubled intersection; *n_failed (may be NULL) counts
 * the cells that gave up, which stay 0 before the dilation.  The result is
 * bit-identical to the reference's loops.  nvert is not installed as the
 * solver's blanking: pass it to vfs_poisson_set_nvert.  Bodies are searched
 * in order from ibi == 0 on the same array, as the reference's loop over the
 * bodies does: a later body then changes only its box of cells (and their
 * neighbours), which is all it passes over. */
int vfs_poisson_ibm_search(vfs_poisson *h, int ibi, int n_v, const double *xyz, int n_elmt, const int32_t *tri,
                           const int *bctype, double *nvert, int *n_failed);

/* One IB node's interpolation record (the reference's IBMInfo, built in
 * ibm_search_advanced, Source/ibm.c:373-508): the node (DA indices), its
 * nearest surface element (nearestcell1, :1373-1518) with the nearest point
 * pmin, the distance d_s and the point's weights cs on the element's
 * vertices; the three cell centres (ip, jp, kp) where the ray from pmin
 * through the node leaves the node's neighbourhood (InterceptionPoint,
 * :1766-2258), their weights cr and the distance d_i; imode, the triangle of
 * the 3x3 patch that ray crosses (-100: none); status 0 = found, 1 = the
 * reference's fallback next to a domain boundary (one k or j neighbour,
 * :423-505), 2 = the reference's search failure (it keeps the previous
 * node's values; here the node itself with zero weights). */
typedef struct {
  int i, j, k;
  int cell;
  double pmin[3];
  double d_s;
  double cs[3];
  int ip[3], jp[3], kp[3];
  double cr[3];
  double d_i;
  int imode;
  int status;
} vfs_ibm_node;

/* vfs_poisson_ibm_search plus the interpolation records of the body's IB
 * nodes (the cells the dilation marks for this body, in k, j, i order),
 * kept in the handle for vfs_poisson_ibm_interpolate.  *n_nodes (may be
 * NULL) receives their number. */
int vfs_poisson_ibm_search_nodes(vfs_poisson *h, int ibi, int n_v, const double *xyz, int n_elmt,
                                 const int32_t *tri, const int *bctype, double *nvert, int *n_failed,
                                 int *n_nodes);

/* Copy up to max_nodes of body ibi's IB node records to nodes (host). */
int vfs_poisson_ibm_nodes(vfs_poisson *h, int ibi, vfs_ibm_node *nodes, int max_nodes, int *n_nodes);

/* ibm_interpolation_advanced (Source/ibm.c:3301-3640) for body ibi with
 * the no-slip reconstruction (Source/wallfunction.c:140-156): at every IB
 * node ucat = Ua + d_s/(d_s + d_i) (Uc - Ua), Ua the surface velocity at
 * pmin (u_surf: n_v x 3 vertex velocities, or NULL for a body at rest),
 * Uc the weighted ucat of the three interception cells -- 0 when any of
 * those is not fluid or the node has nvert > 2.9 -- and p the weighted p of
 * the three cells; then the face fluxes ucont of every cell with
 * (int)(nvert + 0.5) == 1 and of the faces it shares with its -i/-j/-k
 * neighbours from the new ucat (times 0 with immersed == 3; the faces of
 * the -1/-2 walls in bctype set to 0), and Contra2Cart (with the solid
 * zeroing) from the new ucont.  ucat, p, ucont: DA arrays, in/out, host or
 * device; the handle's nvert (set_nvert) is the blanking.  The averaging,
 * level-set, moving-body, inviscid and wall-function branches of the
 * reference routine are momentum-solver options and are not restated. */
int vfs_poisson_ibm_interpolate(vfs_poisson *h, int ibi, const double *u_surf, int immersed, const int *bctype,
                                double *ucat, double *p, double *ucont);

/* IB_BC (Source/momentum.c:2016-2220) with immersed set: the periodic ghost
 * cells of ucat take their partners' values, the face fluxes of the cells
 * with (int)nvert == 1 and of the faces they share with their -i/-j/-k
 * neighbours are formed from ucat (0 with immersed == 3, where the faces
 * between cells whose nvert sum exceeds 1.1 are also zeroed), the faces of
 * the -1/-2 walls in i and j and of the slip (10) walls are set to 0 and
 * the periodic faces take their partners' fluxes.  ucat, ucont: DA arrays,
 * in/out.  The first-step wall marking of nvert (immersed == 0) and the
 * air-flow level-set faces are not restated. */
int vfs_poisson_ib_bc(vfs_poisson *h, int immersed, const int *bctype, double *ucat, double *ucont);

/* ---------------------------------------------------------------------
 * Learned initial guess: a 3-level 3-D U-Net (channels 16/32/64, 3x3x3
 * convolutions with ReLU, 2x2x2 average pooling, nearest upsampling with
 * skip concatenation, 1x1 head) with BF16 weights and activations on the
 * tensor cores and FP32 accumulation.  No counterpart in the reference.
 *
 * Parameters (FP32 master copy, vfs_unet_num_params floats) are laid out
 * layer by layer, encoder e0a e0b e1a e1b e2a e2b then decoder d1a d1b d0a
 * d0b, each as W[tap][cin][cout] (tap = 9 kz + 3 ky + kx, input channel
 * ci of a concatenation: upsampled source first) followed by bias[cout];
 * then the head's 16 weights and its bias.  The first layer has 16 input
 * channels, of which the network feeds 4 (the feature planes) and zeros.
 * --------------------------------------------------------------------- */
typedef struct vfs_unet vfs_unet;

/* A sub-box of feature planes (device memory, FP32): features
 * [4][fz][fy][fx], target and weight [fz][fy][fx] (training only).  The
 * network runs on the sub-box (ox..ox+nx-1, ...); nx, ny, nz multiples of 4.
 * Without `op` the loss is sum(weight * (out - target)^2) / sum(weight).
 * With `op` (the 19 planes [19][fz][fy][fx] of the row-scaled operator, as
 * vfs_poisson_get_operator32 gives them) the loss is
 *   mse_weight * that  +  res_weight * sum_i w_i res_i^2 / sum_i w_i,
 *   res = features[2] - op_scale * (A out)
 * over the sub-box cells whose 19 neighbours lie inside it: the residual of
 * the correction the output stands for, in the units of feature plane 2. */
typedef struct {
  const float *features;
  const float *target;
  const float *weight;
  int fx, fy, fz;
  int ox, oy, oz;
  int nx, ny, nz;
  const float *op;
  float op_scale;
  float mse_weight;
  float res_weight;
} vfs_unet_batch;

int vfs_unet_create(unsigned int seed, vfs_unet **out);
void vfs_unet_destroy(vfs_unet *u);
int vfs_unet_set_stream(vfs_unet *u, void *stream);
int64_t vfs_unet_num_params(vfs_unet *u);
/* host or device pointers of vfs_unet_num_params floats */
int vfs_unet_get_params(vfs_unet *u, float *out);
int vfs_unet_set_params(vfs_unet *u, const float *in);
/* out: [nz][ny][nx] FP32 device memory; asynchronous on the U-Net's stream */
int vfs_unet_forward(vfs_unet *u, const vfs_unet_batch *b, float *out);
/* loss and gradient of the batch (grad: host or device, may be NULL) */
int vfs_unet_gradient(vfs_unet *u, const vfs_unet_batch *b, float *grad, double *loss);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) on the batch's gradient */
int vfs_unet_train_step(vfs_unet *u, const vfs_unet_batch *b, double lr, double *loss);
/* Adam update from the current gradient (as left by vfs_unet_gradient or
 * vfs_unet_set_grads) */
int vfs_unet_adam(vfs_unet *u, double lr, double beta1, double beta2, double eps);
int vfs_unet_set_grads(vfs_unet *u, const float *grad);
int64_t vfs_unet_kernel_launches(vfs_unet *u);

/* Initial guess from a history of solutions (no counterpart in the
 * reference, which restarts from the previous step's Phi2,
 * poisson_hypre.c:577).  The handle keeps the last k converged solutions
 * X_j (1 <= k <= 12; 0 turns it off) and their images A X_j (b - r of the
 * solves that produced them) under the operator assembly current when each
 * was stored, as the newest solution and the differences of consecutive
 * ones.  vfs_poisson_history_guess, after vfs_poisson_rhs, forms two
 * candidates:
 *   - the projection x = sum_j c_j X_j over the solutions of the current
 *     assembly, with c minimising ||b - sum_j c_j A X_j||_2 (Fischer's
 *     projection for successive right-hand sides, CMAME 163 (1998) 193-204),
 *     solved by normal equations in the difference basis, whose Gram entries
 *     are formed from the differences themselves (the raw images of
 *     successive solutions are too nearly parallel for normal equations);
 *     never above the previous step's phi in residual;
 *   - the extrapolation 2 X_0 - X_1 of the newest two solutions (its
 *     residual from the stored images, or by an operator apply when a moving
 *     mask made them stale);
 * and installs the one the judge prefers as the iterate for the next solve
 * (opts.warm_start = 2), with its exact FP64 residual.  The judge: a
 * candidate whose residual exceeds 32x the other's loses outright (the
 * extrapolation is not even formed when the Gram matrix predicts that);
 * otherwise each is rated by its estimated error, the 2-norm of one V-cycle
 * of its residual with the fluid mean removed, and the smaller wins.  A
 * least-squares fit of the residual can leave a smooth error of small
 * residual that the iteration removes slowly (after a mask moves, the
 * projection's error is often several times the extrapolation's); that
 * V-cycle then becomes the solve's first preconditioned vector, so the
 * judging costs one V-cycle per losing candidate.  rel_res gets
 * ||b - A x|| / ||b|| of the installed guess.  Each converged solve appends
 * its solution.  Memory: 2 k + 4 box-sized FP64 vectors.  Up to about 8
 * solutions for sequences solved to rtol 1e-8 by about one V-cycle per
 * step: a fit over more reaches the stored solutions' own errors, and the
 * solutions then drift from step to step while every residual meets rtol. */
int vfs_poisson_set_history(vfs_poisson *h, int k);
int vfs_poisson_history_guess(vfs_poisson *h, double *rel_res);
/* Whether converged solves append to the history (default 1): 0 lets a
 * second solver sequence share the handle without entering it. */
int vfs_poisson_history_record(vfs_poisson *h, int on);

/* With a history, vfs_poisson_learned_guess puts the network's candidate
 * before the same judge as the history's projection and the extrapolation;
 * while the network's candidate keeps losing, the network runs on every
 * `period`-th call only (the others judge the history's candidates alone and
 * report rel_res[1] = -1).  Default 1.  The network is not run either when
 * the projection's residual is below the extrapolation's by more than
 * 1024x. */
int vfs_poisson_set_network_period(vfs_poisson *h, int period);

/* What the last vfs_poisson_history_guess / vfs_poisson_learned_guess
 * installed (no counterpart in the reference).  *chosen: 0 the projection
 * (or the previous step's phi when no history is kept), 1 the network's
 * candidate, 2 the extrapolation.  rel_res[3] and est[3] (either may be
 * NULL), indexed by those codes: each candidate's ||b - A x|| / ||b|| and
 * its estimated error (2-norm of one V-cycle of its residual, fluid mean
 * removed, in units of phi); -1 where the candidate was not formed or not
 * rated. */
int vfs_poisson_guess_report(vfs_poisson *h, int *chosen, double *rel_res, double *est);

/* Learned initial guess for the current right-hand side (vfs_poisson_rhs
 * first), from phi at steps n-1 and n-2 (DA layout, host or device).  The
 * network sees four planes on the half-resolution grid (2x2x2 averages over
 * the dof cells): phi_{n-1}, phi_{n-1} - phi_{n-2}, aj * (b - A phi_ex)
 * with phi_ex = 2 phi_{n-1} - phi_{n-2} (the residual of the linear
 * extrapolation in the aj-scaled system), each divided by its RMS over the
 * dofs, and the dof fraction.  Its output, the correction phi_n - phi_ex in
 * units of kappa * RMS(aj * (b - A phi_ex)), is prolonged trilinearly to the
 * cells and smoothed by two passes of the 27-point binomial filter
 * (environment variable VFS_GUESS_SMOOTH sets the count), and enters in 4
 * wall-distance bands whose weights minimise the residual.  The judge of
 * vfs_poisson_history_guess then chooses among the base (the history's
 * projection; the previous step's phi without a history), the extrapolation
 * phi_ex and the network's guess (formed only when its predicted residual is
 * within 32x of the best).  *chosen: 0 base, 1 network, 2 extrapolation;
 * rel_res[0] = the base's relative residual (-1 without one), rel_res[1] =
 * the network guess's (the extrapolation's when every band weight is 0).
 * Solve from it with opts.warm_start = 2.  The network runs on the handle's
 * stream (its stream is set to it); box dims must be multiples of 8. */
int vfs_poisson_learned_guess(vfs_poisson *h, vfs_unet *u, const double *phi_nm1, const double *phi_nm2,
                              double kappa, int *chosen, double *rel_res);

/* One training sample of the learned guess on the half-resolution grid
 * (box dims / 2): the four feature planes of the current right-hand side
 * (as above), the target (phi_n - phi_ex) / RMS(aj * (b - A phi_ex))
 * averaged over the dof children, and the loss weight (dof fraction); FP32
 * device memory (features 4 planes; target, weight 1 plane). */
int vfs_poisson_guess_sample(vfs_poisson *h, const double *phi_n, const double *phi_nm1, const double *phi_nm2,
                             float *features, float *target, float *weight);

/* The finest level's row-scaled FP32 operator (the aj-scaled PoissonLHSNew
 * rows of the V-cycle): 19 box-layout planes in the slot order C E W N S T
 * B NE SE NW SW TN BN TS BS TE BE TW BW (host or device memory, 19 n). */
int vfs_poisson_get_operator32(vfs_poisson *h, float *planes);

/* ---------------------------------------------------------------------
 * The reference's input files (host code, no GPU).  Two-call pattern:
 * with a NULL output buffer a call only reports the sizes.
 * --------------------------------------------------------------------- */

/* PETSc binary vector (VecView / VecLoadIntoVector of the restart fields
 * vfield / pfield / nvfield, Source/main.c:376-935): big-endian class id
 * 1211214, length, values.  On one rank a DA vector is stored in the DA
 * natural layout, so these are the library's DA arrays (Cmpnts fields
 * interleaved).  *n: in: buffer length; out: the vector's length. */
int vfs_read_petsc_vec(const char *path, int64_t *n, double *values);
int vfs_write_petsc_vec(const char *path, int64_t n, const double *values);

/* Grid nodes (Source/init.c:254-366).  format 0: xyz.dat (IM JM KM, then
 * IM rows "x y z" of which x is used, JM rows for y, KM rows for z: a
 * tensor-product grid); 1: grid.dat as text (block count, then per block
 * IM JM KM and the IM*JM*KM x values, then y, then z, i fastest); 2: the
 * same in native binary.  dims[0..2] = IM, JM, KM of block `block`; coor
 * (may be NULL) is the DA-layout node array [KM+1][JM+1][IM+1][3] (node
 * (i,j,k) at i < IM, the last layer left as is), coordinates / cl * L_dim. */
int vfs_read_grid(const char *path, int format, int block, double L_dim, double cl, int *dims, double *coor);

/* UCD surface (ibmdata%02d, ibm_read_ucd, Source/ibm_io.c:782-1011): three
 * header lines, "n_v n_elmt 0 0 0", n_v rows "id x y z", n_elmt rows
 * "id mat tri n1 n2 n3" (1-based).  place (may be NULL): L_dim, CMx_c,
 * CMy_c, CMz_c, x_r, y_r, z_r, angle_x0, angle_y0, angle_z0 - the
 * reference's scaling, offset and initial rotations, applied in its order.
 * xyz: n_v x 3; tri: n_elmt x 3, 0-based; *n_v / *n_elmt: in: capacities,
 * out: counts. */
int vfs_read_ucd(const char *path, const double *place, int *n_v, int *n_elmt, double *xyz, int32_t *tri);

#ifdef __cplusplus
}
#endif
#endif
