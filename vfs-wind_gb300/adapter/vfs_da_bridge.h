/* vfs_da_bridge.h -- the library's C ABI driven from PETSc 3.1 DA vectors.
 *
 * The reference keeps every field of a block in PETSc DA vectors spread over
 * the MPI ranks of the block's DA (Source/init.c:141-161: box stencil of
 * width 3, periodic wrap for ii/jj/kk_periodic).  This bridge moves the
 * global (non-ghosted) vectors to and from the library's DA-natural layout
 * ([k][j][i], dof interleaved, index 0 and m-1 the boundary layer): every
 * rank takes part in the gather to rank 0 (DAGlobalToNatural +
 * VecScatterCreateToZero), rank 0 alone calls the library on its GPU, and
 * the results go back the same way (SCATTER_REVERSE + DANaturalToGlobal).
 * Ghosted local vectors are never read: with a periodic DA their arrays
 * start at gxs = -3 with rows of gxm = mx + 6 points, so only the global
 * vectors have the library's layout.  After writing a global vector the
 * caller refreshes its ghosted copy (DAGlobalToLocalBegin/End), as the
 * reference does after its own updates.
 *
 * Every function is collective over the DA's communicator and returns 0 or
 * a VFS_* code (the same on every rank; the message is in vfs_last_error()
 * on rank 0).  One bridge per block, single-threaded.
 */
#ifndef VFS_DA_BRIDGE_H
#define VFS_DA_BRIDGE_H

#include "petscda.h"
#include "vfs_poisson.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vfsa_block vfsa_block;

/* A bridge for the block of DA `da` (dof 1) and its vector DA `fda`
 * (dof 3); `desc` gives the periodic flags and bctype[3].  Rank 0 creates
 * the library handle on its current CUDA device. */
int vfsa_create(DA da, DA fda, const vfs_grid_desc *desc, vfsa_block **out);
void vfsa_destroy(vfsa_block *b);
/* The library handle (rank 0; NULL elsewhere). */
vfs_poisson *vfsa_handle(vfsa_block *b);

/* Natural-order copy of a global vector of `da` (dof components per point)
 * on rank 0 (`natural` may be NULL on the other ranks), and its inverse. */
int vfsa_gather(DA da, Vec global, double *natural);
int vfsa_scatter(DA da, const double *natural, Vec global);

/* FormMetrics from the node coordinates (global coordinate vector of the
 * DA, DAGetCoordinates). */
int vfsa_set_grid(vfsa_block *b, Vec coords);
/* setup_lidx2 + PoissonLHSNew + multigrid hierarchy from the global Nvert. */
int vfsa_set_nvert(vfsa_block *b, Vec nvert);
/* VolumeFlux on the global Ucont (in/out): the immersed variant (flg 0)
 * when immersed == 1, the other overload otherwise. */
int vfsa_volume_flux(vfsa_block *b, Vec ucont, int immersed, double *flux, double *area);
/* PoissonRHS2_hypre + the solve + Remove_Nullspace + Convert_Phi2_Phi:
 * phi (global, in: the warm start with opts->warm_start == 1; out: the
 * solution with periodic ghost copies). */
int vfsa_solve(vfsa_block *b, Vec ucont, double dt, double st, double coeff, Vec phi, const vfs_solve_opts *opts,
               vfs_solve_stats *stats);
/* UpdatePressure: p and phi global, in/out. */
int vfsa_update_pressure(vfsa_block *b, Vec p, Vec phi);
/* Projection with the phi of the last solve or update: ucont global, in/out. */
int vfsa_projection(vfsa_block *b, Vec ucont, double dt, double st, double coeff);
/* Divergence maximum of the global Ucont (the same value on every rank). */
int vfsa_divergence(vfsa_block *b, Vec ucont, double *maxdiv);

#ifdef __cplusplus
}
#endif
#endif
