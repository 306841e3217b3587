// vfs_userctx_adapter.cpp -- link-time drop-in for the reference's
// pressure-projection entry points (declared in Source/variables.h:676-704,
// called from Flow_Solver, Source/solvers.c:647-690):
//
//   void PoissonSolver_Hypre(UserCtx *, IBMNodes *, IBMInfo *)   poisson_hypre.c:506
//   PetscErrorCode UpdatePressure(UserCtx *)                      poisson.c:3137
//   PetscErrorCode Projection(UserCtx *)                          poisson.c:2700
//   PetscErrorCode Divergence(UserCtx *)                          main.c:936
//
// Built inside the reference's Source/ directory (it includes variables.h)
// against PETSc 3.1, with the reference's own definitions of these four
// functions renamed at compile time (-DPoissonSolver_Hypre=... on
// poisson_hypre.c, -DUpdatePressure=... -DProjection=... on poisson.c,
// -DDivergence=... on main.c); every other reference function stays as it
// is.  Each block gets a bridge (vfs_da_bridge.h) and a library handle on
// rank 0's GPU at its first call.  Arrays move through the global DA vectors
// (Ucont, Nvert, P, Phi, the DA coordinates); after each update the ghosted
// copies are refreshed the way the reference refreshes them.
//
// Semantics kept: the mask and operator are rebuilt at the first step and
// whenever movefsi, rotatefsi or an unfixed level set moves the mask
// (poisson_hypre.c:548-565); VolumeFlux before the right-hand side
// (:559-561); the warm start from the previous phi (:577); Remove_Nullspace
// and Convert_Phi2_Phi; Projection ends with the reference's own
// Contra2Cart; the timing and Maxdiv lines go to path/Converge_dU.  Not
// supported (the call stops the run with a message): immersed == 2
// (Add_IBMFlux_to_Outlet), level-set runs, free-surface pressure cells.
// A failure of the library stops the run (MPI_Abort): these functions have
// no error path in the reference.
#include <map>

#include "variables.h"
#include "vfs_da_bridge.h"

extern PetscInt ti, tistart, immersed, movefsi, rotatefsi, freesurface;
extern int levelset, fix_level, poisson_it;
extern int i_periodic, ii_periodic, j_periodic, jj_periodic, k_periodic, kk_periodic;
extern double poisson_tol;
extern char path[256];
double time_coeff();               // Source/poisson.c:23
void Contra2Cart(UserCtx *user);   // Source/rhs.c:35

namespace {

struct Block {
  vfsa_block *b = nullptr;
  bool mask_set = false;
};
std::map<UserCtx *, Block> g_blocks;

void stop(const char *where, int rc) {
  int rank = 0;
  MPI_Comm_rank(PETSC_COMM_WORLD, &rank);
  if (rank == 0) fprintf(stderr, "GPU pressure projection: %s failed (%d): %s\n", where, rc, vfs_last_error());
  MPI_Abort(PETSC_COMM_WORLD, 1);
  abort();
}

void check(const char *where, int rc) {
  if (rc != VFS_OK) stop(where, rc);
}

Block &block(UserCtx *user) {
  Block &k = g_blocks[user];
  if (!k.b) {
    if (immersed == 2 || levelset || freesurface) {
      PetscPrintf(PETSC_COMM_WORLD, "GPU pressure projection: immersed 2, level set and free surface are not "
                                    "supported\n");
      stop("set-up", VFS_EINVAL);
    }
    vfs_grid_desc g;
    g.mx = user->info.mx;
    g.my = user->info.my;
    g.mz = user->info.mz;
    g.i_periodic = i_periodic;
    g.j_periodic = j_periodic;
    g.k_periodic = k_periodic;
    g.ii_periodic = ii_periodic;
    g.jj_periodic = jj_periodic;
    g.kk_periodic = kk_periodic;
    g.bctype3 = user->bctype[3];
    check("vfs_poisson_create", vfsa_create(user->da, user->fda, &g, &k.b));
    Vec coords;
    DAGetCoordinates(user->da, &coords);
    check("vfs_poisson_set_grid", vfsa_set_grid(k.b, coords));
  }
  return k;
}

void refresh(DA da, Vec global, Vec local) {
  DAGlobalToLocalBegin(da, global, INSERT_VALUES, local);
  DAGlobalToLocalEnd(da, global, INSERT_VALUES, local);
}

}  // namespace

void PoissonSolver_Hypre(UserCtx *user, IBMNodes *, IBMInfo *) {
  PetscLogDouble ts, te;
  PetscGetTime(&ts);
  Block &k = block(user);
  if (!k.mask_set || movefsi || rotatefsi) {
    check("vfs_poisson_set_nvert", vfsa_set_nvert(k.b, user->Nvert));
    k.mask_set = true;
  }
  double flux = 0., area = 0.;
  check("VolumeFlux", vfsa_volume_flux(k.b, user->Ucont, immersed, &flux, &area));
  refresh(user->fda, user->Ucont, user->lUcont);
  vfs_solve_opts o;
  vfs_poisson_default_opts(&o);
  o.rtol = poisson_tol;
  o.max_it = poisson_it > 20 ? poisson_it : 20;
  o.warm_start = 1;  // the previous step's phi (the reference's Phi2 restart)
  vfs_solve_stats st;
  const int rc = vfsa_solve(k.b, user->Ucont, user->dt, user->st, time_coeff(), user->Phi, &o, &st);
  if (rc != VFS_OK && rc != VFS_ENOCONV) stop("vfs_poisson_solve", rc);
  refresh(user->da, user->Phi, user->lPhi);
  PetscGetTime(&te);
  PetscPrintf(PETSC_COMM_WORLD, "GPU Poisson: %d iterations, relative residual %.3e\n", st.iterations,
              st.rel_residual);
  int rank = 0;
  MPI_Comm_rank(PETSC_COMM_WORLD, &rank);
  if (!rank) {
    char filen[300];
    snprintf(filen, sizeof(filen), "%s/Converge_dU", path);
    FILE *f = fopen(filen, "a");
    if (f) {
      PetscFPrintf(PETSC_COMM_WORLD, f, "%d(poisson)  %.2e(s)", (int)ti, te - ts);
      fclose(f);
    }
  }
}

PetscErrorCode UpdatePressure(UserCtx *user) {
  Block &k = block(user);
  check("vfs_poisson_update_pressure", vfsa_update_pressure(k.b, user->P, user->Phi));
  refresh(user->da, user->P, user->lP);
  refresh(user->da, user->Phi, user->lPhi);
  return 0;
}

PetscErrorCode Projection(UserCtx *user) {
  Block &k = block(user);
  check("vfs_poisson_projection", vfsa_projection(k.b, user->Ucont, user->dt, user->st, time_coeff()));
  refresh(user->fda, user->Ucont, user->lUcont);
  Contra2Cart(user);
  return 0;
}

PetscErrorCode Divergence(UserCtx *user) {
  Block &k = block(user);
  double maxdiv = 0.;
  check("vfs_poisson_divergence", vfsa_divergence(k.b, user->Ucont, &maxdiv));
  PetscPrintf(PETSC_COMM_WORLD, "Maxdiv %d %e\n", (int)ti, maxdiv);
  int rank = 0;
  MPI_Comm_rank(PETSC_COMM_WORLD, &rank);
  if (!rank) {
    char filen[300];
    snprintf(filen, sizeof(filen), "%s/Converge_dU", path);
    FILE *f = fopen(filen, "a");
    if (f) {
      PetscFPrintf(PETSC_COMM_WORLD, f, " Maxdiv=%.2e\n", maxdiv);
      fclose(f);
    }
  }
  return 0;
}
