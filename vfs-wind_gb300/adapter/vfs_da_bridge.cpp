// vfs_da_bridge.cpp -- PETSc 3.1 DA vectors <-> the library's C ABI.
// See vfs_da_bridge.h.  Builds against PETSc 3.1's headers (petscda.h,
// petscvec.h) and links against libvfs_poisson.so.
#include "vfs_da_bridge.h"

#include <string.h>

#include <vector>

#include "petscvec.h"

struct vfsa_block {
  DA da = nullptr, fda = nullptr;
  vfs_poisson *h = nullptr;
  int rank = 0;
  size_t n = 0;  // DA points
  std::vector<double> s1, s2, s3;  // rank-0 staging (natural order)
};

namespace {

int comm_rank() {
  int r = 0;
  MPI_Comm_rank(PETSC_COMM_WORLD, &r);
  return r;
}

// rank 0's status on every rank
int agree(int rc) {
  MPI_Bcast(&rc, 1, MPI_INT, 0, PETSC_COMM_WORLD);
  return rc;
}

size_t da_points(DA da, int *dof) {
  PetscInt M = 0, N = 0, P = 0, d = 1;
  DAGetInfo(da, PETSC_NULL, &M, &N, &P, PETSC_NULL, PETSC_NULL, PETSC_NULL, &d, PETSC_NULL, PETSC_NULL,
            PETSC_NULL);
  if (dof) *dof = d;
  return (size_t)M * N * P;
}

}  // namespace

extern "C" {

int vfsa_gather(DA da, Vec global, double *natural) {
  Vec nat, seq;
  VecScatter sc;
  DACreateNaturalVector(da, &nat);
  DAGlobalToNaturalBegin(da, global, INSERT_VALUES, nat);
  DAGlobalToNaturalEnd(da, global, INSERT_VALUES, nat);
  VecScatterCreateToZero(nat, &sc, &seq);
  VecScatterBegin(sc, nat, seq, INSERT_VALUES, SCATTER_FORWARD);
  VecScatterEnd(sc, nat, seq, INSERT_VALUES, SCATTER_FORWARD);
  int rc = VFS_OK;
  if (comm_rank() == 0) {
    PetscInt n = 0;
    PetscScalar *a;
    VecGetSize(seq, &n);
    VecGetArray(seq, &a);
    if (natural) memcpy(natural, a, sizeof(double) * (size_t)n);
    else rc = VFS_EINVAL;
    VecRestoreArray(seq, &a);
  }
  VecScatterDestroy(sc);
  VecDestroy(seq);
  VecDestroy(nat);
  return agree(rc);
}

int vfsa_scatter(DA da, const double *natural, Vec global) {
  Vec nat, seq;
  VecScatter sc;
  DACreateNaturalVector(da, &nat);
  VecScatterCreateToZero(nat, &sc, &seq);
  int rc = VFS_OK;
  if (comm_rank() == 0) {
    PetscInt n = 0;
    PetscScalar *a;
    VecGetSize(seq, &n);
    VecGetArray(seq, &a);
    if (natural) memcpy(a, natural, sizeof(double) * (size_t)n);
    else rc = VFS_EINVAL;
    VecRestoreArray(seq, &a);
  }
  rc = agree(rc);
  if (rc == VFS_OK) {
    VecScatterBegin(sc, seq, nat, INSERT_VALUES, SCATTER_REVERSE);
    VecScatterEnd(sc, seq, nat, INSERT_VALUES, SCATTER_REVERSE);
    DANaturalToGlobalBegin(da, nat, INSERT_VALUES, global);
    DANaturalToGlobalEnd(da, nat, INSERT_VALUES, global);
  }
  VecScatterDestroy(sc);
  VecDestroy(seq);
  VecDestroy(nat);
  return rc;
}

int vfsa_create(DA da, DA fda, const vfs_grid_desc *desc, vfsa_block **out) {
  if (!out || !desc) return VFS_EINVAL;
  vfsa_block *b = new vfsa_block();
  b->da = da;
  b->fda = fda;
  b->rank = comm_rank();
  b->n = da_points(da, nullptr);
  int rc = VFS_OK;
  if (b->rank == 0) {
    if ((size_t)desc->mx * desc->my * desc->mz != b->n) rc = VFS_EINVAL;
    else rc = vfs_poisson_create(desc, &b->h);
    if (rc == VFS_OK) {
      b->s1.resize(b->n);
      b->s2.resize(b->n);
      b->s3.resize(3 * b->n);
    }
  }
  rc = agree(rc);
  if (rc != VFS_OK) {
    vfsa_destroy(b);
    return rc;
  }
  *out = b;
  return VFS_OK;
}

void vfsa_destroy(vfsa_block *b) {
  if (!b) return;
  if (b->h) vfs_poisson_destroy(b->h);
  delete b;
}

vfs_poisson *vfsa_handle(vfsa_block *b) { return b ? b->h : nullptr; }

int vfsa_set_grid(vfsa_block *b, Vec coords) {
  int rc = vfsa_gather(b->fda, coords, b->rank == 0 ? b->s3.data() : nullptr);
  if (rc != VFS_OK) return rc;
  if (b->rank == 0) rc = vfs_poisson_set_grid(b->h, b->s3.data(), nullptr);
  return agree(rc);
}

int vfsa_set_nvert(vfsa_block *b, Vec nvert) {
  int rc = vfsa_gather(b->da, nvert, b->rank == 0 ? b->s1.data() : nullptr);
  if (rc != VFS_OK) return rc;
  if (b->rank == 0) rc = vfs_poisson_set_nvert(b->h, b->s1.data());
  return agree(rc);
}

int vfsa_volume_flux(vfsa_block *b, Vec ucont, int immersed, double *flux, double *area) {
  int rc = vfsa_gather(b->fda, ucont, b->rank == 0 ? b->s3.data() : nullptr);
  if (rc != VFS_OK) return rc;
  double fa[2] = {0., 0.};
  if (b->rank == 0) {
    rc = immersed == 1 ? vfs_poisson_volume_flux(b->h, b->s3.data(), 0, 0., &fa[0], &fa[1])
                       : vfs_poisson_volume_flux0(b->h, b->s3.data(), immersed, &fa[0], &fa[1]);
  }
  rc = agree(rc);
  if (rc != VFS_OK) return rc;
  MPI_Bcast(fa, 2, MPI_DOUBLE, 0, PETSC_COMM_WORLD);
  if (flux) *flux = fa[0];
  if (area) *area = fa[1];
  return vfsa_scatter(b->fda, b->rank == 0 ? b->s3.data() : nullptr, ucont);
}

int vfsa_solve(vfsa_block *b, Vec ucont, double dt, double st, double coeff, Vec phi, const vfs_solve_opts *opts,
               vfs_solve_stats *stats) {
  int rc = vfsa_gather(b->fda, ucont, b->rank == 0 ? b->s3.data() : nullptr);
  if (rc == VFS_OK) rc = vfsa_gather(b->da, phi, b->rank == 0 ? b->s1.data() : nullptr);
  if (rc != VFS_OK) return rc;
  vfs_solve_stats st_local;
  memset(&st_local, 0, sizeof(st_local));
  if (b->rank == 0) {
    rc = vfs_poisson_rhs(b->h, b->s3.data(), dt, st, coeff);
    if (rc == VFS_OK) rc = vfs_poisson_solve(b->h, b->s1.data(), opts, &st_local);
  }
  rc = agree(rc);
  MPI_Bcast(&st_local, (int)sizeof(st_local), MPI_CHAR, 0, PETSC_COMM_WORLD);
  if (stats) *stats = st_local;
  if (rc != VFS_OK && rc != VFS_ENOCONV) return rc;
  const int rs = vfsa_scatter(b->da, b->rank == 0 ? b->s1.data() : nullptr, phi);
  return rs != VFS_OK ? rs : rc;
}

int vfsa_update_pressure(vfsa_block *b, Vec p, Vec phi) {
  int rc = vfsa_gather(b->da, p, b->rank == 0 ? b->s2.data() : nullptr);
  if (rc == VFS_OK) rc = vfsa_gather(b->da, phi, b->rank == 0 ? b->s1.data() : nullptr);
  if (rc != VFS_OK) return rc;
  if (b->rank == 0) rc = vfs_poisson_update_pressure(b->h, b->s2.data(), b->s1.data());
  rc = agree(rc);
  if (rc != VFS_OK) return rc;
  rc = vfsa_scatter(b->da, b->rank == 0 ? b->s2.data() : nullptr, p);
  if (rc != VFS_OK) return rc;
  return vfsa_scatter(b->da, b->rank == 0 ? b->s1.data() : nullptr, phi);
}

int vfsa_projection(vfsa_block *b, Vec ucont, double dt, double st, double coeff) {
  int rc = vfsa_gather(b->fda, ucont, b->rank == 0 ? b->s3.data() : nullptr);
  if (rc != VFS_OK) return rc;
  if (b->rank == 0) rc = vfs_poisson_projection(b->h, b->s3.data(), dt, st, coeff);
  rc = agree(rc);
  if (rc != VFS_OK) return rc;
  return vfsa_scatter(b->fda, b->rank == 0 ? b->s3.data() : nullptr, ucont);
}

int vfsa_divergence(vfsa_block *b, Vec ucont, double *maxdiv) {
  int rc = vfsa_gather(b->fda, ucont, b->rank == 0 ? b->s3.data() : nullptr);
  if (rc != VFS_OK) return rc;
  double m = 0.;
  if (b->rank == 0) rc = vfs_poisson_divergence(b->h, b->s3.data(), &m);
  rc = agree(rc);
  MPI_Bcast(&m, 1, MPI_DOUBLE, 0, PETSC_COMM_WORLD);
  if (maxdiv) *maxdiv = m;
  return rc;
}

}  // extern "C"
