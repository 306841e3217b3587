// adapter_harness.cpp -- test helper: builds PETSc-DA-shaped inputs for the
// DA bridge (vfs-wind_gb300/adapter/vfs_da_bridge.cpp) on the single-rank
// PETSc stand-in of oracle/refshim/, and reads DA vectors back by their own
// [k][j][i] indexing (DAVecGetArray), independently of the bridge.
#include <string.h>

#include "petscda.h"
#include "petscvec.h"

extern "C" {

// DA of mx x my x mz points, dof components, box stencil of width 3 with
// the wrap of the ii/jj/kk flags (the reference's MGDACreate,
// Source/init.c:141-161)
void *ah_da_create(int mx, int my, int mz, int ii, int jj, int kk, int dof) {
  DAPeriodicType wrap = DA_NONPERIODIC;
  if (ii && jj && kk) wrap = DA_XYZPERIODIC;
  else if (ii && jj) wrap = DA_XYPERIODIC;
  else if (jj && kk) wrap = DA_YZPERIODIC;
  else if (ii && kk) wrap = DA_XZPERIODIC;
  else if (ii) wrap = DA_XPERIODIC;
  else if (jj) wrap = DA_YPERIODIC;
  else if (kk) wrap = DA_ZPERIODIC;
  DA da;
  DACreate3d(PETSC_COMM_WORLD, wrap, DA_STENCIL_BOX, mx, my, mz, 1, 1, 1, dof, 3, PETSC_NULL, PETSC_NULL,
             PETSC_NULL, &da);
  return da;
}
void *ah_coordinate_da(void *da) {
  DA c;
  DASetUniformCoordinates((DA)da, 0., 1., 0., 1., 0., 1.);
  DAGetCoordinateDA((DA)da, &c);
  return c;
}
void *ah_coordinates(void *da) {
  Vec v;
  DAGetCoordinates((DA)da, &v);
  return v;
}
void *ah_global(void *da) {
  Vec v;
  DACreateGlobalVector((DA)da, &v);
  return v;
}
void ah_vec_destroy(void *v) { VecDestroy((Vec)v); }

// global vector <-> natural array through the DA's own [k][j][i] view
void ah_fill(void *da, void *vec, const double *natural, int dof) {
  DALocalInfo info;
  DAGetLocalInfo((DA)da, &info);
  double ***a;
  DAVecGetArray((DA)da, (Vec)vec, &a);
  for (int k = info.zs; k < info.zs + info.zm; k++)
    for (int j = info.ys; j < info.ys + info.ym; j++)
      for (int i = info.xs; i < info.xs + info.xm; i++)
        for (int c = 0; c < dof; c++)
          a[k][j][i * dof + c] = natural[(((size_t)k * info.my + j) * info.mx + i) * dof + c];
  DAVecRestoreArray((DA)da, (Vec)vec, &a);
}
void ah_read(void *da, void *vec, double *natural, int dof) {
  DALocalInfo info;
  DAGetLocalInfo((DA)da, &info);
  double ***a;
  DAVecGetArray((DA)da, (Vec)vec, &a);
  for (int k = info.zs; k < info.zs + info.zm; k++)
    for (int j = info.ys; j < info.ys + info.ym; j++)
      for (int i = info.xs; i < info.xs + info.xm; i++)
        for (int c = 0; c < dof; c++)
          natural[(((size_t)k * info.my + j) * info.mx + i) * dof + c] = a[k][j][i * dof + c];
  DAVecRestoreArray((DA)da, (Vec)vec, &a);
}
// value of component c at (i, j, k) of the ghosted copy of a global
// vector (indices may lie in the ghost layer, e.g. -3 .. -1)
double ah_ghosted(void *da, void *vec, int i, int j, int k, int c, int dof) {
  Vec l;
  DACreateLocalVector((DA)da, &l);
  DAGlobalToLocalBegin((DA)da, (Vec)vec, INSERT_VALUES, l);
  DAGlobalToLocalEnd((DA)da, (Vec)vec, INSERT_VALUES, l);
  double ***a;
  DAVecGetArray((DA)da, l, &a);
  const double v = a[k][j][i * dof + c];
  DAVecRestoreArray((DA)da, l, &a);
  VecDestroy(l);
  return v;
}
void ah_ghost_corners(void *da, int *out6) {
  DALocalInfo info;
  DAGetLocalInfo((DA)da, &info);
  out6[0] = info.gxs; out6[1] = info.gys; out6[2] = info.gzs;
  out6[3] = info.gxm; out6[4] = info.gym; out6[5] = info.gzm;
}

}  // extern "C"
