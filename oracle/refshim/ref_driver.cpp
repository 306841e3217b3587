// ref_driver.cpp -- host harness around the reference's own pressure-Poisson
// functions (Source/metrics.c, Source/poisson.c, Source/poisson_hypre.c,
// Source/main.c compiled unmodified against petsc_shim.h).
//
// Test infrastructure only.  It builds one block's UserCtx the way
// MG_Initial does for one level (Source/init.c:141-161, 591-700: a DA of
// IM+1 x JM+1 x KM+1 points with a box stencil of width 3, periodic wrap for
// the ii/jj/kk flags, the coordinate DA, the global and ghosted vectors),
// calls the reference's functions on it and copies the results out in the
// DA-natural layout, so that tests compare them with the oracle's
// restatement and with the CUDA library.  The exported functions are
// extern "C" for ctypes.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "variables.h"

// globals of the reference (defined in Source/main.c)
extern PetscInt ti, tistart, immersed, movefsi, rotatefsi, block_number;
extern int levelset, fix_level, periodic, poisson;
extern int i_periodic, ii_periodic, j_periodic, jj_periodic, k_periodic, kk_periodic;
extern double poisson_tol;
extern PetscReal poisson_threshold;
extern char path[256];

// functions of the reference's translation units that variables.h does not
// declare
PetscInt setup_lidx2(UserCtx *user);
void PoissonSolver_Hypre(UserCtx *user, IBMNodes *ibm, IBMInfo *ibminfo);
PetscErrorCode FullyBlocked(UserCtx *user);
PetscErrorCode MyNvertRestriction(UserCtx *user_h, UserCtx *user_c);
PetscErrorCode VolumeFlux(UserCtx *user, Vec lUcor, PetscReal *ibm_Flux, PetscReal *ibm_Area);
PetscErrorCode VolumeFlux(UserCtx *user, PetscReal *ibm_Flux, PetscReal *ibm_Area, PetscInt flg);
PetscErrorCode Divergence(UserCtx *user);
PetscErrorCode PoissonNullSpaceFunction_original(MatNullSpace nsp, Vec X, void *ctx);

namespace {

// the inner solve of vr_solver_hypre: records the right-hand side the
// reference hands to HYPRE, then runs the harness's solver
double *g_capture_b = nullptr;
vfs_shim_solve_fn g_inner = nullptr;
int capture_solve(int n, const int *rp, const int *cols, const double *vals, const double *rhs, double *x,
                  double rtol) {
  if (g_capture_b) memcpy(g_capture_b, rhs, sizeof(double) * n);
  return g_inner(n, rp, cols, vals, rhs, x, rtol);
}

struct VecSlot {
  const char *name;
  Vec UserCtx::*field;
  int vector_da;  // 1: fda (3 components), 0: da
  int local;
};

#define G(n, f, v) {n, &UserCtx::f, v, 0}
#define L(n, f, v) {n, &UserCtx::f, v, 1}
const VecSlot kSlots[] = {
    G("csi", Csi, 1), G("eta", Eta, 1), G("zet", Zet, 1), G("icsi", ICsi, 1), G("ieta", IEta, 1),
    G("izet", IZet, 1), G("jcsi", JCsi, 1), G("jeta", JEta, 1), G("jzet", JZet, 1), G("kcsi", KCsi, 1),
    G("keta", KEta, 1), G("kzet", KZet, 1), G("cent", Cent, 1), G("ucont", Ucont, 1), G("ucat", Ucat, 1),
    G("gridspace", GridSpace, 1), G("ucont_o", Ucont_o, 1),
    G("aj", Aj, 0), G("iaj", IAj, 0), G("jaj", JAj, 0), G("kaj", KAj, 0), G("p", P, 0), G("phi", Phi, 0),
    G("nvert", Nvert, 0), G("nvert_o", Nvert_o, 0), G("p_o", P_o, 0),
    L("lcsi", lCsi, 1), L("leta", lEta, 1), L("lzet", lZet, 1), L("licsi", lICsi, 1), L("lieta", lIEta, 1),
    L("lizet", lIZet, 1), L("ljcsi", lJCsi, 1), L("ljeta", lJEta, 1), L("ljzet", lJZet, 1), L("lkcsi", lKCsi, 1),
    L("lketa", lKEta, 1), L("lkzet", lKZet, 1), L("lcent", lCent, 1), L("lucont", lUcont, 1), L("lucat", lUcat, 1),
    L("lgridspace", lGridSpace, 1),
    L("laj", lAj, 0), L("liaj", lIAj, 0), L("ljaj", lJAj, 0), L("lkaj", lKAj, 0), L("lp", lP, 0), L("lphi", lPhi, 0),
    L("lnvert", lNvert, 0), L("lnvert_o", lNvert_o, 0), L("lucat_old", lUcat_old, 1), L("lustar", lUstar, 0),
    G("levelset", Levelset, 0), L("llevelset", lLevelset, 0), L("ldensity", lDensity, 0), L("lmu", lMu, 0),
};
#undef G
#undef L

struct Ctx {
  UserCtx *u = nullptr;
  std::vector<Vec> owned;
  int ndof = 0;
};

const VecSlot *slot(const char *name) {
  for (const VecSlot &s : kSlots)
    if (!strcmp(s.name, name)) return &s;
  return nullptr;
}

void set_globals(const int per[6], int immersed_flag) {
  i_periodic = per[0]; j_periodic = per[1]; k_periodic = per[2];
  ii_periodic = per[3]; jj_periodic = per[4]; kk_periodic = per[5];
  periodic = i_periodic + j_periodic + k_periodic + ii_periodic + jj_periodic + kk_periodic;
  immersed = immersed_flag;
  levelset = 0;
  fix_level = 0;
  movefsi = rotatefsi = 0;
  ti = tistart = 0;
  block_number = 1;
  poisson = 1;
}

// global -> ghosted copy of one vector (DAGlobalToLocal), as the
// reference's driver does after it writes a global field
void refresh_local(Ctx *c, const VecSlot *s) {
  UserCtx *u = c->u;
  std::string ln = std::string("l") + s->name;
  const VecSlot *l = slot(ln.c_str());
  if (!l) return;
  DA d = s->vector_da ? u->fda : u->da;
  DAGlobalToLocalBegin(d, u->*(s->field), INSERT_VALUES, u->*(l->field));
  DAGlobalToLocalEnd(d, u->*(s->field), INSERT_VALUES, u->*(l->field));
}

// FormMetrics keeps its results in the ghosted vectors only (it destroys the
// global metric vectors, Source/metrics.c:1065-1084): these names are read
// from the owned part of their ghosted copies
bool ghosted_result(const char *name) {
  static const char *m[] = {"csi", "eta", "zet", "aj", "icsi", "ieta", "izet", "iaj", "jcsi", "jeta",
                            "jzet", "jaj", "kcsi", "keta", "kzet", "kaj", "cent", "gridspace"};
  for (const char *q : m)
    if (!strcmp(q, name)) return true;
  return false;
}

// owned points of a ghosted vector in DA-natural order
void copy_owned(const DALocalInfo &i, int dof, const double *src, double *out) {
  for (int k = 0; k < i.mz; k++)
    for (int j = 0; j < i.my; j++)
      for (int a = 0; a < i.mx; a++)
        for (int q = 0; q < dof; q++)
          out[(((size_t)k * i.my + j) * i.mx + a) * dof + q] =
              src[(((size_t)(k - i.gzs) * i.gym + (j - i.gys)) * i.gxm + (a - i.gxs)) * dof + q];
}

}  // namespace

extern "C" {

// One block: DA of mx x my x mz points (IM = mx - 1 nodes), periodic flags
// (i, j, k, ii, jj, kk), bctype[6], node coordinates [mz][my][mx][3]
// (DA natural layout), immersed flag.
void *vr_create(int mx, int my, int mz, const int *per, const int *bctype, const double *coor, int immersed_flag) {
  set_globals(per, immersed_flag);
  Ctx *c = new Ctx();
  UserCtx *u = (UserCtx *)calloc(1, sizeof(UserCtx));
  c->u = u;
  DAPeriodicType wrap = DA_NONPERIODIC;
  if (ii_periodic && jj_periodic && kk_periodic) wrap = DA_XYZPERIODIC;
  else if (ii_periodic && jj_periodic) wrap = DA_XYPERIODIC;
  else if (jj_periodic && kk_periodic) wrap = DA_YZPERIODIC;
  else if (ii_periodic && kk_periodic) wrap = DA_XZPERIODIC;
  else if (ii_periodic) wrap = DA_XPERIODIC;
  else if (jj_periodic) wrap = DA_YPERIODIC;
  else if (kk_periodic) wrap = DA_ZPERIODIC;
  DACreate3d(PETSC_COMM_WORLD, wrap, DA_STENCIL_BOX, mx, my, mz, 1, 1, 1, 1, 3, PETSC_NULL, PETSC_NULL, PETSC_NULL,
             &u->da);
  u->aotopetsc = PETSC_FALSE;
  DASetUniformCoordinates(u->da, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0);
  DAGetCoordinateDA(u->da, &u->fda);
  DAGetLocalInfo(u->da, &u->info);
  u->IM = mx - 1;
  u->JM = my - 1;
  u->KM = mz - 1;
  for (int q = 0; q < 6; q++) u->bctype[q] = bctype ? bctype[q] : 0;
  u->dt = 1.;
  u->st = 1.;
  u->ren = 1.;
  u->assignedA = PETSC_FALSE;
  u->thislevel = 0;
  u->mglevels = 1;
  for (const VecSlot &s : kSlots) {
    DA d = s.vector_da ? u->fda : u->da;
    Vec v;
    if (s.local) DACreateLocalVector(d, &v);
    else DACreateGlobalVector(d, &v);
    u->*(s.field) = v;
    vfs_shim_vec_retain(v);  // survives a VecDestroy inside the reference
    c->owned.push_back(v);
  }
  Vec X;
  DAGetCoordinates(u->da, &X);
  int n = 0;
  double *x = vfs_shim_vec_data(X, &n);
  memcpy(x, coor, sizeof(double) * (size_t)n);
  return c;
}

void vr_destroy(void *h) {
  Ctx *c = (Ctx *)h;
  if (!c) return;
  free(c->u->KSKE);
  for (Vec v : c->owned) {
    VecDestroy(v);
    VecDestroy(v);
  }
  free(c->u);
  delete c;
}

// Copy a named vector out in DA-natural layout: "gid" is the numbering
// written by setup_lidx2 (owned points of its ghosted vector), "phi2" the
// compact solution, the metric names the owned part of their ghosted copies,
// every other name the global vector.
int vr_get(void *h, const char *name, double *out, long n) {
  Ctx *c = (Ctx *)h;
  const DALocalInfo &i = c->u->info;
  const long npts = (long)i.mx * i.my * i.mz;
  if (!strcmp(name, "gid")) {
    if (!c->u->Gid) return -2;
    if (n != npts) return -3;
    copy_owned(i, 1, vfs_shim_vec_data(c->u->Gid, nullptr), out);
    return 0;
  }
  if (!strcmp(name, "phi2")) {
    if (!c->u->Phi2) return -2;
    int m = 0;
    const double *d = vfs_shim_vec_data(c->u->Phi2, &m);
    if (m != n) return -3;
    memcpy(out, d, sizeof(double) * (size_t)n);
    return 0;
  }
  const VecSlot *s = slot(name);
  if (!s || s->local) return -1;
  const int dof = s->vector_da ? 3 : 1;
  if (n != npts * dof) return -3;
  if (ghosted_result(name)) {
    std::string ln = std::string("l") + name;
    const VecSlot *l = slot(ln.c_str());
    copy_owned(i, dof, vfs_shim_vec_data(c->u->*(l->field), nullptr), out);
    return 0;
  }
  memcpy(out, vfs_shim_vec_data(c->u->*(s->field), nullptr), sizeof(double) * (size_t)n);
  return 0;
}

// Set a named vector from a DA-natural array.  A global vector's ghosted
// copy is refreshed (DAGlobalToLocal); a ghosted vector named directly gets
// the array on its owned points and its ghosts from them (DALocalToLocal).
int vr_set(void *h, const char *name, const double *in, long n) {
  Ctx *c = (Ctx *)h;
  Vec v = nullptr;
  const VecSlot *ls = slot(name);
  if (ls && ls->local) {
    const DALocalInfo &i = c->u->info;
    const int dof = ls->vector_da ? 3 : 1;
    if (n != (long)i.mx * i.my * i.mz * dof) return -3;
    Vec lv = c->u->*(ls->field);
    double *d = vfs_shim_vec_data(lv, nullptr);
    for (int k = 0; k < i.mz; k++)
      for (int j = 0; j < i.my; j++)
        for (int a = 0; a < i.mx; a++)
          for (int q = 0; q < dof; q++)
            d[(((size_t)(k - i.gzs) * i.gym + (j - i.gys)) * i.gxm + (a - i.gxs)) * dof + q] =
                in[(((size_t)k * i.my + j) * i.mx + a) * dof + q];
    DA da = ls->vector_da ? c->u->fda : c->u->da;
    DALocalToLocalBegin(da, lv, INSERT_VALUES, lv);
    DALocalToLocalEnd(da, lv, INSERT_VALUES, lv);
    return 0;
  }
  if (!strcmp(name, "phi2")) v = c->u->Phi2;
  else {
    const VecSlot *s = slot(name);
    if (!s) return -1;
    v = c->u->*(s->field);
  }
  if (!v) return -2;
  int m = 0;
  double *d = vfs_shim_vec_data(v, &m);
  if (m != n) return -3;
  memcpy(d, in, sizeof(double) * (size_t)n);
  const VecSlot *s = slot(name);
  if (s) refresh_local(c, s);
  return 0;
}

// FormMetrics (Source/metrics.c:12-1355)
int vr_form_metrics(void *h) {
  Ctx *c = (Ctx *)h;
  FormMetrics(c->u);
  return 0;
}

// PoissonLHSNew (Source/poisson.c:977-1688), which numbers the dofs with
// setup_lidx2 on its first call; returns the dof count and the CSR size.
int vr_lhs(void *h, int *ndof, int *nnz) {
  Ctx *c = (Ctx *)h;
  PoissonLHSNew(c->u, nullptr, nullptr);
  int n = 0;
  const int *rp, *cols;
  const double *vals;
  vfs_shim_mat_csr(c->u->A, &n, &rp, &cols, &vals);
  c->ndof = n;
  *ndof = n;
  *nnz = rp[n];
  return 0;
}
int vr_lhs_csr(void *h, int *rowptr, int *cols, double *vals) {
  Ctx *c = (Ctx *)h;
  int n = 0;
  const int *rp, *cc;
  const double *vv;
  vfs_shim_mat_csr(c->u->A, &n, &rp, &cc, &vv);
  memcpy(rowptr, rp, sizeof(int) * (n + 1));
  memcpy(cols, cc, sizeof(int) * rp[n]);
  memcpy(vals, vv, sizeof(double) * rp[n]);
  return 0;
}

// PoissonRHS2 (Source/poisson.c:1780-1906) for -poisson `pflag` into a
// vector of the dof count.
int vr_rhs2(void *h, int pflag, double *b) {
  Ctx *c = (Ctx *)h;
  poisson = pflag;
  Vec B;
  VecDuplicate(c->u->Phi2, &B);
  PoissonRHS2(c->u, B);
  int n = 0;
  const double *d = vfs_shim_vec_data(B, &n);
  memcpy(b, d, sizeof(double) * n);
  VecDestroy(B);
  poisson = 1;
  return 0;
}

// PoissonSolver_Hypre (Source/poisson_hypre.c:506-636) for the first time
// step: LHS, HYPRE matrix copy, VolumeFlux, PoissonRHS2_hypre with
// Remove_Nullspace_Scale, the inner solve (the registered FP64 solver in
// place of HYPRE GMRES + BoomerAMG, to relative tolerance `tol`),
// Remove_Nullspace and Convert_Phi2_Phi.  `b_out` receives the right-hand
// side handed to the solver (dof count), `phi2_out` the compact solution.
int vr_solver_hypre(void *h, vfs_shim_solve_fn solver, double tol, double *b_out, double *phi2_out) {
  Ctx *c = (Ctx *)h;
  poisson_tol = tol;
  g_capture_b = b_out;
  g_inner = solver;
  vfs_shim_set_solver(&capture_solve);
  PoissonSolver_Hypre(c->u, nullptr, nullptr);
  vfs_shim_set_solver(nullptr);
  int n = 0;
  const double *d = vfs_shim_vec_data(c->u->Phi2, &n);
  c->ndof = n;
  if (phi2_out) memcpy(phi2_out, d, sizeof(double) * n);
  return n;
}

// UpdatePressure (Source/poisson.c:3137-3297) and Projection
// (Source/poisson.c:2700-3066) with the current Phi; dt, st and the time
// coefficient come from the UserCtx (1 by default).
int vr_update_pressure(void *h) {
  Ctx *c = (Ctx *)h;
  UpdatePressure(c->u);
  return 0;
}
int vr_projection(void *h, double dt, double st) {
  Ctx *c = (Ctx *)h;
  c->u->dt = dt;
  c->u->st = st;
  Projection(c->u);
  return 0;
}

// Divergence (Source/main.c:936-1074): the maximum it reduces with VecMax.
int vr_divergence(void *h, double *maxdiv) {
  Ctx *c = (Ctx *)h;
  Divergence(c->u);
  *maxdiv = vfs_shim_last_vecmax();
  return 0;
}

// VolumeFlux: the immersed variant (Source/poisson.c:3563-3903) with flg,
// or the immersed == 0 variant on Ucont (Source/poisson.c:3299-3493).
int vr_volume_flux(void *h, int immersed_variant, int flg, double *flux, double *area) {
  Ctx *c = (Ctx *)h;
  int old = immersed;
  if (immersed_variant) {
    immersed = 1;
    VolumeFlux(c->u, flux, area, flg);
  } else {
    immersed = 0;
    VolumeFlux(c->u, c->u->Ucont, flux, area);
  }
  immersed = old;
  return 0;
}

// FullyBlocked (Source/poisson.c:1909-1993) on the current Nvert: the
// multiple-null-space flag and KSKE[2 (j mx + i)] per interior column in
// ksk[j mx + i] (-1 where the reference leaves the entry unset).
int vr_fully_blocked(void *h, int *multi, int *ksk) {
  Ctx *c = (Ctx *)h;
  const DALocalInfo &i = c->u->info;
  const int n = 2 * i.mx * i.my;
  if (!c->u->KSKE) c->u->KSKE = (PetscInt *)malloc(sizeof(PetscInt) * n);
  for (int q = 0; q < n; q++) c->u->KSKE[q] = -1;
  FullyBlocked(c->u);
  *multi = c->u->multinullspace ? 1 : 0;
  for (int q = 0; q < i.mx * i.my; q++) ksk[q] = c->u->KSKE[2 * q];
  return 0;
}

// PoissonNullSpaceFunction_original (Source/poisson.c:757-943) on a
// DA-natural array x (through the global Phi vector), with the flag and
// KSKE of the last vr_fully_blocked.
int vr_nullspace_original(void *h, double *x, long n) {
  Ctx *c = (Ctx *)h;
  int m = 0;
  double *d = vfs_shim_vec_data(c->u->Phi, &m);
  if (m != n) return -3;
  memcpy(d, x, sizeof(double) * (size_t)n);
  PoissonNullSpaceFunction_original(nullptr, c->u->Phi, c->u);
  memcpy(x, d, sizeof(double) * (size_t)n);
  return 0;
}

}  // extern "C"
