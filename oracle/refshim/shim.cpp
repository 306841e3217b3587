// shim.cpp -- single-rank implementation of the PETSc 3.1 / HYPRE / MPI
// subset declared in petsc_shim.h.  Test infrastructure: it exists only so
// that the reference's own translation units can run on the host and pin
// the oracle.  See petsc_shim.h for the semantics.
#include "petsc_shim.h"

#include <execinfo.h>
#include <unistd.h>

#include <chrono>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

[[noreturn]] void unreached(const char *fn) {
  fprintf(stderr, "refshim: %s is not provided by the single-rank stand-in\n", fn);
  void *frames[32];
  const int n = backtrace(frames, 32);
  backtrace_symbols_fd(frames, n, 2);
  abort();
}

bool verbose() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("VFS_SHIM_VERBOSE");
    v = e && e[0] == '1';
  }
  return v == 1;
}

std::map<std::string, std::string> &options() {
  static std::map<std::string, std::string> o;
  return o;
}

vfs_shim_solve_fn g_solver = nullptr;

}  // namespace

// ------------------------------------------------------------ objects ----
struct _p_DA {
  int mx, my, mz, dof, s;
  DAPeriodicType pt;
  bool px, py, pz;
  DA cda = nullptr;    // coordinate DA (dof 3)
  Vec coords = nullptr;  // global coordinate vector
  Vec gcoords = nullptr; // ghosted coordinates (rebuilt on request)
  bool owns_cda = false;
  int gs(int per) const { return per ? -s : 0; }
  int gxs() const { return gs(px); }
  int gys() const { return gs(py); }
  int gzs() const { return gs(pz); }
  int gxm() const { return mx + (px ? 2 * s : 0); }
  int gym() const { return my + (py ? 2 * s : 0); }
  int gzm() const { return mz + (pz ? 2 * s : 0); }
  size_t gsize() const { return (size_t)mx * my * mz * dof; }
  size_t lsize() const { return (size_t)gxm() * gym() * gzm() * dof; }
};

struct _p_Vec {
  std::vector<double> v;
  DA da = nullptr;
  bool local = false;
  int refs = 1;
};

struct _p_Mat {
  int m = 0, n = 0;
  bool shell = false;
  void *ctx = nullptr;
  PetscErrorCode (*mult)(Mat, Vec, Vec) = nullptr;
  std::vector<std::map<int, double>> rows;
  std::vector<int> rowptr, cols;
  std::vector<double> vals;
  void build() {
    rowptr.assign(1, 0);
    cols.clear();
    vals.clear();
    for (auto &r : rows) {
      for (auto &e : r) {
        cols.push_back(e.first);
        vals.push_back(e.second);
      }
      rowptr.push_back((int)cols.size());
    }
  }
};

struct _p_MatNullSpace {
  bool has_cnst = false;
  std::vector<Vec> vecs;
  PetscErrorCode (*fn)(MatNullSpace, Vec, void *) = nullptr;
  void *ctx = nullptr;
};
struct _p_KSP {
  PC pc = nullptr;
};
struct _p_PC {
  int dummy = 0;
};
struct _p_SNES {
  int dummy = 0;
};
struct _p_VecScatter {
  int dummy = 0;
};
struct _p_PetscViewer {
  int dummy = 0;
};

struct hypre_IJVector_struct {
  int lo = 0, hi = -1;
  std::vector<double> v;
};
struct hypre_IJMatrix_struct {
  int lo = 0, hi = -1;
  std::vector<std::map<int, double>> rows;
  std::vector<int> rowptr, cols;
  std::vector<double> vals;
};
struct hypre_Solver_struct {
  double tol = 1e-8;
  int maxit = 1000;
};

// ---------------------------------------------------------------- MPI ----
static size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_CHAR: return 1;
    case MPI_FLOAT: return sizeof(float);
    case MPI_LONG: return sizeof(long);
  }
  return 8;
}
int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
int MPI_Allreduce(void *a, void *b, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (a != MPI_IN_PLACE && a != b) memmove(b, a, n * type_size(t));
  return 0;
}
int MPI_Reduce(void *a, void *b, int n, MPI_Datatype t, MPI_Op o, int, MPI_Comm c) {
  return MPI_Allreduce(a, b, n, t, o, c);
}
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Send(void *, int, MPI_Datatype, int, int, MPI_Comm) { unreached("MPI_Send"); }
int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { unreached("MPI_Recv"); }
int MPI_Gather(void *a, int n, MPI_Datatype t, void *b, int, MPI_Datatype, int, MPI_Comm) {
  memmove(b, a, n * type_size(t));
  return 0;
}
int MPI_Allgather(void *a, int n, MPI_Datatype t, void *b, int, MPI_Datatype, MPI_Comm) {
  memmove(b, a, n * type_size(t));
  return 0;
}
int MPI_Abort(MPI_Comm, int code) {
  fflush(stdout);
  fflush(stderr);
  _exit(code ? code : 1);
}
double MPI_Wtime(void) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ------------------------------------------------------------- system ----
PetscErrorCode PetscInitialize(int *, char ***, const char[], const char[]) { return 0; }
PetscErrorCode PetscFinalize(void) { return 0; }
PetscErrorCode PetscPrintf(MPI_Comm, const char f[], ...) {
  if (!verbose()) return 0;
  va_list a;
  va_start(a, f);
  vfprintf(stderr, f, a);
  va_end(a);
  return 0;
}
PetscErrorCode PetscFPrintf(MPI_Comm, FILE *fp, const char f[], ...) {
  va_list a;
  va_start(a, f);
  if (fp == stdout || fp == stderr) {
    if (verbose()) vfprintf(stderr, f, a);
  } else if (fp) {
    vfprintf(fp, f, a);
  }
  va_end(a);
  return 0;
}
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm c, const char f[], ...) {
  if (!verbose()) return 0;
  va_list a;
  va_start(a, f);
  vfprintf(stderr, f, a);
  va_end(a);
  (void)c;
  return 0;
}
PetscErrorCode PetscSynchronizedFlush(MPI_Comm) { return 0; }
PetscErrorCode PetscBarrier(PetscObject) { return 0; }
PetscErrorCode PetscGetTime(PetscLogDouble *t) {
  *t = MPI_Wtime();
  return 0;
}
PetscErrorCode PetscGlobalSum(const PetscReal *a, PetscReal *b, MPI_Comm) { *b = *a; return 0; }
PetscErrorCode PetscGlobalMax(const PetscReal *a, PetscReal *b, MPI_Comm) { *b = *a; return 0; }
PetscErrorCode PetscGlobalMin(const PetscReal *a, PetscReal *b, MPI_Comm) { *b = *a; return 0; }
PetscErrorCode PetscMallocShim(size_t n, void **p) {
  *p = calloc(n ? n : 1, 1);
  return *p ? 0 : 55;
}
PetscErrorCode PetscFreeShim(void *p) {
  free(p);
  return 0;
}

// options database: "-name value" pairs from PetscOptionsInsertString
PetscErrorCode PetscOptionsInsertString(const char s[]) {
  std::vector<std::string> tok;
  std::string cur;
  for (const char *p = s; ; p++) {
    if (*p == 0 || *p == ' ' || *p == '\t' || *p == '\n') {
      if (!cur.empty()) tok.push_back(cur);
      cur.clear();
      if (*p == 0) break;
    } else {
      cur += *p;
    }
  }
  for (size_t q = 0; q < tok.size(); q++) {
    if (tok[q][0] != '-') continue;
    std::string val;
    if (q + 1 < tok.size() && !(tok[q + 1][0] == '-' && tok[q + 1].size() > 1 && !isdigit(tok[q + 1][1]) &&
                                tok[q + 1][1] != '.'))
      val = tok[++q];
    options()[tok[q - (val.empty() ? 0 : 1)].substr(1)] = val;
  }
  return 0;
}
PetscErrorCode PetscOptionsInsertFile(MPI_Comm, const char[], PetscTruth) { return 0; }
PetscErrorCode PetscOptionsClearValue(const char n[]) {
  options().erase(n[0] == '-' ? n + 1 : n);
  return 0;
}
static const std::string *opt(const char pre[], const char name[]) {
  std::string k = std::string(pre ? pre : "") + (name[0] == '-' ? name + 1 : name);
  auto it = options().find(k);
  return it == options().end() ? nullptr : &it->second;
}
PetscErrorCode PetscOptionsGetInt(const char pre[], const char name[], PetscInt *v, PetscTruth *f) {
  const std::string *s = opt(pre, name);
  if (s && !s->empty()) *v = atoi(s->c_str());
  if (f) *f = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetReal(const char pre[], const char name[], PetscReal *v, PetscTruth *f) {
  const std::string *s = opt(pre, name);
  if (s && !s->empty()) *v = atof(s->c_str());
  if (f) *f = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetString(const char pre[], const char name[], char out[], size_t len, PetscTruth *f) {
  const std::string *s = opt(pre, name);
  if (s && len) {
    strncpy(out, s->c_str(), len - 1);
    out[len - 1] = 0;
  }
  if (f) *f = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetTruth(const char pre[], const char name[], PetscTruth *v, PetscTruth *f) {
  const std::string *s = opt(pre, name);
  if (s) *v = (s->empty() || *s == "1" || *s == "true" || *s == "yes") ? PETSC_TRUE : PETSC_FALSE;
  if (f) *f = s ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetIntArray(const char[], const char[], PetscInt[], PetscInt *n, PetscTruth *f) {
  if (n) *n = 0;
  if (f) *f = PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetRealArray(const char[], const char[], PetscReal[], PetscInt *n, PetscTruth *f) {
  if (n) *n = 0;
  if (f) *f = PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsHasName(const char pre[], const char name[], PetscTruth *f) {
  *f = opt(pre, name) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm, const char[], PetscFileMode, PetscViewer *) {
  unreached("PetscViewerBinaryOpen");
}
PetscErrorCode PetscViewerDestroy(PetscViewer) { return 0; }

// ------------------------------------------------------------ vectors ----
static Vec new_vec(size_t n, DA da, bool local) {
  Vec v = new _p_Vec();
  v->v.assign(n, 0.0);
  v->da = da;
  v->local = local;
  return v;
}
PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt n, PetscInt N, Vec *v) {
  *v = new_vec(N >= 0 ? N : n, nullptr, false);
  return 0;
}
PetscErrorCode VecCreateSeq(MPI_Comm, PetscInt n, Vec *v) {
  *v = new_vec(n, nullptr, false);
  return 0;
}
PetscErrorCode VecDuplicate(Vec a, Vec *b) {
  if (!a) unreached("VecDuplicate of a null vector");
  *b = new_vec(a->v.size(), a->da, a->local);
  return 0;
}
PetscErrorCode VecDestroy(Vec a) {
  if (a && --a->refs == 0) delete a;
  return 0;
}
PetscErrorCode VecSet(Vec a, PetscScalar s) {
  for (auto &x : a->v) x = s;
  return 0;
}
PetscErrorCode VecCopy(Vec a, Vec b) {
  if (a->v.size() != b->v.size()) unreached("VecCopy of vectors of different sizes");
  b->v = a->v;
  return 0;
}
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x) {
  for (size_t q = 0; q < y->v.size(); q++) y->v[q] += a * x->v[q];
  return 0;
}
PetscErrorCode VecAYPX(Vec y, PetscScalar b, Vec x) {
  for (size_t q = 0; q < y->v.size(); q++) y->v[q] = x->v[q] + b * y->v[q];
  return 0;
}
PetscErrorCode VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y) {
  for (size_t q = 0; q < w->v.size(); q++) w->v[q] = a * x->v[q] + y->v[q];
  return 0;
}
PetscErrorCode VecScale(Vec x, PetscScalar a) {
  for (auto &e : x->v) e *= a;
  return 0;
}
PetscErrorCode VecShift(Vec x, PetscScalar a) {
  for (auto &e : x->v) e += a;
  return 0;
}
PetscErrorCode VecSum(Vec x, PetscScalar *s) {
  double t = 0.;
  for (double e : x->v) t += e;
  *s = t;
  return 0;
}
static double g_last_vecmax = 0.;
PetscErrorCode VecMax(Vec x, PetscInt *i, PetscReal *m) {
  double best = -HUGE_VAL;
  int at = -1;
  for (size_t q = 0; q < x->v.size(); q++)
    if (x->v[q] > best) { best = x->v[q]; at = (int)q; }
  if (i) *i = at;
  *m = best;
  g_last_vecmax = best;
  return 0;
}
PetscErrorCode VecMin(Vec x, PetscInt *i, PetscReal *m) {
  double best = HUGE_VAL;
  int at = -1;
  for (size_t q = 0; q < x->v.size(); q++)
    if (x->v[q] < best) { best = x->v[q]; at = (int)q; }
  if (i) *i = at;
  *m = best;
  return 0;
}
PetscErrorCode VecNorm(Vec x, NormType t, PetscReal *r) {
  double s = 0.;
  if (t == NORM_2 || t == NORM_FROBENIUS) {
    for (double e : x->v) s += e * e;
    s = sqrt(s);
  } else if (t == NORM_1) {
    for (double e : x->v) s += fabs(e);
  } else if (t == NORM_INFINITY) {
    for (double e : x->v) s = fabs(e) > s ? fabs(e) : s;
  } else {
    unreached("VecNorm(NORM_1_AND_2)");
  }
  *r = s;
  return 0;
}
PetscErrorCode VecDot(Vec x, Vec y, PetscScalar *r) {
  double s = 0.;
  for (size_t q = 0; q < x->v.size(); q++) s += y->v[q] * x->v[q];
  *r = s;
  return 0;
}
PetscErrorCode VecPointwiseDivide(Vec w, Vec x, Vec y) {
  for (size_t q = 0; q < w->v.size(); q++) w->v[q] = x->v[q] / y->v[q];
  return 0;
}
PetscErrorCode VecPointwiseMult(Vec w, Vec x, Vec y) {
  for (size_t q = 0; q < w->v.size(); q++) w->v[q] = x->v[q] * y->v[q];
  return 0;
}
PetscErrorCode VecGetSize(Vec x, PetscInt *n) { *n = (PetscInt)x->v.size(); return 0; }
PetscErrorCode VecGetLocalSize(Vec x, PetscInt *n) { *n = (PetscInt)x->v.size(); return 0; }
PetscErrorCode VecGetOwnershipRange(Vec x, PetscInt *lo, PetscInt *hi) {
  if (lo) *lo = 0;
  if (hi) *hi = (PetscInt)x->v.size();
  return 0;
}
PetscErrorCode VecGetArray(Vec x, PetscScalar **a) { *a = x->v.data(); return 0; }
PetscErrorCode VecRestoreArray(Vec, PetscScalar **) { return 0; }

// [m][n][p] view with starting indices (mstart, nstart, pstart)
PetscErrorCode VecGetArray3d(Vec x, PetscInt m, PetscInt n, PetscInt p, PetscInt ms, PetscInt ns, PetscInt ps,
                             PetscScalar ****a) {
  if ((size_t)m * n * p > x->v.size()) unreached("VecGetArray3d beyond the vector");
  double ***t = (double ***)malloc(sizeof(double **) * m + sizeof(double *) * m * n);
  double **rows = (double **)(t + m);
  for (int k = 0; k < m; k++) {
    t[k] = rows + (size_t)k * n - ns;
    for (int j = 0; j < n; j++) rows[(size_t)k * n + j] = x->v.data() + ((size_t)k * n + j) * p - ps;
  }
  *a = t - ms;
  return 0;
}
PetscErrorCode VecRestoreArray3d(Vec, PetscInt, PetscInt, PetscInt, PetscInt ms, PetscInt, PetscInt,
                                 PetscScalar ****a) {
  free(*a + ms);
  *a = nullptr;
  return 0;
}
PetscErrorCode VecSetValues(Vec x, PetscInt n, const PetscInt idx[], const PetscScalar val[], InsertMode mode) {
  for (int q = 0; q < n; q++) {
    if (idx[q] < 0) continue;
    if ((size_t)idx[q] >= x->v.size()) unreached("VecSetValues index out of range");
    if (mode == ADD_VALUES) x->v[idx[q]] += val[q];
    else x->v[idx[q]] = val[q];
  }
  return 0;
}
PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
PetscErrorCode VecView(Vec, PetscViewer) { unreached("VecView"); }
PetscErrorCode VecLoadIntoVector(PetscViewer, Vec) { unreached("VecLoadIntoVector"); }
PetscErrorCode VecScatterCreateToZero(Vec x, VecScatter *s, Vec *y) {
  *s = new _p_VecScatter();
  *y = new_vec(x->v.size(), nullptr, false);
  return 0;
}
PetscErrorCode VecScatterCreateToAll(Vec x, VecScatter *s, Vec *y) { return VecScatterCreateToZero(x, s, y); }
// one rank: every scatter is the identity map from the first vector (the
// source, in either direction) to the second
PetscErrorCode VecScatterBegin(VecScatter, Vec a, Vec b, InsertMode mode, ScatterMode) {
  for (size_t q = 0; q < b->v.size() && q < a->v.size(); q++)
    b->v[q] = mode == ADD_VALUES ? b->v[q] + a->v[q] : a->v[q];
  return 0;
}
PetscErrorCode VecScatterEnd(VecScatter, Vec, Vec, InsertMode, ScatterMode) { return 0; }
PetscErrorCode VecScatterDestroy(VecScatter s) {
  delete s;
  return 0;
}

// -------------------------------------------------------- structured grid ----
PetscErrorCode DACreate3d(MPI_Comm, DAPeriodicType pt, DAStencilType, PetscInt M, PetscInt N, PetscInt P, PetscInt,
                          PetscInt, PetscInt, PetscInt dof, PetscInt s, PetscInt *, PetscInt *, PetscInt *, DA *da) {
  DA d = new _p_DA();
  d->mx = M; d->my = N; d->mz = P; d->dof = dof; d->s = s; d->pt = pt;
  d->px = pt == DA_XPERIODIC || pt == DA_XYPERIODIC || pt == DA_XZPERIODIC || pt == DA_XYZPERIODIC;
  d->py = pt == DA_YPERIODIC || pt == DA_XYPERIODIC || pt == DA_YZPERIODIC || pt == DA_XYZPERIODIC;
  d->pz = pt == DA_ZPERIODIC || pt == DA_XZPERIODIC || pt == DA_YZPERIODIC || pt == DA_XYZPERIODIC;
  *da = d;
  return 0;
}
PetscErrorCode DADestroy(DA d) {
  if (!d) return 0;
  if (d->coords) VecDestroy(d->coords);
  if (d->gcoords) VecDestroy(d->gcoords);
  if (d->owns_cda) DADestroy(d->cda);
  delete d;
  return 0;
}
PetscErrorCode DAGetInfo(DA d, PetscInt *dim, PetscInt *M, PetscInt *N, PetscInt *P, PetscInt *m, PetscInt *n,
                         PetscInt *p, PetscInt *dof, PetscInt *s, DAPeriodicType *pt, DAStencilType *st) {
  if (dim) *dim = 3;
  if (M) *M = d->mx;
  if (N) *N = d->my;
  if (P) *P = d->mz;
  if (m) *m = 1;
  if (n) *n = 1;
  if (p) *p = 1;
  if (dof) *dof = d->dof;
  if (s) *s = d->s;
  if (pt) *pt = d->pt;
  if (st) *st = DA_STENCIL_BOX;
  return 0;
}
PetscErrorCode DAGetLocalInfo(DA d, DALocalInfo *i) {
  i->dim = 3; i->dof = d->dof; i->sw = d->s;
  i->mx = d->mx; i->my = d->my; i->mz = d->mz;
  i->xs = i->ys = i->zs = 0;
  i->xm = d->mx; i->ym = d->my; i->zm = d->mz;
  i->gxs = d->gxs(); i->gys = d->gys(); i->gzs = d->gzs();
  i->gxm = d->gxm(); i->gym = d->gym(); i->gzm = d->gzm();
  i->pt = d->pt; i->st = DA_STENCIL_BOX; i->da = d;
  return 0;
}
PetscErrorCode DAGetCorners(DA d, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n, PetscInt *p) {
  if (x) *x = 0;
  if (y) *y = 0;
  if (z) *z = 0;
  if (m) *m = d->mx;
  if (n) *n = d->my;
  if (p) *p = d->mz;
  return 0;
}
PetscErrorCode DAGetGhostCorners(DA d, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n,
                                 PetscInt *p) {
  if (x) *x = d->gxs();
  if (y) *y = d->gys();
  if (z) *z = d->gzs();
  if (m) *m = d->gxm();
  if (n) *n = d->gym();
  if (p) *p = d->gzm();
  return 0;
}
static DA coord_da(DA d) {
  if (!d->cda) {
    DACreate3d(0, d->pt, DA_STENCIL_BOX, d->mx, d->my, d->mz, 1, 1, 1, 3, d->s, 0, 0, 0, &d->cda);
    d->owns_cda = true;
  }
  return d->cda;
}
PetscErrorCode DASetUniformCoordinates(DA d, PetscReal x0, PetscReal x1, PetscReal y0, PetscReal y1, PetscReal z0,
                                       PetscReal z1) {
  DA c = coord_da(d);
  if (!d->coords) d->coords = new_vec(c->gsize(), c, false);
  const double hx = d->mx > 1 ? (x1 - x0) / (d->mx - 1) : 0., hy = d->my > 1 ? (y1 - y0) / (d->my - 1) : 0.,
               hz = d->mz > 1 ? (z1 - z0) / (d->mz - 1) : 0.;
  for (int k = 0; k < d->mz; k++)
    for (int j = 0; j < d->my; j++)
      for (int i = 0; i < d->mx; i++) {
        double *p = &d->coords->v[(((size_t)k * d->my + j) * d->mx + i) * 3];
        p[0] = x0 + i * hx; p[1] = y0 + j * hy; p[2] = z0 + k * hz;
      }
  return 0;
}
PetscErrorCode DAGetCoordinateDA(DA d, DA *c) {
  *c = coord_da(d);
  return 0;
}
PetscErrorCode DAGetCoordinates(DA d, Vec *c) {
  DA cd = coord_da(d);
  if (!d->coords) d->coords = new_vec(cd->gsize(), cd, false);
  *c = d->coords;
  return 0;
}
PetscErrorCode DAGetGhostedCoordinates(DA d, Vec *c) {
  Vec g;
  DAGetCoordinates(d, &g);
  DA cd = d->cda;
  if (!d->gcoords) d->gcoords = new_vec(cd->lsize(), cd, true);
  DAGlobalToLocalBegin(cd, g, INSERT_VALUES, d->gcoords);
  *c = d->gcoords;
  return 0;
}
PetscErrorCode DACreateGlobalVector(DA d, Vec *v) {
  *v = new_vec(d->gsize(), d, false);
  return 0;
}
PetscErrorCode DACreateLocalVector(DA d, Vec *v) {
  *v = new_vec(d->lsize(), d, true);
  return 0;
}
PetscErrorCode DACreateNaturalVector(DA d, Vec *v) {
  *v = new_vec(d->gsize(), d, false);
  return 0;
}
PetscErrorCode DAGetLocalVector(DA d, Vec *v) { return DACreateLocalVector(d, v); }
PetscErrorCode DARestoreLocalVector(DA, Vec *v) {
  VecDestroy(*v);
  *v = nullptr;
  return 0;
}
PetscErrorCode DAGetGlobalVector(DA d, Vec *v) { return DACreateGlobalVector(d, v); }
PetscErrorCode DARestoreGlobalVector(DA, Vec *v) {
  VecDestroy(*v);
  *v = nullptr;
  return 0;
}

// [k][j][i] view of a DA vector in global indices (ghosted extent for local
// vectors); the pointer tables are freed by DAVecRestoreArray
static std::map<void *, void *> &views() {
  static std::map<void *, void *> m;
  return m;
}
PetscErrorCode DAVecGetArray(DA d, Vec v, void *out) {
  if (!v) unreached("DAVecGetArray of a null vector");
  int x0, y0, z0, xm, ym, zm;
  if (v->v.size() == d->lsize() && d->lsize() != d->gsize()) {
    x0 = d->gxs(); y0 = d->gys(); z0 = d->gzs(); xm = d->gxm(); ym = d->gym(); zm = d->gzm();
  } else if (v->v.size() == d->gsize()) {
    x0 = y0 = z0 = 0; xm = d->mx; ym = d->my; zm = d->mz;
  } else {
    unreached("DAVecGetArray of a vector that does not fit the DA");
  }
  const int dof = d->dof;
  char *mem = (char *)malloc(sizeof(double **) * zm + sizeof(double *) * (size_t)zm * ym);
  double ***t = (double ***)mem;
  double **rows = (double **)(mem + sizeof(double **) * zm);
  for (int k = 0; k < zm; k++) {
    t[k] = rows + (size_t)k * ym - y0;
    for (int j = 0; j < ym; j++)
      rows[(size_t)k * ym + j] = v->v.data() + ((size_t)k * ym + j) * xm * dof - (ptrdiff_t)x0 * dof;
  }
  double ***view = t - z0;
  *(double ****)out = view;
  views()[(void *)view] = mem;
  return 0;
}
PetscErrorCode DAVecRestoreArray(DA, Vec, void *out) {
  void *view = *(void **)out;
  auto it = views().find(view);
  if (it == views().end()) unreached("DAVecRestoreArray of an unknown view");
  free(it->second);
  views().erase(it);
  return 0;
}

static inline int wrap(int i, int m) { return ((i % m) + m) % m; }

// local (ghosted) <- global, ghosts of periodic directions wrapped
PetscErrorCode DAGlobalToLocalBegin(DA d, Vec g, InsertMode mode, Vec l) {
  if (g->v.size() != d->gsize() || l->v.size() != d->lsize()) unreached("DAGlobalToLocal sizes");
  const int dof = d->dof, x0 = d->gxs(), y0 = d->gys(), z0 = d->gzs(), xm = d->gxm(), ym = d->gym(),
            zm = d->gzm();
  for (int k = 0; k < zm; k++)
    for (int j = 0; j < ym; j++)
      for (int i = 0; i < xm; i++) {
        const int gi = wrap(i + x0, d->mx), gj = wrap(j + y0, d->my), gk = wrap(k + z0, d->mz);
        const double *s = &g->v[(((size_t)gk * d->my + gj) * d->mx + gi) * dof];
        double *t = &l->v[(((size_t)k * ym + j) * xm + i) * dof];
        for (int c = 0; c < dof; c++) t[c] = mode == ADD_VALUES ? t[c] + s[c] : s[c];
      }
  return 0;
}
PetscErrorCode DAGlobalToLocalEnd(DA, Vec, InsertMode, Vec) { return 0; }
// ghosts of l2 <- owned values of l1 (owned values copied as well)
PetscErrorCode DALocalToLocalBegin(DA d, Vec l1, InsertMode, Vec l2) {
  if (l1->v.size() != d->lsize() || l2->v.size() != d->lsize()) unreached("DALocalToLocal sizes");
  const int dof = d->dof, x0 = d->gxs(), y0 = d->gys(), z0 = d->gzs(), xm = d->gxm(), ym = d->gym(),
            zm = d->gzm();
  std::vector<double> src;
  const double *s0 = l1->v.data();
  if (l1 == l2) {
    src = l1->v;
    s0 = src.data();
  }
  for (int k = 0; k < zm; k++)
    for (int j = 0; j < ym; j++)
      for (int i = 0; i < xm; i++) {
        const int oi = wrap(i + x0, d->mx) - x0, oj = wrap(j + y0, d->my) - y0, ok = wrap(k + z0, d->mz) - z0;
        const double *s = s0 + (((size_t)ok * ym + oj) * xm + oi) * dof;
        double *t = &l2->v[(((size_t)k * ym + j) * xm + i) * dof];
        for (int c = 0; c < dof; c++) t[c] = s[c];
      }
  return 0;
}
PetscErrorCode DALocalToLocalEnd(DA, Vec, InsertMode, Vec) { return 0; }
// owned part of a local vector -> global (ghosts discarded)
PetscErrorCode DALocalToGlobal(DA d, Vec l, InsertMode mode, Vec g) {
  if (g->v.size() != d->gsize() || l->v.size() != d->lsize()) unreached("DALocalToGlobal sizes");
  const int dof = d->dof, x0 = d->gxs(), y0 = d->gys(), z0 = d->gzs(), xm = d->gxm(), ym = d->gym();
  for (int k = 0; k < d->mz; k++)
    for (int j = 0; j < d->my; j++)
      for (int i = 0; i < d->mx; i++) {
        const double *s = &l->v[(((size_t)(k - z0) * ym + (j - y0)) * xm + (i - x0)) * dof];
        double *t = &g->v[(((size_t)k * d->my + j) * d->mx + i) * dof];
        for (int c = 0; c < dof; c++) t[c] = mode == ADD_VALUES ? t[c] + s[c] : s[c];
      }
  return 0;
}
PetscErrorCode DALocalToGlobalBegin(DA d, Vec l, Vec g) { return DALocalToGlobal(d, l, INSERT_VALUES, g); }
PetscErrorCode DALocalToGlobalEnd(DA, Vec, Vec) { return 0; }
// one rank: the natural ordering is the global ordering
PetscErrorCode DAGlobalToNaturalBegin(DA, Vec g, InsertMode, Vec n) { return VecCopy(g, n); }
PetscErrorCode DAGlobalToNaturalEnd(DA, Vec, InsertMode, Vec) { return 0; }
PetscErrorCode DANaturalToGlobalBegin(DA, Vec n, InsertMode, Vec g) { return VecCopy(n, g); }
PetscErrorCode DANaturalToGlobalEnd(DA, Vec, InsertMode, Vec) { return 0; }
// global index of every local (ghosted) entry
PetscErrorCode DAGetGlobalIndices(DA d, PetscInt *n, PetscInt **idx) {
  static std::map<DA, std::vector<PetscInt>> cache;
  std::vector<PetscInt> &v = cache[d];
  const int dof = d->dof, x0 = d->gxs(), y0 = d->gys(), z0 = d->gzs(), xm = d->gxm(), ym = d->gym(),
            zm = d->gzm();
  v.resize(d->lsize());
  for (int k = 0; k < zm; k++)
    for (int j = 0; j < ym; j++)
      for (int i = 0; i < xm; i++)
        for (int c = 0; c < dof; c++) {
          const size_t g = ((size_t)wrap(k + z0, d->mz) * d->my + wrap(j + y0, d->my)) * d->mx + wrap(i + x0, d->mx);
          v[(((size_t)k * ym + j) * xm + i) * dof + c] = (PetscInt)(g * dof + c);
        }
  if (n) *n = (PetscInt)v.size();
  *idx = v.data();
  return 0;
}
PetscErrorCode DAGetAO(DA, AO *) { unreached("DAGetAO"); }
PetscErrorCode AOApplicationToPetsc(AO, PetscInt, PetscInt[]) { return 0; }
PetscErrorCode AOPetscToApplication(AO, PetscInt, PetscInt[]) { return 0; }

// ------------------------------------------------------------ matrices ----
PetscErrorCode MatCreate(MPI_Comm, Mat *A) {
  *A = new _p_Mat();
  return 0;
}
PetscErrorCode MatCreateMPIAIJ(MPI_Comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N, PetscInt, const PetscInt[],
                               PetscInt, const PetscInt[], Mat *A) {
  *A = new _p_Mat();
  MatSetSizes(*A, m, n, M, N);
  return 0;
}
PetscErrorCode MatCreateSeqAIJ(MPI_Comm, PetscInt m, PetscInt n, PetscInt, const PetscInt[], Mat *A) {
  *A = new _p_Mat();
  MatSetSizes(*A, m, n, m, n);
  return 0;
}
PetscErrorCode MatSetSizes(Mat A, PetscInt m, PetscInt n, PetscInt M, PetscInt N) {
  A->m = M >= 0 ? M : m;
  A->n = N >= 0 ? N : n;
  A->rows.assign(A->m, {});
  return 0;
}
PetscErrorCode MatSetType(Mat, MatType) { return 0; }
PetscErrorCode MatSetFromOptions(Mat) { return 0; }
PetscErrorCode MatSetOption(Mat, MatOption, PetscTruth) { return 0; }
PetscErrorCode MatMPIAIJSetPreallocation(Mat, PetscInt, const PetscInt[], PetscInt, const PetscInt[]) { return 0; }
PetscErrorCode MatSeqAIJSetPreallocation(Mat, PetscInt, const PetscInt[]) { return 0; }
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt r[], PetscInt n, const PetscInt c[],
                            const PetscScalar v[], InsertMode mode) {
  for (int a = 0; a < m; a++) {
    if (r[a] < 0) continue;
    if (r[a] >= A->m) unreached("MatSetValues row out of range");
    for (int b = 0; b < n; b++) {
      if (c[b] < 0) continue;
      double &e = A->rows[r[a]][c[b]];
      e = mode == ADD_VALUES ? e + v[(size_t)a * n + b] : v[(size_t)a * n + b];
    }
  }
  return 0;
}
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType) {
  A->build();
  return 0;
}
PetscErrorCode MatZeroEntries(Mat A) {
  for (auto &r : A->rows)
    for (auto &e : r) e.second = 0.;
  A->build();
  return 0;
}
PetscErrorCode MatDestroy(Mat A) {
  delete A;
  return 0;
}
PetscErrorCode MatGetOwnershipRange(Mat A, PetscInt *lo, PetscInt *hi) {
  if (lo) *lo = 0;
  if (hi) *hi = A->m;
  return 0;
}
PetscErrorCode MatGetSize(Mat A, PetscInt *m, PetscInt *n) {
  if (m) *m = A->m;
  if (n) *n = A->n;
  return 0;
}
PetscErrorCode MatGetRow(Mat A, PetscInt r, PetscInt *nc, const PetscInt **c, const PetscScalar **v) {
  if ((int)A->rowptr.size() != A->m + 1) A->build();
  const int b = A->rowptr[r], e = A->rowptr[r + 1];
  if (nc) *nc = e - b;
  if (c) *c = A->cols.data() + b;
  if (v) *v = A->vals.data() + b;
  return 0;
}
PetscErrorCode MatRestoreRow(Mat, PetscInt, PetscInt *, const PetscInt **, const PetscScalar **) { return 0; }
PetscErrorCode MatMult(Mat A, Vec x, Vec y) {
  if (A->shell) {
    if (!A->mult) unreached("MatMult of a shell matrix without MATOP_MULT");
    return A->mult(A, x, y);
  }
  if ((int)A->rowptr.size() != A->m + 1) A->build();
  for (int r = 0; r < A->m; r++) {
    double s = 0.;
    for (int q = A->rowptr[r]; q < A->rowptr[r + 1]; q++) s += A->vals[q] * x->v[A->cols[q]];
    y->v[r] = s;
  }
  return 0;
}
PetscErrorCode MatGetVecs(Mat A, Vec *r, Vec *l) {
  if (r) *r = new_vec(A->n, nullptr, false);
  if (l) *l = new_vec(A->m, nullptr, false);
  return 0;
}
PetscErrorCode MatCreateShell(MPI_Comm, PetscInt m, PetscInt n, PetscInt M, PetscInt N, void *ctx, Mat *A) {
  Mat B = new _p_Mat();
  B->shell = true;
  B->ctx = ctx;
  B->m = M >= 0 ? M : m;
  B->n = N >= 0 ? N : n;
  *A = B;
  return 0;
}
PetscErrorCode MatShellGetContext(Mat A, void **ctx) {
  *ctx = A->ctx;
  return 0;
}
PetscErrorCode MatShellSetOperation(Mat A, MatOperation op, void (*f)(void)) {
  if (op == MATOP_MULT) A->mult = (PetscErrorCode(*)(Mat, Vec, Vec))f;
  return 0;
}
PetscErrorCode MatView(Mat, PetscViewer) { unreached("MatView"); }
PetscErrorCode MatNullSpaceCreate(MPI_Comm, PetscTruth c, PetscInt n, const Vec v[], MatNullSpace *s) {
  MatNullSpace q = new _p_MatNullSpace();
  q->has_cnst = c == PETSC_TRUE;
  for (int a = 0; a < n; a++) q->vecs.push_back(v[a]);
  *s = q;
  return 0;
}
PetscErrorCode MatNullSpaceSetFunction(MatNullSpace s, PetscErrorCode (*f)(MatNullSpace, Vec, void *), void *ctx) {
  s->fn = f;
  s->ctx = ctx;
  return 0;
}
PetscErrorCode MatNullSpaceRemove(MatNullSpace s, Vec x, Vec *out) {
  if (out && *out) unreached("MatNullSpaceRemove into a second vector");
  if (s->has_cnst) {
    double m = 0.;
    for (double e : x->v) m += e;
    m /= (double)x->v.size();
    for (auto &e : x->v) e -= m;
  }
  for (Vec q : s->vecs) {
    double d;
    VecDot(x, q, &d);
    VecAXPY(x, -d, q);
  }
  if (s->fn) s->fn(s, x, s->ctx);
  return 0;
}
PetscErrorCode MatNullSpaceDestroy(MatNullSpace s) {
  delete s;
  return 0;
}

// ---------------------------------------- Krylov set-up (ignored) ----
PetscErrorCode KSPCreate(MPI_Comm, KSP *k) {
  *k = new _p_KSP();
  (*k)->pc = new _p_PC();
  return 0;
}
PetscErrorCode KSPDestroy(KSP k) {
  if (k) {
    delete k->pc;
    delete k;
  }
  return 0;
}
PetscErrorCode KSPSetType(KSP, KSPType) { return 0; }
PetscErrorCode KSPGetPC(KSP k, PC *p) {
  *p = k->pc;
  return 0;
}
PetscErrorCode KSPSetOperators(KSP, Mat, Mat, MatStructure) { return 0; }
PetscErrorCode KSPSetTolerances(KSP, PetscReal, PetscReal, PetscReal, PetscInt) { return 0; }
PetscErrorCode KSPGMRESSetRestart(KSP, PetscInt) { return 0; }
PetscErrorCode KSPSetUp(KSP) { return 0; }
PetscErrorCode KSPSolve(KSP, Vec, Vec) { unreached("KSPSolve"); }
PetscErrorCode KSPSetFromOptions(KSP) { return 0; }
PetscErrorCode KSPSetInitialGuessNonzero(KSP, PetscTruth) { return 0; }
PetscErrorCode KSPSetInitialGuessKnoll(KSP, PetscTruth) { return 0; }
PetscErrorCode KSPSetNullSpace(KSP, MatNullSpace) { return 0; }
PetscErrorCode KSPSetNormType(KSP, KSPNormType) { return 0; }
PetscErrorCode KSPAppendOptionsPrefix(KSP, const char[]) { return 0; }
PetscErrorCode KSPSetOptionsPrefix(KSP, const char[]) { return 0; }
PetscErrorCode KSPMonitorSet(KSP, PetscErrorCode (*)(KSP, PetscInt, PetscReal, void *), void *,
                             PetscErrorCode (*)(void *)) {
  return 0;
}
PetscErrorCode KSPMonitorTrueResidualNorm(KSP, PetscInt, PetscReal, void *) { return 0; }
PetscErrorCode KSPBuildResidual(KSP, Vec, Vec, Vec *) { unreached("KSPBuildResidual"); }
PetscErrorCode KSPGetIterationNumber(KSP, PetscInt *n) {
  *n = 0;
  return 0;
}
PetscErrorCode KSPGetConvergedReason(KSP, KSPConvergedReason *r) {
  *r = KSP_CONVERGED_RTOL;
  return 0;
}
PetscErrorCode KSPGetResidualNorm(KSP, PetscReal *r) {
  *r = 0.;
  return 0;
}
PetscErrorCode PCCreate(MPI_Comm, PC *p) {
  *p = new _p_PC();
  return 0;
}
PetscErrorCode PCSetType(PC, PCType) { return 0; }
PetscErrorCode PCSetOperators(PC, Mat, Mat, MatStructure) { return 0; }
PetscErrorCode PCSetFromOptions(PC) { return 0; }
PetscErrorCode PCSetUp(PC) { return 0; }
PetscErrorCode PCDestroy(PC p) {
  delete p;
  return 0;
}
PetscErrorCode PCBJacobiGetSubKSP(PC, PetscInt *, PetscInt *, KSP **) { unreached("PCBJacobiGetSubKSP"); }
PetscErrorCode PCFactorSetShiftNonzero(PC, PetscReal) { return 0; }
PetscErrorCode PCFactorSetShiftType(PC, MatFactorShiftType) { return 0; }
PetscErrorCode PCFactorSetShiftAmount(PC, PetscReal) { return 0; }
PetscErrorCode PCHYPRESetType(PC, const char[]) { return 0; }
PetscErrorCode PCMGSetLevels(PC, PetscInt, MPI_Comm *) { return 0; }
PetscErrorCode PCMGSetType(PC, PCMGType) { return 0; }
PetscErrorCode PCMGSetCycleType(PC, PCMGCycleType) { return 0; }
PetscErrorCode PCMGSetCycles(PC, PetscInt) { return 0; }
PetscErrorCode PCMGSetNumberSmoothUp(PC, PetscInt) { return 0; }
PetscErrorCode PCMGSetNumberSmoothDown(PC, PetscInt) { return 0; }
static KSP mg_ksp() {
  static KSP k = nullptr;
  if (!k) KSPCreate(0, &k);
  return k;
}
PetscErrorCode PCMGGetSmoother(PC, PetscInt, KSP *k) {
  *k = mg_ksp();
  return 0;
}
PetscErrorCode PCMGGetSmootherUp(PC, PetscInt, KSP *k) {
  *k = mg_ksp();
  return 0;
}
PetscErrorCode PCMGGetSmootherDown(PC, PetscInt, KSP *k) {
  *k = mg_ksp();
  return 0;
}
PetscErrorCode PCMGGetCoarseSolve(PC, KSP *k) {
  *k = mg_ksp();
  return 0;
}
PetscErrorCode PCMGSetInterpolation(PC, PetscInt, Mat) { return 0; }
PetscErrorCode PCMGSetRestriction(PC, PetscInt, Mat) { return 0; }
PetscErrorCode PCMGSetResidual(PC, PetscInt, PetscErrorCode (*)(Mat, Vec, Vec, Vec), Mat) { return 0; }
PetscErrorCode PCMGSetRhs(PC, PetscInt, Vec) { return 0; }
PetscErrorCode PCMGSetX(PC, PetscInt, Vec) { return 0; }
PetscErrorCode PCMGSetR(PC, PetscInt, Vec) { return 0; }
PetscErrorCode PCMGDefaultResidual(Mat, Vec, Vec, Vec) { unreached("PCMGDefaultResidual"); }
PetscErrorCode SNESCreate(MPI_Comm, SNES *s) {
  *s = new _p_SNES();
  return 0;
}
PetscErrorCode SNESDestroy(SNES s) {
  delete s;
  return 0;
}
PetscErrorCode SNESSetFunction(SNES, Vec, PetscErrorCode (*)(SNES, Vec, Vec, void *), void *) {
  unreached("SNESSetFunction");
}
PetscErrorCode MatCreateSNESMF(SNES, Mat *) { unreached("MatCreateSNESMF"); }
PetscErrorCode MatMFFDComputeJacobian(SNES, Vec, Mat *, Mat *, MatStructure *, void *) {
  unreached("MatMFFDComputeJacobian");
}
PetscErrorCode SNESSetJacobian(SNES, Mat, Mat, PetscErrorCode (*)(SNES, Vec, Mat *, Mat *, MatStructure *, void *),
                               void *) {
  unreached("SNESSetJacobian");
}
PetscErrorCode SNESSetType(SNES, SNESType) { unreached("SNESSetType"); }
PetscErrorCode SNESSetMaxLinearSolveFailures(SNES, PetscInt) { unreached("SNESSetMaxLinearSolveFailures"); }
PetscErrorCode SNESSetMaxNonlinearStepFailures(SNES, PetscInt) { unreached("SNESSetMaxNonlinearStepFailures"); }
PetscErrorCode SNESKSPSetUseEW(SNES, PetscTruth) { unreached("SNESKSPSetUseEW"); }
PetscErrorCode SNESKSPSetParametersEW(SNES, PetscInt, PetscReal, PetscReal, PetscReal, PetscReal, PetscReal,
                                      PetscReal) {
  unreached("SNESKSPSetParametersEW");
}
PetscErrorCode SNESSetTolerances(SNES, PetscReal, PetscReal, PetscReal, PetscInt, PetscInt) {
  unreached("SNESSetTolerances");
}
PetscErrorCode SNESGetKSP(SNES, KSP *) { unreached("SNESGetKSP"); }
PetscErrorCode SNESMonitorSet(SNES, PetscErrorCode (*)(SNES, PetscInt, PetscReal, void *), void *,
                              PetscErrorCode (*)(void *)) {
  unreached("SNESMonitorSet");
}
PetscErrorCode SNESSolve(SNES, Vec, Vec) { unreached("SNESSolve"); }
PetscErrorCode SNESGetFunctionNorm(SNES, PetscReal *) { unreached("SNESGetFunctionNorm"); }
PetscErrorCode SNESSetFromOptions(SNES) { unreached("SNESSetFromOptions"); }
PetscErrorCode SNESGetIterationNumber(SNES, PetscInt *) { unreached("SNESGetIterationNumber"); }

// -------------------------------------------------------------- HYPRE ----
HYPRE_Int HYPRE_IJVectorCreate(MPI_Comm, HYPRE_Int lo, HYPRE_Int hi, HYPRE_IJVector *v) {
  *v = new hypre_IJVector_struct();
  (*v)->lo = lo;
  (*v)->hi = hi;
  (*v)->v.assign(hi >= lo ? hi - lo + 1 : 0, 0.);
  return 0;
}
HYPRE_Int HYPRE_IJVectorDestroy(HYPRE_IJVector v) {
  delete v;
  return 0;
}
HYPRE_Int HYPRE_IJVectorSetObjectType(HYPRE_IJVector, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_IJVectorSetMaxOffProcElmts(HYPRE_IJVector, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_IJVectorInitialize(HYPRE_IJVector v) {
  for (auto &e : v->v) e = 0.;
  return 0;
}
static double &hv(HYPRE_IJVector v, int i) {
  if (i < v->lo || i > v->hi) unreached("HYPRE_IJVector index out of range");
  return v->v[i - v->lo];
}
HYPRE_Int HYPRE_IJVectorSetValues(HYPRE_IJVector v, HYPRE_Int n, const HYPRE_Int *idx, const HYPRE_Complex *val) {
  for (int q = 0; q < n; q++) hv(v, idx ? idx[q] : v->lo + q) = val[q];
  return 0;
}
HYPRE_Int HYPRE_IJVectorAddToValues(HYPRE_IJVector v, HYPRE_Int n, const HYPRE_Int *idx, const HYPRE_Complex *val) {
  for (int q = 0; q < n; q++) hv(v, idx ? idx[q] : v->lo + q) += val[q];
  return 0;
}
HYPRE_Int HYPRE_IJVectorGetValues(HYPRE_IJVector v, HYPRE_Int n, const HYPRE_Int *idx, HYPRE_Complex *val) {
  for (int q = 0; q < n; q++) val[q] = hv(v, idx ? idx[q] : v->lo + q);
  return 0;
}
HYPRE_Int HYPRE_IJVectorAssemble(HYPRE_IJVector) { return 0; }
HYPRE_Int HYPRE_IJVectorGetObject(HYPRE_IJVector v, void **o) {
  *o = (void *)v;
  return 0;
}
HYPRE_Int HYPRE_IJMatrixCreate(MPI_Comm, HYPRE_Int lo, HYPRE_Int hi, HYPRE_Int, HYPRE_Int, HYPRE_IJMatrix *A) {
  *A = new hypre_IJMatrix_struct();
  (*A)->lo = lo;
  (*A)->hi = hi;
  (*A)->rows.assign(hi >= lo ? hi - lo + 1 : 0, {});
  return 0;
}
HYPRE_Int HYPRE_IJMatrixDestroy(HYPRE_IJMatrix A) {
  delete A;
  return 0;
}
HYPRE_Int HYPRE_IJMatrixSetObjectType(HYPRE_IJMatrix, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_IJMatrixSetMaxOffProcElmts(HYPRE_IJMatrix, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_IJMatrixSetRowSizes(HYPRE_IJMatrix, const HYPRE_Int *) { return 0; }
HYPRE_Int HYPRE_IJMatrixInitialize(HYPRE_IJMatrix A) {
  for (auto &r : A->rows) r.clear();
  return 0;
}
HYPRE_Int HYPRE_IJMatrixSetValues(HYPRE_IJMatrix A, HYPRE_Int nrows, HYPRE_Int *ncols, const HYPRE_Int *rows,
                                  const HYPRE_Int *cols, const HYPRE_Complex *vals) {
  size_t at = 0;
  for (int a = 0; a < nrows; a++) {
    const int r = rows[a];
    if (r < A->lo || r > A->hi) unreached("HYPRE_IJMatrixSetValues row out of range");
    for (int b = 0; b < ncols[a]; b++, at++) A->rows[r - A->lo][cols[at]] = vals[at];
  }
  return 0;
}
HYPRE_Int HYPRE_IJMatrixAssemble(HYPRE_IJMatrix A) {
  A->rowptr.assign(1, 0);
  A->cols.clear();
  A->vals.clear();
  for (auto &r : A->rows) {
    for (auto &e : r) {
      A->cols.push_back(e.first);
      A->vals.push_back(e.second);
    }
    A->rowptr.push_back((int)A->cols.size());
  }
  return 0;
}
HYPRE_Int HYPRE_IJMatrixGetObject(HYPRE_IJMatrix A, void **o) {
  *o = (void *)A;
  return 0;
}
HYPRE_Int HYPRE_BoomerAMGCreate(HYPRE_Solver *s) {
  *s = new hypre_Solver_struct();
  return 0;
}
HYPRE_Int HYPRE_BoomerAMGDestroy(HYPRE_Solver s) {
  delete s;
  return 0;
}
HYPRE_Int HYPRE_BoomerAMGSetup(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSolve(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector) {
  unreached("HYPRE_BoomerAMGSolve");
}
HYPRE_Int HYPRE_BoomerAMGSetAggNumLevels(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetCoarsenType(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetCycleNumSweeps(HYPRE_Solver, HYPRE_Int, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetCycleType(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetInterpType(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetLevelOuterWt(HYPRE_Solver, HYPRE_Real, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetMaxIter(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetPrintLevel(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetRelaxType(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetRelaxWt(HYPRE_Solver, HYPRE_Real) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetSmoothNumSweeps(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetSmoothType(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetStrongThreshold(HYPRE_Solver, HYPRE_Real) { return 0; }
HYPRE_Int HYPRE_BoomerAMGSetTol(HYPRE_Solver, HYPRE_Real) { return 0; }
HYPRE_Int HYPRE_GMRESSetMaxIter(HYPRE_Solver s, HYPRE_Int n) {
  s->maxit = n;
  return 0;
}
HYPRE_Int HYPRE_GMRESSetPrecond(HYPRE_Solver, HYPRE_PtrToSolverFcn, HYPRE_PtrToSolverFcn, HYPRE_Solver) { return 0; }
HYPRE_Int HYPRE_GMRESSetPrintLevel(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_GMRESSetTol(HYPRE_Solver s, HYPRE_Real t) {
  s->tol = t;
  return 0;
}
HYPRE_Int HYPRE_GMRESSetKDim(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_PCGSetMaxIter(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_PCGSetPrecond(HYPRE_Solver, HYPRE_PtrToSolverFcn, HYPRE_PtrToSolverFcn, HYPRE_Solver) { return 0; }
HYPRE_Int HYPRE_PCGSetPrintLevel(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_PCGSetTol(HYPRE_Solver, HYPRE_Real) { return 0; }
HYPRE_Int HYPRE_ParCSRGMRESCreate(MPI_Comm, HYPRE_Solver *s) {
  *s = new hypre_Solver_struct();
  return 0;
}
HYPRE_Int HYPRE_ParCSRGMRESDestroy(HYPRE_Solver s) {
  delete s;
  return 0;
}
HYPRE_Int HYPRE_ParCSRGMRESSetKDim(HYPRE_Solver, HYPRE_Int) { return 0; }
HYPRE_Int HYPRE_ParCSRGMRESSetAbsoluteTol(HYPRE_Solver, HYPRE_Real) { return 0; }
HYPRE_Int HYPRE_ParCSRGMRESSetup(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector) { return 0; }
// the inner solve: the harness's FP64 solver on the assembled CSR system
HYPRE_Int HYPRE_ParCSRGMRESSolve(HYPRE_Solver s, HYPRE_ParCSRMatrix Am, HYPRE_ParVector bv, HYPRE_ParVector xv) {
  if (!g_solver) unreached("HYPRE_ParCSRGMRESSolve without a registered solver");
  HYPRE_IJMatrix A = (HYPRE_IJMatrix)(void *)Am;
  HYPRE_IJVector b = (HYPRE_IJVector)(void *)bv, x = (HYPRE_IJVector)(void *)xv;
  const int n = A->hi - A->lo + 1;
  return g_solver(n, A->rowptr.data(), A->cols.data(), A->vals.data(), b->v.data(), x->v.data(), s->tol);
}
HYPRE_Int HYPRE_ParCSRPCGCreate(MPI_Comm, HYPRE_Solver *s) { return HYPRE_ParCSRGMRESCreate(0, s); }

// ------------------------------------------------------ harness hooks ----
void vfs_shim_set_solver(vfs_shim_solve_fn fn) { g_solver = fn; }
double vfs_shim_last_vecmax(void) { return g_last_vecmax; }
void vfs_shim_vec_retain(Vec v) { v->refs++; }
double *vfs_shim_vec_data(Vec v, int *n) {
  if (n) *n = (int)v->v.size();
  return v->v.data();
}
int vfs_shim_mat_csr(Mat A, int *nrows, const int **rowptr, const int **cols, const double **vals) {
  if ((int)A->rowptr.size() != A->m + 1) A->build();
  *nrows = A->m;
  *rowptr = A->rowptr.data();
  *cols = A->cols.data();
  *vals = A->vals.data();
  return 0;
}
int vfs_shim_hypre_vec(HYPRE_IJVector v, int *lo, int *hi, double **data) {
  *lo = v->lo;
  *hi = v->hi;
  *data = v->v.data();
  return 0;
}
int vfs_shim_hypre_mat_csr(HYPRE_IJMatrix A, int *nrows, const int **rowptr, const int **cols, const double **vals) {
  *nrows = A->hi - A->lo + 1;
  *rowptr = A->rowptr.data();
  *cols = A->cols.data();
  *vals = A->vals.data();
  return 0;
}
