// petsc_shim.h -- a single-rank stand-in for the parts of PETSc 3.1, HYPRE
// and MPI that the reference's pressure-Poisson translation units use.
//
// Test infrastructure only: it lets the reference's own sources
// (Source/metrics.c, Source/poisson.c, Source/poisson_hypre.c and
// Source/main.c) compile unmodified, so that their output can pin the
// oracle's restatement.  Semantics follow PETSc 3.1 on one MPI rank:
//   * a DA is a structured grid of mx*my*mz points with dof unknowns per
//     point and a box stencil of width s; on one rank the owned range is the
//     whole grid (xs = 0, xm = mx), and a ghosted local vector extends it by
//     s on both sides of each periodic direction (gxs = -s, gxm = mx + 2s)
//     with the values wrapped modulo the grid size; non-periodic directions
//     have no ghosts on one rank (gxs = 0, gxm = mx);
//   * DAVecGetArray returns a [k][j][i] view in global indices (the row of a
//     dof > 1 vector is an array of dof-sized records);
//   * matrices collect MatSetValues entries row by row (CSR on assembly);
//   * HYPRE IJ vectors and matrices are plain arrays; the HYPRE GMRES solve
//     calls a solver the test harness registers (the HYPRE algorithm itself
//     is not part of the reference's sources);
//   * KSP/PC set-up calls are accepted and ignored; a KSPSolve aborts.
// Functions the covered paths never reach abort with their name.
#pragma once

#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

// ---------------------------------------------------------------- MPI ----
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_CHAR 3
#define MPI_FLOAT 4
#define MPI_LONG 5
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_LOR 4
#define MPI_LAND 5
#define MPI_IN_PLACE ((void *)-1)
#define MPIU_REAL MPI_DOUBLE
#define MPIU_INT MPI_INT
int MPI_Comm_rank(MPI_Comm, int *);
int MPI_Comm_size(MPI_Comm, int *);
int MPI_Allreduce(void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Reduce(void *, void *, int, MPI_Datatype, MPI_Op, int, MPI_Comm);
int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm);
int MPI_Barrier(MPI_Comm);
int MPI_Send(void *, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *);
int MPI_Gather(void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm);
int MPI_Allgather(void *, int, MPI_Datatype, void *, int, MPI_Datatype, MPI_Comm);
double MPI_Wtime(void);
int MPI_Abort(MPI_Comm, int);

// -------------------------------------------------------------- PETSc ----
typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef double PetscLogDouble;
typedef enum { PETSC_FALSE, PETSC_TRUE } PetscTruth;
typedef PetscTruth PetscBool;
#define PETSC_NULL 0
#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_COMM_SELF MPI_COMM_SELF
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE PETSC_DECIDE
#define PETSC_DEFAULT (-2)
#define PETSC_MAX_PATH_LEN 4096
#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscAbsScalar(a) fabs(a)
#define PetscAbsReal(a) fabs(a)
#define PetscRealPart(a) (a)
#define CHKERRQ(e) \
  do {             \
    (void)(e);     \
  } while (0)
#define CHKERRABORT(c, e) \
  do {                   \
    (void)(e);           \
  } while (0)
#define SETERRQ(n, s) return (n)
#define PETSC_ERR_SUP 56
#define PETSC_ERR_ARG_OUTOFRANGE 63
#define PetscFunctionBegin
#define PetscFunctionReturn(a) return (a)

typedef struct _p_Vec *Vec;
typedef struct _p_Mat *Mat;
typedef struct _p_DA *DA;
typedef struct _p_KSP *KSP;
typedef struct _p_PC *PC;
typedef struct _p_SNES *SNES;
typedef struct _p_MatNullSpace *MatNullSpace;
typedef struct _p_AO *AO;
typedef struct _p_IS *IS;
typedef struct _p_VecScatter *VecScatter;
typedef struct _p_PetscViewer *PetscViewer;
typedef struct _p_PetscRandom *PetscRandom;
typedef void *PetscObject;

typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES, MAX_VALUES } InsertMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3, NORM_1_AND_2 = 4 } NormType;
#define NORM_MAX NORM_INFINITY
typedef enum { SCATTER_FORWARD = 0, SCATTER_REVERSE = 1 } ScatterMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum {
  SAME_NONZERO_PATTERN,
  DIFFERENT_NONZERO_PATTERN,
  SAME_PRECONDITIONER,
  SUBSET_NONZERO_PATTERN
} MatStructure;
typedef enum { FILE_MODE_READ, FILE_MODE_WRITE, FILE_MODE_APPEND, FILE_MODE_UPDATE, FILE_MODE_APPEND_UPDATE } PetscFileMode;
typedef enum { MAT_SHIFT_NONE, MAT_SHIFT_NONZERO, MAT_SHIFT_POSITIVE_DEFINITE, MAT_SHIFT_INBLOCKS } MatFactorShiftType;
typedef enum { MATOP_MULT = 3, MATOP_MULT_ADD = 5, MATOP_MULT_TRANSPOSE = 4, MATOP_GET_DIAGONAL = 17 } MatOperation;
typedef enum { MAT_NEW_NONZERO_ALLOCATION_ERR, MAT_KEEP_NONZERO_PATTERN, MAT_IGNORE_ZERO_ENTRIES } MatOption;
typedef enum {
  DA_NONPERIODIC,
  DA_XPERIODIC,
  DA_YPERIODIC,
  DA_XYPERIODIC,
  DA_XYZPERIODIC,
  DA_XZPERIODIC,
  DA_YZPERIODIC,
  DA_ZPERIODIC,
  DA_XYZGHOSTED
} DAPeriodicType;
typedef enum { DA_STENCIL_STAR, DA_STENCIL_BOX } DAStencilType;
typedef enum { PC_MG_MULTIPLICATIVE, PC_MG_ADDITIVE, PC_MG_FULL, PC_MG_KASKADE } PCMGType;
typedef enum { PC_MG_CYCLE_V = 1, PC_MG_CYCLE_W = 2 } PCMGCycleType;
typedef enum {
  KSP_NORM_NO = 0,
  KSP_NORM_PRECONDITIONED = 1,
  KSP_NORM_UNPRECONDITIONED = 2,
  KSP_NORM_NATURAL = 3
} KSPNormType;
typedef enum {
  KSP_CONVERGED_ITERATING = 0,
  KSP_CONVERGED_RTOL = 2,
  KSP_DIVERGED_ITS = -3
} KSPConvergedReason;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *MatType;
#define KSPGMRES "gmres"
#define KSPFGMRES "fgmres"
#define KSPCG "cg"
#define KSPBCGS "bcgs"
#define KSPRICHARDSON "richardson"
#define KSPPREONLY "preonly"
#define KSPCHEBYCHEV "chebychev"
#define PCMG "mg"
#define PCLU "lu"
#define PCHYPRE "hypre"
#define PCBJACOBI "bjacobi"
#define PCASM "asm"
#define PCJACOBI "jacobi"
#define PCSOR "sor"
#define PCNONE "none"
#define PCILU "ilu"
#define MATMPIAIJ "mpiaij"
#define MATAIJ "aij"
#define MATSEQAIJ "seqaij"

typedef struct {
  PetscInt dim, dof, sw;
  PetscInt mx, my, mz;
  PetscInt xs, ys, zs;
  PetscInt xm, ym, zm;
  PetscInt gxs, gys, gzs;
  PetscInt gxm, gym, gzm;
  DAPeriodicType pt;
  DAStencilType st;
  DA da;
} DALocalInfo;

// system
PetscErrorCode PetscInitialize(int *, char ***, const char[], const char[]);
PetscErrorCode PetscFinalize(void);
PetscErrorCode PetscPrintf(MPI_Comm, const char[], ...);
PetscErrorCode PetscFPrintf(MPI_Comm, FILE *, const char[], ...);
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm, const char[], ...);
PetscErrorCode PetscSynchronizedFlush(MPI_Comm);
PetscErrorCode PetscBarrier(PetscObject);
PetscErrorCode PetscGetTime(PetscLogDouble *);
PetscErrorCode PetscGlobalSum(const PetscReal *, PetscReal *, MPI_Comm);
PetscErrorCode PetscGlobalMax(const PetscReal *, PetscReal *, MPI_Comm);
PetscErrorCode PetscGlobalMin(const PetscReal *, PetscReal *, MPI_Comm);
PetscErrorCode PetscMallocShim(size_t, void **);
PetscErrorCode PetscFreeShim(void *);
#define PetscMalloc(a, b) PetscMallocShim((size_t)(a), (void **)(b))
#define PetscFree(a) PetscFreeShim((void *)(a))
#define PetscMemzero(a, n) memset((a), 0, (n))
#define PetscMemcpy(a, b, n) memcpy((a), (b), (n))
PetscErrorCode PetscOptionsInsertString(const char[]);
PetscErrorCode PetscOptionsInsertFile(MPI_Comm, const char[], PetscTruth);
PetscErrorCode PetscOptionsClearValue(const char[]);
PetscErrorCode PetscOptionsGetInt(const char[], const char[], PetscInt *, PetscTruth *);
PetscErrorCode PetscOptionsGetReal(const char[], const char[], PetscReal *, PetscTruth *);
PetscErrorCode PetscOptionsGetString(const char[], const char[], char[], size_t, PetscTruth *);
PetscErrorCode PetscOptionsGetTruth(const char[], const char[], PetscTruth *, PetscTruth *);
PetscErrorCode PetscOptionsGetIntArray(const char[], const char[], PetscInt[], PetscInt *, PetscTruth *);
PetscErrorCode PetscOptionsGetRealArray(const char[], const char[], PetscReal[], PetscInt *, PetscTruth *);
PetscErrorCode PetscOptionsHasName(const char[], const char[], PetscTruth *);
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm, const char[], PetscFileMode, PetscViewer *);
PetscErrorCode PetscViewerDestroy(PetscViewer);

// vectors
PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt, PetscInt, Vec *);
PetscErrorCode VecCreateSeq(MPI_Comm, PetscInt, Vec *);
PetscErrorCode VecDuplicate(Vec, Vec *);
PetscErrorCode VecDestroy(Vec);
PetscErrorCode VecSet(Vec, PetscScalar);
PetscErrorCode VecCopy(Vec, Vec);
PetscErrorCode VecAXPY(Vec, PetscScalar, Vec);
PetscErrorCode VecAYPX(Vec, PetscScalar, Vec);
PetscErrorCode VecWAXPY(Vec, PetscScalar, Vec, Vec);
PetscErrorCode VecScale(Vec, PetscScalar);
PetscErrorCode VecShift(Vec, PetscScalar);
PetscErrorCode VecSum(Vec, PetscScalar *);
PetscErrorCode VecMax(Vec, PetscInt *, PetscReal *);
PetscErrorCode VecMin(Vec, PetscInt *, PetscReal *);
PetscErrorCode VecNorm(Vec, NormType, PetscReal *);
PetscErrorCode VecDot(Vec, Vec, PetscScalar *);
PetscErrorCode VecPointwiseDivide(Vec, Vec, Vec);
PetscErrorCode VecPointwiseMult(Vec, Vec, Vec);
PetscErrorCode VecGetSize(Vec, PetscInt *);
PetscErrorCode VecGetLocalSize(Vec, PetscInt *);
PetscErrorCode VecGetOwnershipRange(Vec, PetscInt *, PetscInt *);
PetscErrorCode VecGetArray(Vec, PetscScalar **);
PetscErrorCode VecRestoreArray(Vec, PetscScalar **);
PetscErrorCode VecGetArray3d(Vec, PetscInt, PetscInt, PetscInt, PetscInt, PetscInt, PetscInt, PetscScalar ****);
PetscErrorCode VecRestoreArray3d(Vec, PetscInt, PetscInt, PetscInt, PetscInt, PetscInt, PetscInt, PetscScalar ****);
PetscErrorCode VecSetValues(Vec, PetscInt, const PetscInt[], const PetscScalar[], InsertMode);
#define VecSetValue(v, i, va, mode) \
  do {                              \
    PetscInt _i = (i);              \
    PetscScalar _v = (va);          \
    VecSetValues(v, 1, &_i, &_v, mode); \
  } while (0)
PetscErrorCode VecAssemblyBegin(Vec);
PetscErrorCode VecAssemblyEnd(Vec);
PetscErrorCode VecView(Vec, PetscViewer);
PetscErrorCode VecLoadIntoVector(PetscViewer, Vec);
PetscErrorCode VecScatterCreateToZero(Vec, VecScatter *, Vec *);
PetscErrorCode VecScatterCreateToAll(Vec, VecScatter *, Vec *);
PetscErrorCode VecScatterBegin(VecScatter, Vec, Vec, InsertMode, ScatterMode);
PetscErrorCode VecScatterEnd(VecScatter, Vec, Vec, InsertMode, ScatterMode);
PetscErrorCode VecScatterDestroy(VecScatter);

// structured grids
PetscErrorCode DACreate3d(MPI_Comm, DAPeriodicType, DAStencilType, PetscInt, PetscInt, PetscInt, PetscInt, PetscInt,
                          PetscInt, PetscInt, PetscInt, PetscInt *, PetscInt *, PetscInt *, DA *);
PetscErrorCode DADestroy(DA);
PetscErrorCode DAGetInfo(DA, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *,
                         PetscInt *, PetscInt *, DAPeriodicType *, DAStencilType *);
PetscErrorCode DAGetLocalInfo(DA, DALocalInfo *);
PetscErrorCode DAGetCorners(DA, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *);
PetscErrorCode DAGetGhostCorners(DA, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *, PetscInt *);
PetscErrorCode DASetUniformCoordinates(DA, PetscReal, PetscReal, PetscReal, PetscReal, PetscReal, PetscReal);
PetscErrorCode DAGetCoordinateDA(DA, DA *);
PetscErrorCode DAGetCoordinates(DA, Vec *);
PetscErrorCode DAGetGhostedCoordinates(DA, Vec *);
PetscErrorCode DACreateGlobalVector(DA, Vec *);
PetscErrorCode DACreateLocalVector(DA, Vec *);
PetscErrorCode DACreateNaturalVector(DA, Vec *);
PetscErrorCode DAGetLocalVector(DA, Vec *);
PetscErrorCode DARestoreLocalVector(DA, Vec *);
PetscErrorCode DAGetGlobalVector(DA, Vec *);
PetscErrorCode DARestoreGlobalVector(DA, Vec *);
PetscErrorCode DAVecGetArray(DA, Vec, void *);
PetscErrorCode DAVecRestoreArray(DA, Vec, void *);
PetscErrorCode DAGlobalToLocalBegin(DA, Vec, InsertMode, Vec);
PetscErrorCode DAGlobalToLocalEnd(DA, Vec, InsertMode, Vec);
PetscErrorCode DALocalToLocalBegin(DA, Vec, InsertMode, Vec);
PetscErrorCode DALocalToLocalEnd(DA, Vec, InsertMode, Vec);
PetscErrorCode DALocalToGlobal(DA, Vec, InsertMode, Vec);
PetscErrorCode DALocalToGlobalBegin(DA, Vec, Vec);
PetscErrorCode DALocalToGlobalEnd(DA, Vec, Vec);
PetscErrorCode DAGlobalToNaturalBegin(DA, Vec, InsertMode, Vec);
PetscErrorCode DAGlobalToNaturalEnd(DA, Vec, InsertMode, Vec);
PetscErrorCode DANaturalToGlobalBegin(DA, Vec, InsertMode, Vec);
PetscErrorCode DANaturalToGlobalEnd(DA, Vec, InsertMode, Vec);
PetscErrorCode DAGetGlobalIndices(DA, PetscInt *, PetscInt **);
PetscErrorCode DAGetAO(DA, AO *);
PetscErrorCode AOApplicationToPetsc(AO, PetscInt, PetscInt[]);
PetscErrorCode AOPetscToApplication(AO, PetscInt, PetscInt[]);

// matrices
PetscErrorCode MatCreate(MPI_Comm, Mat *);
PetscErrorCode MatCreateMPIAIJ(MPI_Comm, PetscInt, PetscInt, PetscInt, PetscInt, PetscInt, const PetscInt[], PetscInt,
                               const PetscInt[], Mat *);
PetscErrorCode MatCreateSeqAIJ(MPI_Comm, PetscInt, PetscInt, PetscInt, const PetscInt[], Mat *);
PetscErrorCode MatSetSizes(Mat, PetscInt, PetscInt, PetscInt, PetscInt);
PetscErrorCode MatSetType(Mat, MatType);
PetscErrorCode MatSetFromOptions(Mat);
PetscErrorCode MatSetOption(Mat, MatOption, PetscTruth);
PetscErrorCode MatMPIAIJSetPreallocation(Mat, PetscInt, const PetscInt[], PetscInt, const PetscInt[]);
PetscErrorCode MatSeqAIJSetPreallocation(Mat, PetscInt, const PetscInt[]);
PetscErrorCode MatSetValues(Mat, PetscInt, const PetscInt[], PetscInt, const PetscInt[], const PetscScalar[], InsertMode);
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType);
PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType);
PetscErrorCode MatZeroEntries(Mat);
PetscErrorCode MatDestroy(Mat);
PetscErrorCode MatGetOwnershipRange(Mat, PetscInt *, PetscInt *);
PetscErrorCode MatGetSize(Mat, PetscInt *, PetscInt *);
PetscErrorCode MatGetRow(Mat, PetscInt, PetscInt *, const PetscInt **, const PetscScalar **);
PetscErrorCode MatRestoreRow(Mat, PetscInt, PetscInt *, const PetscInt **, const PetscScalar **);
PetscErrorCode MatMult(Mat, Vec, Vec);
PetscErrorCode MatGetVecs(Mat, Vec *, Vec *);
PetscErrorCode MatCreateShell(MPI_Comm, PetscInt, PetscInt, PetscInt, PetscInt, void *, Mat *);
PetscErrorCode MatShellGetContext(Mat, void **);
PetscErrorCode MatShellSetOperation(Mat, MatOperation, void (*)(void));
PetscErrorCode MatView(Mat, PetscViewer);
PetscErrorCode MatNullSpaceCreate(MPI_Comm, PetscTruth, PetscInt, const Vec[], MatNullSpace *);
PetscErrorCode MatNullSpaceSetFunction(MatNullSpace, PetscErrorCode (*)(MatNullSpace, Vec, void *), void *);
PetscErrorCode MatNullSpaceRemove(MatNullSpace, Vec, Vec *);
PetscErrorCode MatNullSpaceDestroy(MatNullSpace);

// Krylov solvers and preconditioners (accepted and ignored; KSPSolve aborts)
PetscErrorCode KSPCreate(MPI_Comm, KSP *);
PetscErrorCode KSPDestroy(KSP);
PetscErrorCode KSPSetType(KSP, KSPType);
PetscErrorCode KSPGetPC(KSP, PC *);
PetscErrorCode KSPSetOperators(KSP, Mat, Mat, MatStructure);
PetscErrorCode KSPSetTolerances(KSP, PetscReal, PetscReal, PetscReal, PetscInt);
PetscErrorCode KSPGMRESSetRestart(KSP, PetscInt);
PetscErrorCode KSPSetUp(KSP);
PetscErrorCode KSPSolve(KSP, Vec, Vec);
PetscErrorCode KSPSetFromOptions(KSP);
PetscErrorCode KSPSetInitialGuessNonzero(KSP, PetscTruth);
PetscErrorCode KSPSetInitialGuessKnoll(KSP, PetscTruth);
PetscErrorCode KSPSetNullSpace(KSP, MatNullSpace);
PetscErrorCode KSPSetNormType(KSP, KSPNormType);
PetscErrorCode KSPAppendOptionsPrefix(KSP, const char[]);
PetscErrorCode KSPSetOptionsPrefix(KSP, const char[]);
PetscErrorCode KSPMonitorSet(KSP, PetscErrorCode (*)(KSP, PetscInt, PetscReal, void *), void *,
                             PetscErrorCode (*)(void *));
PetscErrorCode KSPMonitorTrueResidualNorm(KSP, PetscInt, PetscReal, void *);
PetscErrorCode KSPBuildResidual(KSP, Vec, Vec, Vec *);
PetscErrorCode KSPGetIterationNumber(KSP, PetscInt *);
PetscErrorCode KSPGetConvergedReason(KSP, KSPConvergedReason *);
PetscErrorCode KSPGetResidualNorm(KSP, PetscReal *);
PetscErrorCode PCCreate(MPI_Comm, PC *);
PetscErrorCode PCSetType(PC, PCType);
PetscErrorCode PCSetOperators(PC, Mat, Mat, MatStructure);
PetscErrorCode PCSetFromOptions(PC);
PetscErrorCode PCSetUp(PC);
PetscErrorCode PCDestroy(PC);
PetscErrorCode PCBJacobiGetSubKSP(PC, PetscInt *, PetscInt *, KSP **);
PetscErrorCode PCFactorSetShiftNonzero(PC, PetscReal);
PetscErrorCode PCFactorSetShiftType(PC, MatFactorShiftType);
PetscErrorCode PCFactorSetShiftAmount(PC, PetscReal);
PetscErrorCode PCHYPRESetType(PC, const char[]);
PetscErrorCode PCMGSetLevels(PC, PetscInt, MPI_Comm *);
PetscErrorCode PCMGSetType(PC, PCMGType);
PetscErrorCode PCMGSetCycleType(PC, PCMGCycleType);
PetscErrorCode PCMGSetCycles(PC, PetscInt);
PetscErrorCode PCMGSetNumberSmoothUp(PC, PetscInt);
PetscErrorCode PCMGSetNumberSmoothDown(PC, PetscInt);
PetscErrorCode PCMGGetSmoother(PC, PetscInt, KSP *);
PetscErrorCode PCMGGetSmootherUp(PC, PetscInt, KSP *);
PetscErrorCode PCMGGetSmootherDown(PC, PetscInt, KSP *);
PetscErrorCode PCMGGetCoarseSolve(PC, KSP *);
PetscErrorCode PCMGSetInterpolation(PC, PetscInt, Mat);
PetscErrorCode PCMGSetRestriction(PC, PetscInt, Mat);
PetscErrorCode PCMGSetResidual(PC, PetscInt, PetscErrorCode (*)(Mat, Vec, Vec, Vec), Mat);
PetscErrorCode PCMGSetRhs(PC, PetscInt, Vec);
PetscErrorCode PCMGSetX(PC, PetscInt, Vec);
PetscErrorCode PCMGSetR(PC, PetscInt, Vec);
PetscErrorCode PCMGDefaultResidual(Mat, Vec, Vec, Vec);
PetscErrorCode SNESCreate(MPI_Comm, SNES *);
PetscErrorCode SNESDestroy(SNES);
// nonlinear solvers (the level-set reinitialisation and momentum paths):
// declared so that those files compile; every call aborts
typedef const char *SNESType;
#define SNESTR "tr"
#define SNESLS "ls"
PetscErrorCode SNESSetFunction(SNES, Vec, PetscErrorCode (*)(SNES, Vec, Vec, void *), void *);
PetscErrorCode MatCreateSNESMF(SNES, Mat *);
PetscErrorCode MatMFFDComputeJacobian(SNES, Vec, Mat *, Mat *, MatStructure *, void *);
PetscErrorCode SNESSetJacobian(SNES, Mat, Mat, PetscErrorCode (*)(SNES, Vec, Mat *, Mat *, MatStructure *, void *),
                               void *);
PetscErrorCode SNESSetType(SNES, SNESType);
PetscErrorCode SNESSetMaxLinearSolveFailures(SNES, PetscInt);
PetscErrorCode SNESSetMaxNonlinearStepFailures(SNES, PetscInt);
PetscErrorCode SNESKSPSetUseEW(SNES, PetscTruth);
PetscErrorCode SNESKSPSetParametersEW(SNES, PetscInt, PetscReal, PetscReal, PetscReal, PetscReal, PetscReal,
                                      PetscReal);
PetscErrorCode SNESSetTolerances(SNES, PetscReal, PetscReal, PetscReal, PetscInt, PetscInt);
PetscErrorCode SNESGetKSP(SNES, KSP *);
PetscErrorCode SNESMonitorSet(SNES, PetscErrorCode (*)(SNES, PetscInt, PetscReal, void *), void *,
                              PetscErrorCode (*)(void *));
PetscErrorCode SNESSolve(SNES, Vec, Vec);
PetscErrorCode SNESGetFunctionNorm(SNES, PetscReal *);
PetscErrorCode SNESSetFromOptions(SNES);
PetscErrorCode SNESGetIterationNumber(SNES, PetscInt *);

// -------------------------------------------------------------- HYPRE ----
typedef int HYPRE_Int;
typedef double HYPRE_Real;
typedef double HYPRE_Complex;
typedef struct hypre_IJVector_struct *HYPRE_IJVector;
typedef struct hypre_IJMatrix_struct *HYPRE_IJMatrix;
typedef struct hypre_ParCSRMatrix_struct *HYPRE_ParCSRMatrix;
typedef struct hypre_ParVector_struct *HYPRE_ParVector;
typedef struct hypre_Solver_struct *HYPRE_Solver;
typedef struct hypre_Matrix_struct *HYPRE_Matrix;
typedef struct hypre_Vector_struct *HYPRE_Vector;
typedef HYPRE_Int (*HYPRE_PtrToSolverFcn)(HYPRE_Solver, HYPRE_Matrix, HYPRE_Vector, HYPRE_Vector);
#define HYPRE_PARCSR 5555

HYPRE_Int HYPRE_IJVectorCreate(MPI_Comm, HYPRE_Int, HYPRE_Int, HYPRE_IJVector *);
HYPRE_Int HYPRE_IJVectorDestroy(HYPRE_IJVector);
HYPRE_Int HYPRE_IJVectorSetObjectType(HYPRE_IJVector, HYPRE_Int);
HYPRE_Int HYPRE_IJVectorSetMaxOffProcElmts(HYPRE_IJVector, HYPRE_Int);
HYPRE_Int HYPRE_IJVectorInitialize(HYPRE_IJVector);
HYPRE_Int HYPRE_IJVectorSetValues(HYPRE_IJVector, HYPRE_Int, const HYPRE_Int *, const HYPRE_Complex *);
HYPRE_Int HYPRE_IJVectorAddToValues(HYPRE_IJVector, HYPRE_Int, const HYPRE_Int *, const HYPRE_Complex *);
HYPRE_Int HYPRE_IJVectorGetValues(HYPRE_IJVector, HYPRE_Int, const HYPRE_Int *, HYPRE_Complex *);
HYPRE_Int HYPRE_IJVectorAssemble(HYPRE_IJVector);
HYPRE_Int HYPRE_IJVectorGetObject(HYPRE_IJVector, void **);
HYPRE_Int HYPRE_IJMatrixCreate(MPI_Comm, HYPRE_Int, HYPRE_Int, HYPRE_Int, HYPRE_Int, HYPRE_IJMatrix *);
HYPRE_Int HYPRE_IJMatrixDestroy(HYPRE_IJMatrix);
HYPRE_Int HYPRE_IJMatrixSetObjectType(HYPRE_IJMatrix, HYPRE_Int);
HYPRE_Int HYPRE_IJMatrixSetMaxOffProcElmts(HYPRE_IJMatrix, HYPRE_Int);
HYPRE_Int HYPRE_IJMatrixSetRowSizes(HYPRE_IJMatrix, const HYPRE_Int *);
HYPRE_Int HYPRE_IJMatrixInitialize(HYPRE_IJMatrix);
HYPRE_Int HYPRE_IJMatrixSetValues(HYPRE_IJMatrix, HYPRE_Int, HYPRE_Int *, const HYPRE_Int *, const HYPRE_Int *,
                                  const HYPRE_Complex *);
HYPRE_Int HYPRE_IJMatrixAssemble(HYPRE_IJMatrix);
HYPRE_Int HYPRE_IJMatrixGetObject(HYPRE_IJMatrix, void **);
HYPRE_Int HYPRE_BoomerAMGCreate(HYPRE_Solver *);
HYPRE_Int HYPRE_BoomerAMGDestroy(HYPRE_Solver);
HYPRE_Int HYPRE_BoomerAMGSetup(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector);
HYPRE_Int HYPRE_BoomerAMGSolve(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector);
HYPRE_Int HYPRE_BoomerAMGSetAggNumLevels(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetCoarsenType(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetCycleNumSweeps(HYPRE_Solver, HYPRE_Int, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetCycleType(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetInterpType(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetLevelOuterWt(HYPRE_Solver, HYPRE_Real, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetMaxIter(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetPrintLevel(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetRelaxType(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetRelaxWt(HYPRE_Solver, HYPRE_Real);
HYPRE_Int HYPRE_BoomerAMGSetSmoothNumSweeps(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetSmoothType(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_BoomerAMGSetStrongThreshold(HYPRE_Solver, HYPRE_Real);
HYPRE_Int HYPRE_BoomerAMGSetTol(HYPRE_Solver, HYPRE_Real);
HYPRE_Int HYPRE_GMRESSetMaxIter(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_GMRESSetPrecond(HYPRE_Solver, HYPRE_PtrToSolverFcn, HYPRE_PtrToSolverFcn, HYPRE_Solver);
HYPRE_Int HYPRE_GMRESSetPrintLevel(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_GMRESSetTol(HYPRE_Solver, HYPRE_Real);
HYPRE_Int HYPRE_GMRESSetKDim(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_PCGSetMaxIter(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_PCGSetPrecond(HYPRE_Solver, HYPRE_PtrToSolverFcn, HYPRE_PtrToSolverFcn, HYPRE_Solver);
HYPRE_Int HYPRE_PCGSetPrintLevel(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_PCGSetTol(HYPRE_Solver, HYPRE_Real);
HYPRE_Int HYPRE_ParCSRGMRESCreate(MPI_Comm, HYPRE_Solver *);
HYPRE_Int HYPRE_ParCSRGMRESDestroy(HYPRE_Solver);
HYPRE_Int HYPRE_ParCSRGMRESSetKDim(HYPRE_Solver, HYPRE_Int);
HYPRE_Int HYPRE_ParCSRGMRESSetAbsoluteTol(HYPRE_Solver, HYPRE_Real);
HYPRE_Int HYPRE_ParCSRGMRESSetup(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector);
HYPRE_Int HYPRE_ParCSRGMRESSolve(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector);
HYPRE_Int HYPRE_ParCSRPCGCreate(MPI_Comm, HYPRE_Solver *);

// ------------------------------------------------ harness-side hooks ----
// The inner FP64 solve that stands in for HYPRE GMRES + BoomerAMG: called
// with the assembled CSR matrix (n rows, 0-based), the right-hand side and
// the initial guess (overwritten with the solution).
typedef int (*vfs_shim_solve_fn)(int n, const int *rowptr, const int *cols, const double *vals, const double *rhs,
                                 double *x, double rtol);
void vfs_shim_set_solver(vfs_shim_solve_fn fn);
// The value of the last VecMax (the reference reduces its divergence with it).
double vfs_shim_last_vecmax(void);
// One more reference to a vector (the harness keeps the UserCtx vectors it
// created alive when a reference function destroys them, as FormMetrics
// does with the global metric vectors once their ghosted copies are set).
void vfs_shim_vec_retain(Vec v);
// Internal views used by the harness: storage of a vector and its DA.
double *vfs_shim_vec_data(Vec v, int *n);
int vfs_shim_mat_csr(Mat A, int *nrows, const int **rowptr, const int **cols, const double **vals);
int vfs_shim_hypre_vec(HYPRE_IJVector v, int *lo, int *hi, double **data);
int vfs_shim_hypre_mat_csr(HYPRE_IJMatrix A, int *nrows, const int **rowptr, const int **cols, const double **vals);
