"""The C code in INTEGRATION.md compiles against include/vfs_poisson.h: the
adapter, the neighbour calls and the learned-guess sequence are extracted,
given stub declarations of the reference's PETSc types and UserCtx fields,
and built with gcc (implicit declarations and pointer mismatches are errors;
CPU)."""
import os
import re
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STUBS = r"""
#include <stddef.h>
typedef double PetscReal;
typedef int PetscInt;
typedef struct { double x, y, z; } Cmpnts;
typedef struct { int mx, my, mz; } DALocalInfo;
typedef struct _DA *DA;
typedef struct _Vec *Vec;
typedef int InsertMode;
#define INSERT_VALUES 0
#define PETSC_COMM_WORLD 0
typedef struct {
  DALocalInfo info; DA da, fda;
  Vec lNvert, lUcont, Ucont, Phi, lPhi, P;
  int bctype[6]; double dt, st, FluxIntpSum;
} UserCtx;
typedef struct { int n_v, n_elmt; } IBMNodes;
int DAGetGhostedCoordinates(DA, Vec *);
int DAVecGetArray(DA, Vec, void *);
int DAVecRestoreArray(DA, Vec, void *);
int DAGlobalToLocalBegin(DA, Vec, InsertMode, Vec);
int DAGlobalToLocalEnd(DA, Vec, InsertMode, Vec);
int PetscPrintf(int, const char *, ...);
int Contra2Cart(UserCtx *);
double time_coeff(void);
int i_periodic, j_periodic, k_periodic, ii_periodic, jj_periodic, kk_periodic;
int ti, tistart, movefsi, rotatefsi, poisson_it;
double poisson_tol;
"""


def _blocks():
    src = open(os.path.join(REPO, "INTEGRATION.md")).read()
    return re.findall(r"```c\n(.*?)```", src, flags=re.S)


def test_integration_c_code_compiles(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    blocks = _blocks()
    adapter = [b for b in blocks if "vfs_gpu_adapter.c" in b]
    neighbours = [b for b in blocks if "vfs_poisson_ibm_search(" in b]
    guess = [b for b in blocks if "vfs_poisson_learned_guess(" in b]
    assert len(adapter) == 1 and len(neighbours) == 1 and len(guess) == 1
    code = STUBS + adapter[0].replace('#include "variables.h"\n', "")
    code += """
static void neighbours(UserCtx *user, int bi, IBMNodes *ibm, int ibi, const double *xyz, const int *tri,
                       PetscReal ***nvert, Cmpnts ***ucont, Cmpnts ***lucont, Cmpnts ***ucat, Cmpnts ***lucat,
                       PetscReal ***lp, int flg, int poisson, int immersed, const double *u_surf) {
  double ibm_Flux = 0., ibm_Area = 0.;
""" + neighbours[0] + "}\n"
    code += """
static void guess(vfs_poisson *h, const double *ucont, const double *phi_nm1, const double *phi_nm2,
                  double *phi, double dt, double st, double coeff, double kappa) {
""" + guess[0] + "}\n"
    src = tmp_path / "snippets.c"
    src.write_text(code)
    p = subprocess.run([gcc, "-std=c99", "-fsyntax-only", "-Werror=implicit-function-declaration",
                        "-Werror=incompatible-pointer-types", "-Werror=int-conversion", "-I",
                        os.path.join(REPO, "include"), str(src)], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
