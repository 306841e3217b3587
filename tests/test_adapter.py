"""The drop-in adapter on the CPU (no GPU needed).

  * The DA bridge reads and writes the reference's global DA vectors in the
    library's DA-natural layout for every periodic-DA family (no wrap, x,
    x+z, x+y+z) and dof 1 and 3, on the single-rank PETSc stand-in whose
    ghosted copies start at gxs = -3 with rows of mx + 6 points
    (Source/init.c:145-161): after a scatter, the ghost layer of the
    refreshed local copy holds the periodic partners' values.
  * Without a GPU the bridge refuses to start with VFS_ECUDA (no fallback).
  * Where the reference's sources exist: the UserCtx adapter compiles
    against the reference's variables.h, links in place of the reference's
    PoissonSolver_Hypre / UpdatePressure / Projection / Divergence (their
    originals renamed at compile time), and a reference call into it stops
    the run with the library's error when no GPU is present.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import adapter_build

WRAPS = {"none": (0, 0, 0), "x": (1, 0, 0), "xz": (1, 0, 1), "xyz": (1, 1, 1)}


@pytest.fixture(scope="module")
def H():
    return adapter_build.harness()


@pytest.mark.parametrize("dof", [1, 3])
@pytest.mark.parametrize("wrap", list(WRAPS))
def test_gather_scatter_global_vectors(H, wrap, dof):
    import ctypes as C
    mx, my, mz = 9, 7, 6
    ii, jj, kk = WRAPS[wrap]
    da = H.ah_da_create(mx, my, mz, ii, jj, kk, dof)
    corners = np.zeros(6, np.int32)
    H.ah_ghost_corners(da, corners.ctypes.data)
    for q, (per, m) in enumerate(zip((ii, jj, kk), (mx, my, mz))):
        assert corners[q] == (-3 if per else 0) and corners[3 + q] == (m + 6 if per else m)
    v = H.ah_global(da)
    rng = np.random.default_rng(5)
    shape = (mz, my, mx) + ((3,) if dof == 3 else ())
    a = rng.standard_normal(shape)
    H.ah_fill(da, v, a.ctypes.data, dof)
    out = np.zeros(shape)
    assert H.vfsa_gather(da, v, out.ctypes.data) == 0
    np.testing.assert_array_equal(out, a)
    b = rng.standard_normal(shape)
    assert H.vfsa_scatter(da, b.ctypes.data, v) == 0
    back = np.zeros(shape)
    H.ah_read(da, v, back.ctypes.data, dof)
    np.testing.assert_array_equal(back, b)
    # ghosts of the refreshed local copy: periodic partners
    c = dof - 1
    bb = b if dof == 3 else b[..., None]
    if ii:
        assert H.ah_ghosted(da, v, -1, 2, 3, c, dof) == bb[3, 2, mx - 1, c]
        assert H.ah_ghosted(da, v, mx + 2, 2, 3, c, dof) == bb[3, 2, 2, c]
    if jj:
        assert H.ah_ghosted(da, v, 4, -3, 1, c, dof) == bb[1, my - 3, 4, c]
    if kk:
        assert H.ah_ghosted(da, v, 4, 2, -2, c, dof) == bb[mz - 2, 2, 4, c]
    H.ah_vec_destroy(v)


def _cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_cuda(), reason="checks the no-GPU refusal")
def test_bridge_refuses_without_gpu(H):
    import ctypes as C
    import vfs_poisson as V
    da = H.ah_da_create(8, 8, 8, 1, 0, 0, 1)
    fda = H.ah_coordinate_da(da)
    desc = V.GridDesc(8, 8, 8, 0, 0, 0, 1, 0, 0, 0)
    b = C.c_void_p()
    rc = H.vfsa_create(da, fda, C.byref(desc), C.byref(b))
    assert rc == V.VFS_ECUDA


@pytest.mark.skipif(_cuda(), reason="checks the no-GPU stop")
def test_full_adapter_links_and_stops_without_gpu(tmp_path):
    lib = adapter_build.full_adapter()
    if lib is None:
        pytest.skip("reference sources not present")
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    for sym in ("_Z19PoissonSolver_HypreP7UserCtxP8IBMNodesP7IBMInfo", "_Z14UpdatePressureP7UserCtx",
                "_Z10ProjectionP7UserCtx", "_Z10DivergenceP7UserCtx", "vfsa_solve"):
        assert sym in out, sym
    for sym in ("vfs_reference_PoissonSolver_Hypre", "vfs_reference_Projection"):
        assert sym in out, sym
    script = f"""
import sys
sys.path[:0] = {[os.path.join(adapter_build.REPO, p) for p in ('oracle', 'vfs-wind_gb300', 'tests')]!r}
import reference as R
R.LIB = {lib!r}
from vfs_poisson import configs as CF
import make_golden
case = CF.cylinder(12, 8, 12)
B = R.Block(case)
B.form_metrics()
B.set("nvert", case.nvert)
B.set("ucont", case.ucont)
B.ndof = 1
B.solver_hypre(make_golden.pinned_solve, 1e-8)
print("returned")
"""
    env = dict(os.environ, PYTHONPATH=os.path.join(adapter_build.REPO, "tests", "golden"))
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, cwd=tmp_path, env=env,
                       timeout=300)
    assert r.returncode != 0 and "returned" not in r.stdout
    assert "GPU pressure projection: vfs_poisson_create failed" in r.stderr, r.stderr[-2000:]
