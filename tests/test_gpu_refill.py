"""Incremental refill of the finest level on a new mask (marked gpu).

A new mask on a handle whose hierarchy is filled refills only the finest
level's rows within two points of a changed nvert value (a row reads nvert
within one point of its own, and a periodic ghost neighbour's dof test reads
its interior partner), the j-line factors of the columns holding one, and
those rows' packed and FP32 copies.  Every result must equal a fresh
handle's for the same mask, bit for bit: the FGMRES operator and its row
types, the finest level's FP32 operator, and the solves in both V-cycle
precisions.  The bodies here cross the periodic seam of the x direction,
where a change on one side alters rows on the other.
"""
import numpy as np
import pytest

from vfs_poisson import configs as CF

pytestmark = pytest.mark.gpu


def _mask(s, case, x0):
    surf = CF.rod_surface((x0, -0.05, 0.5), (0.0, 1.0, 0.0), 1.1, 0.06, 24, 4)
    nv, _ = s.ibm_search(surf, ibi=0)
    return CF.sync_periodic_ghosts(nv, case.periodic)


def _solver(case, incremental):
    import os
    import vfs_poisson as V
    old = os.environ.get("VFS_INCREMENTAL")
    try:
        os.environ["VFS_INCREMENTAL"] = "1" if incremental else "0"
        return V.PoissonSolver(*case.dims, periodic=case.periodic)
    finally:
        if old is None:
            os.environ.pop("VFS_INCREMENTAL", None)
        else:
            os.environ["VFS_INCREMENTAL"] = old


@pytest.mark.parametrize("incremental", [True, False], ids=["incremental", "full"])
@pytest.mark.parametrize("xs", [(0.03, 0.97, 0.5, 0.03), (0.5, 0.52, 0.5)], ids=["seam", "interior"])
def test_refill_matches_fresh(cuda_lib, xs, incremental):
    """(With VFS_INCREMENTAL=0 every row is refilled; both must match.)"""
    import vfs_poisson as V
    case = CF.towers(40, 24, 40, radius=0.05)
    moved = _solver(case, incremental)
    try:
        moved.set_grid(case.coor)
        for step, x0 in enumerate(xs):
            nv = _mask(moved, case, x0)
            moved.set_nvert(nv)
            u = CF._mask_faces(case.ucont, nv)
            fresh = V.PoissonSolver(*case.dims, periodic=case.periodic)
            try:
                fresh.set_grid(case.coor)
                fresh.set_nvert(nv)
                a_m, rt_m = moved.operator()
                a_f, rt_f = fresh.operator()
                np.testing.assert_array_equal(rt_m, rt_f)
                np.testing.assert_array_equal(a_m, a_f)
                np.testing.assert_array_equal(moved.operator32(), fresh.operator32())
                for prec in (0, 1):
                    out = []
                    for s in (moved, fresh):
                        s.rhs(u)
                        phi, st = s.solve(precision=prec, rtol=1e-10)
                        out.append((phi, st.iterations, st.rel_residual))
                    assert out[0][1] == out[1][1] and out[0][2] == out[1][2], (step, prec)
                    np.testing.assert_array_equal(out[0][0], out[1][0])
            finally:
                fresh.close()
    finally:
        moved.close()
