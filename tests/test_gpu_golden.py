"""The CUDA library against the reference's own outputs (marked gpu).

tests/golden/ holds what the reference's functions (Source/metrics.c,
poisson.c, poisson_hypre.c, main.c, rhs.c compiled unmodified against a
single-rank PETSc/HYPRE/MPI stand-in) computed on small seeded grids.  The
library, called through its C ABI, must reproduce them:
  * bit for bit: FormMetrics, the dof numbering, the assembled operator,
    UpdatePressure, Projection, Divergence and the per-face results of both
    VolumeFlux overloads;
  * to 1e-12 of the largest entry where the library reduces in another
    order: the right-hand sides (the mean removals) and the VolumeFlux sums;
  * to 1e-12 of the largest entry as well: PoissonNullSpaceFunction_original
    (its means); FullyBlocked bit for bit;
  * the solve: phi within 1e-6 relative L2 of the phi the reference makes
    from an exact inner solve (Remove_Nullspace + Convert_Phi2_Phi), with the
    true FP64 residual of the reference's own matrix <= 1e-8.
"""
import numpy as np
import pytest

import golden_io
import oracle as O

pytestmark = pytest.mark.gpu

METRICS3 = ("csi", "eta", "zet", "icsi", "ieta", "izet", "jcsi", "jeta", "jzet", "kcsi", "keta", "kzet", "cent")
METRICS1 = ("aj", "iaj", "jaj", "kaj")


@pytest.fixture(scope="module", params=golden_io.names())
def golden(request, cuda_lib):
    import vfs_poisson as V
    case, g = golden_io.load(request.param)
    s = V.PoissonSolver.from_case(case)
    yield case, g, s
    s.close()


def _dof(g, v_da):
    gid = g["gid"].astype(np.int64).ravel()
    mz, my, mx = g["gid"].shape
    inner = np.zeros((mz, my, mx), bool)
    inner[1:-1, 1:-1, 1:-1] = True
    sel = inner.ravel() & (gid >= 0)
    out = np.zeros(int(gid.max()) + 1)
    out[gid[sel]] = v_da.ravel()[sel]
    return out


def test_metrics_numbering_operator(golden):
    case, g, s = golden
    for f in METRICS3 + METRICS1:
        np.testing.assert_array_equal(s.metric(f), g[f], err_msg=f)
    n, gid = s.numbering()
    np.testing.assert_array_equal(gid, g["gid"].astype(np.int32))
    vol, rt = s.operator()
    # the library's coefficients placed by the oracle's column map (which
    # slots hold a matrix entry: the 1e-10 filter, identity rows)
    d = O.dims_of(case)
    col = O.poisson_lhs(d, case.nvert, O.form_metrics(d, case.coor))["col"]
    A = O.csr({"vol": vol, "rowtype": rt, "gid": gid, "ndof": n, "col": col}).tocsr()
    A.sort_indices()
    Ar = golden_io.csr(g)
    np.testing.assert_array_equal(A.indptr, Ar.indptr)
    np.testing.assert_array_equal(A.indices, Ar.indices)
    np.testing.assert_array_equal(A.data, Ar.data)


def test_right_hand_sides(golden):
    case, g, s = golden
    # the reference's solver forms its right-hand side from Ucont after
    # VolumeFlux (the immersed == 0 overload)
    s.rhs(g["vflux_0_ucont"])
    b = _dof(g, s.rhs_array())
    assert np.abs(b - g["b_hypre"]).max() <= 1e-12 * np.abs(g["b_hypre"]).max()
    s.rhs2(case.ucont, 0)
    b = _dof(g, s.rhs_array())
    assert np.abs(b - g["rhs2_0"]).max() <= 1e-12 * np.abs(g["rhs2_0"]).max()


def test_update_pressure_projection_divergence(golden):
    case, g, s = golden
    p = g["p0"].copy()
    s.update_pressure(p, g["phi"].copy())
    np.testing.assert_array_equal(p, g["p"])
    u = g["vflux_0_ucont"].copy()
    s.projection(u)
    np.testing.assert_array_equal(u, g["ucont_proj"])
    assert s.divergence(u) == g["maxdiv_proj"][0]


def test_volume_flux_both_overloads(golden):
    case, g, s = golden
    u = case.ucont.copy()
    flux, area = s.volume_flux(u, 0)
    np.testing.assert_array_equal(u, g["vflux_ib_ucont"])
    f_r, a_r = g["vflux_ib"]
    assert abs(area - a_r) <= 1e-12 * max(abs(a_r), 1.0)
    assert abs(flux - f_r) <= 1e-12 * max(np.abs(case.ucont).max() * max(a_r, 1.0), 1.0)
    u = case.ucont.copy()
    flux, area = s.volume_flux0(u, 0)
    np.testing.assert_array_equal(u, g["vflux_0_ucont"])
    f_r, a_r = g["vflux_0"]
    assert abs(area - a_r) <= 1e-12 * max(abs(a_r), 1.0)
    assert abs(flux - f_r) <= 1e-12 * max(np.abs(case.ucont).max() * max(a_r, 1.0), 1.0)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32mg", "fp64mg"])
def test_solve_against_reference_phi(golden, precision):
    case, g, s = golden
    s.rhs(g["vflux_0_ucont"])
    phi, st = s.solve(precision=precision, rtol=1e-8, max_it=100)
    assert st.status == 0 and st.rel_residual <= 1e-8, st.as_dict()
    A = golden_io.csr(g)
    phi2 = _dof(g, phi)
    b = g["b_hypre"]
    assert np.linalg.norm(b - A @ phi2) / np.linalg.norm(b) <= 1.2e-8
    fl = _dof(g, (case.nvert < 0.1).astype(np.float64)) > 0
    ref = _dof(g, g["phi"])
    assert np.linalg.norm((phi2 - ref)[fl]) / np.linalg.norm(ref[fl]) <= 1e-6


def test_fully_blocked_and_nullspace_original(golden):
    """FullyBlocked bit for bit (the first blocked k per column and the
    multiple-null-space flag, which the channel cut by a solid slab sets),
    and PoissonNullSpaceFunction_original of the fixture's seeded array to
    1e-12 of its largest entry (its means are reduced in another order), on
    host and on device arrays."""
    import torch
    case, g, s = golden
    multi, ksk = s.fully_blocked()
    assert int(multi) == int(g["multinull"][0])
    np.testing.assert_array_equal(ksk, g["ksk"])
    tol = 1e-12 * np.abs(g["ns_x"]).max()
    x = g["ns_x"].copy()
    s.nullspace_original(x)
    np.testing.assert_allclose(x, g["ns_out"], rtol=0, atol=tol)
    xd = torch.from_numpy(g["ns_x"].copy()).cuda()
    s.nullspace_original(xd)
    np.testing.assert_allclose(xd.cpu().numpy(), g["ns_out"], rtol=0, atol=tol)
