"""Load the golden fixtures of tests/golden/ (outputs of the reference's own
functions, written by tests/golden/make_golden.py) and rebuild their inputs
as a configs.Case."""
import glob
import os

import numpy as np

from vfs_poisson import configs as CF

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    g = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    nz, ny, nx = (s - 2 for s in g["nvert"].shape)
    case = CF.Case(name, nx, ny, nz, tuple(int(v) for v in g["periodic"]), g["coor"], g["nvert"], g["ucont"])
    np.testing.assert_array_equal(case.nvert, g["nvert"])  # ghosts already synced
    return case, g


def csr(g):
    import scipy.sparse as sp
    n = len(g["A_rowptr"]) - 1
    A = sp.csr_matrix((g["A_vals"], g["A_cols"], g["A_rowptr"]), shape=(n, n))
    A.sort_indices()
    return A


def check_oracle(case, g):
    """Every stage of the oracle's restatement against the reference's
    outputs `g` on `case`, bit for bit."""
    import oracle as O
    d = O.dims_of(case)
    met = O.form_metrics(d, case.coor)
    for f in ("csi", "eta", "zet", "icsi", "ieta", "izet", "jcsi", "jeta", "jzet", "kcsi", "keta", "kzet", "cent",
              "aj", "iaj", "jaj", "kaj"):
        np.testing.assert_array_equal(met[f], g[f], err_msg=f)
    lhs = O.poisson_lhs(d, case.nvert, met)
    np.testing.assert_array_equal(lhs["gid"].reshape(case.nvert.shape), g["gid"])
    A = O.csr(lhs).tocsr()
    A.sort_indices()
    Ar = csr(g)
    np.testing.assert_array_equal(A.indptr, Ar.indptr)
    np.testing.assert_array_equal(A.indices, Ar.indices)
    np.testing.assert_array_equal(A.data, Ar.data)
    gid = lhs["gid"]
    np.testing.assert_array_equal(O.rhs2(d, case.nvert, gid, case.ucont, met["aj"], 0), g["rhs2_0"])
    np.testing.assert_array_equal(O.rhs2(d, case.nvert, gid, case.ucont, met["aj"], -1), g["rhs2_m1"])
    # PoissonSolver_Hypre applies VolumeFlux (the immersed == 0 overload,
    # poisson_hypre.c:561) to Ucont before its right-hand side
    u_0, flux0, area0 = O.volume_flux0(d, case.nvert, met, case.ucont)
    np.testing.assert_array_equal(u_0, g["vflux_0_ucont"])
    np.testing.assert_array_equal([flux0, area0], g["vflux_0"])
    np.testing.assert_array_equal(O.rhs(d, case.nvert, gid, u_0, met["aj"]), g["b_hypre"])
    phi2 = O.remove_nullspace(d, case.nvert, gid, g["x_solver"])
    np.testing.assert_array_equal(phi2, g["phi2"])
    phi = O.convert_phi2_phi(d, case.nvert, phi2)
    np.testing.assert_array_equal(phi, g["phi"])
    p, _ = O.update_pressure(d, case.nvert, g["p0"].copy(), phi)
    np.testing.assert_array_equal(p, g["p"])
    u = O.projection(d, case.nvert, phi, met, u_0)
    np.testing.assert_array_equal(u, g["ucont_proj"])
    assert O.divergence(d, case.nvert, u, met["aj"]) == g["maxdiv_proj"][0]
    u_ib, flux, area = O.volume_flux(d, case.nvert, met, case.ucont, flg=0)
    np.testing.assert_array_equal(u_ib, g["vflux_ib_ucont"])
    np.testing.assert_array_equal([flux, area], g["vflux_ib"])
    multi, ksk = O.fully_blocked(d, case.nvert)
    assert int(multi) == int(g["multinull"][0])
    np.testing.assert_array_equal(ksk, g["ksk"])
    np.testing.assert_array_equal(O.nullspace_original(d, case.nvert, g["ns_x"], ksk, multi), g["ns_out"])
