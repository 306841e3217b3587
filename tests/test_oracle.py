"""CPU checks of the oracle (no GPU): every stage of the restatement against
the golden fixtures that the reference's own functions produced
(tests/golden/, written by tests/golden/make_golden.py from the reference's
sources compiled against a single-rank PETSc/HYPRE/MPI stand-in), plus the
restated operator's structural properties, the right-hand side's
consistency, the CPU baseline solver against an exact sparse solve and the
transfer operators' algebra."""
import os

import numpy as np
import pytest

import golden_io
import oracle as O
from vfs_poisson import configs as CF



@pytest.fixture(scope="module", params=["channel", "cylinder", "towers"])
def system(request):
    case = {"channel": lambda: CF.channel(12, 10, 12),
            "cylinder": lambda: CF.cylinder(20, 12, 20),
            "towers": lambda: CF.towers(24, 16, 24, radius=0.08)}[request.param]()
    d = O.dims_of(case)
    met = O.form_metrics(d, case.coor)
    lhs = O.poisson_lhs(d, case.nvert, met)
    return case, d, met, lhs


def test_operator_is_conservative_with_constant_nullspace(system):
    case, d, met, lhs = system
    A = O.csr(lhs)
    fluid = O.from_da(d, lhs["gid"], (case.nvert < 0.1).astype(float)) > 0
    # A 1 = 0 on fluid rows (flux form) and column sums vanish (conservation)
    assert np.abs((A @ np.ones(A.shape[0]))[fluid]).max() < 1e-14
    assert np.abs(np.asarray(A.sum(axis=0)).ravel()[fluid]).max() < 1e-14
    assert (A.diagonal()[fluid] < 0).all()


def test_numbering_counts_fluid_cells(system):
    case, d, met, lhs = system
    inner = case.nvert[1:-1, 1:-1, 1:-1]
    assert lhs["ndof"] == int(((inner.astype(int)) <= 0).sum())
    gid = lhs["gid"][1:-1, 1:-1, 1:-1]
    assert sorted(gid[gid >= 0].ravel().tolist()) == list(range(lhs["ndof"]))


def test_rhs_is_consistent(system):
    case, d, met, lhs = system
    b = O.rhs(d, case.nvert, lhs["gid"], case.ucont, met["aj"])
    assert abs(b.sum()) <= 1e-12 * np.abs(b).sum()


def test_cpu_solver_matches_exact(system):
    import scipy.sparse.linalg as spla
    case, d, met, lhs = system
    b = O.rhs(d, case.nvert, lhs["gid"], case.ucont, met["aj"])
    A = O.csr(lhs)
    mg = O.MGSolver(d, case.coor, case.nvert, met, threads=2)
    x, st = mg.solve(O.to_da(d, lhs["gid"], b), rtol=1e-10)
    x2 = O.from_da(d, lhs["gid"], x)
    assert np.linalg.norm(b - A @ x2) / np.linalg.norm(b) <= 1e-10
    Ap = A.tolil()
    Ap[0, :] = 0
    Ap[0, 0] = 1
    bp = b.copy()
    bp[0] = 0
    xe = spla.spsolve(Ap.tocsr(), bp)
    xe = O.remove_nullspace(d, case.nvert, lhs["gid"], xe)
    x2 = O.remove_nullspace(d, case.nvert, lhs["gid"], x2)
    assert np.linalg.norm(x2 - xe) / np.linalg.norm(xe) <= 1e-8


def test_projection_reduces_divergence(system):
    """Solve, update and project: the post-projection divergence of the fluid
    cells away from the body falls to the solver tolerance level."""
    import scipy.sparse.linalg as spla
    case, d, met, lhs = system
    u0 = case.ucont.copy()
    # close the non-periodic walls so that the flux field can be made
    # divergence-free (the synthetic Ucont is random on the wall faces too)
    per = [case.periodic[q] or case.periodic[q + 3] for q in range(3)]
    if not per[0]:
        u0[:, :, 0, 0] = 0
        u0[:, :, -2, 0] = 0
    if not per[1]:
        u0[:, 0, :, 1] = 0
        u0[:, -2, :, 1] = 0
    if not per[2]:
        u0[0, :, :, 2] = 0
        u0[-2, :, :, 2] = 0
    b = O.rhs(d, case.nvert, lhs["gid"], u0, met["aj"])
    A = O.csr(lhs).tolil()
    A[0, :] = 0
    A[0, 0] = 1
    bp = b.copy()
    bp[0] = 0
    x2 = O.remove_nullspace(d, case.nvert, lhs["gid"], spla.spsolve(A.tocsr(), bp))
    phi = O.convert_phi2_phi(d, case.nvert, x2)
    div0 = O.divergence(d, case.nvert, u0, met["aj"])
    u = O.projection(d, case.nvert, phi, met, u0)
    div1 = O.divergence(d, case.nvert, u, met["aj"])
    assert div1 < 1e-6 * div0


def test_restriction_interpolation_weights():
    """MyRestriction of a constant gives 1 on unblanked coarse cells;
    MyInterpolation of a constant reproduces it on the fine grid."""
    case = CF.channel(8, 8, 8)
    d = O.dims_of(case)
    dc = O.dims(6, 6, 6, case.periodic)
    nvc = O.nvert_restriction(d, dc, 0, 0, 0, case.nvert)
    one_f = np.zeros((10, 10, 10))
    one_f[1:-1, 1:-1, 1:-1] = 1
    rc = O.restriction(dc, d, 0, 0, 0, nvc, case.nvert, one_f)
    np.testing.assert_allclose(rc[1:-1, 1:-1, 1:-1], 1.0)
    one_c = np.zeros((6, 6, 6))
    one_c[1:-1, 1:-1, 1:-1] = 1
    f = O.interpolation(d, dc, 0, 0, 0, case.nvert, nvc, one_c)
    np.testing.assert_allclose(f[1:-1, 1:-1, 1:-1], 1.0)


@pytest.mark.parametrize("name", golden_io.names())
def test_golden_fixtures(name):
    """The oracle reproduces the reference's outputs bit for bit: FormMetrics,
    the dof numbering, the assembled operator, PoissonRHS2 (-poisson 0 and
    -1), the right-hand side PoissonSolver_Hypre hands to HYPRE,
    Remove_Nullspace + Convert_Phi2_Phi of the same inner solution,
    UpdatePressure, Projection, Divergence and both VolumeFlux variants."""
    case, g = golden_io.load(name)
    golden_io.check_oracle(case, g)


# --- immersed-boundary classification (ibm_search_advanced) ---

def test_glibc_rand_restatement_matches_libc():
    """The ray directions of point_cell_advanced (Source/ibm.c:1100-1110) use
    the first rand() after srand(searchtimes); the restated generator must
    give the C library's own values."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand.argtypes = [ctypes.c_uint]
    for seed in list(range(0, 130)) + [12345, 2 ** 31 - 1, 2 ** 31, 2 ** 32 - 1]:
        libc.srand(seed)
        assert O.glibc_rand_first(seed) == libc.rand(), seed


def test_ibm_search_cylinder_matches_geometry():
    c = CF.cylinder(24, 16, 24)
    d = O.dims_of(c)
    met = O.form_metrics(d, c.coor)
    n = 24
    surf = CF.rod_surface((0.5, -0.01, 0.5), (0, 1, 0), 1.02, 0.1, n, 8)
    nv, failed = O.ibm_search(d, met["cent"], surf)
    assert failed == 0
    cc = met["cent"][1:-1, 1:-1, 1:-1]
    r = np.hypot(cc[..., 0] - 0.5, cc[..., 2] - 0.5)
    inner = nv[1:-1, 1:-1, 1:-1]
    # inside the inscribed polygon -> solid; outside the circle -> not solid
    assert np.all(inner[r < 0.1 * np.cos(np.pi / n) - 1e-9] == 3)
    assert np.all(inner[r > 0.1 + 1e-9] != 3)
    # interior agrees with the inside/dilation rule used by the generators
    ref = CF.classify(r < 0.1)
    np.testing.assert_array_equal(inner, ref[1:-1, 1:-1, 1:-1])


def test_ibm_search_multibody_and_walls():
    c = CF.towers(32, 24, 32, radius=0.05)
    d = O.dims_of(c)
    met = O.form_metrics(d, c.coor)
    nv = np.zeros((d.mz, d.my, d.mx))
    nv[5, 5, 5] = 7.0                      # >= 5 survives the first body's reset
    bc = (0, 0, -1, 0, 0, 0)
    for ibi, surf in enumerate(CF.tower_surfaces(radius=0.05, height=0.6)):
        nv, failed = O.ibm_search(d, met["cent"], surf, nvert=nv, ibi=ibi, bctype=bc)
        assert failed == 0
    inner = nv[1:-1, 1:-1, 1:-1]
    assert nv[5, 5, 5] == 7.0
    assert np.all(inner[:, 0, :][inner[:, 0, :] != 7.0] == 1.0)   # j == 1 wall row
    assert (inner == 3).sum() > 0 and set(np.unique(inner)) <= {0.0, 1.0, 3.0, 7.0}


def test_rhs2_unweighted_mean(system):
    """PoissonRHS2 (-poisson 0): fluid entries sum to zero; identity-row
    dofs stay 0; the per-cell values equal PoissonRHS2_hypre's before the
    shift (same divergence)."""
    case, d, met, lhs = system
    b2 = O.rhs2(d, case.nvert, lhs["gid"], case.ucont, met["aj"], 0)
    raw = O.rhs_raw(d, case.nvert, lhs["gid"], case.ucont)
    g = lhs["gid"][1:-1, 1:-1, 1:-1]
    fl = (case.nvert[1:-1, 1:-1, 1:-1] < 0.1)
    idx = g[fl]
    assert abs(b2[idx].sum()) <= 1e-10 * np.abs(b2).sum()
    d2 = b2[idx] - raw[idx]
    assert np.ptp(d2) <= 1e-12 * max(1.0, np.abs(d2).max())


def _face_flux_from_velocity(case, met, vel):
    """Contravariant face fluxes of a uniform Cartesian velocity: U.n with
    the face area vectors icsi, jeta, kzet."""
    u = np.zeros(case.nvert.shape + (3,))
    for q, f in enumerate(("icsi", "jeta", "kzet")):
        u[..., q] = met[f] @ np.asarray(vel, np.float64)
    return u


def test_volume_flux_removes_net_ib_flux():
    c = CF.cylinder(20, 12, 20)
    d = O.dims_of(c)
    met = O.form_metrics(d, c.coor)
    rng = np.random.default_rng(2)
    u0 = rng.uniform(-1, 1, c.ucont.shape)
    for flg in (0, 1, 2, 3):
        u, flux, area = O.volume_flux(d, c.nvert, met, u0, flg=flg)
        assert area > 0
        if flg in (0, 2, 3):   # without an interpolation flux the net flux vanishes
            assert abs(flux) <= 1e-10 * np.abs(u0).sum()
        # faces not touching the fluid/IB interface are untouched
        nv = c.nvert
        ib = (nv > 0.1) & (nv < 1.1)
        fl = nv < 0.1
        touch = np.zeros(nv.shape, bool)
        touch[:, :, :-1] |= (fl[:, :, :-1] & ib[:, :, 1:]) | (ib[:, :, :-1] & fl[:, :, 1:])
        far = ~touch
        far[0] = far[-1] = True
        assert np.array_equal(u[..., 0][far & ~touch], u0[..., 0][far & ~touch])


def test_contra2cart_recovers_uniform_velocity():
    # on a uniform Cartesian grid the cell and face metrics agree and the
    # centred flux averages give a uniform velocity back exactly (on
    # stretched grids the reference's cell metrics differ from the face
    # metrics and so does its reconstruction)
    c = CF.channel(12, 10, 12)
    c.coor = CF._nodes(12, 10, 12, lambda e: e, 0.0)
    d = O.dims_of(c)
    met = O.form_metrics(d, c.coor)
    vel = (0.3, -0.2, 0.7)
    ucont = _face_flux_from_velocity(c, met, vel)
    ucat = O.contra2cart(d, c.nvert, met, ucont)
    inner = ucat[1:-1, 1:-1, 1:-1]
    np.testing.assert_allclose(inner, np.broadcast_to(vel, inner.shape), rtol=0, atol=1e-12)


@pytest.mark.parametrize("density", [1.0, 3.0])
def test_levelset_operator_with_uniform_density(system, density):
    """The level-set branch of the restated operator with a uniform density
    and no Dirichlet faces is the plain operator divided by that density
    (harmonic face means of equal densities)."""
    case, d, met, lhs = system
    rho = np.full(case.nvert.shape, density)
    try:
        O.set_levelset(rho, np.zeros_like(rho), (0, 0, 0, 0, 0, 0))
        ls = O.poisson_lhs(d, case.nvert, met)
    finally:
        O.set_levelset(None)
    assert ls["ndof"] == lhs["ndof"]
    np.testing.assert_array_equal(ls["col"], lhs["col"])
    np.testing.assert_allclose(ls["vol"], lhs["vol"] / density, rtol=1e-13, atol=1e-13 * np.abs(lhs["vol"]).max())


def test_levelset_dirichlet_top_makes_rows_regular():
    """With bctype[3] == 4 (zero-Dirichlet j-top faces) the rows next to the
    top face lose their zero row sum and the others keep it."""
    case = CF.channel(12, 10, 12)
    d = O.dims_of(case)
    met = O.form_metrics(d, case.coor)
    rho = np.where(np.arange(case.nvert.shape[1])[None, :, None] < 6, 1000.0, 1.2) * np.ones(case.nvert.shape)
    try:
        O.set_levelset(rho, np.zeros_like(rho), (0, 0, 0, 4, 0, 0))
        lhs = O.poisson_lhs(d, case.nvert, met)
    finally:
        O.set_levelset(None)
    A = O.csr(lhs)
    rs = np.abs(A @ np.ones(A.shape[0]))
    gid = lhs["gid"]
    top = gid[1:-1, -2, 1:-1]
    rest = gid[1:-1, 1:-2, 1:-1]
    scale = np.abs(A.diagonal()).max()
    assert (rs[top[top >= 0]] > 1e-8 * scale).all()
    assert rs[rest[rest >= 0]].max() < 1e-12 * scale
