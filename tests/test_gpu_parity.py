"""CUDA path vs the oracle, through the C ABI (marked gpu).

Bit-exact where the arithmetic is per-cell and ordered (metrics, numbering,
operator coefficients, projection, pressure update, divergence, multigrid
transfers); within stated tolerances where a reduction or an iterative solve
is involved:
  * right-hand side: |b_gpu - b_oracle| <= 1e-12 max|b| (the mean-removal
    sum is reduced in a different order);
  * y = A x: relative max error <= 1e-13 (summation order of 19 products);
  * solve: true FP64 relative residual <= 1e-8 and phi within 1e-6
    relative L2 of the exact sparse solve (both with the fluid mean removed).
"""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF

pytestmark = pytest.mark.gpu


def _cases():
    c1 = CF.channel(12, 10, 12)
    c2 = CF.cylinder(24, 16, 24)
    c3 = CF.towers(32, 24, 32, radius=0.08)
    # explicit-copy periodic flags in i and j, and fractional IB values that
    # make identity rows (nvert in (0.1, 1) keeps a dof, poisson.c:1158)
    c4 = CF.cylinder(16, 12, 16, seed=7)
    c4.nvert = np.where(c4.nvert == 1.0, 0.5, c4.nvert)
    c4.set_periodic((1, 1, 0, 0, 0, 0))
    c4.name = "cylinder_ijper_frac"
    return [c1, c2, c3, c4]


CASES = _cases()


@pytest.fixture(scope="module", params=CASES, ids=[c.name for c in CASES])
def pair(request, cuda_lib):
    import vfs_poisson as V
    case = request.param
    s = V.PoissonSolver.from_case(case)
    d = O.dims_of(case)
    met = O.form_metrics(d, case.coor)
    lhs = O.poisson_lhs(d, case.nvert, met)
    yield case, s, d, met, lhs
    s.close()


def test_metrics_bitexact(pair):
    case, s, d, met, lhs = pair
    for name in ["icsi", "ieta", "izet", "jcsi", "jeta", "jzet", "kcsi", "keta", "kzet", "iaj", "jaj", "kaj",
                 "aj", "cent", "csi", "eta", "zet"]:
        g = s.metric(name)
        np.testing.assert_array_equal(g, met[name], err_msg=name)


def test_numbering_exact(pair):
    case, s, d, met, lhs = pair
    n, gid = s.numbering()
    assert n == lhs["ndof"]
    np.testing.assert_array_equal(gid, lhs["gid"])


def test_operator_bitexact(pair):
    case, s, d, met, lhs = pair
    vol, rt = s.operator()
    np.testing.assert_array_equal(rt, lhs["rowtype"])
    np.testing.assert_array_equal(vol, lhs["vol"])


def test_rhs(pair):
    case, s, d, met, lhs = pair
    s.rhs(case.ucont, 0.5, 1.0, 1.5)
    b_o = O.to_da(d, lhs["gid"], O.rhs(d, case.nvert, lhs["gid"], case.ucont, met["aj"], 0.5, 1.0, 1.5))
    b_g = s.rhs_array()
    assert np.abs(b_g - b_o).max() <= 1e-12 * np.abs(b_o).max()
    # before the mean removal the per-cell values are bit-exact
    raw = O.to_da(d, lhs["gid"], O.rhs_raw(d, case.nvert, lhs["gid"], case.ucont, 0.5, 1.0, 1.5))
    fluid = case.nvert < 0.1
    shift = (b_g - raw)[1:-1, 1:-1, 1:-1][fluid[1:-1, 1:-1, 1:-1]]
    aj = met["aj"][1:-1, 1:-1, 1:-1][fluid[1:-1, 1:-1, 1:-1]]
    ratio = shift / aj
    assert np.ptp(ratio) <= 1e-12 * max(1.0, np.abs(ratio).max())


@pytest.mark.parametrize("poisson", [0, -1])
def test_rhs2(pair, poisson):
    """PoissonRHS2 (-poisson 0 / -1): unweighted mean removal, identity
    rows 0, aj row scaling for -1 (the solver then holds B / aj)."""
    case, s, d, met, lhs = pair
    s.rhs2(case.ucont, poisson, 0.5, 1.0, 1.5)
    b_o = O.to_da(d, lhs["gid"], O.rhs2(d, case.nvert, lhs["gid"], case.ucont, met["aj"], poisson, 0.5, 1.0, 1.5))
    fluid = case.nvert < 0.1
    if poisson == -1:
        b_o = np.where(fluid, b_o / met["aj"], b_o)
    b_g = s.rhs_array()
    assert np.abs(b_g - b_o).max() <= 1e-12 * np.abs(b_o).max()
    # zero-sum over the fluid entries for -poisson 0 (the unweighted removal)
    if poisson == 0:
        assert abs(b_g[fluid].sum()) <= 1e-10 * np.abs(b_g).sum()


def test_apply(pair):
    case, s, d, met, lhs = pair
    A = O.csr(lhs)
    rng = np.random.default_rng(3)
    x2 = rng.standard_normal(lhs["ndof"])
    x = O.convert_phi2_phi(d, case.nvert, x2)
    y = s.apply(x)
    y2 = O.from_da(d, lhs["gid"], y)
    ref = A @ x2
    assert np.abs(y2 - ref).max() <= 1e-13 * np.abs(ref).max()


def _exact(case, d, lhs, b2):
    import scipy.sparse.linalg as spla
    A = O.csr(lhs).tolil()
    A[0, :] = 0
    A[0, 0] = 1.0
    bp = b2.copy()
    bp[0] = 0.0
    xe = spla.spsolve(A.tocsr(), bp)
    return O.remove_nullspace(d, case.nvert, lhs["gid"], xe)


@pytest.mark.parametrize("orth", [0, 1], ids=["cgs", "dcgs2"])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp32mg", "fp64mg"])
def test_solve_matches_exact(pair, precision, orth):
    case, s, d, met, lhs = pair
    s.rhs(case.ucont)
    phi, st = s.solve(precision=precision, rtol=1e-8, orth=orth)
    assert st.status == 0 and st.rel_residual <= 1e-8, st.as_dict()
    b2 = O.rhs(d, case.nvert, lhs["gid"], case.ucont, met["aj"])
    A = O.csr(lhs)
    phi2 = O.from_da(d, lhs["gid"], phi)
    assert np.linalg.norm(b2 - A @ phi2) / np.linalg.norm(b2) <= 1.2e-8
    xe = _exact(case, d, lhs, b2)
    # phi agrees with the exact solve within 1e-6 relative L2 on fluid dofs
    fl = O.from_da(d, lhs["gid"], (case.nvert < 0.1).astype(np.float64)) > 0
    err = np.linalg.norm(phi2[fl] - xe[fl]) / np.linalg.norm(xe[fl])
    assert err <= 1e-6, err
    # Convert_Phi2_Phi layout: identical to the oracle's scatter of the same dofs
    np.testing.assert_array_equal(phi, O.convert_phi2_phi(d, case.nvert, phi2))


def test_projection_pressure_divergence_bitexact(pair):
    case, s, d, met, lhs = pair
    rng = np.random.default_rng(11)
    phi = O.convert_phi2_phi(d, case.nvert, rng.standard_normal(lhs["ndof"]))
    p0 = rng.standard_normal(phi.shape)
    p_o, phi_o = O.update_pressure(d, case.nvert, p0, phi)
    p_g, phi_g = p0.copy(), phi.copy()
    s.update_pressure(p_g, phi_g)
    np.testing.assert_array_equal(p_g, p_o)
    np.testing.assert_array_equal(phi_g, phi_o)
    u_o = O.projection(d, case.nvert, phi_o, met, case.ucont, 0.7, 1.0, 1.5)
    u_g = case.ucont.copy()
    s.projection(u_g, 0.7, 1.0, 1.5)
    np.testing.assert_array_equal(u_g, u_o)
    assert s.divergence(u_g) == O.divergence(d, case.nvert, u_o, met["aj"])


def test_mg_transfers_bitexact(pair):
    case, s, d, met, lhs = pair
    levels = s.mg_levels()
    assert len(levels) >= 2
    rng = np.random.default_rng(5)
    nv_f = case.nvert
    df = d
    for li in range(len(levels) - 1):
        nx, ny, nz, cx, cy, cz = levels[li]
        cnx, cny, cnz = levels[li + 1][:3]
        dc = O.dims(cnx + 2, cny + 2, cnz + 2, case.periodic)
        nv_c = O.nvert_restriction(df, dc, 1 - cx, 1 - cy, 1 - cz, nv_f)
        np.testing.assert_array_equal(s.mg_nvert(li + 1), nv_c)
        xf = np.zeros((nz + 2, ny + 2, nx + 2))
        xf[1:-1, 1:-1, 1:-1] = rng.standard_normal((nz, ny, nx))
        np.testing.assert_array_equal(s.mg_restrict(li, xf), O.restriction(dc, df, 1 - cx, 1 - cy, 1 - cz, nv_c, nv_f, xf))
        xc = np.zeros((cnz + 2, cny + 2, cnx + 2))
        xc[1:-1, 1:-1, 1:-1] = rng.standard_normal((cnz, cny, cnx))
        np.testing.assert_array_equal(s.mg_interpolate(li, xc),
                                      O.interpolation(df, dc, 1 - cx, 1 - cy, 1 - cz, nv_f, nv_c, xc))
        nv_f, df = nv_c, dc


@pytest.mark.parametrize("restart", [6, 20])
def test_orthogonalisation_variants(pair, restart):
    """One-pass classical Gram-Schmidt and DCGS2 reach the same tolerance in
    (nearly) the same iterations.  Line Jacobi with one sweep each way keeps
    a cycle past eight basis vectors (two dots launches per step)."""
    case, s, d, met, lhs = pair
    s.rhs(case.ucont)
    rtol = 1e-9 if restart == 6 else 1e-11
    res = {}
    for orth in (0, 1):
        phi, st = s.solve(rtol=rtol, orth=orth, restart=restart, smoother=0, nu1=1, nu2=1, max_it=400)
        assert st.status == 0 and st.rel_residual <= rtol, (orth, st.as_dict())
        res[orth] = (st.iterations, phi)
    print(case.name, restart, res[0][0], res[1][0])
    assert abs(res[0][0] - res[1][0]) <= max(1, res[1][0] // 10)
    fl = case.nvert < 0.1
    a, b = res[0][1][fl], res[1][1][fl]
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)


def _odd_case(name):
    if name == "channel_odd":  # odd nx and nz, both periodic (the wraps join same-parity columns)
        return CF.channel(13, 10, 11)
    if name == "channel_big":  # level 0 above 2^20 cells: two-kernel sweeps there, fused below
        return CF.channel(128, 96, 96)
    c = CF.cylinder(15, 12, 16, seed=9)  # odd nx, explicit-copy periodic i
    c.set_periodic((1, 0, 0, 0, 0, 0))
    c.name = "cylinder_odd_iper"
    return c


@pytest.mark.parametrize("name", ["channel_odd", "cylinder_odd", "channel_big"])
def test_fused_sweep_bitexact_odd(name, cuda_lib):
    """Smoother 4 (residual formed in the line kernel, x double-buffered)
    reproduces smoother 3 (residual kernel + in-place line kernel) bit for
    bit, on boxes whose periodic wraps put same-parity columns side by side
    and on a box whose finest level keeps the two-kernel sweep."""
    import vfs_poisson as V
    case = _odd_case(name)
    s = V.PoissonSolver.from_case(case)
    try:
        _fused_vs_unfused(case, s)
    finally:
        s.close()


def test_fused_sweep_bitexact(pair):
    case, s, d, met, lhs = pair
    _fused_vs_unfused(case, s)


def _fused_vs_unfused(case, s):
    s.rhs(case.ucont)
    for kw in ({}, {"nu1": 2, "nu2": 1, "omega": 0.9}):
        out = {}
        for sm in (3, 4):
            phi, st = s.solve(precision=0, rtol=1e-9, smoother=sm, **kw)
            assert st.status == 0, (sm, kw, st.as_dict())
            out[sm] = (st.iterations, phi)
        assert out[3][0] == out[4][0], kw
        np.testing.assert_array_equal(out[3][1], out[4][1])
    r = np.random.default_rng(3).standard_normal(phi.shape)
    z4 = s.mg_vcycle(r)  # the default smoother is 4
    assert np.isfinite(z4).all()


def test_warm_start_and_launch_count(pair):
    case, s, d, met, lhs = pair
    s.rhs(case.ucont)
    phi, st = s.solve(rtol=1e-10)
    n0 = s.kernel_launches()
    phi2, st2 = s.solve(phi=phi.copy(), warm_start=1, rtol=1e-10)
    assert st2.iterations <= 1
    assert s.kernel_launches() > n0


@pytest.mark.parametrize("flg", [0, 1, 2, 3])
def test_volume_flux(pair, flg):
    """VolumeFlux (immersed): per-face arithmetic of the reference; the
    three sums are reduced in another order, so the corrected fluxes agree
    to 1e-12 of the largest flux and the returned flux / area to 1e-10."""
    case, s, d, met, lhs = pair
    rng = np.random.default_rng(11 + flg)
    u0 = rng.uniform(-1, 1, case.ucont.shape)
    u_o, f_o, a_o = O.volume_flux(d, case.nvert, met, u0, flg=flg, flux_intp_sum=0.01)
    u_g = u0.copy()
    f_g, a_g = s.volume_flux(u_g, flg=flg, flux_intp_sum=0.01)
    assert np.abs(u_g - u_o).max() <= 1e-12 * np.abs(u0).max()
    assert abs(a_g - a_o) <= 1e-10 * max(abs(a_o), 1e-300)
    assert abs(f_g - f_o) <= 1e-10 * max(np.abs(u0).sum(), 1.0)


@pytest.mark.parametrize("zero_solid", [1, 0])
def test_contra2cart_bitexact(pair, zero_solid):
    case, s, d, met, lhs = pair
    rng = np.random.default_rng(5)
    ucat0 = rng.uniform(-1, 1, case.ucont.shape)
    u_o = O.contra2cart(d, case.nvert, met, case.ucont, ucat0, zero_solid=bool(zero_solid))
    u_g = s.contra2cart(case.ucont, ucat0.copy(), zero_solid=bool(zero_solid))
    np.testing.assert_array_equal(u_g, u_o)


def test_nullspace_scale_quotient_bitexact(cuda_lib):
    """Remove_Nullspace_Scale's per-cell quotient (-sum aj) / sum_aj is formed
    from a reciprocal with two Markstein corrections instead of a division;
    it must give the division's bits.  With integer fluxes and aj on a grid of
    1/256 (aj given as a metric of set_grid) every sum is exact in any order,
    so the right-hand side must equal the oracle's (plain division) bit for
    bit on every cell, across many numerators and two denominators."""
    import vfs_poisson as V
    for seed in (5, 6):
        case = CF.channel(32, 24, 32)
        rng = np.random.default_rng(seed)
        u = rng.integers(-40, 41, case.ucont.shape).astype(np.float64)
        aj = rng.integers(128, 512, case.nvert.shape) / 256.0
        d = O.dims_of(case)
        lhs = O.poisson_lhs(d, case.nvert, O.form_metrics(d, case.coor))
        s = V.PoissonSolver.from_case(case)
        try:
            s.set_grid(case.coor, [None] * 12 + [aj])
            s.set_nvert(case.nvert)
            s.rhs(u)
            b_lib = O.from_da(d, lhs["gid"], s.rhs_array())
        finally:
            s.close()
        b_ref = O.rhs(d, case.nvert, lhs["gid"], u, aj)
        np.testing.assert_array_equal(b_lib, b_ref)
