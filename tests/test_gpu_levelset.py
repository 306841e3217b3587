"""The level-set (two-phase) variant of the operator and the projection vs
the oracle (marked gpu): face coefficients divided by the harmonic mean of
the two cells' densities, the zero-Dirichlet top faces (bctype[3] / [5] ==
4), the bctype[4] == 5000 bottom and the skipped null-space removals
(Source/poisson.c:1171-1561, :2738-2956; poisson_hypre.c:375, :604)."""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF

pytestmark = pytest.mark.gpu

VARIANTS = {
    "density": (0, 0, 0, 0, 0, 0),
    "dirichlet_j": (0, 0, 0, 4, 0, 0),
    "dirichlet_k": (0, 0, 0, 0, 0, 4),
    "bottom5000": (0, 0, 0, 0, 5000, 0),
}


def _case(name):
    c = CF.cylinder(24, 16, 24, seed=21)
    if name == "dirichlet_k" or name == "bottom5000":
        c.set_periodic((0, 0, 0, 1, 0, 0))  # k stays non-periodic (it already is)
    cc = np.zeros(c.nvert.shape + (3,))
    cc[1:-1, 1:-1, 1:-1] = CF.cell_centres(c.coor)
    # wavy water/air interface: level < 0 under it
    level = cc[..., 1] - (0.45 + 0.05 * np.sin(2 * np.pi * cc[..., 0]) * np.cos(2 * np.pi * cc[..., 2]))
    if name == "bottom5000":
        level = cc[..., 2] - 0.5 + 0.0 * level  # the bottom k face sees both signs
    rho = np.where(level < 0, 1000.0, 1.2)
    return c, rho, level


@pytest.fixture(scope="module", params=list(VARIANTS), ids=list(VARIANTS))
def lspair(request, cuda_lib):
    import vfs_poisson as V
    name = request.param
    bc = VARIANTS[name]
    c, rho, level = _case(name)
    s = V.PoissonSolver(*c.dims, periodic=c.periodic)
    s.set_grid(c.coor)
    s.set_levelset(rho, level, bc)
    s.set_nvert(c.nvert)
    d = O.dims_of(c)
    met = O.form_metrics(d, c.coor)
    O.set_levelset(rho, level, bc)
    lhs = O.poisson_lhs(d, c.nvert, met)
    yield name, c, s, d, met, lhs, rho, level, bc
    O.set_levelset(None)
    s.close()


def test_operator_bitexact(lspair):
    name, c, s, d, met, lhs, rho, level, bc = lspair
    O.set_levelset(rho, level, bc)
    vol, rt = s.operator()
    np.testing.assert_array_equal(vol, lhs["vol"])
    if name.startswith("dirichlet"):
        # the Dirichlet rows break the constant null space
        A = O.csr(lhs)
        assert np.abs(A @ np.ones(A.shape[1])).max() > 1e-6


def test_projection_bitexact(lspair):
    name, c, s, d, met, lhs, rho, level, bc = lspair
    O.set_levelset(rho, level, bc)
    rng = np.random.default_rng(4)
    phi2 = rng.standard_normal(lhs["ndof"])
    phi = O.convert_phi2_phi(d, c.nvert, phi2)
    u_o = O.projection(d, c.nvert, phi, met, c.ucont, 0.5, 1.0, 1.5)
    u_g = c.ucont.copy()
    p = np.zeros(c.nvert.shape)
    s.update_pressure(p, phi.copy())
    s.projection(u_g, 0.5, 1.0, 1.5)
    np.testing.assert_array_equal(u_g, u_o)


def test_solve(lspair):
    name, c, s, d, met, lhs, rho, level, bc = lspair
    O.set_levelset(rho, level, bc)
    s.rhs(c.ucont)
    b_g = O.from_da(d, lhs["gid"], s.rhs_array())
    if bc[5] == 4:
        # no null-space removal of the right-hand side (poisson_hypre.c:375)
        np.testing.assert_array_equal(b_g, O.rhs_raw(d, c.nvert, lhs["gid"], c.ucont))
    phi, st = s.solve(precision=0, rtol=1e-8, max_it=100)
    assert st.rel_residual <= 1e-8, st.as_dict()
    A = O.csr(lhs)
    phi2 = O.from_da(d, lhs["gid"], phi)
    r = b_g - A @ phi2
    if bc[5] != 4:
        # the reference removes the fluid mean of phi unless bctype[5] == 4
        # (poisson_hypre.c:604-608), also when a Dirichlet face makes the
        # system regular: the returned phi is the solution shifted by a
        # constant, so the residual lies along A 1
        fl = O.from_da(d, lhs["gid"], (c.nvert < 0.1).astype(np.float64))
        a1 = A @ fl
        if np.linalg.norm(a1) > 0:
            r = r - (r @ a1) / (a1 @ a1) * a1
    assert np.linalg.norm(r) / np.linalg.norm(b_g) <= 1.2e-8


def test_disable_requires_new_operator(cuda_lib):
    """Turning level-set mode off invalidates the density-weighted operator:
    the next right-hand side without a new set_nvert is refused, and after
    set_nvert the operator is the plain one again."""
    import vfs_poisson as V
    c, rho, level = _case("density")
    s = V.PoissonSolver(*c.dims, periodic=c.periodic)
    try:
        s.set_grid(c.coor)
        s.set_levelset(rho, level, VARIANTS["density"])
        s.set_nvert(c.nvert)
        s.rhs(c.ucont)
        s.set_levelset(None, enable=False)
        with pytest.raises(V.VfsError) as e:
            s.rhs(c.ucont)
        assert e.value.code == V.VFS_ESTATE
        s.set_nvert(c.nvert)
        d = O.dims_of(c)
        met = O.form_metrics(d, c.coor)
        O.set_levelset(None)
        lhs = O.poisson_lhs(d, c.nvert, met)
        vol, _ = s.operator()
        np.testing.assert_array_equal(vol, lhs["vol"])
    finally:
        s.close()
