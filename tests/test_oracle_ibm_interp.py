"""The oracle's IB interpolation restatement on its own (no GPU): geometric
properties of the records (Source/ibm.c:373-508, nearestcell1 :1373,
InterceptionPoint :1766), the no-slip profile of ibm_interpolation_advanced
(:3301, wallfunction.c:140) and IB_BC's periodic and wall faces
(Source/momentum.c:2016-2220)."""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF


def _setup(tilted=False):
    if tilted:
        c = CF.cylinder(28, 20, 28)
        c.set_periodic((0, 0, 0, 0, 0, 0))
        surf = CF.rod_surface((0.3, 0.25, 0.35), (0.6, 0.5, 0.62), 0.55, 0.08, 20, 6)
    else:
        c = CF.cylinder(24, 16, 24)
        surf = CF.rod_surface((0.5, -0.01, 0.5), (0, 1, 0), 1.02, 0.1, 24, 8)
    d = O.dims_of(c)
    met = O.form_metrics(d, c.coor)
    marked, _ = O.ibm_mark(d, met["cent"], surf)
    nodes, n = O.ibm_nodes(d, met["cent"], marked, surf)
    nvert = O.ibm_finish(d, marked)
    return c, d, met, surf, marked, nodes, n, nvert


@pytest.mark.parametrize("tilted", [False, True])
def test_records_geometry(tilted):
    c, d, met, surf, marked, nodes, n, nvert = _setup(tilted)
    assert n == int(((marked[1:-1, 1:-1, 1:-1] + 0.5).astype(int) == 2).sum())
    xyz, tri = surf
    keys = []
    for q in range(n):
        r = nodes[q]
        keys.append((r.k, r.j, r.i))
        assert r.status in (0, 1) and r.cell >= 0 and r.d_s > 0
        assert abs(sum(r.cs) - 1) < 1e-12 and abs(sum(r.cr) - 1) < 1e-12
        # the nearest point is the weighted sum of the element's vertices
        v = xyz[tri[r.cell]]
        np.testing.assert_allclose(np.asarray(r.cs) @ v, np.asarray(r.pmin), atol=1e-12)
        assert abs(np.linalg.norm(met["cent"][r.k, r.j, r.i] - np.asarray(r.pmin)) - r.d_s) < 1e-12 * (1 + r.d_s)
        for s in range(3):  # the interception cells are neighbours of the node
            assert max(abs(r.ip[s] - r.i), abs(r.jp[s] - r.j), abs(r.kp[s] - r.k)) == 1
        if r.status == 0:
            assert 0 <= r.imode < 8 and r.d_i > 0
    assert keys == sorted(keys)  # the reference's k, j, i order


def test_noslip_profile():
    c, d, met, surf, marked, nodes, n, nvert = _setup()
    U = np.array([0.7, -0.2, 0.4])
    ucat = np.broadcast_to(U, nvert.shape + (3,)).copy()
    p = np.full(nvert.shape, 2.5)
    ucont = np.zeros(nvert.shape + (3,))
    u2, p2, _ = O.ibm_interpolate(d, nvert, nodes, n, surf, met, ucat, p, ucont)
    checked = 0
    for q in range(n):
        r = nodes[q]
        nb = sum(nvert[r.kp[s], r.jp[s], r.ip[s]] for s in range(3))
        assert abs(p2[r.k, r.j, r.i] - 2.5) < 1e-12
        if nb > 0.1:
            continue  # a blanked interception cell zeroes the node
        checked += 1
        # the node sits at d_s of d_s + d_i between the wall (0) and Uc = U
        np.testing.assert_allclose(u2[r.k, r.j, r.i], r.d_s / (r.d_s + r.d_i) * U, rtol=1e-12, atol=1e-14)
    assert checked > n // 2


def test_ib_bc_faces():
    c, d, met, surf, marked, nodes, n, nvert = _setup()
    rng = np.random.default_rng(3)
    ucat = rng.standard_normal(nvert.shape + (3,))
    ucont = rng.standard_normal(nvert.shape + (3,))
    u2, c2 = O.ib_bc(d, nvert, met, ucat, ucont, bctype=(0, 0, -1, -1, 0, 0))
    # i is periodic in this case: ucat ghosts and the i faces take partners
    np.testing.assert_array_equal(u2[:, :, 0], u2[:, :, -2])
    np.testing.assert_array_equal(c2[:, :, 0, 0], c2[:, :, -2, 0])
    np.testing.assert_array_equal(c2[:, :, -1, 0], c2[:, :, 1, 0])
    # the -1 walls in j close their faces
    assert np.all(c2[1:-1, 0, 1:-1, 1] == 0) and np.all(c2[1:-1, -2, 1:-1, 1] == 0)
    # an IB node's own x face is its averaged ucat dotted with icsi
    r = nodes[0]
    i, j, k = r.i, r.j, r.k
    if i + 1 < d.mx - 1:
        uc = (u2[k, j, i] + u2[k, j, i + 1]) * 0.5
        assert c2[k, j, i, 0] == uc[0] * met["icsi"][k, j, i, 0] + uc[1] * met["icsi"][k, j, i, 1] + \
            uc[2] * met["icsi"][k, j, i, 2]
