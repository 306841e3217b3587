"""IB velocity reconstruction on the GPU vs the oracle (marked gpu).

vfs_poisson_ibm_search_nodes builds the interpolation records of the IB
nodes (ibm_search_advanced, Source/ibm.c:373-508: nearestcell1 :1373-1518,
InterceptionPoint :1766-2258), vfs_poisson_ibm_interpolate applies them
(ibm_interpolation_advanced :3301-3640 with noslip, wallfunction.c:140) and
vfs_poisson_ib_bc restates IB_BC (Source/momentum.c:2016-2220).  Records,
velocities, pressures and fluxes must be bit-identical to the oracle's.
"""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF

pytestmark = pytest.mark.gpu

FIELDS = ["i", "j", "k", "cell", "d_s", "d_i", "imode", "status"]
ARRAYS = ["pmin", "cs", "ip", "jp", "kp", "cr"]


def _records(arr, n):
    out = []
    for q in range(n):
        r = arr[q]
        out.append(tuple(getattr(r, f) for f in FIELDS) + tuple(tuple(getattr(r, a)) for a in ARRAYS))
    return out


def _case(name):
    if name == "cylinder":
        c = CF.cylinder(24, 16, 24)
        surfs = [CF.rod_surface((0.5, -0.01, 0.5), (0, 1, 0), 1.02, 0.1, 24, 8)]
        bc = None
    elif name == "towers":
        c = CF.towers(40, 24, 40, radius=0.05)
        surfs = CF.tower_surfaces(radius=0.05, height=0.6)[:3]
        bc = (0, 0, -1, 0, 0, 0)
    else:  # a tilted rod off every axis, in a box without periodic directions
        c = CF.cylinder(28, 20, 28)
        c.set_periodic((0, 0, 0, 0, 0, 0))
        surfs = [CF.rod_surface((0.3, 0.25, 0.35), (0.6, 0.5, 0.62), 0.55, 0.08, 20, 6)]
        bc = (0, 0, 0, 0, 0, 0)
    return c, surfs, bc


@pytest.fixture(scope="module", params=["cylinder", "towers", "tilted"])
def searched(request, cuda_lib):
    import vfs_poisson as V
    c, surfs, bc = _case(request.param)
    d = O.dims_of(c)
    met = O.form_metrics(d, c.coor)
    s = V.PoissonSolver(*c.dims, periodic=c.periodic)
    s.set_grid(c.coor)
    shape = (d.mz, d.my, d.mx)
    g, o = np.zeros(shape), np.zeros(shape)
    per_body = []
    bcv = bc if bc is not None else (0,) * 6
    for ibi, surf in enumerate(surfs):
        g, fg, ng = s.ibm_search_nodes(surf, nvert=g, ibi=ibi, bctype=bc)
        marked, fo = O.ibm_mark(d, met["cent"], surf, nvert=o, ibi=ibi)
        nodes, no = O.ibm_nodes(d, met["cent"], marked, surf)
        o = O.ibm_finish(d, marked, bcv)
        per_body.append((fg, fo, ng, no, nodes))
    s.set_nvert(g)
    yield request.param, c, d, met, s, surfs, bc, g, o, per_body
    s.close()


def test_search_nodes_nvert_and_counts(searched):
    name, c, d, met, s, surfs, bc, g, o, per_body = searched
    np.testing.assert_array_equal(g, o)
    for ibi, (fg, fo, ng, no, _) in enumerate(per_body):
        assert fg == fo
        assert ng == no and ng > 0


def test_node_records_bitexact(searched):
    name, c, d, met, s, surfs, bc, g, o, per_body = searched
    for ibi, (_, _, ng, no, nodes) in enumerate(per_body):
        arr, n = s.ibm_nodes(ibi)
        assert n == no
        got, want = _records(arr, n), _records(nodes, no)
        bad = [q for q in range(n) if got[q] != want[q]]
        assert not bad, (ibi, got[bad[0]], want[bad[0]])
        st = [r.status for r in nodes[:no]]
        assert st.count(0) > 0.8 * no  # most nodes find their interception


def test_interpolate_bitexact(searched):
    name, c, d, met, s, surfs, bc, g, o, per_body = searched
    rng = np.random.default_rng(11)
    shape = (d.mz, d.my, d.mx)
    ucat = rng.standard_normal(shape + (3,))
    p = rng.standard_normal(shape)
    ucont = rng.standard_normal(shape + (3,))
    bcv = bc if bc is not None else (0,) * 6
    for ibi, (_, _, _, no, nodes) in enumerate(per_body):
        xyz = surfs[ibi][0]
        u_surf = rng.standard_normal(xyz.shape) if ibi % 2 == 0 else None
        for immersed in (1, 3):
            u_o, p_o, c_o = O.ibm_interpolate(d, o, nodes, no, surfs[ibi], met, ucat, p, ucont, u_surf=u_surf,
                                              bctype=bcv, immersed=immersed)
            u_g, p_g, c_g = ucat.copy(), p.copy(), ucont.copy()
            s.ibm_interpolate(u_g, p_g, c_g, ibi=ibi, u_surf=u_surf, immersed=immersed, bctype=bc)
            np.testing.assert_array_equal(p_g, p_o)
            np.testing.assert_array_equal(c_g, c_o)
            np.testing.assert_array_equal(u_g, u_o)
            assert (p_g != p).sum() == no


@pytest.mark.parametrize("bctype", [(0, 0, 0, 0, 0, 0), (-1, -2, -1, -2, 0, 0), (10, 10, 10, 10, 10, 10)])
def test_ib_bc_bitexact(searched, bctype):
    name, c, d, met, s, surfs, bc, g, o, per_body = searched
    rng = np.random.default_rng(12)
    shape = (d.mz, d.my, d.mx)
    ucat = rng.standard_normal(shape + (3,))
    ucont = rng.standard_normal(shape + (3,))
    for immersed in (1, 3):
        u_o, c_o = O.ib_bc(d, o, met, ucat, ucont, bctype=bctype, immersed=immersed)
        u_g, c_g = ucat.copy(), ucont.copy()
        s.ib_bc(u_g, c_g, immersed=immersed, bctype=bctype)
        np.testing.assert_array_equal(u_g, u_o)
        np.testing.assert_array_equal(c_g, c_o)
