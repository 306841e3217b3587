"""Immersed-boundary classification on the GPU vs the oracle (marked gpu).

vfs_poisson_ibm_search restates ibm_search_advanced (Source/ibm.c:92-594)
with the reference's ray directions, intersection test and dilation; the
result must be bit-identical to the oracle's, including the number of cells
whose rays all met a doubled intersection.
"""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF

pytestmark = pytest.mark.gpu


def _run_both(case, surfaces, nvert0=None, bctype=None):
    import vfs_poisson as V
    d = O.dims_of(case)
    met = O.form_metrics(d, case.coor)
    s = V.PoissonSolver(*case.dims, periodic=case.periodic)
    s.set_grid(case.coor)
    shape = (d.mz, d.my, d.mx)
    g = np.zeros(shape) if nvert0 is None else nvert0.copy()
    o = g.copy()
    bc = bctype if bctype is not None else (0,) * 6
    fails = []
    for ibi, surf in enumerate(surfaces):
        g, fg = s.ibm_search(surf, nvert=g, ibi=ibi, bctype=bctype)
        o, fo = O.ibm_search(d, met["cent"], surf, nvert=o, ibi=ibi, bctype=bc)
        fails.append((fg, fo))
    s.close()
    return g, o, fails


def _assert_same(g, o, fails):
    for fg, fo in fails:
        assert fg == fo
    np.testing.assert_array_equal(g, o)


def test_cylinder_body(cuda_lib):
    c = CF.cylinder(24, 16, 24)
    surf = CF.rod_surface((0.5, -0.01, 0.5), (0, 1, 0), 1.02, 0.1, 24, 8)
    g, o, fails = _run_both(c, [surf])
    _assert_same(g, o, fails)
    assert (g == 3).sum() > 0


def test_tower_array_with_walls(cuda_lib):
    c = CF.towers(40, 24, 40, radius=0.05)
    nv0 = np.zeros((c.nz + 2, c.ny + 2, c.nx + 2))
    nv0[4, 6, 8] = 6.0      # kept by the first body's reset (>= 5)
    nv0[7, 3, 2] = 2.5      # cleared by it
    surfs = CF.tower_surfaces(radius=0.05, height=0.6)
    g, o, fails = _run_both(c, surfs, nvert0=nv0, bctype=(0, 0, -1, 0, 0, -2))
    _assert_same(g, o, fails)
    assert g[4, 6, 8] == 6.0


@pytest.mark.parametrize("angle", [0.0, 7.0, 33.0])
def test_rotor_rods(cuda_lib, angle):
    c = CF.rotor(32, 24, 32)
    g, o, fails = _run_both(c, CF.rotor_surfaces(angle_deg=angle))
    _assert_same(g, o, fails)


@pytest.mark.parametrize("kind", ["towers", "rotor"])
def test_later_bodies_on_odd_grids(cuda_lib, kind):
    """Bodies after the first search only the index box of their hash box,
    found through bounds of the cell centres over 8x8x8 blocks: grids whose
    sizes are no multiple of 8 end in partial blocks."""
    if kind == "towers":
        c = CF.towers(37, 21, 43, radius=0.05)
        surfs = CF.tower_surfaces(radius=0.05, height=0.6)
    else:
        c = CF.rotor(29, 19, 35)
        surfs = CF.rotor_surfaces(angle_deg=21.0)
    g, o, fails = _run_both(c, surfs)
    _assert_same(g, o, fails)
    assert (g == 3).sum() > 0


@pytest.mark.parametrize("which", ["side", "cap"])
def test_duplicated_triangles_give_up(cuda_lib, which):
    # a surface with repeated triangles: every ray through them meets a
    # doubled intersection, all 64 directions give up, and the cell is
    # counted and left at 0 (then dilated like any other)
    c = CF.channel(24, 20, 24)
    if which == "side":
        xyz, tri = CF.rod_surface((0.5, 0.2, 0.5), (0, 1, 0), 0.6, 0.2, 8, 4)
        tri = np.concatenate([tri, tri[[0, 1, 5, 9]]])
    else:
        xyz, tri = CF.rod_surface((0.5, 0.5, 0.3), (0, 0, 1), 0.4, 0.15, 12, 3)
        tri = np.concatenate([tri, tri[-24:]])
    g, o, fails = _run_both(c, [(xyz, tri)])
    _assert_same(g, o, fails)
    assert fails[0][0] > 0


def test_device_arrays(cuda_lib):
    import torch
    import vfs_poisson as V
    c = CF.cylinder(24, 16, 24)
    surf = CF.rod_surface((0.5, -0.01, 0.5), (0, 1, 0), 1.02, 0.1, 24, 8)
    s = V.PoissonSolver(*c.dims, periodic=c.periodic)
    s.set_grid(c.coor)
    host, _ = s.ibm_search(surf)
    dev = torch.zeros(host.shape, dtype=torch.float64, device="cuda")
    s.ibm_search(surf, nvert=dev)
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    # the classified blanking drives the solver like a generated one
    s.set_nvert(host)
    n, gid = s.numbering()
    d = O.dims_of(c)
    lhs = O.poisson_lhs(d, host, O.form_metrics(d, c.coor))
    assert n == lhs["ndof"]
    np.testing.assert_array_equal(gid, lhs["gid"])
    s.close()


def test_surface_from_ucd_file(cuda_lib, tmp_path):
    """A UCD surface file read by the library's reader and classified on the
    GPU equals the oracle's classification of the same surface; a restart
    field written and read back as a PETSc binary vector gives the same
    right-hand side."""
    import vfs_poisson as V
    c = CF.cylinder(24, 16, 24)
    xyz, tri = CF.rod_surface((0.5, -0.01, 0.5), (0, 1, 0), 1.02, 0.1, 24, 8)
    p = tmp_path / "ibmdata00"
    with open(p, "w") as f:
        f.write("#\n#\n#\n%d %d 0 0 0\n" % (len(xyz), len(tri)))
        for q, v in enumerate(xyz):
            f.write("%d %.17e %.17e %.17e\n" % (q + 1, *v))
        for e, t in enumerate(tri):
            f.write("%d 0 tri %d %d %d\n" % (e + 1, t[0] + 1, t[1] + 1, t[2] + 1))
    surf = V.read_ucd(str(p))
    g, o, fails = _run_both(c, [surf])
    _assert_same(g, o, fails)
    s = V.PoissonSolver.from_case(c)
    vf = tmp_path / "vfield000000_0.dat"
    V.write_petsc_vec(str(vf), c.ucont)
    u = V.read_petsc_vec(str(vf)).reshape(c.ucont.shape)
    s.rhs(c.ucont)
    b1 = s.rhs_array()
    s.rhs(u)
    np.testing.assert_array_equal(s.rhs_array(), b1)
    s.close()
