"""The drop-in adapter's DA bridge on the GPU (marked gpu).

A block's fields live in PETSc DA vectors (the single-rank PETSc stand-in of
oracle/refshim/, with the reference's periodic ghost layout).  The bridge
(vfs-wind_gb300/adapter/vfs_da_bridge.cpp) gathers them, drives the library
and scatters the results back; the same steps through the library on
natural arrays must give bit-identical fields: VolumeFlux (both overloads),
the right-hand side and solve (warm start from the DA's phi), UpdatePressure,
Projection and the Divergence maximum.  This is the sequence the UserCtx
adapter runs for PoissonSolver_Hypre, UpdatePressure, Projection and
Divergence (Source/solvers.c:647-690).
"""
import ctypes as C

import numpy as np
import pytest

import adapter_build
from vfs_poisson import configs as CF

pytestmark = pytest.mark.gpu


def _cases():
    c = CF.cylinder(24, 16, 24, seed=9)
    c.set_periodic((0, 0, 0, 1, 0, 1))
    return {"towers_ii_kk": CF.towers(32, 24, 32, radius=0.08), "cylinder_ii_kk": c,
            "channel_ii_kk": CF.channel(16, 12, 16)}


CASES = _cases()


@pytest.mark.parametrize("immersed", [0, 1])
@pytest.mark.parametrize("name", list(CASES))
def test_bridge_matches_library(cuda_lib, name, immersed):
    import vfs_poisson as V
    H = adapter_build.harness()
    case = CASES[name]
    mx, my, mz = case.dims
    per = case.periodic
    da = H.ah_da_create(mx, my, mz, per[3], per[4], per[5], 1)
    fda = H.ah_coordinate_da(da)
    coords = H.ah_coordinates(da)
    H.ah_fill(fda, coords, np.ascontiguousarray(case.coor).ctypes.data, 3)
    vecs = {k: H.ah_global(fda if k == "ucont" else da) for k in ("nvert", "ucont", "phi", "p")}
    rng = np.random.default_rng(3)
    p0 = rng.standard_normal(case.nvert.shape)
    H.ah_fill(da, vecs["nvert"], np.ascontiguousarray(case.nvert).ctypes.data, 1)
    H.ah_fill(fda, vecs["ucont"], np.ascontiguousarray(case.ucont).ctypes.data, 3)
    H.ah_fill(da, vecs["phi"], np.zeros(case.nvert.shape).ctypes.data, 1)
    H.ah_fill(da, vecs["p"], p0.ctypes.data, 1)
    desc = V.GridDesc(mx, my, mz, *[int(p) for p in per], 0)
    b = C.c_void_p()
    assert H.vfsa_create(da, fda, C.byref(desc), C.byref(b)) == 0
    try:
        assert H.vfsa_set_grid(b, coords) == 0
        assert H.vfsa_set_nvert(b, vecs["nvert"]) == 0
        f, a = C.c_double(), C.c_double()
        assert H.vfsa_volume_flux(b, vecs["ucont"], immersed, C.byref(f), C.byref(a)) == 0
        opts = V.default_opts(rtol=1e-8, warm_start=1)
        st = V.SolveStats()
        assert H.vfsa_solve(b, vecs["ucont"], 1.0, 1.0, 1.0, vecs["phi"], C.byref(opts), C.byref(st)) == 0
        assert H.vfsa_update_pressure(b, vecs["p"], vecs["phi"]) == 0
        assert H.vfsa_projection(b, vecs["ucont"], 1.0, 1.0, 1.0) == 0
        md = C.c_double()
        assert H.vfsa_divergence(b, vecs["ucont"], C.byref(md)) == 0

        def read(k, dof):
            out = np.zeros(case.nvert.shape + ((3,) if dof == 3 else ()))
            H.ah_read(fda if dof == 3 else da, vecs[k], out.ctypes.data, dof)
            return out

        s = V.PoissonSolver.from_case(case)
        try:
            u = case.ucont.copy()
            f2, a2 = s.volume_flux(u, 0) if immersed == 1 else s.volume_flux0(u, immersed)
            assert (f.value, a.value) == (f2, a2)
            s.rhs(u)
            phi = np.zeros(case.nvert.shape)
            phi, st2 = s.solve(phi, opts=opts)
            assert st.iterations == st2.iterations and st.rel_residual == st2.rel_residual
            p = p0.copy()
            s.update_pressure(p, phi)
            s.projection(u)
            np.testing.assert_array_equal(read("phi", 1), phi)
            np.testing.assert_array_equal(read("p", 1), p)
            np.testing.assert_array_equal(read("ucont", 3), u)
            assert md.value == s.divergence(u)
        finally:
            s.close()
    finally:
        H.vfsa_destroy(b)
        for v in vecs.values():
            H.ah_vec_destroy(v)
