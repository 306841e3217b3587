"""Regenerate the golden fixtures in this directory from the reference itself.

Each fixture holds a small seeded grid (node coordinates, nvert, Ucont, a
pressure field) and the outputs of the reference's own functions on it:
Source/metrics.c, poisson.c, poisson_hypre.c, main.c and rhs.c compiled
unmodified against the single-rank PETSc/HYPRE/MPI stand-in of
oracle/refshim/ (oracle/reference.py).  Recorded per case:

  * FormMetrics: the 17 metric arrays (owned points of the ghosted copies);
  * setup_lidx2 / PoissonLHSNew: the dof numbering Gid and the assembled
    matrix (CSR, dof order);
  * PoissonRHS2 for -poisson 0 and -1;
  * PoissonSolver_Hypre: the right-hand side it hands to HYPRE
    (PoissonRHS2_hypre + Remove_Nullspace_Scale), the inner solution `x`
    (an exact FP64 solve standing in for HYPRE GMRES + BoomerAMG, which the
    reference does not ship) and what the reference makes of it:
    Remove_Nullspace -> Phi2, Convert_Phi2_Phi -> Phi;
  * UpdatePressure of a seeded P, Projection of Ucont with that Phi, and the
    Divergence maximum after it;
  * VolumeFlux, the immersed variant (flg 0) and the immersed == 0 variant,
    on the input Ucont;
  * FullyBlocked (the first blocked k of every column and the multiple
    null space flag) and PoissonNullSpaceFunction_original of a seeded
    array (the -poisson -1 path's null-space removal).

The CPU tests check the oracle's restatement against these, the GPU tests
check the CUDA library against them.  Needs the reference sources (the
library is built from them in place):

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "oracle"), os.path.join(REPO, "vfs-wind_gb300")]

import reference as R  # noqa: E402
from vfs_poisson import configs as CF  # noqa: E402


def cases():
    """The fixture grids: a periodic channel, the curvilinear cylinder, two
    towers with both periodic DA directions, and a cylinder with the
    explicit-copy i/j periodic flags and fractional IB values (nvert 0.5:
    dofs with identity rows), and a channel cut by a solid k-slab (every
    column blocked: the multiple null space of FullyBlocked)."""
    c4 = CF.cylinder(10, 8, 10, seed=7)
    c4.nvert = np.where(c4.nvert == 1.0, 0.5, c4.nvert)
    c4.set_periodic((1, 1, 0, 0, 0, 0))
    c4.name = "cylinder_ijper_frac"
    c5 = CF.channel(8, 8, 8)
    nv = c5.nvert.copy()
    nv[5] = 1.0
    c5.nvert = CF.sync_periodic_ghosts(nv, c5.periodic)
    c5.ucont = CF._mask_faces(c5.ucont, c5.nvert)
    c5.name = "channel_slab"
    return {
        "channel_8": CF.channel(8, 8, 8),
        "cylinder_12": CF.cylinder(12, 8, 12),
        "towers_10": CF.towers(10, 8, 10, radius=0.12, array=(2, 1)),
        "cylinder_ijper_frac_10": c4,
        "channel_slab_8": c5,
    }


def pinned_solve(A, b, x0=None, rtol=0.0):
    """Exact FP64 solve of the singular system: one row of every connected
    component of the matrix graph pinned to zero."""
    import scipy.sparse as sp
    import scipy.sparse.csgraph as cg
    import scipy.sparse.linalg as spla
    n = A.shape[0]
    ncomp, lab = cg.connected_components(A + A.T, directed=False)
    first = np.full(ncomp, -1)
    for i in range(n):
        if first[lab[i]] < 0:
            first[lab[i]] = i
    A = A.tolil(copy=True)
    bp = b.copy()
    for r in first:
        A.rows[r] = [r]
        A.data[r] = [1.0]
        bp[r] = 0.0
    return spla.spsolve(sp.csr_matrix(A), bp)


def reference_outputs(case, seed):
    """The reference's outputs on `case` (a dict of arrays, the fixture)."""
    rng = np.random.default_rng(seed)
    p0 = rng.standard_normal(case.nvert.shape)
    out = {"coor": case.coor, "nvert": case.nvert, "ucont": case.ucont, "p0": p0,
           "periodic": np.asarray(case.periodic, np.int32)}
    # VolumeFlux variants on the input Ucont, each on a block of its own
    for variant, key in ((True, "vflux_ib"), (False, "vflux_0")):
        B = R.Block(case, immersed=1 if variant else 0)
        B.form_metrics()
        B.set("nvert", case.nvert)
        B.set("nvert_o", case.nvert)
        B.set("ucont", case.ucont)
        f, a = B.volume_flux(variant, 0)
        out[key] = np.array([f, a])
        out[key + "_ucont"] = B.get("ucont", 3)
        B.close()
    B = R.Block(case)
    B.form_metrics()
    for f in ("csi", "eta", "zet", "icsi", "ieta", "izet", "jcsi", "jeta", "jzet", "kcsi", "keta", "kzet", "cent"):
        out[f] = B.get(f, 3)
    for f in ("aj", "iaj", "jaj", "kaj"):
        out[f] = B.get(f)
    B.set("nvert", case.nvert)
    B.set("nvert_o", case.nvert)
    B.set("ucont", case.ucont)
    n, rp, cols, vals = B.lhs()
    out.update(gid=B.get("gid"), A_rowptr=rp, A_cols=cols, A_vals=vals)
    out["rhs2_0"] = B.rhs2(0)
    out["rhs2_m1"] = B.rhs2(-1)
    solved = {}

    def solve(A, b, x0, rtol):
        solved["x"] = pinned_solve(A, b)
        return solved["x"]

    b, phi2, _ = B.solver_hypre(solve, 1e-8)
    out.update(b_hypre=b, x_solver=solved["x"], phi2=phi2, phi=B.get("phi"))
    B.set("p", p0)
    B.update_pressure()
    out["p"] = B.get("p")
    B.projection()
    out["ucont_proj"] = B.get("ucont", 3)
    out["maxdiv_proj"] = np.array([B.divergence()])
    multi, ksk = B.fully_blocked()
    out["multinull"] = np.array([int(multi)], np.int32)
    out["ksk"] = ksk
    out["ns_x"] = rng.standard_normal(case.nvert.shape)
    out["ns_out"] = B.nullspace_original(out["ns_x"])
    B.close()
    return out


def make(name, case):
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **reference_outputs(case, sum(name.encode())))


if __name__ == "__main__":
    if R.build() is None:
        sys.exit("the reference sources are not available: cannot regenerate the fixtures")
    for name, case in cases().items():
        make(name, case)
        print("written", name)
