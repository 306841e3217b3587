"""The reach of a mask change in the operator (CPU, the oracle's PoissonLHSNew).

The incremental refill of a new mask (vfs_poisson_set_nvert on a filled
hierarchy) re-assembles only the rows within two points of a changed nvert
value, a periodic axis wrapping.  That rests on a row reading nvert within
one point of its own: the one-sided differences next to blanked cells and the
neighbours' dof tests, where a periodic ghost neighbour's test reads its
interior partner.  Here single cells change between fluid and solid, at the
periodic seams, next to a body and inside the domain, and every row whose
coefficients, type or column pattern changes must lie within one point of the
changed cell, in both assemblies the library keeps (the FGMRES operator,
unscaled with the reference's insertion filter, and the aj-scaled multigrid
operator without it).
"""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF


@pytest.fixture(scope="module")
def setup():
    case = CF.towers(12, 10, 12, radius=0.12, array=(2, 1))
    d = O.dims_of(case)
    met = O.form_metrics(d, case.coor)
    return case, d, met


def _rows(d, nv, met, scaled):
    lhs = O.poisson_lhs(d, nv, met, scale_by_aj=scaled, apply_filter=not scaled)
    return lhs["rowtype"], lhs["vol"], lhs["col"] >= 0


def _pdist(a, b, m, periodic):
    dd = abs(a - b)
    return min(dd, (m - 2) - dd) if periodic else dd


@pytest.mark.parametrize("scaled", [False, True], ids=["fgmres", "multigrid"])
def test_row_reach_of_a_mask_change(setup, scaled):
    case, d, met = setup
    nv0 = CF.sync_periodic_ghosts(case.nvert.copy(), case.periodic)
    px, pz = bool(case.periodic[0] or case.periodic[3]), bool(case.periodic[2] or case.periodic[5])
    rt0, vol0, has0 = _rows(d, nv0, met, scaled)
    rng = np.random.default_rng(7)
    cells = [(1, 5, 6), (d.mx - 2, 5, 6), (6, 5, 1), (6, 5, d.mz - 2), (1, 1, 1), (d.mx - 2, d.my - 2, d.mz - 2),
             (6, 5, 6)]
    solid = np.argwhere(nv0[1:-1, 1:-1, 1:-1] > 0.1)
    for q in solid[rng.choice(len(solid), 3, replace=False)]:
        cells.append((int(q[2]) + 1, int(q[1]) + 1, int(q[0]) + 1))
    for _ in range(4):
        cells.append(tuple(int(rng.integers(1, m - 1)) for m in (d.mx, d.my, d.mz)))
    reach = 0
    for (i0, j0, k0) in cells:
        nv = nv0.copy()
        nv[k0, j0, i0] = 0.0 if nv0[k0, j0, i0] > 0.1 else 3.0
        nv = CF.sync_periodic_ghosts(nv, case.periodic)
        rt, vol, has = _rows(d, nv, met, scaled)
        changed = (rt != rt0) | np.any(vol != vol0, axis=-1) | np.any(has != has0, axis=-1)
        for k, j, i in np.argwhere(changed):
            if not (0 < i < d.mx - 1 and 0 < j < d.my - 1 and 0 < k < d.mz - 1):
                continue  # ghost points carry no row
            dist = max(_pdist(i, i0, d.mx, px), abs(int(j) - j0), _pdist(k, k0, d.mz, pz))
            reach = max(reach, dist)
            assert dist <= 1, ((i0, j0, k0), (i, j, k))
    assert reach == 1  # the neighbours of a changed cell do change
