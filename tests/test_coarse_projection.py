"""The algebra of the coarsest-level solve, modelled in numpy (CPU): for a
singular system with zero row sums (one null vector per connected
component), pinning one row per component, inverting, and projecting the
right-hand side with the component's left null vector
w^T = e_r0^T I - m_r0^T I gives a solution of the projected system that is
zero at the pinned cell, whatever the right-hand side's inconsistency."""
import numpy as np
import pytest


def _component(rng, nd):
    M = -np.abs(rng.random((nd, nd))) * (rng.random((nd, nd)) < 0.25)
    for i in range(nd - 1):  # a chain keeps the component connected
        M[i, i + 1] = M[i, i + 1] or -0.5
        M[i + 1, i] = M[i + 1, i] or -0.3
    np.fill_diagonal(M, 0.0)
    np.fill_diagonal(M, -M.sum(1))
    return M * rng.uniform(0.5, 2.0, size=(nd, 1))  # row scaling (aj)


def _coarsest_inverse(M, comps):
    nd = len(M)
    Mp = M.copy()
    pins = []
    for c in comps:
        r0 = c[0]
        pins.append((r0, M[r0].copy(), c))
        Mp[r0] = 0.0
        Mp[r0, r0] = 1.0
    I = np.linalg.inv(Mp)
    ws = [I[r0] - m0 @ I for r0, m0, _ in pins]
    for r0, _, _ in pins:
        I[:, r0] = 0.0
    for (r0, _, c), w in zip(pins, ws):
        mask = np.zeros(nd, bool)
        mask[c] = True
        s1 = w[mask].sum()
        rs = I[:, mask].sum(1)
        I[:, mask] -= np.outer(rs, w[mask]) / s1
    return I, pins, ws


@pytest.mark.parametrize("sizes", [(24,), (40, 17), (12, 30, 9)])
def test_projected_coarsest_solve(sizes):
    rng = np.random.default_rng(sum(sizes))
    nd = sum(sizes)
    M = np.zeros((nd, nd))
    comps, o = [], 0
    for s in sizes:
        M[o:o + s, o:o + s] = _component(rng, s)
        comps.append(list(range(o, o + s)))
        o += s
    Dinv, pins, ws = _coarsest_inverse(M, comps)
    for (r0, _, c), w in zip(pins, ws):
        assert abs(w[r0] - 1.0) < 1e-12
        assert np.abs(w[c] @ M[np.ix_(c, c)]).max() < 1e-10 * np.abs(M).max()  # left null vector
    b = rng.standard_normal(nd)  # inconsistent on every component
    x = Dinv @ b
    for (r0, _, c), w in zip(pins, ws):
        bp = b[c] - (w[c] @ b[c]) / w[c].sum()  # b projected evenly onto the range
        assert np.abs(M[np.ix_(c, c)] @ x[c] - bp).max() < 1e-9 * np.abs(b).max()
        assert abs(x[r0]) < 1e-12
