"""Numpy model of the history projection of the initial guess (CPU).

The library's projection (vfs_poisson_history_guess) solves the normal
equations of min ||b - sum_j c_j A X_j|| in the basis of the newest image
Y_0 and the differences Y_0 - Y_1, Y_1 - Y_2, ... (Gram entries formed from
the difference vectors), by a Cholesky factorisation in that order that
drops a vector whose pivot falls below 1e-13 of its Gram diagonal.  This
model restates that step and checks it on an advected towers sequence solved
by the oracle's CPU solver: the projection is never worse than the previous
step's phi, it reaches the least-squares optimum of a QR solution over the
same solutions up to 8 of them, and over 6 solutions it cuts the initial
residual of the sequence by more than 1000x.
"""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF


def greedy_projection(G, g, order):
    """Coefficients of the library's projection (order: slots newest first)."""
    k = len(order)
    L = np.zeros((k, k))
    acc = []
    for sl in order:
        row = np.zeros(len(acc))
        for q in range(len(acc)):
            v = G[sl, acc[q]] - row[:q] @ L[q, :q]
            row[q] = v / L[q, q]
        piv = G[sl, sl] - row @ row
        if not piv > 1e-13 * G[sl, sl]:
            continue
        p = len(acc)
        L[p, :p] = row
        L[p, p] = np.sqrt(piv)
        acc.append(sl)
    na = len(acc)
    c = np.zeros(G.shape[0])
    if na:
        Ls = L[:na, :na]
        z = np.linalg.solve(Ls, g[acc])
        c[acc] = np.linalg.solve(Ls.T, z)
    return c


@pytest.fixture(scope="module")
def sequence():
    import bench
    nx, ny, nz = 48, 32, 48
    case0, d, met = bench.cpu_sequence_case(nx, ny, nz, 0)
    lhs = O.poisson_lhs(d, case0.nvert, met)
    A = O.csr(lhs).tocsr()
    mg = bench.cpu_solver(d, case0.coor, case0.nvert, met)
    bs, xs = [], []
    for s in range(12):
        u = CF._mask_faces(CF._fourier_ucont(np.random.default_rng(1003), nx, ny, nz, shift=0.5 * s), case0.nvert)
        b2 = O.rhs(d, case0.nvert, lhs["gid"], u, met["aj"])
        x, st = mg.solve(O.to_da(d, lhs["gid"], b2), rtol=1e-10, max_it=100, nu1=1, nu2=2, omega=1.0,
                         restart=20)
        bs.append(b2)
        xs.append(O.from_da(d, lhs["gid"], x))
    return A, bs, xs


def _rel(A, b, x):
    return np.linalg.norm(b - A @ x) / np.linalg.norm(b)


def difference_basis(V):
    """V_0, V_0 - V_1, V_1 - V_2, ... of vectors given newest first."""
    return [V[0]] + [V[i] - V[i + 1] for i in range(len(V) - 1)]


@pytest.mark.parametrize("k", [2, 4, 6, 8])
def test_projection_model(sequence, k):
    A, bs, xs = sequence
    n = 11
    b = bs[n]
    X = [xs[n - 1 - i] for i in range(k)]          # i-th newest
    Y = [A @ x for x in X]
    BX, BY = difference_basis(X), difference_basis(Y)
    G = np.array([[yi @ yj for yj in BY] for yi in BY])
    g = np.array([y @ b for y in BY])
    c = greedy_projection(G, g, list(range(k)))
    xg = sum(ci * xi for ci, xi in zip(c, BX))
    r_proj = _rel(A, b, xg)
    r_prev = _rel(A, b, xs[n - 1])
    assert r_proj <= r_prev * (1 + 1e-9)
    cq, *_ = np.linalg.lstsq(np.stack(Y, 1), b, rcond=None)
    r_ls = _rel(A, b, np.stack(X, 1) @ cq)
    assert r_proj <= 1.01 * r_ls, (k, r_proj, r_ls)
    if k >= 6:
        assert r_proj < 1e-3 * r_prev, (r_proj, r_prev)
