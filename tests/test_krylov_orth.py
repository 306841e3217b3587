"""The FGMRES orthogonalisations of the library, modelled in numpy (CPU):
one-pass classical Gram-Schmidt with the basis kept unnormalised and scaled
by its norms (orth 0, the default), delayed reorthogonalisation (DCGS2,
orth 1) and classical Gram-Schmidt with full reorthogonalisation converge in
the same number of iterations on an anisotropic system with a preconditioner
rounded to FP32 (the FP32 V-cycle's role)."""
import numpy as np
import pytest

sp = pytest.importorskip("scipy.sparse")
spl = pytest.importorskip("scipy.sparse.linalg")


def _system(n=14, seed=0):
    rng = np.random.default_rng(seed)
    I = sp.identity(n)
    e = np.ones(n)
    T = sp.diags([-e[:-1], 2 * e, -e[:-1]], [-1, 0, 1])
    A = sp.kron(sp.kron(I, I), T) + 3e4 * sp.kron(sp.kron(I, T), I) + 0.3 * sp.kron(sp.kron(T, I), I)
    A = (A + sp.diags(1e-9 * rng.random(n ** 3)) + 0.01 * sp.random(n ** 3, n ** 3, density=1e-4, random_state=1))
    A = A.tocsr()
    b = rng.standard_normal(n ** 3)
    ilu = spl.spilu(A.tocsc(), drop_tol=1e-2, fill_factor=2)
    return A, b, lambda v: ilu.solve(v).astype(np.float32).astype(np.float64)


def _fgmres(A, b, M, mode, m, rtol, maxit=300):
    N = len(b)
    x = np.zeros(N)
    bn = np.linalg.norm(b)
    it = 0
    r = b - A @ x
    beta = np.linalg.norm(r)
    rel = beta / bn
    while rel > rtol and it < maxit:
        V, Z, nrm2 = [r.copy()], [], [beta * beta]
        H = np.zeros((m + 1, m))
        R = np.zeros((m + 1, m))
        cs, sn, g = np.zeros(m), np.zeros(m), np.zeros(m + 1)
        g[0] = beta
        gsave = None

        def rotate(j):
            R[:j + 2, j] = H[:j + 2, j]
            for i in range(j):
                a, c = R[i, j], R[i + 1, j]
                R[i, j], R[i + 1, j] = cs[i] * a + sn[i] * c, -sn[i] * a + cs[i] * c
            a, c = R[j, j], R[j + 1, j]
            den = np.hypot(a, c)
            cs[j], sn[j] = a / den, c / den
            R[j, j], R[j + 1, j] = den, 0.0
            g[j + 1], g[j] = -sn[j] * g[j], cs[j] * g[j]

        jj = 0
        while jj < m and it < maxit:
            Z.append(M(V[jj] / np.sqrt(nrm2[jj])))
            w = A @ Z[jj]
            if mode == "cgs":  # one pass, unnormalised basis scaled by its norms
                Q = np.array(V[:jj + 1])
                sinv = 1 / np.sqrt(np.array(nrm2[:jj + 1]))
                h = (Q @ w) * sinv
                w = w - (h * sinv) @ Q
                wn = np.linalg.norm(w)
                H[:jj + 1, jj], H[jj + 1, jj] = h, wn
            elif mode == "dcgs2":  # delayed reorthogonalisation
                Q = np.array(V[:jj]) if jj else np.zeros((0, N))
                u = V[jj]
                a, bb, uu, uw = Q @ u, Q @ w, u @ u, u @ w
                rr = np.sqrt(uu - a @ a)
                hj = (uw - a @ bb) / rr
                V[jj] = (u - a @ Q) / rr
                w = w - bb @ Q - hj * V[jj]
                wn = np.linalg.norm(w)
                if jj > 0:
                    H[:jj, jj - 1] += a
                    H[jj, jj - 1] = rr
                    g[:] = gsave
                    rotate(jj - 1)
                H[:jj, jj], H[jj, jj], H[jj + 1, jj] = bb, hj, wn
            else:  # classical with full reorthogonalisation, normalised basis
                if jj == 0:
                    V[0] = V[0] / np.sqrt(nrm2[0])
                Q = np.array(V[:jj + 1])
                h1 = Q @ w
                w = w - h1 @ Q
                h2 = Q @ w
                w = w - h2 @ Q
                wn = np.linalg.norm(w)
                H[:jj + 1, jj], H[jj + 1, jj] = h1 + h2, wn
                w = w / wn
            it += 1
            V.append(w)
            nrm2.append(wn * wn if mode != "cgs2" else 1.0)
            gsave = g.copy()
            rotate(jj)
            jj += 1
            if abs(g[jj]) / bn <= rtol or wn == 0:
                break
        y = np.zeros(jj)
        for i in range(jj - 1, -1, -1):
            y[i] = (g[i] - R[i, i + 1:jj] @ y[i + 1:jj]) / R[i, i]
        x = x + np.array(Z[:jj]).T @ y
        r = b - A @ x
        beta = np.linalg.norm(r)
        rel = beta / bn
    return it, rel


@pytest.mark.parametrize("m,rtol", [(5, 1e-10), (20, 1e-10), (20, 1e-12)])
def test_orthogonalisations_converge_alike(m, rtol):
    A, b, M = _system()
    res = {mode: _fgmres(A, b, M, mode, m, rtol) for mode in ("cgs", "dcgs2", "cgs2")}
    its = {k: v[0] for k, v in res.items()}
    assert max(its.values()) - min(its.values()) <= 1, its
    for mode, (it, rel) in res.items():
        assert rel <= rtol * 1.5, (mode, rel)
