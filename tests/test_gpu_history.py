"""History projection of the initial guess on the GPU (marked gpu).

On an advected towers sequence (48x32x48, the bench's generator on the host):
  * the residual the projection reports is the true FP64 residual of the
    iterate it installs (checked with the oracle's operator);
  * it is never worse than the previous step's phi, and over 6 stored
    solutions it cuts the initial residual by more than 1000x;
  * after a new operator assembly the stored images are recomputed, so the
    reported residual stays exact;
  * the learned guess judges its candidate against the projection, and with
    a network period the network sits out the calls in between.
"""
import numpy as np
import pytest

import oracle as O
from vfs_poisson import configs as CF

pytestmark = pytest.mark.gpu

NX, NY, NZ = 48, 32, 48


@pytest.fixture(scope="module")
def seq():
    import bench
    case0, d, met = bench.cpu_sequence_case(NX, NY, NZ, 0)
    lhs = O.poisson_lhs(d, case0.nvert, met)
    us = [CF._mask_faces(CF._fourier_ucont(np.random.default_rng(1003), NX, NY, NZ, shift=0.5 * s), case0.nvert)
          for s in range(10)]
    return case0, d, met, lhs, us


def _true_rel(d, lhs, case, met, u, phi):
    A = O.csr(lhs)
    b2 = O.rhs(d, case.nvert, lhs["gid"], u, met["aj"])
    x2 = O.from_da(d, lhs["gid"], phi)
    return np.linalg.norm(b2 - A @ x2) / np.linalg.norm(b2)


def test_projection_exact_and_never_worse(cuda_lib, seq):
    import vfs_poisson as V
    case0, d, met, lhs, us = seq
    s = V.PoissonSolver.from_case(case0)
    try:
        s.set_history(6)
        phi_prev = None
        for step, u in enumerate(us):
            s.rhs(u)
            if step == 0:
                phi_prev, st = s.solve(rtol=1e-10)
                continue
            rel = s.history_guess()
            # the installed iterate itself: a solve that stops at once
            s.history_record(False)
            phi_g, st0 = s.solve(opts=V.default_opts(rtol=0.99, warm_start=2))
            s.history_record(True)
            assert st0.iterations == 0 and abs(st0.initial_rel_residual - rel) <= 1e-12 * rel + 1e-300
            true = _true_rel(d, lhs, case0, met, u, phi_g)
            assert abs(true - rel) <= 1e-6 * rel + 1e-14, (true, rel)
            prev = _true_rel(d, lhs, case0, met, u, phi_prev)
            assert rel <= prev * (1 + 1e-6), (rel, prev)
            if step >= 7:
                assert rel < 1e-3 * prev, (step, rel, prev)
            s.history_guess()
            phi_prev, st = s.solve(opts=V.default_opts(rtol=1e-10, warm_start=2))
            assert st.rel_residual <= 1e-10
    finally:
        s.close()


def test_projection_after_new_operator(cuda_lib, seq):
    import vfs_poisson as V
    case0, d, met, lhs, us = seq
    s = V.PoissonSolver.from_case(case0)
    try:
        s.set_history(4)
        for u in us[:4]:
            s.rhs(u)
            s.solve(rtol=1e-10)
        # a different mask: the towers moved by two cells in x
        nv = np.roll(case0.nvert, 2, axis=2)
        nv = CF.sync_periodic_ghosts(nv, case0.periodic)
        case1 = CF.Case("towers_moved", NX, NY, NZ, case0.periodic, case0.coor, nv, CF._mask_faces(us[4], nv))
        s.set_nvert(case1.nvert)
        s.rhs(case1.ucont)
        rel = s.history_guess()
        s.history_record(False)
        phi_g, _ = s.solve(opts=V.default_opts(rtol=0.99, warm_start=2))
        lhs1 = O.poisson_lhs(d, case1.nvert, met)
        true = _true_rel(d, lhs1, case1, met, case1.ucont, phi_g)
        assert abs(true - rel) <= 1e-6 * rel + 1e-14, (true, rel)
    finally:
        s.close()


def test_learned_guess_against_projection(cuda_lib, seq):
    import vfs_poisson as V
    case0, d, met, lhs, us = seq
    s = V.PoissonSolver.from_case(case0)
    net = V.UNet(0)
    try:
        hist = []
        for u in us[:4]:
            s.rhs(u)
            phi, _ = s.solve(rtol=1e-10)
            hist.append(phi.copy())
        s.set_history(6)
        s.set_network_period(3)
        calls = []
        for u in us[4:10]:
            s.rhs(u)
            ch, rr = s.learned_guess(net, hist[-1], hist[-2], 1.0)
            calls.append((ch, rr))
            phi, st = s.solve(opts=V.default_opts(rtol=1e-8, warm_start=2))
            assert st.rel_residual <= 1e-8
            hist.append(phi.copy())
        # after a call whose network candidate lost to the projection, the
        # next period - 1 = 2 calls install the projection without the network
        evaluated = [rr[1] >= 0. for ch, rr in calls]
        for i, (ch, rr) in enumerate(calls[1:-2], start=1):
            if evaluated[i] and ch == 0:
                assert not evaluated[i + 1] and not evaluated[i + 2], calls
        assert sum(evaluated) >= 2 and not all(evaluated), calls
        # the projection's residual shrinks as the history fills
        assert calls[-1][1][0] < calls[0][1][0]
    finally:
        s.close()
        net.close()
