"""Initial guess from the solution history on the GPU (marked gpu).

On an advected towers sequence (48x32x48, the bench's generator on the host)
and a rotating rotor (64x48x64, a new mask every step):
  * the residual the guess reports is the true FP64 residual of the iterate
    it installs (checked with the oracle's operator);
  * the projection is never worse than the previous step's phi, and over 6
    stored solutions it cuts the initial residual by more than 1000x;
  * after a new operator assembly the projection has no solution of the
    current operator: the extrapolation of the newest two is installed, with
    its residual formed by an operator apply;
  * the judge: the estimated error it reports for the installed guess is the
    2-norm of one V-cycle of that guess's residual with the fluid mean
    removed, and the installed candidate has the smallest estimate among the
    rated ones; solves from it converge;
  * the learned guess puts its network before the same judge, and with a
    network period the network sits out the calls in between;
  * over 10 stored solutions the projection reaches the least-squares
    optimum of their images, and on a 128x96x128 towers sequence the error
    of solves started from an 8-solution history stays bounded.
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
            ch, rels, ests = s.guess_report()
            assert rels[ch] == pytest.approx(rel, rel=1e-12)
            # the installed iterate itself: a solve that stops at once (any
            # initial residual passes rtol 1e30)
            s.history_record(False)
            phi_g, st0 = s.solve(opts=V.default_opts(rtol=1e30, warm_start=2))
            s.history_record(True)
            assert st0.iterations == 0 and abs(st0.initial_rel_residual - rel) <= 1e-12 * rel + 1e-300
            true = _true_rel(d, lhs, case0, met, u, phi_g)
            assert abs(true - rel) <= 1e-6 * rel + 1e-14, (true, rel)
            prev = _true_rel(d, lhs, case0, met, u, phi_prev)
            assert rels[0] <= prev * (1 + 1e-6), (rels[0], prev)    # the projection
            if step >= 7:
                assert rels[0] < 1e-3 * prev, (step, rels[0], prev)
            _check_judge(ch, rels, ests)
            s.history_guess()
            phi_prev, st = s.solve(opts=V.default_opts(rtol=1e-10, warm_start=2))
            assert st.rel_residual <= 1e-10
    finally:
        s.close()


def test_projection_reaches_least_squares(cuda_lib, seq):
    """With 10 stored solutions the projection's residual is the least-squares
    optimum over the images of the stored solutions (numpy lstsq with the
    oracle's operator) within 1 %: the basis of the newest solution and the
    differences of consecutive ones keeps the directions that normal
    equations on the nearly parallel images themselves would lose."""
    import vfs_poisson as V
    case0, d, met, lhs, _ = seq
    A = O.csr(lhs)
    us = [CF._mask_faces(CF._fourier_ucont(np.random.default_rng(1003), NX, NY, NZ, shift=0.5 * t), case0.nvert)
          for t in range(13)]
    s = V.PoissonSolver.from_case(case0)
    try:
        s.set_history(10)
        X = []
        for step, u in enumerate(us[:-1]):
            s.rhs(u)
            if step:
                s.history_guess()
            phi, st = s.solve(opts=V.default_opts(rtol=1e-10, warm_start=2 if step else 0))
            assert st.rel_residual <= 1e-10
            X.append(O.from_da(d, lhs["gid"], phi))
        s.rhs(us[-1])
        s.history_guess()
        ch, rels, _ = s.guess_report()
        b2 = O.rhs(d, case0.nvert, lhs["gid"], us[-1], met["aj"])
        Y = np.stack([A @ x for x in X[-10:]], 1)
        c, *_ = np.linalg.lstsq(Y, b2, rcond=None)
        r_ls = np.linalg.norm(b2 - Y @ c) / np.linalg.norm(b2)
        assert rels[0] <= 1.01 * r_ls, (rels[0], r_ls)
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
        ch, rels, _ = s.guess_report()
        # no stored solution of the new operator: the extrapolation alone
        assert ch == 2 and rels[0] == -1.
        s.history_record(False)
        phi_g, _ = s.solve(opts=V.default_opts(rtol=1e30, warm_start=2))
        lhs1 = O.poisson_lhs(d, case1.nvert, met)
        true = _true_rel(d, lhs1, case1, met, case1.ucont, phi_g)
        assert abs(true - rel) <= 1e-6 * rel + 1e-14, (true, rel)
        # one solve under the new operator: the projection is back
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
            if evaluated[i] and ch != 1:
                assert not evaluated[i + 1] and not evaluated[i + 2], calls
        assert sum(evaluated) >= 2 and not all(evaluated), calls
        # the projection's residual shrinks as the history fills
        base = [rr[0] for ch, rr in calls if rr[0] >= 0.]
        assert base[-1] < base[0]
    finally:
        s.close()
        net.close()


def _check_judge(ch, rels, ests):
    """The installed candidate: the smallest estimated error among the rated
    ones, else (nothing rated) the smallest residual among the formed ones."""
    rated = [c for c in range(3) if ests[c] >= 0.]
    if len(rated) >= 2:
        assert ch in rated and ests[ch] == min(ests[c] for c in rated), (ch, rels, ests)
    else:
        formed = [c for c in range(3) if rels[c] >= 0.]
        assert rels[ch] == min(rels[c] for c in formed), (ch, rels, ests)


def test_judge_on_moving_rotor(cuda_lib):
    """A 64x48x64 rotor turning 2 degrees per step: every step has a new
    operator, so the guess is the extrapolation of the newest two solutions
    (residual by an operator apply); the reported error estimate of the
    installed guess equals one V-cycle of its residual with the fluid mean
    removed, formed independently through the library's V-cycle entry."""
    import torch
    import vfs_poisson as V
    from vfs_poisson import sequence as S
    seq = S.RotorSequence(64, 48, 64, n_theta=16)
    s = V.PoissonSolver(*seq.dims, periodic=seq.periodic)
    try:
        s.set_grid(seq.coor)
        s.set_history(4)
        for n in range(6):
            nv = seq.classify(s, n)
            s.set_nvert(nv)
            u = seq.mask_faces(seq.ucont(n), nv)
            s.rhs(u)
            if n < 2:
                phi, st = s.solve(rtol=1e-10)
                continue
            rel = s.history_guess()
            ch, rels, ests = s.guess_report()
            assert ch == 2 and rels[0] == -1. and rels[2] == pytest.approx(rel, rel=1e-12)
            s.history_record(False)
            phi_g, _ = s.solve(opts=V.default_opts(rtol=1e30, warm_start=2))
            s.history_record(True)
            # the installed iterate's residual, on the host
            b = s.rhs_array()
            ax = s.apply(phi_g)
            nvh = nv.cpu().numpy()
            fluid = np.zeros(nvh.shape, bool)
            fluid[1:-1, 1:-1, 1:-1] = nvh[1:-1, 1:-1, 1:-1] < 0.1
            r = np.where(fluid, b - ax, 0.)
            assert np.linalg.norm(r) / np.linalg.norm(b) == pytest.approx(rel, rel=1e-6)
            s.rhs(u)
            s.history_guess()
            phi, st = s.solve(opts=V.default_opts(rtol=1e-10, warm_start=2))
            assert st.rel_residual <= 1e-10
    finally:
        s.close()


def test_judge_estimate_matches_vcycle(cuda_lib):
    """On the static towers sequence with two stored solutions the
    extrapolation is within the gate of the projection, so both are rated:
    the estimate of the installed one is the 2-norm of one V-cycle of its
    residual, fluid mean removed (formed again through the library's V-cycle
    entry), the smaller estimate wins, and the solve that starts from the
    judge's V-cycle converges to the phi of a solve from the same iterate
    that forms its own first V-cycle."""
    import vfs_poisson as V
    case0, d, met, lhs, us = _seq_cache()
    fl = np.zeros(case0.nvert.shape, bool)
    fl[1:-1, 1:-1, 1:-1] = case0.nvert[1:-1, 1:-1, 1:-1] < 0.1
    s = V.PoissonSolver.from_case(case0)
    rated_steps = 0
    try:
        s.set_history(2)
        for u in us[:2]:
            s.rhs(u)
            s.solve(rtol=1e-10)
        for u in us[2:6]:
            s.rhs(u)
            s.history_guess()
            ch, rels, ests = s.guess_report()
            _check_judge(ch, rels, ests)
            s.history_record(False)
            phi_g, _ = s.solve(opts=V.default_opts(rtol=1e30, warm_start=2))
            if ests[ch] >= 0.:
                rated_steps += 1
                r = np.where(fl, s.rhs_array() - s.apply(phi_g), 0.)
                z = s.mg_vcycle(r)
                zc = z[fl] - z[fl].mean()
                assert np.linalg.norm(zc) == pytest.approx(ests[ch], rel=1e-4)
            # the judged start against a start from the same iterate
            s.rhs(u)
            s.history_guess()
            phi_a, st_a = s.solve(opts=V.default_opts(rtol=1e-9, warm_start=2))
            s.rhs(u)
            phi_b, st_b = s.solve(phi_g.copy(), opts=V.default_opts(rtol=1e-9, warm_start=1))
            assert st_a.rel_residual <= 1e-9 and st_b.rel_residual <= 1e-9
            err = np.linalg.norm((phi_a - phi_b)[fl]) / np.linalg.norm(phi_b[fl])
            assert err < 1e-6, err
            # the step enters the history once
            s.history_record(True)
            s.rhs(u)
            s.history_guess()
            s.solve(opts=V.default_opts(rtol=1e-10, warm_start=2))
        assert rated_steps >= 1
    finally:
        s.close()


_CACHE = {}


def _seq_cache():
    if "seq" not in _CACHE:
        import bench
        case0, d, met = bench.cpu_sequence_case(NX, NY, NZ, 0)
        lhs = O.poisson_lhs(d, case0.nvert, met)
        us = [CF._mask_faces(CF._fourier_ucont(np.random.default_rng(1003), NX, NY, NZ, shift=0.5 * s), case0.nvert)
              for s in range(10)]
        _CACHE["seq"] = (case0, d, met, lhs, us)
    return _CACHE["seq"]


def test_new_mask_refills_hierarchy_bitexact(cuda_lib):
    """A second mask on a handle refills its multigrid hierarchy in place
    (same levels, buffers and coarse metrics; the coarsest inverse and the
    V-cycle graphs formed anew).  Its solves must match a fresh handle built
    for that mask bit for bit, in both V-cycle precisions, and back again
    for the first mask."""
    import vfs_poisson as V
    from vfs_poisson import sequence as S
    seq = S.RotorSequence(48, 32, 48, n_theta=16)
    moved = V.PoissonSolver(*seq.dims, periodic=seq.periodic)
    try:
        moved.set_grid(seq.coor)
        masks = [seq.classify(moved, n) for n in (0, 7, 0)]
        for step, nv in enumerate(masks):
            moved.set_nvert(nv)
            u = seq.mask_faces(seq.ucont(step), nv)
            fresh = V.PoissonSolver(*seq.dims, periodic=seq.periodic)
            try:
                fresh.set_grid(seq.coor)
                fresh.set_nvert(nv)
                for prec in (0, 1):
                    out = []
                    for s in (moved, fresh):
                        s.rhs(u)
                        phi, st = s.solve(precision=prec, rtol=1e-10)
                        out.append((phi, st.iterations, st.rel_residual))
                    assert out[0][1] == out[1][1] and out[0][2] == out[1][2], (step, prec)
                    np.testing.assert_array_equal(out[0][0], out[1][0])
            finally:
                fresh.close()
    finally:
        moved.close()


def test_projection_error_stays_bounded(cuda_lib):
    """A towers sequence (128x96x128) in the bench's order: 10 plain FP64
    solves fill an 8-solution history, then 30 solves start from the history
    guess with the FP32 V-cycle.  Their phi stays within 1e-8 relative L2 of
    an independent FP64 solve to 1e-11, with no growth over the sequence, and
    no solve needs more than 3 iterations.  (A fit over too many solutions of
    a sequence solved to rtol reaches the solutions' own errors, whose
    differences have almost no image: the least-squares fit then adds them
    freely, and the error grows from step to step.)"""
    import torch
    import vfs_poisson as V
    from vfs_poisson import sequence as S
    seq = S.TowerSequence(128, 96, 128)
    stream = torch.cuda.current_stream()
    solvers = []
    try:
        for _ in range(2):
            h = V.PoissonSolver(*seq.dims, periodic=seq.periodic)
            h.set_stream(stream.cuda_stream)
            h.set_grid(seq.coor)
            solvers.append(h)
        s, ref = solvers
        nv = seq.classify(s, 0)
        s.set_nvert(nv)
        ref.set_nvert(nv)
        s.set_history(8)
        fluid = torch.zeros_like(nv, dtype=torch.bool)
        fluid[1:-1, 1:-1, 1:-1] = nv[1:-1, 1:-1, 1:-1] < 0.1
        phi = torch.zeros_like(nv)
        errs, its = [], []
        for n in range(40):
            u = seq.mask_faces(seq.ucont(n), nv)
            s.rhs(u)
            ref.rhs(u)
            pr, _ = ref.solve(torch.zeros_like(nv), opts=V.default_opts(precision=1, rtol=1e-11))
            if n < 10:
                phi, st = s.solve(phi.clone(), opts=V.default_opts(precision=1, rtol=1e-8, warm_start=1))
                continue
            s.history_guess()
            phi, st = s.solve(torch.empty_like(nv), opts=V.default_opts(precision=0, rtol=1e-8, warm_start=2))
            assert st.rel_residual <= 1e-8
            its.append(st.iterations)
            errs.append(((phi - pr)[fluid].norm() / pr[fluid].norm()).item())
        assert max(its) <= 3, its
        assert max(errs) <= 1e-8, errs
        assert max(errs[-10:]) <= 10 * max(max(errs[:10]), 1e-10), errs
    finally:
        for h in solvers:
            h.close()
