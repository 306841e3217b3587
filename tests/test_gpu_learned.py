"""The learned initial guess end to end on a small advected-towers sequence
(marked gpu): samples from the plain solver, training by the library's own
kernels, then held-out steps where the plain solver judges the guess.

What the test pins: the network's guess is never worse in residual than
the linear extrapolation it corrects (its band weights are a least-squares
fit on the FP64 residual, and zero weights give the extrapolation back);
the judge installs the network's guess or the extrapolation rather than the
previous-step warm start (the reference's Phi2 restart), and the solve from
it converges in fewer iterations than from the previous step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_guess_on_sequence(cuda_lib):
    import torch
    import vfs_poisson as V
    from vfs_poisson import learned as LG, sequence as S
    seq = S.TowerSequence(nx=64, ny=48, nz=64, n_theta=24)
    s = V.PoissonSolver(*seq.dims, periodic=seq.periodic)
    s.set_grid(seq.coor)
    pool = LG.SamplePool((seq.nx, seq.ny, seq.nz), 10)
    o64 = V.default_opts(precision=1)
    hist, recs = LG.run_sequence(seq, s, 12, o64, guess="prev", pool=pool)
    assert pool.size == 10
    assert all(r["rel"] <= 1e-8 for r in recs)
    # sample planes: finite features, weights are dof fractions
    assert torch.isfinite(pool.feat[:pool.size]).all()
    assert float(pool.wt.min()) >= 0.0 and float(pool.wt.max()) <= 1.0
    net = V.UNet(1)
    losses = LG.train(net, pool, 300, crop=(32, 24, 32), lr=1e-3, lr_end=1e-4)
    assert np.mean(losses[-30:]) < losses[0]
    fresh = V.UNet(1)
    fresh.kappa = net.kappa
    o32 = V.default_opts(precision=0)
    _, learned = LG.run_sequence(seq, s, 3, o32, guess="learned", net=net, start=12, history=hist)
    _, untrained = LG.run_sequence(seq, s, 3, o32, guess="learned", net=fresh, start=12, history=hist)
    _, prev = LG.run_sequence(seq, s, 3, o32, guess="prev", start=12, history=hist)
    for a, u, p in zip(learned, untrained, prev):
        assert a["rel"] <= 1e-8
        assert a["rel_learned"] <= u["rel_learned"] * (1 + 1e-6)   # never worse than the extrapolation
        assert a["chosen"] in (1, 2) and a["rel_learned"] < a["rel_prev"]
        assert a["iterations"] < p["iterations"]
    s.close()
    net.close()
    fresh.close()


def test_speculative_first_step_bitexact(cuda_lib, monkeypatch):
    """A learned guess that expects the plain extrapolation to win runs the
    next solve's first Arnoldi step on the handle's stream while the network
    runs on a side stream.  Solves that resume from it match solves that
    form every step themselves bit for bit, step after step; and a solve
    whose options differ from the step's, or that needs a larger Krylov
    basis, forms its own first step."""
    import torch
    import vfs_poisson as V
    from vfs_poisson import learned as LG, sequence as S
    seq = S.TowerSequence(nx=64, ny=48, nz=64, n_theta=24)
    o64 = V.default_opts(precision=1)
    o32 = V.default_opts(precision=0)
    runs = {}
    for spec in ("1", "0"):
        monkeypatch.setenv("VFS_GUESS_SPECULATE", spec)
        s = V.PoissonSolver(*seq.dims, periodic=seq.periodic)
        s.set_grid(seq.coor)
        hist, _ = LG.run_sequence(seq, s, 4, o64, guess="prev")
        net = V.UNet(0)
        net.kappa = 1e-4
        hist2, recs = LG.run_sequence(seq, s, 3, o32, guess="learned", net=net, start=4, history=hist)
        # a solve with other options after a speculative guess
        u = seq.mask_faces(seq.ucont(7), seq.classify(s, 7))
        s.rhs(u)
        s.learned_guess(net, hist2[-1], hist2[-2], net.kappa)
        phi = torch.empty_like(hist2[-1])
        _, st = s.solve(phi, opts=V.default_opts(precision=0, warm_start=2, nu2=3))
        # and one whose restart length needs a larger basis than the step's
        s.learned_guess(net, hist2[-1], hist2[-2], net.kappa)
        phi2 = torch.empty_like(hist2[-1])
        _, st2 = s.solve(phi2, opts=V.default_opts(precision=0, warm_start=2, restart=30))
        runs[spec] = ([r["iterations"] for r in recs], [h.clone() for h in hist2], st.iterations, phi.clone(),
                      st2.iterations, phi2.clone())
        assert all(r["rel"] <= 1e-8 for r in recs) and st.rel_residual <= 1e-8 and st2.rel_residual <= 1e-8
        assert all(r["chosen"] == 2 for r in recs)   # the extrapolation (band weights 0)
        s.close()
        net.close()
    a, b = runs["1"], runs["0"]
    assert a[0] == b[0] and a[2] == b[2]
    for x, y in zip(a[1], b[1]):
        assert torch.equal(x, y)
    assert torch.equal(a[3], b[3])
    assert a[4] == b[4] and torch.equal(a[5], b[5])
