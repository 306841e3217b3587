"""The learned initial guess end to end on a small advected-towers sequence
(marked gpu): samples from the plain solver, training by the library's own
kernels, then held-out steps where the plain solver judges the guess.

What the test pins: the guess is never worse than the linear
extrapolation it corrects (its band weights are a least-squares fit on the
FP64 residual, and zero weights give the extrapolation back), it beats the
previous-step warm start (the reference's Phi2 restart, the fallback), and
the solve from it converges in fewer iterations than from the previous
step.
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
        assert a["chosen"] == 1 and a["rel_learned"] < a["rel_prev"]
        assert a["iterations"] < p["iterations"]
    s.close()
    net.close()
    fresh.close()
