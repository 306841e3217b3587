"""Training and use of the learned initial guess.

The plain solver generates the data: after each solved step n (n >= 2) the
library writes the network's feature planes and the target
(phi_n - phi_ex) / RMS(aj (b - A phi_ex)), phi_ex = 2 phi_{n-1} - phi_{n-2},
into device-resident sample slots (`vfs_poisson_guess_sample`).  The U-Net
is then trained on random sub-boxes of random samples by the library's own
forward, backward and Adam kernels.  The target scale kappa (the RMS of the
raw targets) is fixed from the first samples and kept with the network.
At use, `vfs_poisson_learned_guess` builds the same features, runs the
network and keeps whichever of the learned guess and phi_{n-1} has the
smaller FP64 residual, so the previous-step guess remains the fallback.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import UNet


class SamplePool:
    """Device-resident training samples of one grid (its cell box dims; the
    samples live on the half-resolution grid the network runs on)."""

    def __init__(self, box, capacity, device="cuda", operators=0):
        """operators: how many row-scaled operators to keep for the residual
        loss (0: MSE training on the half-resolution targets)."""
        import torch
        self.torch = torch
        nx, ny, nz = (c // 2 for c in box)
        box = (nx, ny, nz)
        self.box = box
        self.feat = torch.zeros((capacity, 4, nz, ny, nx), dtype=torch.float32, device=device)
        self.tgt = torch.zeros((capacity, nz, ny, nx), dtype=torch.float32, device=device)
        self.wt = torch.zeros((capacity, nz, ny, nx), dtype=torch.float32, device=device)
        self.op = torch.zeros((operators, 19, nz, ny, nx), dtype=torch.float32, device=device) if operators else None
        self.n = 0
        self.kappa = None

    def add(self, solver, phi_n, phi_nm1, phi_nm2):
        """Store the sample of the solver's current right-hand side."""
        q = self.n % self.feat.shape[0]
        solver.guess_sample(phi_n, phi_nm1, phi_nm2, self.feat[q], self.tgt[q], self.wt[q])
        if self.op is not None and (self.n < self.op.shape[0] or self.op.shape[0] > 1):
            solver.operator32(self.op[q % self.op.shape[0]])
        if self.kappa is not None:
            self.tgt[q] /= self.kappa
        self.n += 1

    def operator(self, q):
        return None if self.op is None else self.op[q % self.op.shape[0]]

    @property
    def size(self):
        return min(self.n, self.feat.shape[0])

    def fix_kappa(self):
        """Target scale from the stored samples (RMS over dofs)."""
        torch = self.torch
        k = self.size
        num = (self.tgt[:k] ** 2 * self.wt[:k]).sum()
        den = self.wt[:k].sum().clamp(min=1.0)
        self.kappa = float(torch.sqrt(num / den))
        if not self.kappa > 0:
            self.kappa = 1.0
        self.tgt[:k] /= self.kappa
        return self.kappa


def train(net: UNet, pool: SamplePool, steps, crop=(64, 64, 64), lr=2e-3, lr_end=1e-4, seed=0, log_every=0,
          time_limit=None, mse_weight=0.1, res_weight=1.0):
    """Adam on random crops; learning rate decays geometrically from lr to
    lr_end.  With the pool's operators the loss is the residual of the
    predicted correction (what the solver judges a guess by) plus
    mse_weight times the error against the solved target.  Returns the list
    of losses."""
    if pool.kappa is None:
        net.kappa = pool.fix_kappa()
    else:
        net.kappa = pool.kappa
    rng = np.random.default_rng(seed)
    nx, ny, nz = pool.box
    cx, cy, cz = (min(c, n) // 4 * 4 for c, n in zip(crop, pool.box))
    losses = []
    t0 = time.time()
    for it in range(steps):
        q = int(rng.integers(pool.size))
        o = (int(rng.integers(0, nx - cx + 1)), int(rng.integers(0, ny - cy + 1)), int(rng.integers(0, nz - cz + 1)))
        op = pool.operator(q)
        b = UNet.batch(pool.feat[q], pool.tgt[q], pool.wt[q], origin=o, size=(cx, cy, cz), op=op,
                       op_scale=net.kappa, mse_weight=mse_weight if op is not None else 1.0,
                       res_weight=res_weight if op is not None else 0.0)
        a = lr * (lr_end / lr) ** (it / max(steps - 1, 1))
        losses.append(net.train_step(b, a))
        if log_every and it % log_every == 0:
            print(f"train step {it} lr {a:.2e} loss {losses[-1]:.4e}", flush=True)
        if time_limit is not None and time.time() - t0 > time_limit:
            break
    return losses


def run_sequence(seq, solver, steps, opts, guess="prev", net=None, pool=None, start=0, history=None, stats=None):
    """Solve steps start..start+steps-1 of a sequence on `solver`.

    guess: "zero", "prev" (phi_{n-1}, the reference's warm start), "extrap"
    (2 phi_{n-1} - phi_{n-2}) or "learned" (the library's judge among
    phi_{n-1} or the history's projection, the extrapolation and the
    network's guess).  With `pool`, every step with two predecessors adds a
    training sample.  Returns (history [phi_{n-1}, phi_n] as CUDA tensors,
    per-step records)."""
    import torch
    hist = list(history or [])
    recs = []
    nv = None
    for n in range(start, start + steps):
        if nv is None or seq.moving:
            nv = seq.classify(solver, n)
            solver.set_nvert(nv)
        u = seq.mask_faces(seq.ucont(n), nv)
        solver.rhs(u)
        phi = torch.zeros_like(nv)
        rec = {"step": n}
        o = opts
        if guess == "learned" and len(hist) >= 2:
            ch, rr = solver.learned_guess(net, hist[-1], hist[-2], net.kappa)
            rec.update(chosen=ch, rel_prev=rr[0], rel_learned=rr[1])
            _, st = solver.solve(phi, opts=_with(o, warm_start=2))
        elif guess in ("prev", "learned") and len(hist) >= 1:
            phi.copy_(hist[-1])
            _, st = solver.solve(phi, opts=_with(o, warm_start=1))
        elif guess == "extrap" and len(hist) >= 2:
            phi.copy_(2 * hist[-1] - hist[-2])
            _, st = solver.solve(phi, opts=_with(o, warm_start=1))
        else:
            _, st = solver.solve(phi, opts=_with(o, warm_start=0))
        rec.update(iterations=st.iterations, initial=st.initial_rel_residual, rel=st.rel_residual, ms=st.ms_total)
        if pool is not None and len(hist) >= 2:
            pool.add(solver, phi, hist[-1], hist[-2])
        hist = (hist + [phi])[-2:]
        recs.append(rec)
        if stats is not None:
            stats.append(rec)
    return hist, recs


def _with(opts, **kw):
    from . import SolveOpts
    o = SolveOpts()
    for f, _ in SolveOpts._fields_:
        setattr(o, f, getattr(opts, f))
    for k, v in kw.items():
        setattr(o, k, v)
    return o
