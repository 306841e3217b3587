"""Time sequences of pressure solves: the moving-rotor case and the advected
towers case, generated on the GPU.

A step n has its own blanking (a 3-rod rotor turned by 2 degrees per step,
classified by the library's immersed-boundary search from closed rod
surfaces, or static towers) and its own contravariant fluxes (the Fourier
pattern of the configurations advected by 0.5 cells per step in x, with the
faces next to blanked cells zeroed).  The Fourier sums are evaluated with
torch on the device so that long sequences are cheap to generate; the mode
parameters are drawn with numpy in the order ``configs._fourier_ucont`` uses.
"""
from __future__ import annotations

import math

import numpy as np

from . import configs as CF


def _draw_modes(rng, modes=32, kmax=8):
    out = []
    for comp in range(3):
        lst = []
        while len(lst) < modes:
            kv = rng.integers(-kmax, kmax + 1, size=3)
            kn = math.sqrt(float((kv ** 2).sum()))
            if kn < 1 or kn > kmax:
                continue
            lst.append((int(kv[0]), int(kv[1]), int(kv[2]), rng.normal() / kn, rng.uniform(0, 2 * np.pi)))
        out.append(lst)
    return out


class _Sequence:
    """Common part: grid, Fourier modes, per-step fluxes and face masking."""

    periodic = (0, 0, 0, 1, 0, 0)
    moving = True  # the blanking changes every step

    def __init__(self, nx, ny, nz, coor, seed, device="cuda", noise=0.1, advect=0.5):
        import torch
        self.torch = torch
        self.nx, self.ny, self.nz = nx, ny, nz
        self.coor = coor
        self.device = device
        self.advect = advect
        rng = np.random.default_rng(seed)
        self.modes = _draw_modes(rng)
        shape = (nz + 2, ny + 2, nx + 2, 3)
        self.noise = torch.from_numpy(rng.uniform(-noise, noise, size=shape)).to(device)
        self.ii = torch.arange(nx + 2, dtype=torch.float64, device=device)
        self.jj = torch.arange(ny + 2, dtype=torch.float64, device=device)
        self.kk = torch.arange(nz + 2, dtype=torch.float64, device=device)

    @property
    def dims(self):
        return (self.nx + 2, self.ny + 2, self.nz + 2)

    def ucont(self, step):
        """Unmasked fluxes of step `step`, DA layout [mz][my][mx][3] (device)."""
        torch = self.torch
        u = torch.zeros((self.nz + 2, self.ny + 2, self.nx + 2, 3), dtype=torch.float64, device=self.device)
        shift = self.advect * step
        for comp in range(3):
            fx = (self.ii - (0.0 if comp == 0 else 0.5) - shift) / self.nx
            fy = (self.jj - (0.0 if comp == 1 else 0.5)) / self.ny
            fz = (self.kk - (0.0 if comp == 2 else 0.5)) / self.nz
            acc = u[..., comp]
            for kx, ky, kz, a, ph in self.modes[comp]:
                acc += a * torch.cos(2 * math.pi * (kz * fz[:, None, None] + ky * fy[None, :, None]
                                                    + kx * fx[None, None, :]) + ph)
        u += self.noise
        return u

    def mask_faces(self, u, nvert):
        """Zero every face flux next to a blanked cell (nvert > 0.1)."""
        b = nvert > 0.1
        u[:, :, :-1, 0][b[:, :, :-1] | b[:, :, 1:]] = 0.0
        u[:, :-1, :, 1][b[:, :-1, :] | b[:, 1:, :]] = 0.0
        u[:-1, :, :, 2][b[:-1, :, :] | b[1:, :, :]] = 0.0
        return u

    def bodies(self, step):
        return []

    def classify(self, solver, step):
        """nvert of step `step` through the library's surface search (device)."""
        torch = self.torch
        nv = torch.zeros((self.nz + 2, self.ny + 2, self.nx + 2), dtype=torch.float64, device=self.device)
        for ibi, surf in enumerate(self.bodies(step)):
            solver.ibm_search(surf, nvert=nv, ibi=ibi)
        # periodic ghost layers take their partner cells' values, as the
        # ghost points of a periodic DA do after the search
        per = [self.periodic[q] or self.periodic[q + 3] for q in range(3)]
        if per[0]:
            nv[:, :, 0] = nv[:, :, -2]
            nv[:, :, -1] = nv[:, :, 1]
        if per[1]:
            nv[:, 0, :] = nv[:, -2, :]
            nv[:, -1, :] = nv[:, 1, :]
        if per[2]:
            nv[0, :, :] = nv[-2, :, :]
            nv[-1, :, :] = nv[1, :, :]
        return nv


class RotorSequence(_Sequence):
    """The rotor: 192x128x192, the cylinder case's curvilinear grid (tanh
    beta 2 in eta, amplitude 0.05, periodic x), a 3-rod rotor (radius 3
    cells, length 30 cells) rotating 2 degrees per step about a z-axis hub at
    the domain centre, Fourier fluxes advected 0.5 cells per step in x."""

    def __init__(self, nx=192, ny=128, nz=192, seed=1004, amp=0.05, device="cuda", n_theta=32):
        coor = CF._nodes(nx, ny, nz, lambda e: CF._tanh_stretch(e, 2.0), amp)
        super().__init__(nx, ny, nz, coor, seed, device)
        self.h = 1.0 / nz
        self.n_theta = n_theta

    def bodies(self, step):
        return CF.rotor_surfaces(centre=(0.5, 0.5, 0.5), angle_deg=2.0 * step, rods=3, radius=3 * self.h,
                                 length=30 * self.h, hub=0.0, n_theta=self.n_theta, n_len=30)


class TowerSequence(_Sequence):
    """The towers case (256x192x256, geometric 1.03 wall stretching,
    amplitude 0.02, periodic x and z, 3x2 towers of radius 0.02 spanning the
    height) as a sequence: static towers, Fourier fluxes advected 0.5 cells
    per step in x."""

    periodic = (0, 0, 0, 1, 0, 1)
    moving = False

    def __init__(self, nx=256, ny=192, nz=256, seed=1003, amp=0.02, ratio=1.03, device="cuda", n_theta=64):
        yc = CF._geometric(ny, ratio)
        coor = CF._nodes(nx, ny, nz, lambda e: np.interp(e, np.arange(ny + 1) / ny, yc), amp, physical=True)
        super().__init__(nx, ny, nz, coor, seed, device)
        self.n_theta = n_theta

    def bodies(self, step):
        return CF.tower_surfaces(radius=0.02, y0=-0.05, height=1.1, n_theta=self.n_theta, n_len=4)


class FarmSequence(_Sequence):
    """The wind farm: 512x256x512, geometric 1.02 wall stretching,
    amplitude 0.02, periodic x and z; a 4x3 array of towers (the towers
    case's radius 0.02 and 0.25 streamwise spacing, 0.3 spanwise, filling the
    domain) from below the wall to the hub height 0.5, each carrying a 3-rod
    rotor (rod radius 3 cells, length 0.08) at its top that rotates 2 degrees
    per step about the z axis, as the rotor case's does; Fourier fluxes
    advected 0.5 cells per step in x."""

    periodic = (0, 0, 0, 1, 0, 1)
    moving = True
    XS = (0.125, 0.375, 0.625, 0.875)
    ZS = (0.2, 0.5, 0.8)
    HUB = 0.5

    def __init__(self, nx=512, ny=256, nz=512, seed=1005, amp=0.02, ratio=1.02, device="cuda", n_theta=32):
        yc = CF._geometric(ny, ratio)
        coor = CF._nodes(nx, ny, nz, lambda e: np.interp(e, np.arange(ny + 1) / ny, yc), amp, physical=True)
        super().__init__(nx, ny, nz, coor, seed, device)
        self.n_theta = n_theta
        self.h = 1.0 / nx

    def bodies(self, step):
        out = []
        for x0 in self.XS:
            for z0 in self.ZS:
                out.append(CF.rod_surface((x0, -0.05, z0), (0.0, 1.0, 0.0), self.HUB + 0.05, 0.02, self.n_theta, 4))
                out += CF.rotor_surfaces(centre=(x0, self.HUB, z0), angle_deg=2.0 * step, rods=3,
                                         radius=3 * self.h, length=0.08, hub=0.0, n_theta=16, n_len=12)
        return out
