"""Synthetic wind-farm-like inputs for the pressure-Poisson solve.

The reference is benchmarked on no public dataset.  These generators build
seeded stand-ins for the five solver configurations (channel, curvilinear
cylinder, wind-farm towers, rotating rotor) in the reference's own data
layout: node coordinates, immersed-boundary flags ``nvert`` (0 fluid, 1 IB
node, 3 solid, as written by ibm_search_advanced, Source/ibm.c:514-522) and
contravariant face fluxes ``ucont`` (Cmpnts AoS), all as PETSc-DA-shaped
``[mz][my][mx]`` arrays with one boundary layer on each side
(Source/init.c:157-161: the DA holds IM+1 points for IM nodes).

The domain is the unit cube (the configurations give no lengths).  Seeds
follow ``numpy.random.default_rng(1000 + config)``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Case:
    name: str
    nx: int
    ny: int
    nz: int
    periodic: tuple  # (i, j, k, ii, jj, kk) flags, reference globals
    coor: np.ndarray  # [mz][my][mx][3] node coordinates (node (i,j,k) for i<=nx)
    nvert: np.ndarray  # [mz][my][mx]
    ucont: np.ndarray  # [mz][my][mx][3]
    dt: float = 1.0
    st: float = 1.0
    coeff: float = 1.0
    extra: dict = field(default_factory=dict)

    def set_periodic(self, periodic):
        """Change the periodic flags and re-sync the nvert ghost layers."""
        self.periodic = tuple(periodic)
        self.nvert = sync_periodic_ghosts(self.nvert, self.periodic)

    def __post_init__(self):
        self.nvert = sync_periodic_ghosts(self.nvert, self.periodic)

    @property
    def dims(self):
        return (self.nx + 2, self.ny + 2, self.nz + 2)

    @property
    def cells(self):
        return self.nx * self.ny * self.nz


def _tanh_stretch(eta, beta):
    return 0.5 * (1.0 + np.tanh(beta * (2.0 * eta - 1.0)) / np.tanh(beta))


def _geometric(n, ratio):
    j = np.arange(n + 1, dtype=np.float64)
    return (ratio ** j - 1.0) / (ratio ** n - 1.0)


def _nodes(nx, ny, nz, yfun, amp, physical=False):
    """Node coordinates on the DA-shaped array; the last layer stays zero.

    x = xi + amp sin(2 pi e) sin(2 pi zeta), y = ys(eta) + amp sin(2 pi zeta)
    sin(2 pi xi), z = zeta + amp sin(2 pi xi) sin(2 pi e), where e is the
    computational coordinate eta, or with `physical` the stretched height
    ys(eta) itself, so that the perturbation is smooth in physical space and
    the wall-resolving cells stay unskewed (terrain-following grid)."""
    xi = np.arange(nx + 1) / nx
    et = np.arange(ny + 1) / ny
    ze = np.arange(nz + 1) / nz
    Z, Y, X = np.meshgrid(ze, et, xi, indexing="ij")  # [k][j][i]
    ys = yfun(Y)
    E = ys if physical else Y
    tp = 2.0 * np.pi
    coor = np.zeros((nz + 2, ny + 2, nx + 2, 3))
    coor[: nz + 1, : ny + 1, : nx + 1, 0] = X + amp * np.sin(tp * E) * np.sin(tp * Z)
    coor[: nz + 1, : ny + 1, : nx + 1, 1] = ys + amp * np.sin(tp * Z) * np.sin(tp * X)
    coor[: nz + 1, : ny + 1, : nx + 1, 2] = Z + amp * np.sin(tp * X) * np.sin(tp * E)
    return coor


def cell_centres(coor):
    """Interior cell centres (average of the 8 nodes), shape [nz][ny][nx][3]."""
    c = coor[:-1, :-1, :-1]
    return 0.125 * (c[1:, 1:, 1:] + c[1:, :-1, 1:] + c[:-1, 1:, 1:] + c[:-1, :-1, 1:]
                    + c[1:, 1:, :-1] + c[1:, :-1, :-1] + c[:-1, 1:, :-1] + c[:-1, :-1, :-1])


def classify(inside):
    """nvert from an inside/outside flag on interior cells: 3 inside, 1 for
    cells whose 27-neighbourhood touches an inside cell (the dilation of
    Source/ibm.c:326-348 followed by the 4->3 / 2->1 mapping of :514-522)."""
    nz, ny, nx = inside.shape
    nv = np.zeros((nz + 2, ny + 2, nx + 2))
    ins = np.zeros_like(nv, dtype=bool)
    ins[1:-1, 1:-1, 1:-1] = inside
    near = np.zeros_like(ins)
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                near |= np.roll(np.roll(np.roll(ins, dk, 0), dj, 1), di, 2)
    nv[near] = 1.0
    nv[ins] = 3.0
    nv[0, :, :] = nv[-1, :, :] = 0.0
    nv[:, 0, :] = nv[:, -1, :] = 0.0
    nv[:, :, 0] = nv[:, :, -1] = 0.0
    return nv


def sync_periodic_ghosts(nvert, periodic):
    """Give the boundary layer of each periodic direction its partner cells'
    values (index 0 <- m-2, m-1 <- 1), as the ghost points of a periodic DA
    hold them.  The operator reads nvert at these ghosts
    (Source/poisson.c:1167-1561), so this keeps blanking consistent across
    the periodic seam."""
    nv = nvert.copy()
    per = [periodic[q] or periodic[q + 3] for q in range(3)]
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


def _mask_faces(ucont, nvert):
    """Zero every face flux touching a blanked cell (nvert > 0.1)."""
    b = nvert > 0.1
    u = ucont.copy()
    bx = b[:, :, :-1] | b[:, :, 1:]
    u[:, :, :-1, 0][bx] = 0.0
    by = b[:, :-1, :] | b[:, 1:, :]
    u[:, :-1, :, 1][by] = 0.0
    bz = b[:-1, :, :] | b[1:, :, :]
    u[:-1, :, :, 2][bz] = 0.0
    return u


def _uniform_ucont(rng, nx, ny, nz):
    u = np.zeros((nz + 2, ny + 2, nx + 2, 3))
    u[...] = rng.uniform(-1.0, 1.0, size=u.shape)
    return u


def _fourier_ucont(rng, nx, ny, nz, modes=32, kmax=8, noise=0.1, shift=0.0):
    """Sum of `modes` random Fourier modes with integer wavevectors
    1 <= |k| <= kmax, amplitudes N(0,1)/|k|, per velocity component,
    evaluated at face positions in computational space, plus uniform
    noise.  `shift` advects the pattern in x by that many cells."""
    u = np.zeros((nz + 2, ny + 2, nx + 2, 3))
    ii = np.arange(nx + 2, dtype=np.float64)
    jj = np.arange(ny + 2, dtype=np.float64)
    kk = np.arange(nz + 2, dtype=np.float64)
    for comp in range(3):
        fx = (ii - (0.0 if comp == 0 else 0.5) - shift) / nx
        fy = (jj - (0.0 if comp == 1 else 0.5)) / ny
        fz = (kk - (0.0 if comp == 2 else 0.5)) / nz
        acc = np.zeros((nz + 2, ny + 2, nx + 2))
        n = 0
        while n < modes:
            kv = rng.integers(-kmax, kmax + 1, size=3)
            kn = np.sqrt((kv ** 2).sum())
            if kn < 1 or kn > kmax:
                continue
            a = rng.normal() / kn
            ph = rng.uniform(0, 2 * np.pi)
            acc += a * np.cos(2 * np.pi * (kv[2] * fz[:, None, None] + kv[1] * fy[None, :, None]
                                           + kv[0] * fx[None, None, :]) + ph)
            n += 1
        u[..., comp] = acc
    u += rng.uniform(-noise, noise, size=u.shape)
    return u


def channel(nx=64, ny=64, nz=64, seed=1001):
    """The channel: Cartesian, tanh wall stretching (beta 1.5) in y,
    periodic x and z (periodic DA), Neumann y walls, no body."""
    rng = np.random.default_rng(seed)
    coor = _nodes(nx, ny, nz, lambda e: _tanh_stretch(e, 1.5), 0.0)
    nvert = np.zeros((nz + 2, ny + 2, nx + 2))
    ucont = _uniform_ucont(rng, nx, ny, nz)
    return Case("channel", nx, ny, nz, (0, 0, 0, 1, 0, 1), coor, nvert, ucont)


def cylinder(nx=128, ny=96, nz=128, seed=1002, amp=0.05):
    """The cylinder case: curvilinear grid (amplitude 0.05, tanh beta 2 in eta),
    periodic x, vertical cylinder of radius 0.1 at the domain centre."""
    rng = np.random.default_rng(seed)
    coor = _nodes(nx, ny, nz, lambda e: _tanh_stretch(e, 2.0), amp)
    cc = cell_centres(coor)
    r2 = (cc[..., 0] - 0.5) ** 2 + (cc[..., 2] - 0.5) ** 2
    nvert = classify(r2 < 0.1 ** 2)
    ucont = _mask_faces(_uniform_ucont(rng, nx, ny, nz), nvert)
    return Case("cylinder", nx, ny, nz, (0, 0, 0, 1, 0, 0), coor, nvert, ucont)


def towers(nx=256, ny=192, nz=256, seed=1003, amp=0.02, ratio=1.03, array=(3, 2),
           radius=0.02, physical=True):
    """The towers: wind-farm-like grid, geometric wall stretching (ratio 1.03)
    in y, perturbation amplitude 0.02, periodic x and z, a 3x2 array of
    vertical tower cylinders (radius 0.02, 0.25 streamwise and 0.3 spanwise
    spacing); Fourier-mode Ucont plus noise."""
    rng = np.random.default_rng(seed)
    yc = _geometric(ny, ratio)
    coor = _nodes(nx, ny, nz, lambda e: np.interp(e, np.arange(ny + 1) / ny, yc), amp, physical=physical)
    cc = cell_centres(coor)
    inside = np.zeros(cc.shape[:3], dtype=bool)
    ax, az = array
    xs = 0.5 + 0.25 * (np.arange(ax) - (ax - 1) / 2)
    zs = 0.5 + 0.3 * (np.arange(az) - (az - 1) / 2)
    for x0 in xs:
        for z0 in zs:
            inside |= (cc[..., 0] - x0) ** 2 + (cc[..., 2] - z0) ** 2 < radius ** 2
    nvert = classify(inside)
    ucont = _mask_faces(_fourier_ucont(rng, nx, ny, nz), nvert)
    return Case("towers", nx, ny, nz, (0, 0, 0, 1, 0, 1), coor, nvert, ucont)


def rotor_mask(coor, centre, angle_deg, rods=3, rod_radius_cells=3, rod_length_cells=30,
               hub_axis=2):
    """Inside flags of a rotor of `rods` cylindrical rods (radius and length
    in cells of the local spacing) on a hub at `centre`, rotated by
    `angle_deg` about the z axis."""
    cc = cell_centres(coor)
    h = 1.0 / cc.shape[2]
    rr = rod_radius_cells * h
    L = rod_length_cells * h
    inside = np.zeros(cc.shape[:3], dtype=bool)
    d = cc - np.asarray(centre)[None, None, None, :]
    for r in range(rods):
        th = np.deg2rad(angle_deg + 360.0 * r / rods)
        ax = np.array([np.cos(th), np.sin(th), 0.0])
        t = d @ ax
        perp = d - t[..., None] * ax
        inside |= (t >= 0) & (t <= L) & ((perp ** 2).sum(-1) < rr ** 2)
    return inside


def rotor(nx=192, ny=128, nz=192, step=0, seed=1004, amp=0.05):
    """The rotor: the cylinder case's geometry with a 3-rod rotor (radius 3 cells,
    length 30 cells) rotating 2 degrees per step about a z-axis hub at the
    domain centre; Fourier RHS advected 0.5 cells per step in x."""
    rng = np.random.default_rng(seed)
    coor = _nodes(nx, ny, nz, lambda e: _tanh_stretch(e, 2.0), amp)
    inside = rotor_mask(coor, (0.5, 0.5, 0.5), 2.0 * step)
    nvert = classify(inside)
    ucont = _mask_faces(_fourier_ucont(rng, nx, ny, nz, shift=0.5 * step), nvert)
    return Case(f"rotor_step{step}", nx, ny, nz, (0, 0, 0, 1, 0, 0), coor, nvert, ucont,
                extra={"step": step})


def rod_surface(base, axis, length, radius, n_theta=24, n_len=8, up=(0.0, 0.0, 1.0)):
    """Closed triangulated circular rod (the reference reads such bodies as
    UCD surfaces, Source/ibm_io.c): rings of `n_theta` vertices at `n_len`+1
    stations from `base` along the unit `axis`, closed by two fan caps.
    Returns (xyz[n_v, 3], tri[n_elmt, 3]) with outward-facing windings."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    u = np.cross(a, up)
    if np.linalg.norm(u) < 1e-12:
        u = np.cross(a, (1.0, 0.0, 0.0))
    u /= np.linalg.norm(u)
    w = np.cross(a, u)
    th = 2.0 * np.pi * np.arange(n_theta) / n_theta
    ring = radius * (np.cos(th)[:, None] * u + np.sin(th)[:, None] * w)
    base = np.asarray(base, np.float64)
    pts = [base + s * length * a + ring for s in np.arange(n_len + 1) / n_len]
    xyz = np.concatenate(pts + [base[None], (base + length * a)[None]])
    c0, c1 = len(xyz) - 2, len(xyz) - 1
    tri = []
    for s in range(n_len):
        for t in range(n_theta):
            p00, p01 = s * n_theta + t, s * n_theta + (t + 1) % n_theta
            p10, p11 = p00 + n_theta, p01 + n_theta
            tri += [(p00, p01, p11), (p00, p11, p10)]
    top = n_len * n_theta
    for t in range(n_theta):
        tri.append((c0, (t + 1) % n_theta, t))
        tri.append((c1, top + t, top + (t + 1) % n_theta))
    return xyz, np.asarray(tri, np.int32)


def tower_surfaces(array=(3, 2), radius=0.02, height=0.6, n_theta=24, n_len=12, y0=0.0):
    """Closed vertical tower cylinders at the positions of the towers case
    (0.25 streamwise, 0.3 spanwise spacing about the domain centre), from
    y = `y0` to `y0 + height`: one surface per tower (body ibi)."""
    ax, az = array
    xs = 0.5 + 0.25 * (np.arange(ax) - (ax - 1) / 2)
    zs = 0.5 + 0.3 * (np.arange(az) - (az - 1) / 2)
    return [rod_surface((x0, y0, z0), (0.0, 1.0, 0.0), height, radius, n_theta, n_len)
            for x0 in xs for z0 in zs]


def rotor_surfaces(centre=(0.5, 0.5, 0.5), angle_deg=0.0, rods=3, radius=0.03, length=0.25, hub=0.04,
                   n_theta=16, n_len=10):
    """The rotor of the rotor case as closed surfaces, one per rod (body
    ibi): rods of `radius` and `length` in the x-y plane starting `hub` from
    the centre, rotated by `angle_deg` about the z axis."""
    out = []
    c = np.asarray(centre, np.float64)
    for r in range(rods):
        th = np.deg2rad(angle_deg + 360.0 * r / rods)
        a = np.array([np.cos(th), np.sin(th), 0.0])
        out.append(rod_surface(c + hub * a, a, length, radius, n_theta, n_len))
    return out


CONFIGS = {
    "c1": channel,
    "c2": cylinder,
    "c3": towers,
    "c4": rotor,
}


def make(name, **kw):
    return CONFIGS[name](**kw)
