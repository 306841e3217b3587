"""ctypes front end of the CPU oracle (oracle/vfs_oracle.c, oracle/mg_solver.c).

TEST INFRASTRUCTURE ONLY: used by tests/, by bench.py's cpu_baseline and
reference arm, and by __graft_entry__.smoke() as the checker.  The product
never imports it.  Parity unpinned: see the header of oracle/vfs_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = [os.path.join(HERE, "vfs_oracle.c"), os.path.join(HERE, "mg_solver.c"),
           os.path.join(HERE, "ibm_oracle.c"), os.path.join(HERE, "ibm_interp_oracle.c")]


def build(force=False):
    """Compile the oracle with IEEE source-order evaluation (no contraction),
    and, where the reference's sources are present, the reference's own
    pressure-Poisson units against the PETSc/HYPRE/MPI stand-in
    (oracle/_ref, the oracle's pin; see reference.py)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES + [os.path.join(HERE, "vfs_oracle.h")])
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB_PATH,
               *SOURCES, "-lm"]
        subprocess.check_call(cmd)
    import reference
    reference.build(force=force)
    return LIB_PATH


class Dims(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("mz", C.c_int),
                ("i_periodic", C.c_int), ("j_periodic", C.c_int), ("k_periodic", C.c_int),
                ("ii_periodic", C.c_int), ("jj_periodic", C.c_int), ("kk_periodic", C.c_int)]


METRIC_FIELDS = ["cent", "csi", "eta", "zet", "aj", "icsi", "ieta", "izet", "iaj",
                 "jcsi", "jeta", "jzet", "jaj", "kcsi", "keta", "kzet", "kaj"]
VECTOR_FIELDS = {"cent", "csi", "eta", "zet", "icsi", "ieta", "izet", "jcsi", "jeta", "jzet",
                 "kcsi", "keta", "kzet"}


class Metrics(C.Structure):
    _fields_ = [(f, C.POINTER(C.c_double)) for f in METRIC_FIELDS]


class SolveOpts(C.Structure):
    _fields_ = [("max_it", C.c_int), ("restart", C.c_int), ("rtol", C.c_double),
                ("nu1", C.c_int), ("nu2", C.c_int), ("omega", C.c_double),
                ("threads", C.c_int), ("coarsest_max", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double),
                ("setup_ms", C.c_double), ("solve_ms", C.c_double), ("levels", C.c_int)]


class IbmNode(C.Structure):
    """One IB node's interpolation record (or_ibm_node)."""
    _fields_ = [("i", C.c_int), ("j", C.c_int), ("k", C.c_int), ("cell", C.c_int),
                ("pmin", C.c_double * 3), ("d_s", C.c_double), ("cs", C.c_double * 3),
                ("ip", C.c_int * 3), ("jp", C.c_int * 3), ("kp", C.c_int * 3),
                ("cr", C.c_double * 3), ("d_i", C.c_double), ("imode", C.c_int), ("status", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        dp, ip = P(C.c_double), P(C.c_int)
        L.or_form_metrics.argtypes = [P(Dims), dp, P(Metrics)]
        L.or_setup_lidx2.argtypes = [P(Dims), dp, ip]
        L.or_setup_lidx2.restype = C.c_int
        L.or_poisson_lhs.argtypes = [P(Dims), dp, P(Metrics), C.c_int, C.c_int, ip, ip, dp, ip]
        L.or_poisson_lhs.restype = C.c_int
        L.or_poisson_rhs2_hypre.argtypes = [P(Dims), dp, ip, dp, C.c_double, C.c_double, C.c_double, dp]
        L.or_poisson_rhs2.argtypes = [P(Dims), dp, ip, dp, dp, C.c_double, C.c_double, C.c_double, C.c_int, dp]
        L.or_set_levelset.argtypes = [dp, dp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.or_volume_flux.argtypes = [P(Dims), dp, dp, dp, dp, dp, C.c_int, C.c_double, dp]
        L.or_volume_flux0.argtypes = [P(Dims), dp, dp, dp, dp, dp, C.c_int, dp]
        L.or_contra2cart.argtypes = [P(Dims), dp, dp, dp, dp, dp, dp, C.c_int]
        L.or_remove_nullspace_scale.argtypes = [P(Dims), dp, ip, dp, dp, C.c_int]
        L.or_remove_nullspace.argtypes = [P(Dims), dp, ip, dp, C.c_int]
        L.or_fully_blocked.argtypes = [P(Dims), dp, ip]
        L.or_fully_blocked.restype = C.c_int
        L.or_nullspace_original.argtypes = [P(Dims), dp, ip, C.c_int, dp]
        L.or_convert_phi2_phi.argtypes = [P(Dims), dp, dp, dp]
        L.or_update_pressure.argtypes = [P(Dims), dp, dp, dp]
        L.or_projection.argtypes = [P(Dims), dp, dp, P(Metrics), C.c_double, C.c_double, C.c_double, dp]
        L.or_divergence.argtypes = [P(Dims), dp, dp, dp]
        L.or_divergence.restype = C.c_double
        L.or_my_nvert_restriction.argtypes = [P(Dims), P(Dims), C.c_int, C.c_int, C.c_int, dp, dp]
        L.or_my_restriction.argtypes = [P(Dims), P(Dims), C.c_int, C.c_int, C.c_int, dp, dp, dp, dp]
        L.or_my_interpolation.argtypes = [P(Dims), P(Dims), C.c_int, C.c_int, C.c_int, dp, dp, dp, dp]
        L.or_mg_create.argtypes = [P(Dims), dp, dp, P(Metrics), P(SolveOpts)]
        L.or_mg_create.restype = C.c_void_p
        L.or_mg_solve.argtypes = [C.c_void_p, dp, dp, P(SolveOpts), P(SolveStats)]
        L.or_mg_solve.restype = C.c_int
        L.or_mg_vcycle.argtypes = [C.c_void_p, dp, dp, C.c_int, C.c_int, C.c_double]
        L.or_mg_level_info.argtypes = [C.c_void_p, C.c_int, ip]
        L.or_mg_level_info.restype = C.c_int
        L.or_mg_destroy.argtypes = [C.c_void_p]
        L.or_mg_set_smoother.argtypes = [C.c_int]
        L.or_glibc_rand_first.argtypes = [C.c_uint]
        L.or_glibc_rand_first.restype = C.c_uint
        L.or_triangle_normals.argtypes = [C.c_int, ip, dp, dp, dp, dp]
        L.or_ibm_search.argtypes = [P(Dims), dp, C.c_int, C.c_int, dp, dp, dp, C.c_int, ip, ip, dp, C.c_int]
        L.or_ibm_search.restype = C.c_int
        L.or_ibm_mark.argtypes = [P(Dims), dp, C.c_int, C.c_int, dp, dp, dp, C.c_int, ip, dp, C.c_int]
        L.or_ibm_mark.restype = C.c_int
        L.or_ibm_finish.argtypes = [P(Dims), ip, dp]
        L.or_bounding_sphere.argtypes = [C.c_int, ip, dp, dp, dp, dp, dp]
        L.or_ibm_nodes.argtypes = [P(Dims), dp, dp, C.c_int, dp, dp, dp, C.c_int, ip, P(IbmNode), C.c_int]
        L.or_ibm_nodes.restype = C.c_int
        L.or_ibm_interpolate.argtypes = [P(Dims), dp, P(IbmNode), C.c_int, ip, dp, dp, dp, dp, dp, dp, dp, ip,
                                         C.c_int, dp, dp, dp]
        L.or_ib_bc.argtypes = [P(Dims), dp, dp, dp, dp, ip, C.c_int, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int))


def dims(mx, my, mz, periodic):
    return Dims(mx, my, mz, *[int(p) for p in periodic])


def dims_of(case):
    mx, my, mz = case.dims
    return dims(mx, my, mz, case.periodic)


def form_metrics(d, coor):
    shape = (d.mz, d.my, d.mx)
    out = {f: np.zeros(shape + ((3,) if f in VECTOR_FIELDS else ()), dtype=np.float64)
           for f in METRIC_FIELDS}
    m = metrics_struct(out)
    lib().or_form_metrics(C.byref(d), _dp(np.ascontiguousarray(coor)), C.byref(m))
    return out


def metrics_struct(met):
    return Metrics(*[_dp(met[f]) for f in METRIC_FIELDS])


def poisson_lhs(d, nvert, met, scale_by_aj=False, apply_filter=True):
    n = d.mx * d.my * d.mz
    gid = np.zeros(n, np.int32)
    rt = np.zeros(n, np.int32)
    vol = np.zeros(n * 19)
    col = np.zeros(n * 19, np.int32)
    m = metrics_struct(met)
    ndof = lib().or_poisson_lhs(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), C.byref(m),
                                int(scale_by_aj), int(apply_filter), _ip(gid), _ip(rt), _dp(vol), _ip(col))
    shape = (d.mz, d.my, d.mx)
    return dict(ndof=ndof, gid=gid.reshape(shape), rowtype=rt.reshape(shape),
                vol=vol.reshape(shape + (19,)), col=col.reshape(shape + (19,)))


def csr(lhs):
    """Assemble the reference's matrix (MatSetValues INSERT semantics) as CSR."""
    import scipy.sparse as sp
    rt = lhs["rowtype"].ravel()
    gid = lhs["gid"].ravel()
    vol = lhs["vol"].reshape(-1, 19)
    col = lhs["col"].reshape(-1, 19)
    rows, cols, vals = [], [], []
    cells = np.nonzero(rt > 0)[0]
    for s in range(19):
        c = col[cells, s]
        keep = c >= 0
        rows.append(gid[cells][keep])
        cols.append(c[keep])
        vals.append(vol[cells, s][keep])
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    vals = np.concatenate(vals)
    n = lhs["ndof"]
    # INSERT semantics: a later slot with the same column replaces the value
    order = np.lexsort((np.arange(len(rows)), cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    last = np.ones(len(rows), bool)
    last[:-1] = (rows[1:] != rows[:-1]) | (cols[1:] != cols[:-1])
    return sp.csr_matrix((vals[last], (rows[last], cols[last])), shape=(n, n))


def rhs(d, nvert, gid, ucont, aj, dt=1.0, st=1.0, coeff=1.0, bctype3=0):
    n = int(gid.max()) + 1
    b = np.zeros(max(n, 1))
    g = np.ascontiguousarray(gid, np.int32).ravel()
    nv = np.ascontiguousarray(nvert, np.float64)
    lib().or_poisson_rhs2_hypre(C.byref(d), _dp(nv), _ip(g), _dp(np.ascontiguousarray(ucont)), dt, st, coeff, _dp(b))
    lib().or_remove_nullspace_scale(C.byref(d), _dp(nv), _ip(g), _dp(np.ascontiguousarray(aj)), _dp(b), bctype3)
    return b[:n]


def rhs2(d, nvert, gid, ucont, aj, poisson=0, dt=1.0, st=1.0, coeff=1.0):
    """PoissonRHS2 (the -poisson 0 / -1 right-hand side), one entry per dof."""
    n = int(gid.max()) + 1
    b = np.zeros(max(n, 1))
    lib().or_poisson_rhs2(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)),
                          _ip(np.ascontiguousarray(gid, np.int32).ravel()), _dp(np.ascontiguousarray(ucont)),
                          _dp(np.ascontiguousarray(aj, np.float64)), dt, st, coeff, int(poisson), _dp(b))
    return b[:n]


_ls_keep = None


def set_levelset(rho=None, level=None, bctype=(0, 0, 0, 0, 0, 0)):
    """Level-set context of poisson_lhs / projection (rho None: off)."""
    global _ls_keep
    if rho is None:
        _ls_keep = None
        lib().or_set_levelset(None, None, 0, 0, 0, 0)
        return
    r = np.ascontiguousarray(rho, np.float64)
    lv = np.ascontiguousarray(level if level is not None else np.zeros_like(r), np.float64)
    _ls_keep = (r, lv)
    lib().or_set_levelset(_dp(r), _dp(lv), 1, int(bctype[3]), int(bctype[4]), int(bctype[5]))


def volume_flux(d, nvert, met, ucont, flg=0, flux_intp_sum=0.0):
    """VolumeFlux (immersed == 1); returns (corrected ucont, flux, area)."""
    u = np.ascontiguousarray(ucont, np.float64).copy()
    out = np.zeros(2)
    lib().or_volume_flux(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), _dp(met["csi"]),
                         _dp(met["eta"]), _dp(met["zet"]), _dp(u), int(flg), float(flux_intp_sum), _dp(out))
    return u, out[0], out[1]


def volume_flux0(d, nvert, met, ucont, immersed=0):
    """VolumeFlux, the overload for immersed != 1, 2; returns (ucont, flux, area)."""
    u = np.ascontiguousarray(ucont, np.float64).copy()
    out = np.zeros(2)
    lib().or_volume_flux0(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), _dp(met["csi"]),
                          _dp(met["eta"]), _dp(met["zet"]), _dp(u), int(immersed), _dp(out))
    return u, out[0], out[1]


def contra2cart(d, nvert, met, ucont, ucat=None, zero_solid=True):
    """Contra2Cart's change of basis; returns ucat."""
    out = np.zeros((d.mz, d.my, d.mx, 3)) if ucat is None else np.ascontiguousarray(ucat, np.float64).copy()
    lib().or_contra2cart(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), _dp(met["csi"]),
                         _dp(met["eta"]), _dp(met["zet"]), _dp(np.ascontiguousarray(ucont, np.float64)), _dp(out),
                         int(zero_solid))
    return out


def rhs_raw(d, nvert, gid, ucont, dt=1.0, st=1.0, coeff=1.0):
    n = int(gid.max()) + 1
    b = np.zeros(max(n, 1))
    g = np.ascontiguousarray(gid, np.int32).ravel()
    lib().or_poisson_rhs2_hypre(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), _ip(g),
                                _dp(np.ascontiguousarray(ucont)), dt, st, coeff, _dp(b))
    return b[:n]


def remove_nullspace(d, nvert, gid, phi2, bctype3=0):
    p = np.ascontiguousarray(phi2, np.float64).copy()
    lib().or_remove_nullspace(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)),
                              _ip(np.ascontiguousarray(gid, np.int32).ravel()), _dp(p), bctype3)
    return p


def fully_blocked(d, nvert):
    """FullyBlocked: (multi, ksk[my, mx]) -- the first blocked k of every
    interior column (-1 where none)."""
    ksk = np.zeros((d.my, d.mx), np.int32)
    multi = lib().or_fully_blocked(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), _ip(ksk))
    return bool(multi), ksk


def nullspace_original(d, nvert, x, ksk=None, multi=None):
    """PoissonNullSpaceFunction_original on a DA-layout copy of x."""
    if ksk is None:
        multi, ksk = fully_blocked(d, nvert)
    out = np.ascontiguousarray(x, np.float64).copy()
    lib().or_nullspace_original(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)),
                                _ip(np.ascontiguousarray(ksk, np.int32)), int(bool(multi)), _dp(out))
    return out


def convert_phi2_phi(d, nvert, phi2):
    phi = np.zeros((d.mz, d.my, d.mx))
    lib().or_convert_phi2_phi(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)),
                              _dp(np.ascontiguousarray(phi2, np.float64)), _dp(phi))
    return phi


def update_pressure(d, nvert, p, phi):
    p = np.ascontiguousarray(p, np.float64).copy()
    phi = np.ascontiguousarray(phi, np.float64).copy()
    lib().or_update_pressure(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), _dp(p), _dp(phi))
    return p, phi


def projection(d, nvert, phi, met, ucont, dt=1.0, st=1.0, coeff=1.0):
    u = np.ascontiguousarray(ucont, np.float64).copy()
    m = metrics_struct(met)
    lib().or_projection(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)),
                        _dp(np.ascontiguousarray(phi, np.float64)), C.byref(m), dt, st, coeff, _dp(u))
    return u


def divergence(d, nvert, ucont, aj):
    return lib().or_divergence(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)),
                               _dp(np.ascontiguousarray(ucont, np.float64)), _dp(np.ascontiguousarray(aj)))


def nvert_restriction(dh, dc, isc, jsc, ksc, nvert_h):
    out = np.zeros((dc.mz, dc.my, dc.mx))
    lib().or_my_nvert_restriction(C.byref(dh), C.byref(dc), isc, jsc, ksc,
                                  _dp(np.ascontiguousarray(nvert_h, np.float64)), _dp(out))
    return out


def restriction(dc, df, isc, jsc, ksc, nvert_c, nvert_f, xf):
    out = np.zeros((dc.mz, dc.my, dc.mx))
    lib().or_my_restriction(C.byref(dc), C.byref(df), isc, jsc, ksc, _dp(np.ascontiguousarray(nvert_c)),
                            _dp(np.ascontiguousarray(nvert_f)), _dp(np.ascontiguousarray(xf)), _dp(out))
    return out


def interpolation(df, dc, isc, jsc, ksc, nvert_f, nvert_c, xc):
    out = np.zeros((df.mz, df.my, df.mx))
    lib().or_my_interpolation(C.byref(df), C.byref(dc), isc, jsc, ksc, _dp(np.ascontiguousarray(nvert_f)),
                              _dp(np.ascontiguousarray(nvert_c)), _dp(np.ascontiguousarray(xc)), _dp(out))
    return out


def glibc_rand_first(seed):
    return lib().or_glibc_rand_first(seed)


def ibm_search(d, cent, surface, nvert=None, ibi=0, bctype=(0, 0, 0, 0, 0, 0), max_tries=64):
    """ibm_search_advanced for one body; `surface` = (xyz[n_v,3], tris[n_elmt,3] 0-based)."""
    xyz, tris = surface
    x = np.ascontiguousarray(xyz[:, 0], np.float64)
    y = np.ascontiguousarray(xyz[:, 1], np.float64)
    z = np.ascontiguousarray(xyz[:, 2], np.float64)
    nv = np.ascontiguousarray(tris, np.int32).ravel()
    out = np.zeros((d.mz, d.my, d.mx)) if nvert is None else np.ascontiguousarray(nvert, np.float64).copy()
    bc = np.ascontiguousarray(bctype, np.int32)
    failed = lib().or_ibm_search(C.byref(d), _dp(np.ascontiguousarray(cent, np.float64)), ibi, len(x), _dp(x),
                                 _dp(y), _dp(z), len(nv) // 3, _ip(nv), _ip(bc), _dp(out), max_tries)
    return out, failed


def set_smoother(zebra):
    """CPU solver smoother: 1 zebra j-line Gauss-Seidel over checkerboard
    columns (the GPU V-cycle's), 2 over k-planes, 0 damped line Jacobi."""
    lib().or_mg_set_smoother(int(zebra))


class MGSolver:
    """FP64 FGMRES + geometric V-cycle on the CPU (timed CPU baseline)."""

    def __init__(self, d, coor, nvert, met=None, threads=0, coarsest_max=128):
        self.d = d
        self.opts = SolveOpts(max_it=200, restart=30, rtol=1e-8, nu1=2, nu2=2, omega=0.8,
                              threads=threads, coarsest_max=coarsest_max)
        self._met = met
        m = C.byref(metrics_struct(met)) if met is not None else None
        self.h = lib().or_mg_create(C.byref(d), _dp(np.ascontiguousarray(coor)),
                                    _dp(np.ascontiguousarray(nvert, np.float64)), m, C.byref(self.opts))

    def levels(self):
        v = np.zeros(7, np.int32)
        n = lib().or_mg_level_info(self.h, 0, _ip(v))
        out = []
        for li in range(n):
            lib().or_mg_level_info(self.h, li, _ip(v))
            out.append(tuple(int(x) for x in v))
        return out

    def solve(self, b_da, x0_da=None, rtol=1e-8, max_it=200, restart=30, nu1=2, nu2=2, omega=0.8):
        self.opts.rtol, self.opts.max_it, self.opts.restart = rtol, max_it, restart
        self.opts.nu1, self.opts.nu2, self.opts.omega = nu1, nu2, omega
        x = np.zeros((self.d.mz, self.d.my, self.d.mx)) if x0_da is None else np.ascontiguousarray(x0_da).copy()
        st = SolveStats()
        lib().or_mg_solve(self.h, _dp(np.ascontiguousarray(b_da)), _dp(x), C.byref(self.opts), C.byref(st))
        return x, st

    def vcycle(self, r_da, nu1=2, nu2=2, omega=0.8):
        z = np.zeros((self.d.mz, self.d.my, self.d.mx))
        lib().or_mg_vcycle(self.h, _dp(np.ascontiguousarray(r_da)), _dp(z), nu1, nu2, omega)
        return z

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_mg_destroy(self.h)
            self.h = None


def to_da(d, gid, v2):
    """Scatter a dof vector onto the DA layout (zero where there is no dof)."""
    out = np.zeros(d.mz * d.my * d.mx)
    g = gid.ravel()
    inner = np.zeros((d.mz, d.my, d.mx), bool)
    inner[1:-1, 1:-1, 1:-1] = True
    sel = inner.ravel() & (g >= 0)
    out[sel] = v2[g[sel]]
    return out.reshape(d.mz, d.my, d.mx)


def from_da(d, gid, v):
    g = gid.ravel()
    inner = np.zeros((d.mz, d.my, d.mx), bool)
    inner[1:-1, 1:-1, 1:-1] = True
    sel = inner.ravel() & (g >= 0)
    n = int(g.max()) + 1
    out = np.zeros(n)
    out[g[sel]] = v.ravel()[sel]
    return out


def _surface_arrays(surface):
    xyz, tris = surface
    x = np.ascontiguousarray(xyz[:, 0], np.float64)
    y = np.ascontiguousarray(xyz[:, 1], np.float64)
    z = np.ascontiguousarray(xyz[:, 2], np.float64)
    nv = np.ascontiguousarray(tris, np.int32).ravel()
    return x, y, z, nv


def ibm_mark(d, cent, surface, nvert=None, ibi=0, max_tries=64):
    """Classification and dilation of one body (4 inside, 2 IB node)."""
    x, y, z, nv = _surface_arrays(surface)
    out = np.zeros((d.mz, d.my, d.mx)) if nvert is None else np.ascontiguousarray(nvert, np.float64).copy()
    failed = lib().or_ibm_mark(C.byref(d), _dp(np.ascontiguousarray(cent, np.float64)), ibi, len(x), _dp(x),
                               _dp(y), _dp(z), len(nv) // 3, _ip(nv), _dp(out), max_tries)
    return out, failed


def ibm_finish(d, nvert, bctype=(0, 0, 0, 0, 0, 0)):
    out = np.ascontiguousarray(nvert, np.float64).copy()
    lib().or_ibm_finish(C.byref(d), _ip(np.ascontiguousarray(bctype, np.int32)), _dp(out))
    return out


def bounding_sphere(surface):
    x, y, z, nv = _surface_arrays(surface)
    ne = len(nv) // 3
    q = np.zeros((ne, 3))
    r = np.zeros(ne)
    lib().or_bounding_sphere(ne, _ip(nv), _dp(x), _dp(y), _dp(z), _dp(q), _dp(r))
    return q, r


def ibm_nodes(d, cent, nvert_marked, surface):
    """The IB nodes (cells marked 2) of one body with their records."""
    x, y, z, nv = _surface_arrays(surface)
    marked = np.ascontiguousarray(nvert_marked, np.float64)
    c = np.ascontiguousarray(cent, np.float64)
    n = lib().or_ibm_nodes(C.byref(d), _dp(c), _dp(marked), len(x), _dp(x), _dp(y), _dp(z), len(nv) // 3, _ip(nv),
                           None, 0)
    arr = (IbmNode * max(n, 1))()
    lib().or_ibm_nodes(C.byref(d), _dp(c), _dp(marked), len(x), _dp(x), _dp(y), _dp(z), len(nv) // 3, _ip(nv),
                       arr, n)
    return arr, n


def ibm_interpolate(d, nvert, nodes, n_nodes, surface, met, ucat, p, ucont, u_surf=None,
                    bctype=(0, 0, 0, 0, 0, 0), immersed=1):
    """ibm_interpolation_advanced + noslip for one body; returns (ucat, p, ucont)."""
    _, _, _, nv = _surface_arrays(surface)
    uc = np.ascontiguousarray(ucat, np.float64).copy()
    pp = np.ascontiguousarray(p, np.float64).copy()
    uo = np.ascontiguousarray(ucont, np.float64).copy()
    us = None if u_surf is None else _dp(np.ascontiguousarray(u_surf, np.float64))
    lib().or_ibm_interpolate(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), nodes, n_nodes, _ip(nv), us,
                             _dp(met["icsi"]), _dp(met["jeta"]), _dp(met["kzet"]), _dp(met["csi"]),
                             _dp(met["eta"]), _dp(met["zet"]), _ip(np.ascontiguousarray(bctype, np.int32)),
                             int(immersed), _dp(uc), _dp(pp), _dp(uo))
    return uc, pp, uo


def ib_bc(d, nvert, met, ucat, ucont, bctype=(0, 0, 0, 0, 0, 0), immersed=1):
    """IB_BC's face fluxes and boundary faces; returns (ucat, ucont)."""
    uc = np.ascontiguousarray(ucat, np.float64).copy()
    uo = np.ascontiguousarray(ucont, np.float64).copy()
    lib().or_ib_bc(C.byref(d), _dp(np.ascontiguousarray(nvert, np.float64)), _dp(met["icsi"]), _dp(met["jeta"]),
                   _dp(met["kzet"]), _ip(np.ascontiguousarray(bctype, np.int32)), int(immersed), _dp(uc), _dp(uo))
    return uc, uo
