"""Python binding of libvfs_poisson.so (the C ABI in include/vfs_poisson.h).

The class ``PoissonSolver`` mirrors the reference's per-block entry points
(Source/poisson_hypre.c:506 PoissonSolver_Hypre, Source/poisson.c:3137
UpdatePressure, :2700 Projection, Source/main.c:936 Divergence) on arrays in
the reference's DA layout.  Arrays may be numpy arrays (host) or CUDA
tensors / device pointers; the library detects which.

There is no CPU fallback: loading fails loudly when the CUDA library has not
been built, and every call fails when no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import configs  # noqa: F401  (synthetic inputs)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libvfs_poisson.so")

VFS_OK, VFS_EINVAL, VFS_ECUDA, VFS_ESTATE, VFS_ENOCONV, VFS_ENOMEM, VFS_ETIMEOUT = 0, -1, -2, -3, -4, -5, -6

# Exported symbols (every one is declared in include/vfs_poisson.h).
EXPORTS = [
    "vfs_last_error", "vfs_poisson_default_opts", "vfs_poisson_create", "vfs_poisson_destroy",
    "vfs_poisson_set_grid", "vfs_poisson_set_nvert", "vfs_poisson_rhs", "vfs_poisson_solve",
    "vfs_poisson_solver_hypre", "vfs_poisson_update_pressure", "vfs_poisson_projection",
    "vfs_poisson_divergence", "vfs_poisson_get_numbering", "vfs_poisson_get_operator",
    "vfs_poisson_get_metric", "vfs_poisson_get_rhs", "vfs_poisson_apply", "vfs_poisson_mg_levels",
    "vfs_poisson_mg_level_info", "vfs_poisson_mg_get_nvert", "vfs_poisson_mg_restrict",
    "vfs_poisson_mg_interpolate", "vfs_poisson_mg_vcycle", "vfs_poisson_kernel_launches",
    "vfs_poisson_set_stream", "vfs_poisson_profile", "vfs_poisson_profile_read",
    "vfs_divergence_noalloc", "vfs_poisson_ibm_search",
    "vfs_unet_create", "vfs_unet_destroy", "vfs_unet_set_stream", "vfs_unet_num_params", "vfs_unet_get_params",
    "vfs_unet_set_params", "vfs_unet_forward", "vfs_unet_gradient", "vfs_unet_train_step", "vfs_unet_adam",
    "vfs_unet_set_grads", "vfs_unet_kernel_launches", "vfs_poisson_learned_guess", "vfs_poisson_guess_sample",
    "vfs_poisson_get_operator32", "vfs_poisson_rhs2", "vfs_poisson_volume_flux", "vfs_poisson_volume_flux0", "vfs_poisson_contra2cart",
    "vfs_read_petsc_vec", "vfs_write_petsc_vec", "vfs_read_grid", "vfs_read_ucd", "vfs_poisson_set_levelset",
    "vfs_poisson_ibm_search_nodes", "vfs_poisson_ibm_nodes", "vfs_poisson_ibm_interpolate", "vfs_poisson_ib_bc",
    "vfs_poisson_set_history", "vfs_poisson_history_guess", "vfs_poisson_set_network_period",
    "vfs_poisson_history_record", "vfs_poisson_guess_report", "vfs_poisson_fully_blocked",
    "vfs_poisson_nullspace_original",
]


class IbmNode(C.Structure):
    """One IB node's interpolation record (vfs_ibm_node)."""
    _fields_ = [("i", C.c_int), ("j", C.c_int), ("k", C.c_int), ("cell", C.c_int),
                ("pmin", C.c_double * 3), ("d_s", C.c_double), ("cs", C.c_double * 3),
                ("ip", C.c_int * 3), ("jp", C.c_int * 3), ("kp", C.c_int * 3),
                ("cr", C.c_double * 3), ("d_i", C.c_double), ("imode", C.c_int), ("status", C.c_int)]


class GridDesc(C.Structure):
    _fields_ = [("mx", C.c_int), ("my", C.c_int), ("mz", C.c_int),
                ("i_periodic", C.c_int), ("j_periodic", C.c_int), ("k_periodic", C.c_int),
                ("ii_periodic", C.c_int), ("jj_periodic", C.c_int), ("kk_periodic", C.c_int),
                ("bctype3", C.c_int)]


class SolveOpts(C.Structure):
    _fields_ = [("rtol", C.c_double), ("max_it", C.c_int), ("restart", C.c_int), ("precision", C.c_int),
                ("nu1", C.c_int), ("nu2", C.c_int), ("omega", C.c_double), ("use_graphs", C.c_int),
                ("coarsest_max", C.c_int), ("warm_start", C.c_int), ("smoother", C.c_int), ("orth", C.c_int),
                ("nu2_near", C.c_int)]


class UNetBatch(C.Structure):
    _fields_ = [("features", C.c_void_p), ("target", C.c_void_p), ("weight", C.c_void_p),
                ("fx", C.c_int), ("fy", C.c_int), ("fz", C.c_int), ("ox", C.c_int), ("oy", C.c_int),
                ("oz", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("op", C.c_void_p), ("op_scale", C.c_float), ("mse_weight", C.c_float), ("res_weight", C.c_float)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double), ("initial_rel_residual", C.c_double),
                ("ms_total", C.c_double), ("levels", C.c_int), ("status", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


METRIC_INDEX = {name: q for q, name in enumerate(
    ["icsi", "ieta", "izet", "jcsi", "jeta", "jzet", "kcsi", "keta", "kzet", "csi", "eta", "zet", "cent",
     "iaj", "jaj", "kaj", "aj"])}

_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() "
                           "(there is no CPU fallback)")
    L = C.CDLL(path)
    P, vp, dp, ip = C.POINTER, C.c_void_p, C.c_void_p, C.c_void_p
    L.vfs_last_error.restype = C.c_char_p
    L.vfs_poisson_default_opts.argtypes = [P(SolveOpts)]
    L.vfs_poisson_create.argtypes = [P(GridDesc), P(vp)]
    L.vfs_poisson_destroy.argtypes = [vp]
    L.vfs_poisson_set_grid.argtypes = [vp, dp, vp]
    L.vfs_poisson_set_nvert.argtypes = [vp, dp]
    L.vfs_poisson_rhs.argtypes = [vp, dp, C.c_double, C.c_double, C.c_double]
    L.vfs_poisson_solve.argtypes = [vp, dp, P(SolveOpts), P(SolveStats)]
    L.vfs_poisson_solver_hypre.argtypes = [vp, dp, C.c_double, C.c_double, C.c_double, dp, P(SolveOpts),
                                           P(SolveStats)]
    L.vfs_poisson_update_pressure.argtypes = [vp, dp, dp]
    L.vfs_poisson_projection.argtypes = [vp, dp, C.c_double, C.c_double, C.c_double]
    L.vfs_poisson_divergence.argtypes = [vp, dp, P(C.c_double)]
    L.vfs_poisson_get_numbering.argtypes = [vp, P(C.c_int), ip]
    L.vfs_poisson_get_operator.argtypes = [vp, dp, ip]
    L.vfs_poisson_get_metric.argtypes = [vp, C.c_int, dp]
    L.vfs_poisson_get_rhs.argtypes = [vp, dp]
    L.vfs_poisson_apply.argtypes = [vp, dp, dp]
    L.vfs_poisson_mg_levels.argtypes = [vp, P(C.c_int)]
    L.vfs_poisson_mg_level_info.argtypes = [vp, C.c_int, P(C.c_int)]
    L.vfs_poisson_mg_get_nvert.argtypes = [vp, C.c_int, dp]
    L.vfs_poisson_mg_restrict.argtypes = [vp, C.c_int, dp, dp]
    L.vfs_poisson_mg_interpolate.argtypes = [vp, C.c_int, dp, dp]
    L.vfs_poisson_mg_vcycle.argtypes = [vp, C.c_int, dp, dp]
    L.vfs_poisson_kernel_launches.argtypes = [vp]
    L.vfs_poisson_kernel_launches.restype = C.c_int64
    L.vfs_poisson_set_stream.argtypes = [vp, vp]
    L.vfs_poisson_profile.argtypes = [vp, C.c_int]
    L.vfs_poisson_profile_read.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_int64)]
    L.vfs_divergence_noalloc.argtypes = [P(GridDesc), vp, vp, vp, vp, vp]
    L.vfs_poisson_ibm_search.argtypes = [vp, C.c_int, C.c_int, vp, C.c_int, vp, vp, vp, P(C.c_int)]
    L.vfs_poisson_ibm_search_nodes.argtypes = [vp, C.c_int, C.c_int, vp, C.c_int, vp, vp, vp, P(C.c_int),
                                               P(C.c_int)]
    L.vfs_poisson_ibm_nodes.argtypes = [vp, C.c_int, vp, C.c_int, P(C.c_int)]
    L.vfs_poisson_ibm_interpolate.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, vp, vp]
    L.vfs_poisson_ib_bc.argtypes = [vp, C.c_int, vp, vp, vp]
    L.vfs_unet_create.argtypes = [C.c_uint, P(vp)]
    L.vfs_unet_destroy.argtypes = [vp]
    L.vfs_unet_destroy.restype = None
    L.vfs_unet_set_stream.argtypes = [vp, vp]
    L.vfs_unet_num_params.argtypes = [vp]
    L.vfs_unet_num_params.restype = C.c_int64
    L.vfs_unet_get_params.argtypes = [vp, vp]
    L.vfs_unet_set_params.argtypes = [vp, vp]
    L.vfs_unet_forward.argtypes = [vp, P(UNetBatch), vp]
    L.vfs_unet_gradient.argtypes = [vp, P(UNetBatch), vp, P(C.c_double)]
    L.vfs_unet_train_step.argtypes = [vp, P(UNetBatch), C.c_double, P(C.c_double)]
    L.vfs_unet_adam.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
    L.vfs_unet_set_grads.argtypes = [vp, vp]
    L.vfs_unet_kernel_launches.argtypes = [vp]
    L.vfs_unet_kernel_launches.restype = C.c_int64
    L.vfs_poisson_learned_guess.argtypes = [vp, vp, vp, vp, C.c_double, P(C.c_int), vp]
    L.vfs_poisson_guess_sample.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.vfs_poisson_get_operator32.argtypes = [vp, vp]
    L.vfs_poisson_rhs2.argtypes = [vp, dp, C.c_double, C.c_double, C.c_double, C.c_int]
    L.vfs_poisson_volume_flux.argtypes = [vp, dp, C.c_int, C.c_double, P(C.c_double), P(C.c_double)]
    L.vfs_poisson_volume_flux0.argtypes = [vp, dp, C.c_int, P(C.c_double), P(C.c_double)]
    L.vfs_poisson_set_history.argtypes = [vp, C.c_int]
    L.vfs_poisson_history_guess.argtypes = [vp, P(C.c_double)]
    L.vfs_poisson_set_network_period.argtypes = [vp, C.c_int]
    L.vfs_poisson_history_record.argtypes = [vp, C.c_int]
    L.vfs_poisson_guess_report.argtypes = [vp, P(C.c_int), vp, vp]
    L.vfs_poisson_fully_blocked.argtypes = [vp, P(C.c_int), vp]
    L.vfs_poisson_nullspace_original.argtypes = [vp, vp]
    L.vfs_poisson_contra2cart.argtypes = [vp, dp, dp, C.c_int]
    L.vfs_poisson_set_levelset.argtypes = [vp, dp, dp, vp, C.c_int]
    L.vfs_read_petsc_vec.argtypes = [C.c_char_p, P(C.c_int64), vp]
    L.vfs_write_petsc_vec.argtypes = [C.c_char_p, C.c_int64, vp]
    L.vfs_read_grid.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_double, C.c_double, vp, vp]
    L.vfs_read_ucd.argtypes = [C.c_char_p, vp, P(C.c_int), P(C.c_int), vp, vp]
    _lib = L
    return L


class VfsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"vfs_poisson error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc != VFS_OK:
        raise VfsError(rc, load().vfs_last_error().decode())
    return rc


def _ptr(a, writable=False):
    """Address of a numpy array (C-contiguous float64) or a CUDA tensor."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):  # torch tensor
        assert a.is_contiguous()
        return a.data_ptr()
    assert isinstance(a, np.ndarray) and a.flags.c_contiguous, "arrays must be C-contiguous"
    if writable:
        assert a.flags.writeable
    return a.ctypes.data


def default_opts(**kw):
    o = SolveOpts()
    load().vfs_poisson_default_opts(C.byref(o))
    for k, v in kw.items():
        if not any(k == f for f, _ in SolveOpts._fields_):
            raise TypeError(f"unknown solver option {k!r}")
        setattr(o, k, v)
    return o


class PoissonSolver:
    """One block's pressure-Poisson projection on the GPU."""

    def __init__(self, mx, my, mz, periodic=(0, 0, 0, 0, 0, 0), bctype3=0):
        L = load()
        self.dims = (mx, my, mz)
        g = GridDesc(mx, my, mz, *[int(p) for p in periodic], bctype3)
        h = C.c_void_p()
        _check(L.vfs_poisson_create(C.byref(g), C.byref(h)))
        self.h = h

    @classmethod
    def from_case(cls, case):
        s = cls(*case.dims, periodic=case.periodic)
        s.set_grid(case.coor)
        s.set_nvert(case.nvert)
        return s

    def close(self):
        if getattr(self, "h", None):
            load().vfs_poisson_destroy(self.h)
            self.h = None

    __del__ = close

    def _shape(self, comps=0):
        mx, my, mz = self.dims
        return (mz, my, mx) + ((comps,) if comps else ())

    # --- set-up ---
    def set_grid(self, coor, face_metrics=None):
        fm = None
        if face_metrics is not None:
            arr = (C.c_void_p * 13)(*[_ptr(a) for a in face_metrics])
            fm = C.cast(arr, C.c_void_p)
            self._fm_keep = (arr, face_metrics)
        _check(load().vfs_poisson_set_grid(self.h, _ptr(coor), fm))

    def set_levelset(self, rho, level=None, bctype=(0, 0, 0, 0, 0, 0), enable=True):
        """Level-set (two-phase) operator: densities rho, level-set field and
        the six bctype codes; call before set_nvert."""
        bc = np.ascontiguousarray(bctype, np.int32)
        _check(load().vfs_poisson_set_levelset(self.h, _ptr(rho), _ptr(level), _ptr(bc), int(enable)))

    def set_nvert(self, nvert):
        _check(load().vfs_poisson_set_nvert(self.h, _ptr(nvert)))

    # --- per step ---
    def rhs(self, ucont, dt=1.0, st=1.0, coeff=1.0):
        _check(load().vfs_poisson_rhs(self.h, _ptr(ucont), dt, st, coeff))

    def rhs2(self, ucont, poisson=0, dt=1.0, st=1.0, coeff=1.0):
        """PoissonRHS2, the -poisson 0 / -1 right-hand side."""
        _check(load().vfs_poisson_rhs2(self.h, _ptr(ucont), dt, st, coeff, int(poisson)))

    def volume_flux(self, ucont, flg=0, flux_intp_sum=0.0):
        """VolumeFlux (immersed): corrects ucont in place; returns (flux, area)."""
        f, a = C.c_double(), C.c_double()
        _check(load().vfs_poisson_volume_flux(self.h, _ptr(ucont, True), int(flg), float(flux_intp_sum),
                                              C.byref(f), C.byref(a)))
        return f.value, a.value

    def volume_flux0(self, ucont, immersed=0):
        """VolumeFlux, the overload for immersed != 1: corrects (immersed 3,
        other) or zeroes (immersed 0, 3) the fluid/blanked faces of ucont in
        place; returns (flux, area) formed afterwards."""
        f, a = C.c_double(), C.c_double()
        _check(load().vfs_poisson_volume_flux0(self.h, _ptr(ucont, True), int(immersed), C.byref(f), C.byref(a)))
        return f.value, a.value

    def contra2cart(self, ucont, ucat=None, zero_solid=True):
        """Contra2Cart's change of basis; returns ucat (DA Cmpnts)."""
        out = np.zeros(self._shape(3)) if ucat is None else ucat
        _check(load().vfs_poisson_contra2cart(self.h, _ptr(ucont), _ptr(out, True), int(zero_solid)))
        return out

    def solve(self, phi=None, opts=None, **kw):
        o = opts if opts is not None else default_opts(**kw)
        st = SolveStats()
        out = phi if phi is not None else np.zeros(self._shape())
        rc = load().vfs_poisson_solve(self.h, _ptr(out, True), C.byref(o), C.byref(st))
        if rc not in (VFS_OK, VFS_ENOCONV):
            _check(rc)
        return out, st

    def solver_hypre(self, ucont, dt=1.0, st=1.0, coeff=1.0, phi=None, opts=None, **kw):
        self.rhs(ucont, dt, st, coeff)
        return self.solve(phi, opts, **kw)

    def update_pressure(self, p, phi=None):
        _check(load().vfs_poisson_update_pressure(self.h, _ptr(p, True), _ptr(phi, True)))
        return p, phi

    def projection(self, ucont, dt=1.0, st=1.0, coeff=1.0):
        _check(load().vfs_poisson_projection(self.h, _ptr(ucont, True), dt, st, coeff))
        return ucont

    def divergence(self, ucont):
        v = C.c_double()
        _check(load().vfs_poisson_divergence(self.h, _ptr(ucont), C.byref(v)))
        return v.value

    def ibm_search(self, surface, nvert=None, ibi=0, bctype=None):
        """Classify the cells against one closed triangulated surface
        (xyz[n_v, 3], tri[n_elmt, 3]); returns (nvert, cells that gave up)."""
        xyz = np.ascontiguousarray(surface[0], np.float64)
        tri = np.ascontiguousarray(surface[1], np.int32)
        out = np.zeros(self._shape()) if nvert is None else nvert
        bc = None if bctype is None else (C.c_int * 6)(*[int(b) for b in bctype])
        nf = C.c_int()
        _check(load().vfs_poisson_ibm_search(self.h, ibi, xyz.shape[0], _ptr(xyz), tri.shape[0], _ptr(tri),
                                             bc, _ptr(out, True), C.byref(nf)))
        return out, nf.value

    def ibm_search_nodes(self, surface, nvert=None, ibi=0, bctype=None):
        """ibm_search plus the interpolation records of the body's IB nodes
        (kept in the handle); returns (nvert, cells that gave up, nodes)."""
        xyz = np.ascontiguousarray(surface[0], np.float64)
        tri = np.ascontiguousarray(surface[1], np.int32)
        out = np.zeros(self._shape()) if nvert is None else nvert
        bc = None if bctype is None else (C.c_int * 6)(*[int(b) for b in bctype])
        nf, nn = C.c_int(), C.c_int()
        _check(load().vfs_poisson_ibm_search_nodes(self.h, ibi, xyz.shape[0], _ptr(xyz), tri.shape[0], _ptr(tri),
                                                   bc, _ptr(out, True), C.byref(nf), C.byref(nn)))
        return out, nf.value, nn.value

    def ibm_nodes(self, ibi=0):
        """The IB node records of body ibi (a ctypes array of IbmNode)."""
        n = C.c_int()
        _check(load().vfs_poisson_ibm_nodes(self.h, ibi, None, 0, C.byref(n)))
        arr = (IbmNode * max(n.value, 1))()
        _check(load().vfs_poisson_ibm_nodes(self.h, ibi, C.cast(arr, C.c_void_p), n.value, C.byref(n)))
        return arr, n.value

    def ibm_interpolate(self, ucat, p, ucont, ibi=0, u_surf=None, immersed=1, bctype=None):
        """ibm_interpolation_advanced with no-slip for body ibi; ucat, p,
        ucont in/out (DA layout)."""
        bc = None if bctype is None else (C.c_int * 6)(*[int(b) for b in bctype])
        us = None if u_surf is None else np.ascontiguousarray(u_surf, np.float64)
        _check(load().vfs_poisson_ibm_interpolate(self.h, ibi, _ptr(us), int(immersed), bc, _ptr(ucat, True),
                                                  _ptr(p, True), _ptr(ucont, True)))
        return ucat, p, ucont

    def ib_bc(self, ucat, ucont, immersed=1, bctype=None):
        """IB_BC: face fluxes around the IB nodes and the wall / slip /
        periodic faces; ucat (periodic ghosts) and ucont in/out."""
        bc = None if bctype is None else (C.c_int * 6)(*[int(b) for b in bctype])
        _check(load().vfs_poisson_ib_bc(self.h, int(immersed), bc, _ptr(ucat, True), _ptr(ucont, True)))
        return ucat, ucont

    # --- inspection ---
    def numbering(self):
        n = C.c_int()
        gid = np.zeros(self._shape(), np.int32)
        _check(load().vfs_poisson_get_numbering(self.h, C.byref(n), _ptr(gid, True)))
        return n.value, gid

    def operator(self):
        vol = np.zeros(self._shape(19))
        rt = np.zeros(self._shape(), np.int32)
        _check(load().vfs_poisson_get_operator(self.h, _ptr(vol, True), _ptr(rt, True)))
        return vol, rt

    def metric(self, name):
        q = METRIC_INDEX[name]
        out = np.zeros(self._shape(3 if q < 13 else 0))
        _check(load().vfs_poisson_get_metric(self.h, q, _ptr(out, True)))
        return out

    def rhs_array(self):
        out = np.zeros(self._shape())
        _check(load().vfs_poisson_get_rhs(self.h, _ptr(out, True)))
        return out

    def apply(self, x):
        y = np.zeros(self._shape())
        _check(load().vfs_poisson_apply(self.h, _ptr(np.ascontiguousarray(x, np.float64)), _ptr(y, True)))
        return y

    def mg_levels(self):
        n = C.c_int()
        _check(load().vfs_poisson_mg_levels(self.h, C.byref(n)))
        out = []
        for li in range(n.value):
            d = (C.c_int * 6)()
            _check(load().vfs_poisson_mg_level_info(self.h, li, d))
            out.append(tuple(d))
        return out

    def mg_nvert(self, level):
        nx, ny, nz = self.mg_levels()[level][:3]
        out = np.zeros((nz + 2, ny + 2, nx + 2))
        _check(load().vfs_poisson_mg_get_nvert(self.h, level, _ptr(out, True)))
        return out

    def mg_restrict(self, fine, xf):
        nx, ny, nz = self.mg_levels()[fine + 1][:3]
        out = np.zeros((nz + 2, ny + 2, nx + 2))
        _check(load().vfs_poisson_mg_restrict(self.h, fine, _ptr(np.ascontiguousarray(xf)), _ptr(out, True)))
        return out

    def mg_interpolate(self, fine, xc):
        nx, ny, nz = self.mg_levels()[fine][:3]
        out = np.zeros((nz + 2, ny + 2, nx + 2))
        _check(load().vfs_poisson_mg_interpolate(self.h, fine, _ptr(np.ascontiguousarray(xc)), _ptr(out, True)))
        return out

    def mg_vcycle(self, r, precision=0):
        z = np.zeros(self._shape())
        _check(load().vfs_poisson_mg_vcycle(self.h, precision, _ptr(np.ascontiguousarray(r)), _ptr(z, True)))
        return z

    def kernel_launches(self):
        return load().vfs_poisson_kernel_launches(self.h)

    def set_stream(self, stream):
        """Run on a caller's CUDA stream (an int handle, e.g.
        torch.cuda.current_stream().cuda_stream); None for a private one."""
        _check(load().vfs_poisson_set_stream(self.h, stream))

    def profile(self, enable=True):
        _check(load().vfs_poisson_profile(self.h, int(enable)))

    def profile_read(self):
        ms, b, n = C.c_double(), C.c_double(), C.c_int64()
        _check(load().vfs_poisson_profile_read(self.h, C.byref(ms), C.byref(b), C.byref(n)))
        return ms.value, b.value, n.value

    # --- learned initial guess ---
    def guess_sample(self, phi_n, phi_nm1, phi_nm2, features, target, weight):
        """Training sample for the current right-hand side: feature planes
        [4][nz][ny][nx], target and weight [nz][ny][nx] (FP32 CUDA tensors,
        box layout, written in place)."""
        _check(load().vfs_poisson_guess_sample(self.h, _ptr(phi_n), _ptr(phi_nm1), _ptr(phi_nm2), _ptr(features),
                                               _ptr(target), _ptr(weight)))

    def operator32(self, out=None):
        """The finest level's row-scaled FP32 operator, [19][nz][ny][nx]."""
        if out is None:
            mx, my, mz = self.dims
            out = np.zeros((19, mz - 2, my - 2, mx - 2), np.float32)
        _check(load().vfs_poisson_get_operator32(self.h, _ptr(out, True)))
        return out

    def set_history(self, k):
        """Keep the last k converged solutions for the history projection of
        the initial guess (0 turns it off)."""
        _check(load().vfs_poisson_set_history(self.h, int(k)))

    def history_guess(self):
        """Install the history's projection or extrapolation, whichever the
        judge prefers, as the iterate (solve with warm_start=2 next); returns
        its relative residual (guess_report tells which)."""
        r = C.c_double()
        _check(load().vfs_poisson_history_guess(self.h, C.byref(r)))
        return r.value

    def history_record(self, on=True):
        """Whether converged solves append to the history."""
        _check(load().vfs_poisson_history_record(self.h, int(bool(on))))

    def set_network_period(self, period):
        _check(load().vfs_poisson_set_network_period(self.h, int(period)))

    def fully_blocked(self):
        """FullyBlocked: (multinullspace, ksk[my, mx]) -- the first k of every
        interior column with nvert > 0.1 (-1 where none)."""
        m = C.c_int()
        ksk = np.zeros(self._shape()[1:], np.int32)
        _check(load().vfs_poisson_fully_blocked(self.h, C.byref(m), _ptr(ksk, True)))
        return bool(m.value), ksk

    def nullspace_original(self, x):
        """PoissonNullSpaceFunction_original on x (DA layout, in place for a
        CUDA tensor; a numpy array is changed in place too)."""
        _check(load().vfs_poisson_nullspace_original(self.h, _ptr(x, True)))
        return x

    def guess_report(self):
        """What the last guess installed: (chosen, rel_res[3], est[3]) with
        codes 0 projection / previous phi, 1 network, 2 extrapolation, and
        per code the relative residual and the estimated error (-1 where the
        candidate was not formed or not rated)."""
        ch = C.c_int()
        rr = (C.c_double * 3)()
        es = (C.c_double * 3)()
        _check(load().vfs_poisson_guess_report(self.h, C.byref(ch), C.cast(rr, C.c_void_p), C.cast(es, C.c_void_p)))
        return ch.value, list(rr), list(es)

    def learned_guess(self, unet, phi_nm1, phi_nm2, kappa):
        """Install the judge's choice among the base (history projection, or
        phi_{n-1} without a history), the extrapolation and the network's
        guess as the iterate; returns (chosen, [rel_res_base,
        rel_res_network]) with chosen 0 base, 1 network, 2 extrapolation.
        Solve with warm_start=2 next."""
        ch = C.c_int()
        rr = (C.c_double * 2)()
        _check(load().vfs_poisson_learned_guess(self.h, unet.u, _ptr(phi_nm1), _ptr(phi_nm2), float(kappa),
                                                C.byref(ch), C.cast(rr, C.c_void_p)))
        return ch.value, [rr[0], rr[1]]


class UNet:
    """The learned-guess network (3 levels, 16/32/64 channels, BF16 tensor
    cores), trained and run by the library's own kernels."""

    def __init__(self, seed=0):
        L = load()
        u = C.c_void_p()
        _check(L.vfs_unet_create(seed, C.byref(u)))
        self.u = u
        self.kappa = 1.0

    def close(self):
        if getattr(self, "u", None):
            load().vfs_unet_destroy(self.u)
            self.u = None

    __del__ = close

    @property
    def num_params(self):
        return load().vfs_unet_num_params(self.u)

    def get_params(self):
        out = np.zeros(self.num_params, np.float32)
        _check(load().vfs_unet_get_params(self.u, _ptr(out, True)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32) if isinstance(p, np.ndarray) else p
        _check(load().vfs_unet_set_params(self.u, _ptr(p)))

    def set_grads(self, g):
        g = np.ascontiguousarray(g, np.float32) if isinstance(g, np.ndarray) else g
        _check(load().vfs_unet_set_grads(self.u, _ptr(g)))

    def set_stream(self, stream):
        _check(load().vfs_unet_set_stream(self.u, stream))

    @staticmethod
    def batch(features, target=None, weight=None, origin=(0, 0, 0), size=None, op=None, op_scale=1.0,
              mse_weight=1.0, res_weight=0.0):
        """features: CUDA float32 tensor [4][fz][fy][fx]; target/weight
        [fz][fy][fx]; origin (ox, oy, oz) and size (nx, ny, nz) of the
        sub-box; op: the row-scaled operator planes [19][fz][fy][fx] for the
        residual loss."""
        fz, fy, fx = features.shape[1:]
        nx, ny, nz = size if size is not None else (fx, fy, fz)
        return UNetBatch(_ptr(features), _ptr(target), _ptr(weight), fx, fy, fz, *origin, nx, ny, nz, _ptr(op),
                         op_scale, mse_weight, res_weight)

    def forward(self, batch, out):
        _check(load().vfs_unet_forward(self.u, C.byref(batch), _ptr(out)))
        return out

    def gradient(self, batch, grad=None):
        loss = C.c_double()
        _check(load().vfs_unet_gradient(self.u, C.byref(batch), _ptr(grad), C.byref(loss)))
        return loss.value

    def train_step(self, batch, lr):
        loss = C.c_double()
        _check(load().vfs_unet_train_step(self.u, C.byref(batch), float(lr), C.byref(loss)))
        return loss.value

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(load().vfs_unet_adam(self.u, float(lr), float(beta1), float(beta2), float(eps)))

    def kernel_launches(self):
        return load().vfs_unet_kernel_launches(self.u)


# --- the reference's input files (host) ---
def read_petsc_vec(path):
    """A PETSc binary vector (restart field) as a float64 array."""
    L = load()
    n = C.c_int64(0)
    _check(L.vfs_read_petsc_vec(path.encode(), C.byref(n), None))
    out = np.zeros(n.value)
    _check(L.vfs_read_petsc_vec(path.encode(), C.byref(n), _ptr(out, True)))
    return out


def write_petsc_vec(path, values):
    v = np.ascontiguousarray(values, np.float64).ravel()
    _check(load().vfs_write_petsc_vec(path.encode(), v.size, _ptr(v)))


GRID_XYZ, GRID_TEXT, GRID_BINARY = 0, 1, 2


def read_grid(path, fmt=GRID_XYZ, block=0, L_dim=1.0, cl=1.0):
    """Grid nodes as the DA-layout array [KM+1][JM+1][IM+1][3]."""
    L = load()
    dims = np.zeros(3, np.int32)
    _check(L.vfs_read_grid(path.encode(), fmt, block, L_dim, cl, _ptr(dims, True), None))
    IM, JM, KM = (int(v) for v in dims)
    coor = np.zeros((KM + 1, JM + 1, IM + 1, 3))
    _check(L.vfs_read_grid(path.encode(), fmt, block, L_dim, cl, _ptr(dims, True), _ptr(coor, True)))
    return coor


def read_ucd(path, L_dim=1.0, cm=(0.0, 0.0, 0.0), centre=(0.0, 0.0, 0.0), angles=(0.0, 0.0, 0.0)):
    """A UCD surface as (xyz[n_v, 3], tri[n_elmt, 3] 0-based), placed like
    the reference's ibm_read_ucd."""
    L = load()
    nv, ne = C.c_int(0), C.c_int(0)
    _check(L.vfs_read_ucd(path.encode(), None, C.byref(nv), C.byref(ne), None, None))
    xyz = np.zeros((nv.value, 3))
    tri = np.zeros((ne.value, 3), np.int32)
    place = np.array([L_dim, *cm, *centre, *angles], np.float64)
    _check(L.vfs_read_ucd(path.encode(), _ptr(place), C.byref(nv), C.byref(ne), _ptr(xyz, True), _ptr(tri, True)))
    return xyz, tri
