"""ctypes binding of oracle/_ref/libvfs_ref.so: the reference's own
pressure-Poisson functions (Source/metrics.c, poisson.c, poisson_hypre.c,
main.c, rhs.c, momentum.c, level.c), compiled unmodified against the
single-rank PETSc/HYPRE/MPI stand-in of oracle/refshim/.

Test infrastructure: the CPU tests use it to pin the oracle's restatement to
the reference itself.  The library is built by oracle/refshim/build_ref.py
where the reference sources exist (the GPU host has none); `available()`
tells whether it has been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libvfs_ref.so")
_lib = None
SOLVE_FN = C.CFUNCTYPE(C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                       C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double)


def build(force=False):
    import importlib.util
    spec = importlib.util.spec_from_file_location("vfs_build_ref", os.path.join(HERE, "refshim", "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    if not mod.available():
        return None
    return mod.build(force=force)


def available():
    return os.path.exists(LIB)


def reference_dir():
    """The reference tree the library was built from (None if not built)."""
    p = os.path.join(HERE, "_ref", "REFERENCE_DIR")
    if not os.path.exists(p):
        return None
    return open(p).read().strip()


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.vr_create.restype = vp
        L.vr_create.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_int]
        L.vr_destroy.argtypes = [vp]
        L.vr_get.argtypes = [vp, C.c_char_p, vp, C.c_long]
        L.vr_set.argtypes = [vp, C.c_char_p, vp, C.c_long]
        L.vr_form_metrics.argtypes = [vp]
        L.vr_lhs.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.vr_lhs_csr.argtypes = [vp, vp, vp, vp]
        L.vr_rhs2.argtypes = [vp, C.c_int, vp]
        L.vr_solver_hypre.argtypes = [vp, SOLVE_FN, C.c_double, vp, vp]
        L.vr_update_pressure.argtypes = [vp]
        L.vr_projection.argtypes = [vp, C.c_double, C.c_double]
        L.vr_divergence.argtypes = [vp, C.POINTER(C.c_double)]
        L.vr_volume_flux.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.vr_fully_blocked.argtypes = [vp, C.POINTER(C.c_int), vp]
        L.vr_nullspace_original.argtypes = [vp, vp, C.c_long]
        _lib = L
    return _lib


class Block:
    """One block's UserCtx built the way MG_Initial builds one level
    (Source/init.c:141-161, 591-700), driven through the reference's own
    functions.  Arrays use the DA-natural layout [mz][my][mx](x3)."""

    def __init__(self, case, bctype=(0, 0, 0, 0, 0, 0), immersed=0):
        self.dims = case.dims
        mx, my, mz = self.dims
        per = np.ascontiguousarray(case.periodic, np.int32)
        bc = np.ascontiguousarray(bctype, np.int32)
        coor = np.ascontiguousarray(case.coor, np.float64)
        self.h = lib().vr_create(mx, my, mz, per.ctypes.data, bc.ctypes.data, coor.ctypes.data, int(immersed))
        self.ndof = None

    def close(self):
        if getattr(self, "h", None):
            lib().vr_destroy(self.h)
            self.h = None

    __del__ = close

    def _shape(self, comps):
        mx, my, mz = self.dims
        return (mz, my, mx) + ((comps,) if comps > 1 else ())

    def get(self, name, comps=1):
        out = np.zeros(self._shape(comps))
        rc = lib().vr_get(self.h, name.encode(), out.ctypes.data, out.size)
        if rc != 0:
            raise RuntimeError(f"vr_get({name}) = {rc}")
        return out

    def get_phi2(self):
        out = np.zeros(self.ndof)
        rc = lib().vr_get(self.h, b"phi2", out.ctypes.data, out.size)
        if rc != 0:
            raise RuntimeError(f"vr_get(phi2) = {rc}")
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, np.float64)
        rc = lib().vr_set(self.h, name.encode(), a.ctypes.data, a.size)
        if rc != 0:
            raise RuntimeError(f"vr_set({name}) = {rc}")

    def form_metrics(self):
        lib().vr_form_metrics(self.h)

    def lhs(self):
        """PoissonLHSNew: (ndof, rowptr, cols, vals) of the assembled matrix."""
        n, nnz = C.c_int(), C.c_int()
        lib().vr_lhs(self.h, C.byref(n), C.byref(nnz))
        self.ndof = n.value
        rp = np.zeros(n.value + 1, np.int32)
        cols = np.zeros(nnz.value, np.int32)
        vals = np.zeros(nnz.value)
        lib().vr_lhs_csr(self.h, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data)
        return n.value, rp, cols, vals

    def rhs2(self, poisson=0):
        b = np.zeros(self.ndof)
        lib().vr_rhs2(self.h, int(poisson), b.ctypes.data)
        return b

    def solver_hypre(self, solve, tol=1e-8):
        """PoissonSolver_Hypre with `solve(A_csr, b, x0, rtol) -> x` in place of
        HYPRE GMRES + BoomerAMG.  Returns (b handed to the solve, Phi2)."""
        import scipy.sparse as sp
        captured = {}

        def cb(n, rp, cols, vals, rhs, x, rtol):
            try:
                nnz = rp[n]
                A = sp.csr_matrix((np.ctypeslib.as_array(vals, (nnz,)).copy(),
                                   np.ctypeslib.as_array(cols, (nnz,)).copy(),
                                   np.ctypeslib.as_array(rp, (n + 1,)).copy()), shape=(n, n))
                b = np.ctypeslib.as_array(rhs, (n,)).copy()
                xv = np.ctypeslib.as_array(x, (n,))
                xv[:] = solve(A, b, xv.copy(), rtol)
                captured["A"] = A
                return 0
            except Exception as e:  # noqa: BLE001 -- reported after the call
                captured["error"] = e
                return 1

        fn = SOLVE_FN(cb)
        n = self.ndof if self.ndof is not None else int(np.prod(self.dims))
        b = np.zeros(n)
        phi2 = np.zeros(n)
        got = lib().vr_solver_hypre(self.h, fn, float(tol), b.ctypes.data, phi2.ctypes.data)
        if "error" in captured:
            raise captured["error"]
        self.ndof = got
        return b[:got], phi2[:got], captured.get("A")

    def update_pressure(self):
        lib().vr_update_pressure(self.h)

    def projection(self, dt=1.0, st=1.0):
        lib().vr_projection(self.h, float(dt), float(st))

    def divergence(self):
        v = C.c_double()
        lib().vr_divergence(self.h, C.byref(v))
        return v.value

    def fully_blocked(self):
        """FullyBlocked: (multi, ksk[my, mx]) with -1 where KSKE is unset."""
        m = C.c_int()
        ksk = np.zeros((self.dims[1], self.dims[0]), np.int32)
        lib().vr_fully_blocked(self.h, C.byref(m), ksk.ctypes.data)
        return bool(m.value), ksk

    def nullspace_original(self, x):
        """PoissonNullSpaceFunction_original on a copy of the DA array x
        (after fully_blocked)."""
        a = np.ascontiguousarray(x, np.float64).copy()
        rc = lib().vr_nullspace_original(self.h, a.ctypes.data, a.size)
        if rc != 0:
            raise RuntimeError(f"vr_nullspace_original = {rc}")
        return a

    def volume_flux(self, immersed_variant=True, flg=0):
        f, a = C.c_double(), C.c_double()
        lib().vr_volume_flux(self.h, int(bool(immersed_variant)), int(flg), C.byref(f), C.byref(a))
        return f.value, a.value
