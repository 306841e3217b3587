"""vfs_divergence_noalloc: the Divergence entry point for callers that may
not allocate device memory (inside a stream capture, or under their own
device-memory pool).  It keeps its scratch in a fixed device array inside
the library instead of allocating.

Called through the C ABI and compared with the handle-based
vfs_poisson_divergence on two calls in a row (the shared scratch keeps the
first call's partial maxima).  Both evaluate the same per-cell expression
and a max reduction, so the tolerance is zero: the values must be equal.
This file sorts last so that a stop-at-first-failure run has already run
every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_divergence_noalloc_matches_handle(cuda_lib):
    import torch

    import vfs_poisson as V
    from vfs_poisson import configs as CF

    case = CF.cylinder(24, 16, 24)
    s = V.PoissonSolver.from_case(case)
    try:
        aj = s.metric("aj")
        L = V.load()

        def dev(a):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()

        nv, ajd = dev(case.nvert), dev(aj)
        out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        g = V.GridDesc(*case.dims, *case.periodic, 0)
        rng = np.random.default_rng(2)
        u2 = case.ucont + 0.3 * rng.standard_normal(case.ucont.shape)
        for u in (case.ucont, u2):
            ref = s.divergence(u)
            ud = dev(u)
            rc = L.vfs_divergence_noalloc(ctypes.byref(g), ud.data_ptr(), nv.data_ptr(), ajd.data_ptr(),
                                          out.data_ptr(), None)
            torch.cuda.synchronize()
            assert rc == V.VFS_OK, L.vfs_last_error()
            assert out.item() == ref
        # grids beyond the scratch capacity are refused before any launch
        big = V.GridDesc(4100, 4100, 20, 0, 0, 0, 0, 0, 0, 0)
        rc = L.vfs_divergence_noalloc(ctypes.byref(big), ud.data_ptr(), nv.data_ptr(), ajd.data_ptr(),
                                      out.data_ptr(), None)
        assert rc == V.VFS_EINVAL and b"at most" in L.vfs_last_error()
        # host pointers are refused (copying them would need device memory)
        rc = L.vfs_divergence_noalloc(ctypes.byref(g), u2.ctypes.data, nv.data_ptr(), ajd.data_ptr(),
                                      out.data_ptr(), None)
        assert rc == V.VFS_EINVAL
    finally:
        s.close()
