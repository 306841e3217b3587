"""The C-ABI library builds for sm_103a, loads without a GPU and exports
every entry point that include/vfs_poisson.h declares (no compute calls)."""
import ctypes
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(REPO, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(REPO, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(vfs_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(cuda_lib):
    import vfs_poisson
    declared = _declared()
    assert "vfs_poisson_solve" in declared and len(declared) >= 20
    lib = ctypes.CDLL(vfs_poisson.LIB_PATH)
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(vfs_poisson.EXPORTS) <= declared


def test_no_cpu_fallback_without_gpu(cuda_lib):
    import torch
    import vfs_poisson
    if torch.cuda.is_available():
        return
    try:
        vfs_poisson.PoissonSolver(6, 6, 6)
    except vfs_poisson.VfsError as e:
        assert e.code in (vfs_poisson.VFS_ECUDA, vfs_poisson.VFS_ENOMEM)
    else:
        raise AssertionError("the library must fail loudly without a GPU")
