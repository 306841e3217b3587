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


def test_python_structs_match_the_header(tmp_path):
    """Every ctypes mirror of a struct in include/vfs_poisson.h has the C
    layout: a small C program built with gcc against the header prints each
    field's offset and each struct's size."""
    import shutil
    import subprocess
    import pytest
    import vfs_poisson as V
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    mirrors = {"vfs_grid_desc": V.GridDesc, "vfs_solve_opts": V.SolveOpts, "vfs_solve_stats": V.SolveStats,
               "vfs_ibm_node": V.IbmNode, "vfs_unet_batch": V.UNetBatch}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "vfs_poisson.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, field, val = ln.split()
        got[(cname, field)] = int(val)
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)
