"""Build oracle/_ref/libvfs_ref.so: the reference's own pressure-Poisson
translation units (Source/metrics.c, poisson.c, poisson_hypre.c, main.c),
compiled unmodified against the single-rank PETSc/HYPRE/MPI stand-in in this
folder, plus the host harness ref_driver.cpp.

Test infrastructure: the library pins the oracle's restatement (tests/), it
is never part of the product.  It needs the reference's sources, so it is
built only where they are present (the reference directory comes from
VFS_REFERENCE_DIR, default /root/reference); nothing is copied out of them.

Symbols that the four units reference but that live in the reference's other
files (the momentum solver, FSI, turbine models, I/O) are resolved by
generated stubs: a function stub aborts with its name if it is ever called;
a global variable stub is a zero-filled block.  The harness never reaches
those functions on the covered paths (metrics, numbering, operator,
right-hand sides, the HYPRE driver around an injected inner solve,
UpdatePressure, Projection, Divergence, VolumeFlux).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libvfs_ref.so")
UNITS = ["metrics.c", "poisson.c", "poisson_hypre.c", "main.c", "rhs.c", "momentum.c", "level.c"]
# the reference builds as C++ (mpicxx); no FMA contraction, so that every
# operation rounds in source order like the oracle and the CUDA kernels
REF_FLAGS = ["-x", "c++", "-std=gnu++98", "-O2", "-fPIC", "-w", "-ffp-contract=off",
             "-Dmain=vfs_reference_main_unused"]
OWN_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-ffp-contract=off"]


def reference_dir():
    return os.environ.get("VFS_REFERENCE_DIR", "/root/reference")


def available():
    src = os.path.join(reference_dir(), "Source")
    return all(os.path.exists(os.path.join(src, u)) for u in UNITS + ["variables.h"])


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd[:3])} ... failed:\n{r.stdout[-4000:]}\n{r.stderr[-4000:]}")
    return r


def _sources():
    src = os.path.join(reference_dir(), "Source")
    own = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".h", ".cpp", ".py"))]
    return [os.path.join(src, u) for u in UNITS + ["variables.h"]] + own


def build(force=False, verbose=False):
    if not available():
        raise FileNotFoundError(f"reference sources not found under {reference_dir()}")
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in _sources()):
        return LIB
    src = os.path.join(reference_dir(), "Source")
    inc = ["-I", HERE, "-I", src]
    jobs = []
    for u in UNITS:
        jobs.append(["g++", *REF_FLAGS, *inc, "-c", os.path.join(src, u),
                     "-o", os.path.join(OUT, "obj", os.path.splitext(u)[0] + ".o")])
    for f in ("shim.cpp", "ref_driver.cpp"):
        flags = OWN_FLAGS + (["-w", "-std=gnu++17"] if f == "ref_driver.cpp" else [])
        jobs.append(["g++", *flags, *inc, "-c", os.path.join(HERE, f),
                     "-o", os.path.join(OUT, "obj", os.path.splitext(f)[0] + ".o")])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    objs = [j[-1] for j in jobs]
    # symbols the units need from the reference's other files -> stubs
    probe = subprocess.run(["g++", "-shared", "-o", os.path.join(OUT, "probe.so"), *objs,
                            "-Wl,--no-undefined", "-Wl,--no-demangle"], capture_output=True, text=True)
    missing = sorted(set(re.findall(r"undefined reference to `([^']+)'", probe.stderr)))
    stub = os.path.join(OUT, "stubs.c")
    with open(stub, "w") as f:
        f.write("/* generated by build_ref.py: symbols of the reference's other files */\n"
                "#include <stdio.h>\n#include <stdlib.h>\n"
                "static void unreached(const char *s) {\n"
                "  fprintf(stderr, \"reference function %s is outside the compiled units\\n\", s);\n"
                "  abort();\n}\n")
        for s in missing:
            if s.startswith("_Z"):
                f.write(f"void {s}(void) {{ unreached(\"{s}\"); }}\n")
            else:
                f.write(f"char {s}[4096] __attribute__((aligned(64)));\n")
    _run(["gcc", "-O1", "-fPIC", "-w", "-c", stub, "-o", os.path.join(OUT, "obj", "stubs.o")])
    tmp = LIB + ".tmp"
    _run(["g++", "-shared", "-o", tmp, *objs, os.path.join(OUT, "obj", "stubs.o"), "-Wl,--no-undefined"])
    os.replace(tmp, LIB)
    if os.path.exists(os.path.join(OUT, "probe.so")):
        os.remove(os.path.join(OUT, "probe.so"))
    with open(os.path.join(OUT, "REFERENCE_DIR"), "w") as f:
        f.write(reference_dir() + "\n")
    if verbose:
        print(f"{LIB}: {len(missing)} stubbed symbols")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
