"""Build helpers for the drop-in adapter tests.

  * harness(): tests/adapter_harness.cpp + the DA bridge
    (vfs-wind_gb300/adapter/vfs_da_bridge.cpp) + the single-rank PETSc
    stand-in (oracle/refshim/shim.cpp), linked against libvfs_poisson.so;
  * full_adapter(): where the reference's sources exist, the reference's
    pressure-Poisson units with their PoissonSolver_Hypre, UpdatePressure,
    Projection and Divergence renamed at compile time (the link-time drop-in
    of INTEGRATION.md), the UserCtx adapter, the bridge, the stand-in and the
    oracle's UserCtx harness (oracle/refshim/ref_driver.cpp), so that the
    reference's own calls reach the adapter.
Outputs go to oracle/_build/ (git-ignored).
"""
import ctypes as C
import os
import re
import subprocess

TESTS = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(TESTS)
SHIM = os.path.join(REPO, "oracle", "refshim")
ADAPTER = os.path.join(REPO, "vfs-wind_gb300", "adapter")
LIBDIR = os.path.join(REPO, "vfs-wind_gb300", "lib")
OUT = os.path.join(REPO, "oracle", "_build")

RENAMES = {
    "poisson_hypre.c": ["-DPoissonSolver_Hypre=vfs_reference_PoissonSolver_Hypre"],
    "poisson.c": ["-DUpdatePressure=vfs_reference_UpdatePressure", "-DProjection=vfs_reference_Projection"],
    "main.c": ["-DDivergence=vfs_reference_Divergence", "-Dmain=vfs_reference_main_unused"],
}


def _newer(target, sources):
    return os.path.exists(target) and os.path.getmtime(target) >= max(os.path.getmtime(s) for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}")


def harness():
    from vfs_poisson import _build
    _build.build()
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libvfs_adapter_harness.so")
    srcs = [os.path.join(TESTS, "adapter_harness.cpp"), os.path.join(ADAPTER, "vfs_da_bridge.cpp"),
            os.path.join(SHIM, "shim.cpp")]
    deps = srcs + [os.path.join(ADAPTER, "vfs_da_bridge.h"), os.path.join(SHIM, "petsc_shim.h"),
                   os.path.join(LIBDIR, "libvfs_poisson.so")]
    if not _newer(lib, deps):
        _run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I", SHIM, "-I", ADAPTER,
              "-I", os.path.join(REPO, "include"), *srcs, "-o", lib, "-L", LIBDIR, "-lvfs_poisson",
              f"-Wl,-rpath,{LIBDIR}"])
    L = C.CDLL(lib)
    vp = C.c_void_p
    L.ah_da_create.restype = vp
    L.ah_da_create.argtypes = [C.c_int] * 7
    for f in ("ah_coordinate_da", "ah_coordinates", "ah_global"):
        getattr(L, f).restype = vp
        getattr(L, f).argtypes = [vp]
    L.ah_vec_destroy.argtypes = [vp]
    L.ah_fill.argtypes = [vp, vp, vp, C.c_int]
    L.ah_read.argtypes = [vp, vp, vp, C.c_int]
    L.ah_ghosted.restype = C.c_double
    L.ah_ghosted.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.ah_ghost_corners.argtypes = [vp, vp]
    L.vfsa_gather.argtypes = [vp, vp, vp]
    L.vfsa_scatter.argtypes = [vp, vp, vp]
    L.vfsa_create.argtypes = [vp, vp, vp, C.POINTER(vp)]
    L.vfsa_destroy.argtypes = [vp]
    L.vfsa_set_grid.argtypes = [vp, vp]
    L.vfsa_set_nvert.argtypes = [vp, vp]
    L.vfsa_volume_flux.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.vfsa_solve.argtypes = [vp, vp, C.c_double, C.c_double, C.c_double, vp, vp, vp]
    L.vfsa_update_pressure.argtypes = [vp, vp, vp]
    L.vfsa_projection.argtypes = [vp, vp, C.c_double, C.c_double, C.c_double]
    L.vfsa_divergence.argtypes = [vp, vp, C.POINTER(C.c_double)]
    return L


def full_adapter():
    """The reference with the adapter linked in (None without the reference
    sources)."""
    import reference
    if reference.build() is None:
        return None
    from vfs_poisson import _build
    _build.build()
    src = os.path.join(reference.reference_dir(), "Source")
    obj = os.path.join(OUT, "adapter_obj")
    os.makedirs(obj, exist_ok=True)
    lib = os.path.join(OUT, "libvfs_ref_adapter.so")
    units = ["metrics.c", "poisson.c", "poisson_hypre.c", "main.c", "rhs.c", "momentum.c", "level.c"]
    own = [os.path.join(ADAPTER, "vfs_userctx_adapter.cpp"), os.path.join(ADAPTER, "vfs_da_bridge.cpp"),
           os.path.join(SHIM, "shim.cpp"), os.path.join(SHIM, "ref_driver.cpp")]
    deps = [os.path.join(src, u) for u in units] + own + [os.path.join(LIBDIR, "libvfs_poisson.so"),
                                                          os.path.join(SHIM, "petsc_shim.h")]
    if _newer(lib, deps):
        return lib
    inc = ["-I", SHIM, "-I", src, "-I", ADAPTER, "-I", os.path.join(REPO, "include")]
    objs = []
    for u in units:
        o = os.path.join(obj, os.path.splitext(u)[0] + ".o")
        _run(["g++", "-x", "c++", "-std=gnu++98", "-O1", "-fPIC", "-w", "-ffp-contract=off", *inc,
              *RENAMES.get(u, ["-Dmain=vfs_reference_main_unused"] if u == "main.c" else []),
              "-c", os.path.join(src, u), "-o", o])
        objs.append(o)
    for f in own:
        o = os.path.join(obj, os.path.splitext(os.path.basename(f))[0] + ".o")
        _run(["g++", "-std=gnu++17", "-O1", "-fPIC", "-w", *inc, "-c", f, "-o", o])
        objs.append(o)
    probe = subprocess.run(["g++", "-shared", "-o", os.path.join(obj, "probe.so"), *objs, "-L", LIBDIR,
                            "-lvfs_poisson", "-Wl,--no-undefined", "-Wl,--no-demangle"],
                           capture_output=True, text=True)
    missing = sorted(set(re.findall(r"undefined reference to `([^']+)'", probe.stderr)))
    stub = os.path.join(obj, "stubs.c")
    with open(stub, "w") as f:
        f.write("#include <stdio.h>\n#include <stdlib.h>\n"
                "static void unreached(const char *s) { fprintf(stderr, \"%s unreached\\n\", s); abort(); }\n")
        for s in missing:
            if s.startswith("_Z"):
                f.write(f"void {s}(void) {{ unreached(\"{s}\"); }}\n")
            else:
                f.write(f"char {s}[4096] __attribute__((aligned(64)));\n")
    _run(["gcc", "-O1", "-fPIC", "-w", "-c", stub, "-o", os.path.join(obj, "stubs.o")])
    _run(["g++", "-shared", "-o", lib, *objs, os.path.join(obj, "stubs.o"), "-L", LIBDIR, "-lvfs_poisson",
          f"-Wl,-rpath,{LIBDIR}", "-Wl,--no-undefined"])
    return lib
