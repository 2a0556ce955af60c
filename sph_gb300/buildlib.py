"""Build recipe of the sph_gb300 shared library (sm_103a, nvcc, no cmake).

The translation units compile in parallel and link into
``sph_gb300/lib/libsph_gb300.so``, which the Python host layer and any C/C++
caller load.  The FP64 parity form is compiled without FMA contraction so its
sums round as the reference's own (non-fast-math) build does; host code is
compiled without contraction on every architecture for the same reason.

``build(variant="checked")`` makes ``libsph_gb300_checked.so`` from the same
sources with ``-DSPH_BOUNDS_CHECK``: neighbour indices read from device data
are checked and an out-of-range one sets SPH_STATUS_BOUNDS instead of being
read (a test build; the arithmetic is the same).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libsph_gb300.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
COMMON = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
UNITS = {
    "sph_api.cu": [],
    "sph_scene_f32.cu": [],
    "sph_scene_f64.cu": ["-fmad=false"],
    "sph_noalloc.cu": [],
    "sph_pool.cu": [],
    "sph_scene_io.cpp": [],
    "sph_mesh.cpp": [],
    "sph_serve.cpp": [],
}
HEADERS = ["sph_device.cuh", "sph_kernels.cuh", "sph_lists.cuh", "sph_scene.cuh", "sph_scene_base.h", "sph_ctx.h",
           "sph_phase.cuh"]
VARIANTS = {"": ([], OBJDIR, LIB),
            "checked": (["-DSPH_BOUNDS_CHECK"], OBJDIR + "_checked", os.path.join(LIBDIR, "libsph_gb300_checked.so"))}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "sph_gb300.h")]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None, variant: str = "") -> str:
    vflags, objdir, lib = VARIANTS[variant]
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(objdir, exist_ok=True)
    cc = nvcc()
    jobs = []
    for unit, flags in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(objdir, os.path.splitext(unit)[0] + ".o")
        if force or _stale(obj, src):
            jobs.append([cc, *COMMON, *flags, *vflags, *(extra or []), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(objdir, os.path.splitext(u)[0] + ".o") for u in UNITS]
    if jobs or not os.path.exists(lib):
        run([cc, ARCH, "-shared", "-o", lib, *objs, "-lcudart"])
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
