"""Build the native parts of parm_gb300 in-tree.

* ``parm_gb300/_lib/libparm_gb300.so`` — the CUDA kernels and the C ABI
  declared in ``include/parm_gb300.h`` (sm_103a only).
* ``parm_gb300/_lib/libparm_host.so`` (3D) and ``libparm_host2d.so`` (2D) —
  the C++ host API of ``parm_gb300/host/`` that mirrors the reference's
  classes (Box, AtomVec, NeighborList, NListed, Collection...) on top of the
  C ABI.

Each translation unit is compiled by its own nvcc/g++ process in parallel.
The FP64 translation units use ``-fmad=false`` so that no multiply-add is
contracted: their arithmetic must round exactly like the reference's CPU
code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
LIB = PKG / "_lib"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
               f"-I{INCLUDE}", f"-I{CSRC}", "--expt-relaxed-constexpr"]
# translation unit -> extra flags
CUDA_UNITS = {
    "nlist.cu": ["-fmad=false"],
    "integrate.cu": ["-fmad=false"],
    "pair64.cu": ["-fmad=false"],
    "pair32.cu": [],
    "staged.cu": [],
    "capi.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "nlcg.cu": ["-fmad=false"],
}
HOST_UNITS = ["parm_host.cpp"]
# the host API is built once per dimension, like the reference (-DVEC3D / -DVEC2D)
HOST_LIBS = {"libparm_host.so": [], "libparm_host2d.so": ["-DVEC2D"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build parm_gb300")


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile everything that is out of date; returns the CUDA library path."""
    LIB.mkdir(exist_ok=True)
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + [INCLUDE / "parm_gb300.h"]
    nv = nvcc()
    jobs = jobs or max(1, min(len(CUDA_UNITS) + len(HOST_UNITS), os.cpu_count() or 4))
    tasks = []
    objs = []
    for unit, extra in CUDA_UNITS.items():
        src = CSRC / unit
        obj = BUILD / (unit + ".o")
        objs.append(obj)
        if _stale(obj, [src, *headers, Path(__file__)]):
            tasks.append([nv, *ARCH, *NVCC_COMMON, *extra, "-c", str(src), "-o", str(obj)])
    host_objs = {}
    host_headers = sorted(HOST.glob("*.hpp")) + [INCLUDE / "parm_gb300.h"]
    for libname, defs in HOST_LIBS.items():
        host_objs[libname] = []
        for unit in HOST_UNITS:
            src = HOST / unit
            if not src.exists():
                continue
            obj = BUILD / (unit + ("".join(defs) + ".o"))
            host_objs[libname].append(obj)
            if _stale(obj, [src, *host_headers, Path(__file__)]):
                tasks.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", *defs, f"-I{INCLUDE}",
                              f"-I{HOST}", "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(jobs) as ex:
        for cmd in tasks:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, tasks))
    lib = LIB / "libparm_gb300.so"
    if _stale(lib, objs):
        cudalib = cuda_home() / "lib64"
        if not cudalib.exists():
            cudalib = cuda_home() / "lib"
        _run([nv, *ARCH, "-shared", "-o", str(lib), *map(str, objs), f"-L{cudalib}", "-lcudart",
              "-Xlinker", f"-rpath={cudalib}"])
    for libname, objs_h in host_objs.items():
        if not objs_h:
            continue
        hlib = LIB / libname
        if _stale(hlib, objs_h + [lib]):
            _run(["g++", "-shared", "-o", str(hlib), *map(str, objs_h), f"-L{LIB}", "-lparm_gb300",
                  "-Wl,-rpath,$ORIGIN"])
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", LIB)
