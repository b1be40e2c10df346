"""Building programs against the C++ host API (parm_gb300/host)."""
from __future__ import annotations

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HOST = ROOT / "parm_gb300" / "host"
INCLUDE = ROOT / "include"
LIB = ROOT / "parm_gb300" / "_lib"
DECK_DRIVER = ROOT / "oracle" / "refbuild" / "ref_driver.cpp"


def compile_program(src: Path, out: Path, ndim: int = 3, link: bool = True) -> subprocess.CompletedProcess:
    """g++ a program written against the reference's headers, with this library's headers instead."""
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{HOST}", f"-I{INCLUDE}"]
    if ndim == 2:
        cmd.append("-DVEC2D")
    if link:
        lib = "parm_host" if ndim == 3 else "parm_host2d"
        cmd += [str(src), "-o", str(out), f"-L{LIB}", f"-l{lib}", "-lparm_gb300", f"-Wl,-rpath,{LIB}"]
    else:
        cmd += ["-c", str(src), "-o", str(out)]
    return subprocess.run(cmd, capture_output=True, text=True)
