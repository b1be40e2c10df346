"""Compile the oracle (oracle.cpp) into oracle/_build/liboracle.so.

-ffp-contract=off is required: the restatement must round like the
reference's unfused double arithmetic on any host (aarch64 compilers contract
a*b+c into fma by default).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def build() -> Path:
    src = HERE / "oracle.cpp"
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime >= max(src.stat().st_mtime, Path(__file__).stat().st_mtime):
        return OUT
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17", str(src), "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return OUT


REFBUILD = HERE / "refbuild"
REF_OUT = HERE / "_ref"
# the reference's src/ directory; PARM_REFERENCE_SRC overrides the default location
REF_SRC = Path(os.environ.get("PARM_REFERENCE_SRC", "/root/reference/src"))


def build_ref(ref_src: Path = REF_SRC) -> Path | None:
    """Compile the reference's own sources into oracle/_ref (fixture drivers).

    Only possible where the reference sources are present; returns None
    elsewhere.  The drivers regenerate tests/golden/*.npz; no test runs them.
    """
    if not (ref_src / "collection.cpp").exists():
        return None
    r = subprocess.run(["make", "-C", str(REFBUILD), f"REF={ref_src}", f"OUT={REF_OUT}", "-j2"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    return REF_OUT


if __name__ == "__main__":
    print(build())
    print(build_ref())
