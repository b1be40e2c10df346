"""Compile the oracle (oracle.cpp) into oracle/_build/liboracle.so.

-ffp-contract=off is required: the restatement must round like the
reference's unfused double arithmetic on any host (aarch64 compilers contract
a*b+c into fma by default).
"""
from __future__ import annotations

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


if __name__ == "__main__":
    print(build())
