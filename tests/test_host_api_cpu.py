"""The C++ host API compiles the programs written against the reference.

The deck driver of the golden fixtures (oracle/refbuild/ref_driver.cpp) is
one source that builds against the reference's own headers and, unchanged,
against parm_gb300/host; the reference's example program src/bin/LJatoms.cpp
does too where the reference sources are present.  (Running them needs a GPU:
tests/test_gpu_host_api.py.)
"""
import os
from pathlib import Path

import pytest

from host_api import DECK_DRIVER, compile_program

REF_SRC = Path(os.environ.get("PARM_REFERENCE_SRC", "/root/reference/src"))


@pytest.mark.parametrize("ndim", [3, 2])
def test_deck_driver_builds_against_host_api(tmp_path, built_lib, ndim):
    r = compile_program(DECK_DRIVER, tmp_path / f"drv{ndim}", ndim=ndim)
    assert r.returncode == 0, r.stderr[-3000:]
    assert (tmp_path / f"drv{ndim}").exists()


@pytest.mark.parametrize("prog", ["LJatoms.cpp", "packer.cpp"])
def test_reference_programs_build_against_host_api(tmp_path, built_lib, prog):
    """The reference's example programs (src/bin/LJatoms.cpp: CollectionVerlet; src/bin/packer.cpp:
    CollectionNLCG) compile and link unchanged against the host API."""
    src = REF_SRC / "bin" / prog
    if not src.exists():
        pytest.skip("reference sources not present")
    r = compile_program(src, tmp_path / prog.replace(".cpp", ""))
    assert r.returncode == 0, r.stderr[-3000:]


def test_packing_program_builds(tmp_path, built_lib):
    """The CollectionNLCG packing program of the GPU tests builds against the host API."""
    src = Path(__file__).resolve().parent / "programs" / "nlcg_packing.cpp"
    r = compile_program(src, tmp_path / "packing")
    assert r.returncode == 0, r.stderr[-3000:]


def test_rsq_tracker_program_builds(tmp_path, built_lib):
    """A program using RsqTracker inside a Collection builds against the host API."""
    src = Path(__file__).resolve().parent / "programs" / "rsq_tracker.cpp"
    r = compile_program(src, tmp_path / "rsq")
    assert r.returncode == 0, r.stderr[-3000:]


def test_energy_tracker_program_builds(tmp_path, built_lib):
    """EnergyTracker and a caller-defined tracker in a Collection build against the host API."""
    src = Path(__file__).resolve().parent / "programs" / "energy_tracker.cpp"
    r = compile_program(src, tmp_path / "et")
    assert r.returncode == 0, r.stderr[-3000:]
