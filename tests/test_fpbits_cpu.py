"""The bit-pattern float <-> double conversions of the mixed-precision update
(parm_gb300/csrc/fpbits.cuh) equal the host's IEEE conversions: edge cases,
exact rounding ties, carries into the exponent, the ends of the float range
and 4M seeded random values of each kind (tests/programs/fpbits_check.cpp)."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_fpbits_match_host_conversions(tmp_path):
    exe = tmp_path / "fpbits_check"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'parm_gb300' / 'csrc'}",
                        str(ROOT / "tests" / "programs" / "fpbits_check.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok "), r.stdout + r.stderr
