"""The C ABI library loads and exports every declared entry point (no GPU calls)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(parm_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "parm_create" in names and "parm_verlet" in names and len(names) >= 30


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_matches_header(built_lib):
    from parm_gb300 import capi
    assert set(declared_functions()) <= set(capi.SIGNATURES), set(declared_functions()) - set(capi.SIGNATURES)


def test_argument_errors_without_device(built_lib):
    """Argument validation happens before any CUDA call and maps to ValueError."""
    from parm_gb300 import capi
    lib = capi.load()
    assert lib.parm_version() == 100
    h = ctypes.c_void_p()
    n = (ctypes.c_uint32 * 1)(10)
    assert lib.parm_create(ctypes.byref(h), 4, 1, n, 0) == capi.PARM_ERR_ARG
    assert b"ndim" in lib.parm_last_error()
    assert lib.parm_create(ctypes.byref(h), 3, 1, n, 7) == capi.PARM_ERR_ARG
    with pytest.raises(ValueError):
        capi.check(capi.PARM_ERR_ARG)


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from parm_gb300 import capi
    monkeypatch.setattr(capi, "_lib", None)
    monkeypatch.setattr(capi, "LIBPATH", tmp_path / "nope.so")
    with pytest.raises(ImportError):
        capi.load()
