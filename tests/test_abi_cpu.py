"""CPU checks of the drop-in boundary: libgbfe.so loads and exports every
symbol declared in include/gbfe.h (no compute call without a GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    hdr = (ROOT / "include" / "gbfe.h").read_text()
    return sorted(set(re.findall(r"^int\s+(gbfe_\w+)\s*\(", hdr, flags=re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gbfe_apply" in syms and "gbfe_ks_eigen_solve" in syms and "gbfe_cg_solve" in syms


def test_library_exports_declared_symbols():
    from gbfe.build import build

    lib_path = build()
    lib = ctypes.CDLL(str(lib_path))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from gbfe import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_no_cpu_fallback_when_library_missing(tmp_path):
    import pytest
    from gbfe import _lib

    with pytest.raises(ImportError):
        _lib.load(tmp_path / "absent.so")
