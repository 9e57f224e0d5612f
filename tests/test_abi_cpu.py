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


def test_operator_context_adapter_compiles_against_reference_headers(tmp_path):
    """The C++ drop-in (include/gbfe_operator_context.hpp) type-checks against
    the reference's own OperatorContext / MultiVector headers, instantiated
    for HOST and DEVICE memory spaces.  Skipped where the reference sources are
    not present."""
    import shutil
    import subprocess

    import pytest

    found = subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh"), "--source"], capture_output=True,
                           text=True)
    ref = Path(found.stdout.strip()) if found.returncode == 0 else None
    if ref is None or not ref.is_dir() or not shutil.which("g++"):
        pytest.skip("reference sources not available")
    src = tmp_path / "adapter.cpp"
    src.write_text(
        "#include <gbfe_operator_context.hpp>\n"
        "using namespace dftefe;\n"
        "template class dftefe::gb300::GpuCellOperatorContext<double, double, utils::MemorySpace::HOST>;\n"
        "template class dftefe::gb300::GpuDiagonalOperatorContext<double, double, utils::MemorySpace::HOST>;\n"
        "template class dftefe::gb300::GpuCellOperatorContext<float, float, utils::MemorySpace::HOST>;\n"
        "int main() { return 0; }\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-DNDEBUG", "-w", f"-I{ROOT / 'include'}",
                        f"-I{ROOT / 'oracle' / 'ref_harness' / 'shadow'}", f"-I{ref}", str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
