"""The host symmetric eigen-decomposition used for the small Rayleigh-Ritz
matrices (csrc/gbfe_host_eig.cpp), compiled on its own and checked against
numpy.linalg.eigh: eigenvalues within 1e-13 ||A||, residual ||A V - V L|| and
orthogonality ||V^T V - I|| within 1e-13 (||A|| for the residual)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

SRC = Path(__file__).resolve().parent.parent / "dft-efe_gb300" / "csrc" / "gbfe_host_eig.cpp"


@pytest.fixture(scope="module")
def eig(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("host_eig")
    wrap = d / "wrap.cpp"
    wrap.write_text(f'#include "{SRC}"\nextern "C" int eig(int n, double *a, double *w) '
                    '{ return gbfe::host_sym_eig(n, a, w); }\n')
    lib = d / "libeig.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", str(wrap), "-o", str(lib)], check=True)
    L = C.CDLL(str(lib))
    L.eig.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    L.eig.restype = C.c_int

    def run(A):
        n = A.shape[0]
        a = np.asfortranarray(A.copy())
        w = np.empty(n)
        rc = L.eig(n, a.ctypes.data, w.ctypes.data)
        return rc, w, a

    return run


def _cases():
    rng = np.random.default_rng(3)
    out = []
    for n in (1, 2, 3, 10, 64, 100):
        B = rng.standard_normal((n, n))
        out.append((f"random{n}", B + B.T))
    Q, _ = np.linalg.qr(rng.standard_normal((48, 48)))
    out.append(("clustered", Q @ np.diag(np.repeat([1.0, 2.0, 2.0 + 1e-12, 5.0], 12)) @ Q.T))
    out.append(("diagonal", np.diag(rng.standard_normal(20))))
    out.append(("zero", np.zeros((8, 8))))
    G = np.diag(10.0 ** np.linspace(-8, 8, 40))
    Q2, _ = np.linalg.qr(rng.standard_normal((40, 40)))
    out.append(("graded", Q2 @ G @ Q2.T))
    T = np.diag(np.full(30, 2.0)) + np.diag(np.full(29, -1.0), 1) + np.diag(np.full(29, -1.0), -1)
    out.append(("laplacian1d", T))
    return out


@pytest.mark.parametrize("name,A", _cases(), ids=[c[0] for c in _cases()])
def test_host_sym_eig_matches_eigh(eig, name, A):
    A = 0.5 * (A + A.T)
    rc, w, V = eig(A)
    assert rc == 0
    n = A.shape[0]
    nrm = max(np.abs(A).max(), 1e-300)
    ref = np.linalg.eigvalsh(A)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - ref).max() <= 1e-13 * nrm * max(1, n / 10)
    assert np.abs(A @ V - V * w).max() <= 1e-13 * nrm * max(1, n / 10)
    assert np.abs(V.T @ V - np.eye(n)).max() <= 1e-13 * max(1, n / 10)
