"""The host dense kernels of the small Rayleigh-Ritz block
(csrc/gbfe_host_eig.cpp), compiled on their own and checked against numpy:
the symmetric eigen-decomposition (eigenvalues within 1e-13 ||A||, residual
||A V - V L|| and orthogonality ||V^T V - I|| within 1e-13, ||A|| for the
residual), the Cholesky factor (1e-13 relative, LAPACK potrf's info on a
matrix that is not positive definite) and the solves L^-1 A L^-T and L^-T B
(1e-12 relative)."""
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
                    '{ return gbfe::host_sym_eig(n, a, w); }\n'
                    'extern "C" int chol(int n, double *a) { return gbfe::host_cholesky(n, a); }\n'
                    'extern "C" void sandwich(int n, const double *L, double *A) { gbfe::host_sandwich(n, L, A); }\n'
                    'extern "C" void trsm_lt(int n, const double *L, double *B) { gbfe::host_trsm_lower_t(n, L, B); }\n'
                    'extern "C" void arm(int on) { gbfe::host_pool_arm(on != 0); }\n')
    lib = d / "libeig.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", str(wrap), "-o", str(lib)], check=True)
    L = C.CDLL(str(lib))
    L.eig.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    L.eig.restype = C.c_int
    L.chol.argtypes = [C.c_int, C.c_void_p]
    L.chol.restype = C.c_int
    L.sandwich.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    L.trsm_lt.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    L.arm.argtypes = [C.c_int]

    def run(A):
        n = A.shape[0]
        a = np.asfortranarray(A.copy())
        w = np.empty(n)
        rc = L.eig(n, a.ctypes.data, w.ctypes.data)
        return rc, w, a

    run.lib = L
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


@pytest.mark.parametrize("n", [1, 2, 7, 64, 128])
def test_host_cholesky_and_solves(eig, n):
    L_ = eig.lib
    rng = np.random.default_rng(n)
    G = rng.standard_normal((n, n))
    A = G @ G.T + n * np.eye(n)
    Lh = np.asfortranarray(A.copy())
    assert L_.chol(n, Lh.ctypes.data) == 0
    Lr = np.linalg.cholesky(A)
    assert np.abs(Lh - Lr).max() <= 1e-13 * np.abs(Lr).max()
    H = rng.standard_normal((n, n))
    H = H + H.T
    S = np.asfortranarray(H.copy())
    L_.sandwich(n, Lh.ctypes.data, S.ctypes.data)
    Li = np.linalg.inv(Lr)
    Sr = Li @ H @ Li.T
    assert np.abs(S - Sr).max() <= 1e-12 * np.abs(Sr).max()
    assert np.array_equal(S, S.T)
    B = np.asfortranarray(rng.standard_normal((n, n)))
    Br = np.linalg.solve(Lr.T, B)
    L_.trsm_lt(n, Lh.ctypes.data, B.ctypes.data)
    assert np.abs(B - Br).max() <= 1e-12 * np.abs(Br).max()


def test_host_cholesky_reports_the_failing_minor(eig):
    A = np.asfortranarray(np.diag([1.0, 2.0, -1.0, 4.0]))
    assert eig.lib.chol(4, A.ctypes.data) == 3


def test_host_block_is_deterministic_under_threads(eig):
    """The pool splits a job by problem size only and any thread may run any
    part: repeated decompositions and solves of the same 64 x 64 block (the
    size that uses the pool) give the same bits every time."""
    rng = np.random.default_rng(11)
    n = 64
    Q = rng.standard_normal((n, n))
    A = Q + Q.T + n * np.eye(n)
    ref = eig(A)
    for _ in range(25):
        rc, w, v = eig(A)
        assert rc == ref[0] and np.array_equal(w, ref[1]) and np.array_equal(v, ref[2])


def test_host_pool_armed_and_sleeping_give_the_same_bits(eig):
    """The pool's workers spin while armed and sleep otherwise; jobs run the
    same either way (and arming without a job, or twice, is harmless)."""
    rng = np.random.default_rng(12)
    n = 64
    Q = rng.standard_normal((n, n))
    A = Q + Q.T
    ref = eig(A)
    L = eig.lib
    L.arm(1)
    L.arm(1)
    try:
        for _ in range(5):
            rc, w, v = eig(A)
            assert rc == ref[0] and np.array_equal(w, ref[1]) and np.array_equal(v, ref[2])
    finally:
        L.arm(0)
    L.arm(0)
    rc, w, v = eig(A)
    assert np.array_equal(w, ref[1]) and np.array_equal(v, ref[2])
