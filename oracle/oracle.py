"""CPU oracle for the ChFSI / Poisson hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this module; the product library never does.

* ``fe_oracle.c`` (built here into ``liboracle.so``) restates the reference's
  apply, constraints, Chebyshev filters and CG line by line (see its header
  for the reference file:line of every routine).  Its per-cell product calls
  the same Fortran ``dgemm`` the reference calls (scipy's bundled OpenBLAS,
  reached through ``scipy.linalg.cython_blas``), so the oracle is also the
  reference-speed CPU baseline.
* The FP64 dense stages are restated here with numpy/scipy LAPACK:
  - ``cholesky_gram_schmidt``: OrthonormalizationFunctions.t.cpp:356-415
    (computeXTransOpX -> potrf('L') -> trtri('L','N') -> gemm('N','N'));
  - ``rayleigh_ritz``: RayleighRitzEigenSolver.t.cpp:233-301
    (computeXTransOpX -> heevd('V','L') -> gemm('T','N'));
  - ``eigen_residual_norms``: KohnShamEigenSolver.t.cpp:574-684;
  - ``chfsi_pass``: ChebyshevFilteredEigenSolver.t.cpp:194-437;
  - ``ks_eigen_solve``: the pass loop of KohnShamEigenSolver.t.cpp:319-487
    (without the Fermi-level step) and its bound heuristics :262-300;
  - ``lanczos_bounds``: LanczosExtremeEigenSolver.t.cpp:230-440.
* Either side of the eigensolve (module functions, numpy FP64):
  - ``assemble_cells``: KohnShamOperatorContextFE::reinit
    (ksdft/KohnShamOperatorContextFE.t.cpp:1253-1311) with the kinetic part
    (ksdft/KineticFE.t.cpp:90-97) passed as fixed matrices and the local
    potential part int N_i V N_j (ksdft/ElectrostaticLocalFE.t.cpp:1625-1660);
  - ``density_cells``: DensityCalculator's interpolation of psi to the
    quadrature points and rho = sum_i 2 |psi_i|^2 f_i
    (ksdft/DensityCalculator.t.cpp:37-100, 283-345).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import scipy.linalg as sla

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build(force: bool = False) -> Path:
    src = HERE / "fe_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        cc = os.environ.get("CC", "gcc")
        subprocess.run([cc, "-O3", "-fPIC", "-shared", "-std=c99", str(src), "-o", str(LIB), "-lm"], check=True)
    return LIB


class _Mesh(C.Structure):
    _fields_ = [("n_dofs", C.c_uint64), ("n_cells", C.c_uint32), ("nd", C.c_void_p), ("ids", C.c_void_p),
                ("cell_off", C.c_void_p), ("mat_off", C.c_void_p)]


class _Cons(C.Structure):
    _fields_ = [("nrows", C.c_uint32), ("row_ids", C.c_void_p), ("row_sizes", C.c_void_p), ("col_ids", C.c_void_p),
                ("row_acc", C.c_void_p), ("col_vals", C.c_void_p), ("inh", C.c_void_p)]


class _Op(C.Structure):
    _fields_ = [("kind", C.c_int), ("mesh", C.c_void_p), ("cons", C.c_void_p), ("mats", C.c_void_p),
                ("diag", C.c_void_p), ("blk_begin", C.c_uint64), ("blk_n", C.c_uint64), ("blk", C.c_void_p),
                ("nl", C.c_void_p)]


class _NonLocal(C.Structure):
    _fields_ = [("n_proj", C.c_uint32), ("np", C.c_void_p), ("pids", C.c_void_p), ("p_off", C.c_void_p),
                ("c_off", C.c_void_p), ("cmat", C.c_void_p), ("v", C.c_void_p)]


_lib = None


def _dgemm_pointer() -> int:
    """Address of scipy's LP64 Fortran dgemm (the BLAS the reference links)."""
    from scipy.linalg import cython_blas

    cap = cython_blas.__pyx_capi__["dgemm"]
    get_name = C.pythonapi.PyCapsule_GetName
    get_name.restype = C.c_char_p
    get_name.argtypes = [C.py_object]
    get_ptr = C.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = C.c_void_p
    get_ptr.argtypes = [C.py_object, C.c_char_p]
    return get_ptr(cap, get_name(cap))


def load(use_blas: bool = True):
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        P = C.c_void_p
        lib.orc_apply.argtypes = [P, P, P, C.c_uint32]
        lib.orc_p2c.argtypes = [P, P, C.c_uint32]
        lib.orc_c2p.argtypes = [P, P, C.c_uint32]
        lib.orc_set_dgemm.argtypes = [P]
        lib.orc_residual_chebyshev_filter.argtypes = [P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                                      C.c_double, P]
        lib.orc_chebyshev_filter.argtypes = [P, P, P, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, P]
        lib.orc_cg.argtypes = [P, P, P, P, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                               C.POINTER(C.c_uint32), P]
        lib.orc_sweep.argtypes = [C.c_uint64, C.c_uint32, C.c_double, P, C.c_double, P, P, P]
        lib.orc_sweep.restype = None
        _lib = lib
    _lib.orc_set_dgemm(C.c_void_p(_dgemm_pointer()) if use_blas else None)
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class OracleSystem:
    """Holds one mesh + constraints and builds oracle operators on it."""

    def __init__(self, nd_per_cell, cell_dof_ids, n_dofs, constraints=None, use_blas: bool = True):
        self.lib = load(use_blas)
        self.keep = []
        nd = np.ascontiguousarray(nd_per_cell, dtype=np.uint32)
        ids = np.ascontiguousarray(cell_dof_ids, dtype=np.uint32)
        coff = np.zeros(nd.size + 1, np.uint64)
        np.cumsum(nd.astype(np.uint64), out=coff[1:])
        moff = np.zeros(nd.size + 1, np.uint64)
        np.cumsum(nd.astype(np.uint64) ** 2, out=moff[1:])
        self.keep += [nd, ids, coff, moff]
        self.mesh = _Mesh(int(n_dofs), nd.size, _p(nd).value, _p(ids).value, _p(coff).value, _p(moff).value)
        self.n_dofs = int(n_dofs)
        self.cons = None
        if constraints is not None:
            arrs = [np.ascontiguousarray(a, dtype=t) for a, t in (
                (constraints.row_ids, np.uint32), (constraints.row_sizes, np.uint32),
                (constraints.col_ids, np.uint32), (constraints.row_acc, np.uint32),
                (constraints.col_values, np.float64), (constraints.inhomogeneities, np.float64))]
            self.keep += arrs
            self.cons = _Cons(arrs[0].size, *[_p(a).value for a in arrs])

    @classmethod
    def from_problem(cls, prob, **kw):
        return cls(prob.nd_per_cell, prob.cell_dof_ids, prob.n_dofs, prob.constraints, **kw)

    def _op(self, kind, mats=None, diag=None, use_cons=True):
        arr = np.ascontiguousarray(mats if mats is not None else diag, dtype=np.float64)
        self.keep.append(arr)
        op = _Op(kind, C.addressof(self.mesh), C.addressof(self.cons) if (self.cons is not None and use_cons) else None,
                 _p(arr).value if mats is not None else None, _p(arr).value if diag is not None else None)
        self.keep.append(op)
        return op

    def cell_op(self, mats, use_cons=True, nonlocal_part=None):
        op = self._op(0, mats=mats, use_cons=use_cons)
        if nonlocal_part is not None:
            op.nl = C.addressof(nonlocal_part)
        return op

    def nonlocal_part(self, data):
        """Projector data (gbfe.nonlocal_psp.NonLocalData) as an oracle structure."""
        nd = self.keep[0].astype(np.uint64)
        npc = np.ascontiguousarray(data.proj_per_cell, dtype=np.uint32)
        poff = np.zeros(npc.size + 1, np.uint64)
        np.cumsum(npc.astype(np.uint64), out=poff[1:])
        coff = np.zeros(npc.size + 1, np.uint64)
        np.cumsum(npc.astype(np.uint64) * nd, out=coff[1:])
        pids = np.ascontiguousarray(data.proj_ids, dtype=np.uint32)
        cm = np.ascontiguousarray(data.cell_c, dtype=np.float64)
        v = np.ascontiguousarray(data.coupling, dtype=np.float64)
        self.keep += [npc, poff, coff, pids, cm, v]
        nl = _NonLocal(int(data.n_proj), _p(npc).value, _p(pids).value, _p(poff).value, _p(coff).value,
                       _p(cm).value, _p(v).value)
        self.keep.append(nl)
        return nl

    def nonlocal_op(self, nonlocal_part, use_cons=True):
        """AtomCenterNonLocalOpContextFE::apply alone (no cell matrices)."""
        op = _Op(0, C.addressof(self.mesh), C.addressof(self.cons) if (self.cons is not None and use_cons) else None,
                 None, None)
        op.nl = C.addressof(nonlocal_part)
        self.keep.append(op)
        return op

    def diag_op(self, diag, use_cons=True):
        return self._op(1, diag=diag, use_cons=use_cons)

    def jacobi_op(self, diagonal):
        return self._op(2, diag=1.0 / np.asarray(diagonal, dtype=np.float64), use_cons=False)

    def diag_block_op(self, diag, blk_begin, blk, use_cons=True):
        """OrthoEFE inverse overlap: diagonal + dense block on [blk_begin, blk_begin + n)."""
        op = self._op(3, diag=diag, use_cons=use_cons)
        b = np.ascontiguousarray(np.asarray(blk, dtype=np.float64).T)  # store column-major
        self.keep.append(b)
        op.blk_begin, op.blk_n, op.blk = int(blk_begin), int(b.shape[0]), b.ctypes.data
        return op

    # ---- operations (row-major [N][m] float64 arrays, modified like the reference)
    def apply(self, op, X: np.ndarray) -> np.ndarray:
        assert X.dtype == np.float64 and X.flags.c_contiguous
        m = X.shape[1]
        Y = np.empty_like(X)
        rc = self.lib.orc_apply(C.byref(op), _p(X), _p(Y), m)
        if rc:
            raise RuntimeError(f"orc_apply failed ({rc})")
        return Y

    def p2c(self, X):
        self.lib.orc_p2c(C.byref(self.cons), _p(X), X.shape[1])

    def c2p(self, X):
        self.lib.orc_c2p(C.byref(self.cons), _p(X), X.shape[1])

    def residual_filter(self, A, B, BInv, eig, X, degree, wl, wu, uu) -> np.ndarray:
        eig = np.ascontiguousarray(eig, dtype=np.float64)
        Y = np.zeros_like(X)
        rc = self.lib.orc_residual_chebyshev_filter(C.byref(A), C.byref(B), C.byref(BInv), _p(eig), _p(X),
                                                    X.shape[1], int(degree), wl, wu, uu, _p(Y))
        if rc:
            raise RuntimeError("oracle filter failed")
        return Y

    def chebyshev_filter(self, A, BInv, X, degree, wl, wu, uu) -> np.ndarray:
        Y = np.zeros_like(X)
        self.lib.orc_chebyshev_filter(C.byref(A), C.byref(BInv), _p(X), X.shape[1], int(degree), wl, wu, uu, _p(Y))
        return Y

    def cg(self, A, PC, b, x0, max_iter, abs_tol, rel_tol, div_tol):
        x = np.ascontiguousarray(x0, dtype=np.float64).copy()
        it = C.c_uint32()
        rn = np.empty(b.shape[1])
        rc = self.lib.orc_cg(C.byref(A), C.byref(PC), _p(np.ascontiguousarray(b)), _p(x), b.shape[1], int(max_iter),
                             abs_tol, rel_tol, div_tol, C.byref(it), _p(rn))
        return rc, x, int(it.value), rn

    # ---- FP64 dense stages (serial LAPACK branches)
    def cholesky_gram_schmidt(self, B, X):
        """Returns (status, X_ortho).  status 0 ok, 4 not orthonormalizable, 5 lapack error."""
        N, m = X.shape
        if N < m:
            return 4, None
        BX = self.apply(B, X)
        S = X.T @ BX  # S(i,j) = x_i . (B x_j); lower triangle used
        S = np.tril(S)
        try:
            L = sla.cholesky(S + np.tril(S, -1).T, lower=True)
        except sla.LinAlgError:
            return 5, None
        Linv = sla.solve_triangular(L, np.eye(m), lower=True)
        return 0, X @ Linv.T

    def rayleigh_ritz(self, A, X):
        AX = self.apply(A, X)
        P = X.T @ AX
        P = np.tril(P) + np.tril(P, -1).T
        w, Q = sla.eigh(P, driver="evd")
        return w, X @ Q

    def eigen_residual_norms(self, A, B, X, eig):
        HX = self.apply(A, X)
        MX = self.apply(B, X)
        R = -HX + MX * np.asarray(eig)[None, :]
        return np.sqrt((R * R).sum(axis=0))

    def chfsi_pass(self, A, B, BInv, X, eig, degree, wl, wu, uu):
        Y = self.residual_filter(A, B, BInv, eig, X, degree, wl, wu, uu)
        st, Xo = self.cholesky_gram_schmidt(B, Y)
        if st:
            raise RuntimeError(f"oracle Cholesky-GS failed ({st})")
        return self.rayleigh_ritz(A, Xo)

    def sweep(self, a, x, b, coef, y, z):
        """z = a x + b coef[j] y (one vector update of the filter's kind, in C)."""
        self.lib.orc_sweep(x.size, x.shape[1], float(a), _p(x), float(b), _p(np.ascontiguousarray(coef)), _p(y), _p(z))

    def lanczos_bounds(self, A, B, BInv, steps=20, seed=7, start=None):
        """start: the initial vector (n_dofs values); None draws MT19937(seed) uniform [0, 1)."""
        if start is None:
            rng = np.random.Generator(np.random.MT19937(seed))
            x0 = rng.random((self.n_dofs, 1))
        else:
            x0 = np.ascontiguousarray(start, dtype=np.float64).reshape(self.n_dofs, 1).copy()
        temp = self.apply(B, x0)
        alpha = np.sqrt(float((x0 * temp).sum()))
        q = x0 / alpha
        qprev = np.zeros_like(q)
        beta = 0.0
        av, bv = [], []
        for _ in range(steps):
            temp = self.apply(A, q)
            v = self.apply(BInv, temp.copy())
            alpha = float((q * temp).sum())
            av.append(alpha)
            v = v - alpha * q
            v = v - beta * qprev
            temp = self.apply(B, v)
            beta = float(np.sqrt((v * temp).sum()))
            bv.append(beta)
            qprev = q.copy()
            if beta < 1e-14:
                break
            q = v / beta
        k = len(av)
        T = np.diag(av) + np.diag(bv[: k - 1], 1) + np.diag(bv[: k - 1], -1)
        w = np.linalg.eigvalsh(T)
        return np.array([w[0], w[-1], bv[-1]])

    def ks_eigen_solve(self, A, B, BInv, X0, degree, max_passes, n_wanted, tol, bounds=None, eig0=None,
                       fixed_passes=False, lanczos_steps=20, lanczos_seed=7, lanczos_start=None):
        X = np.ascontiguousarray(X0, dtype=np.float64).copy()
        m = X.shape[1]
        if bounds is None:
            b = self.lanczos_bounds(A, B, BInv, lanczos_steps, lanczos_seed, start=lanczos_start)
            res = b[2] / 10.0
            wl, uu = b[0], b[1] + res
            wu = (b[1] + res - b[0]) * (m * 200.0 / self.n_dofs) + b[0]
            if wu >= uu:
                wu = (uu + b[0]) * 0.5
        else:
            wl, wu, uu = bounds
        eig = np.zeros(m) if eig0 is None else np.asarray(eig0, dtype=np.float64).copy()
        status, passes, resid = 6, 0, None
        for it in range(max_passes):
            eig, X = self.chfsi_pass(A, B, BInv, X, eig, degree, wl, wu, uu)
            resid = self.eigen_residual_norms(A, B, X, eig)
            passes = it + 1
            conv = bool(np.all(resid[:n_wanted] <= tol))
            if conv and not fixed_passes:
                status = 0
                break
            if fixed_passes and passes == max_passes:
                status = 0 if conv else 6
            wl, wu = eig[0], eig[m - 1]
        return status, eig, X, resid, passes


def _cell_blocks(nd, nq_per_cell, basis_values):
    off = 0
    for k, q in zip(np.asarray(nd, np.int64), np.asarray(nq_per_cell, np.int64)):
        yield k, q, basis_values[off: off + q * k].reshape(q, k)
        off += q * k


def assemble_cells(nd, nq_per_cell, basis_values, weights, fixed_mats=None, alpha=1.0):
    """Cell matrices A_c = alpha F_c + B_c^T diag(w_c) B_c, column-major per
    cell, cells concatenated (the layout of d_hamiltonianInAllCells)."""
    out, moff, qoff = [], 0, 0
    for k, q, Bc in _cell_blocks(nd, nq_per_cell, basis_values):
        A = Bc.T @ (weights[qoff: qoff + q, None] * Bc)
        if fixed_mats is not None:
            A = A + alpha * fixed_mats[moff: moff + k * k].reshape(k, k).T
        out.append(A.T.ravel())
        moff += k * k
        qoff += q
    return np.concatenate(out)


def density_cells(nd, ids, Psi, occupation, nq_per_cell, basis_values):
    """rho at each cell's quadrature points, cells concatenated."""
    out, doff = [], 0
    occ = np.asarray(occupation, dtype=np.float64)
    for k, q, Bc in _cell_blocks(nd, nq_per_cell, basis_values):
        psi = Bc @ Psi[np.asarray(ids[doff: doff + k], np.int64)]  # nq_c x m
        out.append((2.0 * psi * psi * occ[None, :]).sum(axis=1))
        doff += k
    return np.concatenate(out)
