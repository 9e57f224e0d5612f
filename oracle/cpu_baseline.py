"""CPU baseline of a whole ChFSI solve, measured on a sample -- TEST
INFRASTRUCTURE ONLY (used by bench.py's CPU legs; the product never imports
it).

A full FP64 solve of the large workloads takes hours on one host core (one
Hamiltonian apply of the 24^3-cell degree-5 case is ~660 GFLOP), so the
baseline is measured per operation and multiplied out:

* the operations of one FP64 pass in the reference's call sequence are
  counted from the code the oracle restates (``pass_counts``):
  ResidualChebyshevFilterGEP (linearAlgebra/ChebyshevFilter.t.cpp:242-444:
  one B and one A apply for the initial residual, then per degree step one
  B^-1 and one A apply and three vector updates, one final B^-1 apply and
  update), Cholesky-Gram-Schmidt (OrthonormalizationFunctions.t.cpp:356-415:
  B apply, X^T B X, potrf, trtri, X L^-T), Rayleigh-Ritz
  (RayleighRitzEigenSolver.t.cpp:233-301: A apply, X^T A X, syevd, X Q) and
  the residual of KohnShamEigenSolver.t.cpp:574-684 (A and B applies, one
  update, the norms); the Lanczos bounds of a solve
  (LanczosExtremeEigenSolver.t.cpp:296-440) add 20 single-vector A, B^-1, B
  applies;
* each operation is timed once with the oracle on a slab of the same
  workload -- the first layer(s) of cells of the mesh with every vector of
  the block (``slab``) -- and scaled to the whole mesh by cell-matrix entries
  (cell applies) or rows (vector updates, the tall-skinny products); the
  m x m factorisations are timed at full size;
* solve time = Lanczos + passes x pass time.

``predicted_vs_measured`` checks the model on a workload small enough for a
whole oracle solve.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np
import scipy.linalg as sla

from . import oracle as O


def pass_counts(degree: int) -> dict:
    """Operations of one FP64 pass of the reference (see module docstring)."""
    d = int(degree)
    return {
        # filter: B, A (initial residual) + (d-1) A + CholGS B + RR A + residual A, B
        "cell": (2 + (d - 1)) + 1 + 1 + 2,
        "diag": (d - 1) + 1,
        # filter: residual, copy, scale + 3 per degree step + final; residual update + norms
        "sweep": 3 + 3 * (d - 1) + 1 + 2,
        "gram": 2,  # X^T B X, X^T A X
        "rot": 2,  # X L^-T, X Q
        "chol": 1,  # potrf + trtri of the m x m Gram matrix
        "eig": 1,  # syevd of the m x m projected matrix
    }


LANCZOS_STEPS = 20


def lanczos_counts(steps: int = LANCZOS_STEPS) -> dict:
    return {"cell1": 2 * steps + 1, "diag1": steps}


@dataclass
class Slab:
    """A sub-mesh made of the first cells of a mesh, with its own dof numbering."""
    nd: np.ndarray
    ids: np.ndarray
    n_dofs: int
    H: np.ndarray
    minv: np.ndarray
    cons_rows: np.ndarray
    cell_scale: float  # whole-mesh cell-matrix entries / slab's
    row_scale: float  # whole-mesh rows / slab's


def slab(prob, min_rows: int, layers: int = 1) -> Slab:
    """The first `layers` z-layers of cells (cells are numbered x fastest, so a
    layer is a contiguous run of cells), grown until the slab has at least
    `min_rows` dofs (a Cholesky of the m x m Gram matrix needs N >= m)."""
    C = prob.n_cells
    per_layer = max(1, int(round(prob.n_side ** 2))) if getattr(prob, "n_side", 0) else C
    nd = prob.nd_per_cell.astype(np.int64)
    off = np.zeros(C + 1, np.int64)
    np.cumsum(nd, out=off[1:])
    moff = np.zeros(C + 1, np.int64)
    np.cumsum(nd * nd, out=moff[1:])
    while True:
        nc = min(C, layers * per_layer)
        ids = prob.cell_dof_ids[: off[nc]].astype(np.int64)
        uniq, inv = np.unique(ids, return_inverse=True)
        if uniq.size >= min_rows or nc == C:
            break
        layers += 1
    rows = np.isin(prob.constraints.row_ids.astype(np.int64), uniq)
    keep_rows = np.searchsorted(uniq, prob.constraints.row_ids.astype(np.int64)[rows])
    return Slab(nd=prob.nd_per_cell[:nc].copy(), ids=inv.astype(np.uint32), n_dofs=int(uniq.size),
                H=np.ascontiguousarray(prob.H[: moff[nc]]), minv=1.0 / prob.m_gll_diag[uniq],
                cons_rows=keep_rows.astype(np.uint32), cell_scale=float(moff[C]) / float(moff[nc]),
                row_scale=float(prob.n_dofs) / float(uniq.size))


def slab_arrays(s: Slab) -> dict:
    return dict(nd=s.nd, ids=s.ids, n_dofs=s.n_dofs, H=s.H, minv=s.minv, cons_rows=s.cons_rows,
                cell_scale=s.cell_scale, row_scale=s.row_scale)


def time_operations(z: dict, m: int, seed: int = 5) -> dict:
    """Seconds of one of each operation on the slab (one thread).  Each input
    is a fresh copy, as in the reference's pass (the applies modify X)."""
    import gbfe.mesh as M  # the input generator's Constraints container

    nr = z["cons_rows"].size
    cons = M.Constraints(z["cons_rows"].astype(np.uint32), np.zeros(nr, np.uint32), np.zeros(0, np.uint32),
                         np.zeros(nr, np.uint32), np.zeros(0), np.zeros(nr))
    s = O.OracleSystem(z["nd"], z["ids"], int(z["n_dofs"]), cons)
    H = s.cell_op(z["H"])
    Mi = s.diag_op(z["minv"])
    N = int(z["n_dofs"])
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N, m))
    Y = rng.standard_normal((N, m))
    coef = rng.standard_normal(m)
    out = {}

    def timed(key, fn):
        # short operations are repeated (median of up to 7) so that one-off
        # costs (first touch, cold caches) do not dominate them
        ts = []
        while len(ts) < 7:
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
            if sum(ts) > 0.25:
                break
        out[key] = float(np.median(ts))

    timed("cell", lambda: s.apply(H, X.copy()))
    timed("diag", lambda: s.apply(Mi, X.copy()))
    Z = np.empty_like(X)
    timed("sweep", lambda: s.sweep(1.0, X, -1.0, coef, Y, Z))
    # the dense stages as the oracle computes them (numpy / LAPACK, FP64)
    timed("gram", lambda: X.T @ Y)
    S = X.T @ X / N + np.eye(m)
    timed("chol", lambda: sla.solve_triangular(sla.cholesky(S, lower=True), np.eye(m), lower=True))
    T = rng.standard_normal((m, m))
    timed("rot", lambda: X @ T)
    timed("eig", lambda: sla.eigh(S, driver="evd"))
    x1 = X[:, :1].copy()
    timed("cell1", lambda: s.apply(H, x1.copy()))
    timed("diag1", lambda: s.apply(Mi, x1.copy()))
    return out


SCALE = {"cell": "cell", "diag": "row", "sweep": "row", "gram": "row", "rot": "row", "chol": None, "eig": None,
         "cell1": "cell", "diag1": "row"}


def solve_seconds(t: dict, cell_scale: float, row_scale: float, degree: int, passes: float) -> dict:
    """Whole-workload seconds of a pass and of a solve from slab timings."""
    def full(key):
        sc = SCALE[key]
        return t[key] * (cell_scale if sc == "cell" else row_scale if sc == "row" else 1.0)

    per_pass = sum(n * full(k) for k, n in pass_counts(degree).items())
    lanczos = sum(n * full(k) for k, n in lanczos_counts().items())
    return {"pass_s": per_pass, "lanczos_s": lanczos, "solve_s": lanczos + passes * per_pass}


def worker(args):
    """One single-threaded process: time the operations on the slab file."""
    path, m = args
    z = dict(np.load(path))
    return time_operations(z, m)
