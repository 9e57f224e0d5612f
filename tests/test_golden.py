"""Golden vectors produced by the reference's own CPU implementation
(tests/golden/make_golden.py drives oracle/_ref/ref_driver, built from the
reference sources).  They pin the oracle port (CPU tests) and the CUDA path
(GPU tests).

Tolerances: applies 1e-12 relative max-norm; X after the constraint
distribution 1e-15 (one rounding: the reference's daxpy may fuse the
multiply-add); filters (degree 5-8) 1e-10; CG solution 1e-9.
"""
from pathlib import Path

import numpy as np
import pytest

import gbfe.mesh as M
from oracle import oracle as O
from conftest import rel_maxnorm

GOLDEN = sorted((Path(__file__).resolve().parent / "golden").glob("case_*.npz"))


def load(path):
    z = dict(np.load(path))
    cons = M.Constraints(z["cons_rows"], z["cons_sizes"], z["cons_cols"], z["cons_acc"], z["cons_vals"],
                         z["cons_inh"])
    deg, wl, wu, uu, max_iter, abs_tol, rel_tol, div_tol = z["params"]
    z["cons"] = cons
    z["filter"] = (int(deg), float(wl), float(wu), float(uu))
    z["cg"] = (int(max_iter), float(abs_tol), float(rel_tol), float(div_tol))
    return z


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 4


@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_oracle_port_matches_reference(path):
    z = load(path)
    s = O.OracleSystem(z["nd"], z["ids"], int(z["n_dofs"]), z["cons"])
    H, Mm, K = s.cell_op(z["H"]), s.cell_op(z["M"]), s.cell_op(z["K"])
    Mi = s.diag_op(z["minv"])
    X = z["X"].copy()
    assert rel_maxnorm(s.apply(H, X), z["Y_H"]) <= 1e-13
    assert rel_maxnorm(X, z["X_after"]) <= 1e-15  # the reference's daxpy may fuse multiply-adds
    assert rel_maxnorm(s.apply(Mm, z["X"].copy()), z["Y_M"]) <= 1e-13
    assert rel_maxnorm(s.apply(Mi, z["X"].copy()), z["Y_Minv"]) <= 1e-15
    deg, wl, wu, uu = z["filter"]
    assert rel_maxnorm(s.residual_filter(H, Mm, Mi, z["eig"], z["X"].copy(), deg, wl, wu, uu), z["Y_rfilter"]) <= 1e-10
    assert rel_maxnorm(s.chebyshev_filter(H, Mi, z["X"].copy(), deg, wl, wu, uu), z["Y_filter"]) <= 1e-10
    mi, at, rt, dt = z["cg"]
    rc, x, it, rn = s.cg(K, s.jacobi_op(z["jacdiag"]), z["b"], np.zeros_like(z["b"]), mi, at, rt, dt)
    assert (rc == 0) == bool(z["cg_ok"])
    assert rel_maxnorm(x, z["x_cg"]) <= 1e-9 if np.abs(z["x_cg"]).max() > 0 else np.abs(x).max() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_gpu_matches_reference(gpu_ctx, path):
    from gbfe import api

    z = load(path)
    basis = api.FEBasisManager(gpu_ctx, z["nd"], z["ids"], int(z["n_dofs"]), z["cons"])
    H = api.KohnShamOperatorContextFE(basis, z["H"])
    Mm = api.CFEOverlapOperatorContext(basis, z["M"])
    K = api.LaplaceOperatorContextFE(basis, z["K"])
    Mi = api.DiagonalOperatorContext(basis, z["minv"])
    m = z["X"].shape[1]
    X = api.MultiVector(basis, m, init=z["X"])
    Y = api.MultiVector(basis, m)
    H.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_H"]) <= 1e-12
    assert rel_maxnorm(X.numpy(), z["X_after"]) <= 1e-15
    X.copy_from(z["X"])
    Mm.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_M"]) <= 1e-12
    X.copy_from(z["X"])
    Mi.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_Minv"]) <= 1e-15
    deg, wl, wu, uu = z["filter"]
    X.copy_from(z["X"])
    api.ResidualChebyshevFilterGEP(H, Mm, Mi, z["eig"], X, deg, wl, wu, uu, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_rfilter"]) <= 1e-10
    X.copy_from(z["X"])
    api.ChebyshevFilter(H, Mi, X, deg, wl, wu, uu, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_filter"]) <= 1e-10
    mi, at, rt, dt = z["cg"]
    nrhs = z["b"].shape[1]
    b = api.MultiVector(basis, nrhs, init=z["b"])
    x = api.MultiVector(basis, nrhs)
    J = api.PreconditionerJacobi(basis, z["jacdiag"])
    rc, it, rn = api.CGLinearSolver(mi, at, rt, dt).solve(K, J, b, x)
    assert (rc == 0) == bool(z["cg_ok"])
    if np.abs(z["x_cg"]).max() > 0:
        assert rel_maxnorm(x.numpy(), z["x_cg"]) <= 1e-9


NONLOCAL = [p for p in GOLDEN if "nonlocal" in p.stem]


class _NL:
    """Nonlocal arrays of a fixture in the shape gbfe.nonlocal_psp.NonLocalData has."""

    def __init__(self, z):
        self.n_proj = int(z["nl_n_proj"])
        self.proj_per_cell, self.proj_ids = z["nl_np"], z["nl_pids"]
        self.cell_c, self.coupling = z["nl_c"], z["nl_v"]


def test_nonlocal_fixtures_present():
    assert len(NONLOCAL) >= 2


@pytest.mark.parametrize("path", NONLOCAL, ids=[p.stem for p in NONLOCAL])
def test_oracle_nonlocal_matches_reference(path):
    """AtomCenterNonLocalOpContextFE::apply and the KS apply with the
    nonlocal part fused in, as the reference computes them."""
    z = load(path)
    s = O.OracleSystem(z["nd"], z["ids"], int(z["n_dofs"]), z["cons"])
    nl = s.nonlocal_part(_NL(z))
    assert rel_maxnorm(s.apply(s.nonlocal_op(nl), z["X"].copy()), z["Y_nl"]) <= 1e-13
    assert rel_maxnorm(s.apply(s.cell_op(z["H"], nonlocal_part=nl), z["X"].copy()), z["Y_Hnl"]) <= 1e-13
    # the nonlocal term is not negligible in these cases
    assert rel_maxnorm(z["Y_Hnl"], z["Y_H"]) > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("path", NONLOCAL, ids=[p.stem for p in NONLOCAL])
def test_gpu_nonlocal_matches_reference(gpu_ctx, path):
    from gbfe import api

    z = load(path)
    basis = api.FEBasisManager(gpu_ctx, z["nd"], z["ids"], int(z["n_dofs"]), z["cons"])
    nl = api.AtomCenterNonLocalOpContextFE(basis, _NL(z))
    H = api.KohnShamOperatorContextFE(basis, z["H"], nonlocal_part=nl)
    m = z["X"].shape[1]
    X, Y = api.MultiVector(basis, m, init=z["X"]), api.MultiVector(basis, m)
    nl.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_nl"]) <= 1e-12
    X.copy_from(z["X"])
    H.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_Hnl"]) <= 1e-12


ENRICHED = [p for p in GOLDEN if "enriched" in p.stem]


def test_enriched_fixtures_present():
    assert len(ENRICHED) >= 1


@pytest.mark.parametrize("path", ENRICHED, ids=[p.stem for p in ENRICHED])
def test_oracle_ortho_efe_inverse_matches_reference(path):
    """OrthoEFEOverlapInverseOpContextGLL::apply (direct branch) as the
    reference computes it: GLL diagonal inverse on every dof, the enrichment
    rows replaced by the dense inverse block times X's enrichment rows."""
    z = load(path)
    s = O.OracleSystem(z["nd"], z["ids"], int(z["n_dofs"]), z["cons"])
    op = s.diag_block_op(z["minv"], int(z["enr_begin"]), z["enr_blk"])
    assert rel_maxnorm(s.apply(op, z["X"].copy()), z["Y_Minv_efe"]) <= 1e-14
    # the block changes the enrichment rows
    assert rel_maxnorm(z["Y_Minv_efe"], z["Y_Minv"]) > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("path", ENRICHED, ids=[p.stem for p in ENRICHED])
def test_gpu_ortho_efe_inverse_matches_reference(gpu_ctx, path):
    from gbfe import api

    z = load(path)
    basis = api.FEBasisManager(gpu_ctx, z["nd"], z["ids"], int(z["n_dofs"]), z["cons"])
    Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, 1.0 / z["minv"], int(z["enr_begin"]), z["enr_blk"])
    m = z["X"].shape[1]
    X, Y = api.MultiVector(basis, m, init=z["X"]), api.MultiVector(basis, m)
    Mi.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), z["Y_Minv_efe"]) <= 1e-14
