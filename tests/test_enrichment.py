"""Orthogonalised enriched inputs (uneven cell sizes) and the OrthoEFE
inverse overlap: oracle against a dense generalized eigensolve (CPU), and the
GPU path against the oracle (apply 1e-12, eigenvalues 1e-8 Ha FP64 and 1e-6 Ha
mixed)."""
import numpy as np
import pytest
import scipy.linalg as sla

import gbfe.enrichment as E
import gbfe.mesh as M
from oracle import oracle as O
from conftest import rel_maxnorm


@pytest.fixture(scope="module")
def enriched():
    return E.enriched_problem(4, 3, 12.0, 2, 6.0, 0.4, seed=3)


def dense(prob, mats):
    N = prob.n_dofs
    A = np.zeros((N, N))
    nd = prob.nd_per_cell.astype(np.int64)
    moff = np.concatenate([[0], np.cumsum(nd * nd)])
    coff = np.concatenate([[0], np.cumsum(nd)])
    for c in range(prob.n_cells):
        ids = prob.cell_dof_ids[coff[c]:coff[c + 1]].astype(np.int64)
        A[np.ix_(ids, ids)] += mats[moff[c]:moff[c + 1]].reshape(nd[c], nd[c]).T
    return A


def test_enriched_cells_are_uneven(enriched):
    nd = np.unique(enriched.nd_per_cell)
    assert nd.size >= 2 and nd.min() == 64
    assert enriched.extra["n_enrichment"] == 10


def test_oracle_chfsi_on_enriched_matches_dense(enriched):
    p = enriched
    s = O.OracleSystem.from_problem(p)
    H, Mo = s.cell_op(p.H), s.cell_op(p.M)
    Mi = s.diag_block_op(1.0 / p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"])
    st, eig, X, res, passes = s.ks_eigen_solve(H, Mo, Mi, M.random_block(p.n_dofs, 10, 4), 14, 60, 5, 1e-8)
    free = np.setdiff1d(np.arange(p.n_dofs), p.constraints.row_ids)
    w = sla.eigh(dense(p, p.H)[np.ix_(free, free)], dense(p, p.M)[np.ix_(free, free)], eigvals_only=True)
    assert st == 0
    assert np.abs(eig[:5] - w[:5]).max() < 1e-9


@pytest.mark.gpu
def test_gpu_enriched_apply_and_inverse(gpu_ctx, enriched):
    from gbfe import api

    p = enriched
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H)
    Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"])
    s = O.OracleSystem.from_problem(p)
    X0 = M.random_block(p.n_dofs, 8, 5)
    for op, oop in ((H, s.cell_op(p.H)),
                    (Mi, s.diag_block_op(1.0 / p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"]))):
        X = api.MultiVector(basis, 8, init=X0)
        Y = api.MultiVector(basis, 8)
        op.apply(X, Y)
        assert rel_maxnorm(Y.numpy(), s.apply(oop, X0.copy())) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_enriched_ks_solve(gpu_ctx, enriched, mixed):
    from gbfe import api

    p = enriched
    s = O.OracleSystem.from_problem(p)
    oH, oM = s.cell_op(p.H), s.cell_op(p.M)
    oMi = s.diag_block_op(1.0 / p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"])
    X0 = M.random_block(p.n_dofs, 10, 6)
    b = s.lanczos_bounds(oH, oM, oMi)
    bounds = (b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10)
    st, eig_ref, _, _, _ = s.ks_eigen_solve(oH, oM, oMi, X0, 14, 80, 5, 1e-8, bounds=bounds)
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H, mixed=mixed)
    Mo = api.CFEOverlapOperatorContext(basis, p.M, mixed=mixed)
    Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"])
    X = api.MultiVector(basis, 10, init=X0)
    rc, eig, res, passes = api.KohnShamEigenSolver(5, 14, 80, 1e-8, mixed=mixed, bounds=bounds).solve(H, X, Mo, Mi)
    gpu_ctx.check_status()
    assert rc == 0 and st == 0
    assert np.abs(eig[:5] - eig_ref[:5]).max() <= (1e-6 if mixed else 1e-8)


@pytest.mark.gpu
def test_gpu_enriched_fused_filter_matches_separate(gpu_ctx, enriched):
    """The fused mixed filter step with the OrthoEFE inverse (diagonal folded
    into the split-BF16 tiles, the enrichment block applied beforehand and
    substituted in the gather) against the separate launches: within 1e-3
    relative (split-BF16 rounding of A diag(B^-1) versus A)."""
    from gbfe import api

    p = enriched
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H, mixed=True)
    Mo = api.CFEOverlapOperatorContext(basis, p.M, mixed=True)
    Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"])
    X0 = M.random_block(p.n_dofs, 12, 8)
    eig0 = np.linspace(-2.0, 0.5, 12)
    s = O.OracleSystem.from_problem(p)
    b = s.lanczos_bounds(s.cell_op(p.H), s.cell_op(p.M),
                         s.diag_block_op(1.0 / p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"]))
    wl, wu, uu = b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10
    outs = {}
    for fused, tc in ((True, 2), (False, 2), (True, 3)):
        gpu_ctx.set_fused_filter(fused)
        gpu_ctx.set_tensor_cores(tc)
        try:
            X = api.MultiVector(basis, 12, init=X0)
            Y = api.MultiVector(basis, 12)
            api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig0, X, 9, wl, wu, uu, Y, mixed=True)
            gpu_ctx.check_status()
            outs[fused, tc] = Y.numpy()
        finally:
            gpu_ctx.set_fused_filter(True)
            gpu_ctx.set_tensor_cores(2)
    err = rel_maxnorm(outs[True, 2], outs[False, 2])
    print(f"enriched fused filter vs separate: {err:.2e}, bitwise {np.array_equal(outs[True, 2], outs[False, 2])}")
    assert err <= 1e-3
    # the 16-byte and the 4-byte gathers (enrichment rows substituted in both)
    # hand the same operands to the same MMAs
    assert np.array_equal(outs[True, 2], outs[True, 3])
