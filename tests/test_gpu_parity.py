"""GPU parity of the FP64 path against the oracle, through the C ABI.

Tolerances (stated per test):
  * FP64 apply: relative max-norm error <= 1e-12 (the bar for the plain path);
  * filters / orthonormalisation / Rayleigh-Ritz: <= 1e-10 relative;
  * converged eigenvalues: <= 1e-8 Ha;
  * FP32 mixed apply: <= 2e-6 relative max-norm against FP64.
"""
import numpy as np
import pytest

import gbfe.mesh as M
from oracle import oracle as O
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu


def _setup(ctx, p, mixed=False):
    from gbfe import api

    basis = api.FEBasisManager.from_problem(ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H, mixed=mixed)
    Mo = api.CFEOverlapOperatorContext(basis, p.M, mixed=mixed)
    Mi = api.CFEOverlapInverseOpContextGLL(basis, p.m_gll_diag)
    s = O.OracleSystem.from_problem(p)
    return basis, H, Mo, Mi, s, s.cell_op(p.H), s.cell_op(p.M), s.diag_op(1.0 / p.m_gll_diag)


@pytest.mark.parametrize("m", [1, 7, 24, 64])
def test_apply_fp64_dirichlet(gpu_ctx, small_problem, m):
    from gbfe import api

    p = small_problem
    basis, H, _, _, s, oH, _, _ = _setup(gpu_ctx, p)
    X0 = M.random_block(p.n_dofs, m, 100 + m)
    X = api.MultiVector(basis, m, init=X0)
    Y = api.MultiVector(basis, m)
    H.apply(X, Y)
    Xo = X0.copy()
    Yo = s.apply(oH, Xo)
    assert rel_maxnorm(Y.numpy(), Yo) <= 1e-12
    assert np.array_equal(X.numpy(), Xo)  # constraints modified X identically


def test_apply_fp64_hanging_inhomogeneous(gpu_ctx):
    from gbfe import api

    p = M.ks_box(3, 3, 8.0, 2, 4.0, 0.5, seed=21)
    p.constraints = M.add_synthetic_hanging(p.constraints, 3, 3, np.random.default_rng(2), 0.15, inhomogeneous=True)
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    K = api.LaplaceOperatorContextFE(basis, p.K)
    s = O.OracleSystem.from_problem(p)
    X0 = M.random_block(p.n_dofs, 6, 3)
    X = api.MultiVector(basis, 6, init=X0)
    Y = api.MultiVector(basis, 6)
    K.apply(X, Y)
    Xo = X0.copy()
    Yo = s.apply(s.cell_op(p.K), Xo)
    assert rel_maxnorm(X.numpy(), Xo) <= 1e-14
    assert rel_maxnorm(Y.numpy(), Yo) <= 1e-12


def test_apply_variable_cell_sizes(gpu_ctx):
    """Uneven nd_c (enriched-cell-like): random dof maps and cell matrices."""
    from gbfe import api

    rng = np.random.default_rng(7)
    C, N = 60, 900
    nd = rng.integers(20, 41, size=C).astype(np.uint32)
    ids = np.concatenate([rng.choice(N, size=k, replace=False) for k in nd]).astype(np.uint32)
    mats = rng.standard_normal(int((nd.astype(np.int64) ** 2).sum()))
    cons = M.Constraints(np.array([0, 5, 17], np.uint32), np.zeros(3, np.uint32), np.zeros(0, np.uint32),
                         np.zeros(3, np.uint32), np.zeros(0), np.zeros(3))
    basis = api.FEBasisManager(gpu_ctx, nd, ids, N, cons)
    A = api.CellMatrixOperatorContext(basis, mats)
    s = O.OracleSystem(nd, ids, N, cons)
    X0 = M.random_block(N, 9, 1)
    X = api.MultiVector(basis, 9, init=X0)
    Y = api.MultiVector(basis, 9)
    A.apply(X, Y)
    Yo = s.apply(s.cell_op(mats), X0.copy())
    assert rel_maxnorm(Y.numpy(), Yo) <= 1e-12


def test_apply_deterministic(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis, H, *_ = _setup(gpu_ctx, p)
    X0 = M.random_block(p.n_dofs, 16, 4)
    outs = []
    for _ in range(2):
        X = api.MultiVector(basis, 16, init=X0)
        Y = api.MultiVector(basis, 16)
        H.apply(X, Y)
        outs.append(Y.numpy())
    assert np.array_equal(outs[0], outs[1])


def test_diag_and_jacobi(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis, _, _, Mi, s, _, _, oMi = _setup(gpu_ctx, p)
    X0 = M.random_block(p.n_dofs, 5, 6)
    X = api.MultiVector(basis, 5, init=X0)
    Y = api.MultiVector(basis, 5)
    Mi.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), s.apply(oMi, X0.copy())) <= 1e-15
    d = np.abs(M.random_block(p.n_dofs, 1, 8)[:, 0]) + 1.0
    J = api.PreconditionerJacobi(basis, d)
    J.apply(X, Y)
    assert rel_maxnorm(Y.numpy(), s.apply(s.jacobi_op(d), X.numpy())) <= 1e-15


def test_residual_filter_fp64(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p)
    m, deg = 8, 10
    b = s.lanczos_bounds(oH, oM, oMi)
    wl, wu, uu = b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10
    eig = np.linspace(-2, 1, m)
    X0 = M.random_block(p.n_dofs, m, 12)
    X = api.MultiVector(basis, m, init=X0)
    Y = api.MultiVector(basis, m)
    api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig, X, deg, wl, wu, uu, Y)
    Yo = s.residual_filter(oH, oM, oMi, eig, X0.copy(), deg, wl, wu, uu)
    assert rel_maxnorm(Y.numpy(), Yo) <= 1e-10


def test_chebyshev_filter_standard(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p)
    b = s.lanczos_bounds(oH, oM, oMi)
    wl, wu, uu = b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10
    X0 = M.random_block(p.n_dofs, 4, 13)
    X = api.MultiVector(basis, 4, init=X0)
    Y = api.MultiVector(basis, 4)
    api.ChebyshevFilter(H, Mi, X, 7, wl, wu, uu, Y)
    Yo = s.chebyshev_filter(oH, oMi, X0.copy(), 7, wl, wu, uu)
    assert rel_maxnorm(Y.numpy(), Yo) <= 1e-10


def test_ortho_and_rayleigh_ritz(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p)
    m = 12
    X0 = M.random_block(p.n_dofs, m, 14)
    X0[p.constraints.row_ids] = 0.0
    X = api.MultiVector(basis, m, init=X0)
    Xo = api.MultiVector(basis, m)
    api.OrthonormalizationFunctions.CholeskyGramSchmidt(X, Xo, Mo)
    st, Xo_ref = s.cholesky_gram_schmidt(oM, X0.copy())
    assert st == 0
    assert rel_maxnorm(Xo.numpy(), Xo_ref) <= 1e-10
    Psi = api.MultiVector(basis, m)
    ev = api.RayleighRitzEigenSolver.solve(H, Xo, Psi)
    ev_ref, Psi_ref = s.rayleigh_ritz(oH, Xo_ref.copy())
    assert np.abs(ev - ev_ref).max() <= 1e-10 * max(1.0, np.abs(ev_ref).max())


def test_ortho_not_orthonormalizable(gpu_ctx):
    """Linearly dependent block -> Cholesky failure status, not a crash."""
    from gbfe import api
    from gbfe._lib import GBFEError

    p = M.ks_box(2, 2, 4.0, 0, 4.0, 0.5, seed=1)
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    Mo = api.CFEOverlapOperatorContext(basis, p.M)
    X0 = np.repeat(M.random_block(p.n_dofs, 1, 2), 3, axis=1)
    X = api.MultiVector(basis, 3, init=X0)
    Xo = api.MultiVector(basis, 3)
    with pytest.raises(GBFEError) as e:
        api.OrthonormalizationFunctions.CholeskyGramSchmidt(X, Xo, Mo)
    assert e.value.status in ("ERR_LAPACK", "ERR_NOT_ORTHONORMALIZABLE")


def test_ks_eigen_solve_fp64_matches_oracle(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p)
    m, nw = 10, 6
    X0 = M.random_block(p.n_dofs, m, 15)
    b = s.lanczos_bounds(oH, oM, oMi)
    res = b[2] / 10
    bounds = (b[0], (b[1] + res - b[0]) * (m * 200.0 / p.n_dofs) + b[0], b[1] + res)
    if bounds[1] >= bounds[2]:
        bounds = (b[0], (bounds[2] + b[0]) * 0.5, bounds[2])
    st, eig_ref, _, res_ref, passes_ref = s.ks_eigen_solve(oH, oM, oMi, X0, 12, 40, nw, 1e-9, bounds=bounds)
    X = api.MultiVector(basis, m, init=X0)
    solver = api.KohnShamEigenSolver(nw, 12, 40, 1e-9, bounds=bounds)
    rc, eig, resid, passes = solver.solve(H, X, Mo, Mi)
    assert rc == 0 and st == 0
    assert np.abs(eig[:nw] - eig_ref[:nw]).max() <= 1e-8
    assert abs(passes - passes_ref) <= 1


def test_cg_fp64_matches_oracle(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    s = O.OracleSystem.from_problem(p)
    K = api.LaplaceOperatorContextFE(basis, p.K)
    oK = s.cell_op(p.K)
    C, nd = p.n_cells, p.nd
    diag = np.zeros(p.n_dofs)
    np.add.at(diag, p.cell_dof_ids.astype(np.int64), np.tile(np.diag(p.K[: nd * nd].reshape(nd, nd)), C))
    diag[p.constraints.row_ids] = 1.0
    J = api.PreconditionerJacobi(basis, diag)
    rng = np.random.default_rng(3)
    b0 = rng.standard_normal((p.n_dofs, 2))
    b0[p.constraints.row_ids] = 0.0
    b = api.MultiVector(basis, 2, init=b0)
    x = api.MultiVector(basis, 2)
    rc, iters, rn = api.CGLinearSolver(2000, 1e-14, 1e-10, 1e6).solve(K, J, b, x)
    rc_o, x_o, it_o, rn_o = s.cg(oK, s.jacobi_op(diag), b0, np.zeros_like(b0), 2000, 1e-14, 1e-10, 1e6)
    assert rc == 0 and rc_o == 0
    assert abs(iters - it_o) <= 1
    assert rel_maxnorm(x.numpy(), x_o) <= 1e-8


def test_mixed_apply_fp32(gpu_ctx, small_problem):
    from gbfe import api

    p = small_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H, mixed=True)
    X0 = M.random_block(p.n_dofs, 32, 16)
    X = api.MultiVector(basis, 32, init=X0)
    Y = api.MultiVector(basis, 32)
    H.apply(X, Y)
    Xf = api.MultiVector(basis, 32, dtype=np.float32, init=X0.astype(np.float32))
    Yf = api.MultiVector(basis, 32, dtype=np.float32)
    H.apply(Xf, Yf)
    assert rel_maxnorm(Yf.numpy(), Y.numpy()) <= 2e-6
