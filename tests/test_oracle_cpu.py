"""CPU checks of the oracle against independent computations and known answers.

The oracle (oracle/fe_oracle.c + oracle/oracle.py) restates the reference's
algorithms; these tests pin it against a dense numpy assembly, the analytic
spectrum of the Dirichlet box, and a CG known-solution case mirroring
test/linearAlgebra/src/TestCGLinearSolverSerialHostDouble.cpp:381-506.
"""
import numpy as np
import pytest
import scipy.linalg as sla

import gbfe.mesh as M
from oracle import oracle as O


def dense_assemble(prob, mats):
    C, nd, N = prob.n_cells, prob.nd, prob.n_dofs
    ids = prob.cell_dof_ids.reshape(C, nd).astype(np.int64)
    A = np.zeros((N, N))
    Mc = mats.reshape(C, nd, nd)
    for c in range(C):
        A[np.ix_(ids[c], ids[c])] += Mc[c].T  # stored column-major
    return A


@pytest.mark.parametrize("use_blas", [True, False])
def test_apply_matches_dense(small_problem, use_blas):
    p = small_problem
    s = O.OracleSystem.from_problem(p, use_blas=use_blas)
    H = s.cell_op(p.H)
    X = M.random_block(p.n_dofs, 5, 3)
    Y = s.apply(H, X.copy())
    Xc = X.copy()
    Xc[p.constraints.row_ids] = 0.0
    Yd = dense_assemble(p, p.H) @ Xc
    Yd[p.constraints.row_ids] = 0.0
    assert np.abs(Y - Yd).max() <= 1e-12 * np.abs(Yd).max()


def test_apply_hanging_constraints():
    p = M.ks_box(3, 2, 6.0, 1, 4.0, 0.5, seed=3)
    rng = np.random.default_rng(5)
    p.constraints = M.add_synthetic_hanging(p.constraints, 3, 2, rng, fraction=0.2, inhomogeneous=True)
    c = p.constraints
    s = O.OracleSystem.from_problem(p)
    K = s.cell_op(p.K)
    X = M.random_block(p.n_dofs, 3, 4)
    Xm = X.copy()
    Y = s.apply(K, Xm)
    # dense restatement: P maps free -> full, x_r = inh + sum w x_c
    N = p.n_dofs
    Xe = X.copy()
    for i in range(c.nrows):
        r, a, sz = c.row_ids[i], c.row_acc[i], c.row_sizes[i]
        Xe[r] = c.inhomogeneities[i] + sum(c.col_values[a + j] * X[c.col_ids[a + j]] for j in range(sz))
    assert np.abs(Xm - Xe).max() < 1e-14  # X modified exactly like distributeParentToChild
    Yd = dense_assemble(p, p.K) @ Xe
    for i in range(c.nrows):
        r, a, sz = c.row_ids[i], c.row_acc[i], c.row_sizes[i]
        for j in range(sz):
            Yd[c.col_ids[a + j]] += c.col_values[a + j] * Yd[r]
        Yd[r] = 0.0
    assert np.abs(Y - Yd).max() <= 1e-12 * np.abs(Yd).max()


def test_chfsi_matches_dense_generalized_eigensolve(small_problem):
    p = small_problem
    s = O.OracleSystem.from_problem(p)
    H, Mo, Mi = s.cell_op(p.H), s.cell_op(p.M), s.diag_op(1.0 / p.m_gll_diag)
    st, eig, X, res, passes = s.ks_eigen_solve(H, Mo, Mi, M.random_block(p.n_dofs, 10, 2), 12, 40, 5, 1e-9)
    free = np.setdiff1d(np.arange(p.n_dofs), p.constraints.row_ids)
    Hd, Md = dense_assemble(p, p.H), dense_assemble(p, p.M)
    w = sla.eigh(Hd[np.ix_(free, free)], Md[np.ix_(free, free)], eigvals_only=True)
    assert st == 0
    assert np.abs(eig[:5] - w[:5]).max() < 1e-10


def test_dirichlet_box_spectrum_known_answer():
    """V = 0: lambda = (pi^2 / 2 L^2)(nx^2 + ny^2 + nz^2); lowest = 3 pi^2 / (2 L^2)."""
    L = 20.0
    p = M.build_problem(4, 4, L, np.zeros((0, 3)), np.zeros(0), 0.5)
    s = O.OracleSystem.from_problem(p)
    H, Mo, Mi = s.cell_op(p.H), s.cell_op(p.M), s.diag_op(1.0 / p.m_gll_diag)
    st, eig, X, res, passes = s.ks_eigen_solve(H, Mo, Mi, M.random_block(p.n_dofs, 8, 1), 15, 40, 4, 1e-9)
    exact = np.pi ** 2 / (2 * L * L) * np.array([3, 6, 6, 6])
    assert np.abs(eig[:4] - exact).max() < 1e-5  # FE discretisation error at p=4, h=5


def test_cg_known_solution(small_problem):
    p = small_problem
    s = O.OracleSystem.from_problem(p)
    K = s.cell_op(p.K)
    Kd = dense_assemble(p, p.K)
    diag = np.diag(Kd).copy()
    diag[p.constraints.row_ids] = 1.0
    PC = s.jacobi_op(diag)
    rng = np.random.default_rng(9)
    xs = rng.standard_normal((p.n_dofs, 2))
    xs[p.constraints.row_ids] = 0.0
    b = s.apply(K, xs.copy())
    rc, x, iters, rn = s.cg(K, PC, b, np.zeros_like(b), 1000, 1e-14, 1e-12, 1e6)
    assert rc == 0
    assert np.abs(x - xs).max() / np.abs(xs).max() < 1e-9


def test_residual_filter_reduces_unwanted(small_problem):
    p = small_problem
    s = O.OracleSystem.from_problem(p)
    H, Mo, Mi = s.cell_op(p.H), s.cell_op(p.M), s.diag_op(1.0 / p.m_gll_diag)
    b = s.lanczos_bounds(H, Mo, Mi)
    X = M.random_block(p.n_dofs, 6, 5)
    Y = s.residual_filter(H, Mo, Mi, np.zeros(6), X.copy(), 8, b[0], b[0] + 0.2 * (b[1] - b[0]), b[1] + b[2] / 10)
    assert np.isfinite(Y).all() and np.abs(Y).max() > 0


@pytest.mark.parametrize("use_blas", [True, False])
def test_nonlocal_matches_dense_projector_form(use_blas):
    """The oracle's nonlocal part (cell-wise C_c blocks, scatter, V scale,
    beta = 1 add) equals the dense form P^T C^T diag(V) C P X on a Dirichlet
    box, standalone and fused into the Kohn-Sham apply."""
    from gbfe import nonlocal_psp as NL

    p = M.ks_box(3, 3, 8.0, 2, 4.0, 0.5, seed=31)
    d = NL.projectors(p)
    assert d.n_proj == 2 * d.per_atom and d.proj_per_cell.max() > 0
    s = O.OracleSystem.from_problem(p, use_blas=use_blas)
    nl = s.nonlocal_part(d)
    X0 = M.random_block(p.n_dofs, 5, 3)
    Cg = d.dense(p.nd_per_cell, p.cell_dof_ids, p.n_dofs)
    rows = p.constraints.row_ids.astype(np.int64)
    Xp = X0.copy()
    Xp[rows] = 0.0
    Yd = Cg.T @ (d.coupling[:, None] * (Cg @ Xp))
    Yd[rows] = 0.0
    Ynl = s.apply(s.nonlocal_op(nl), X0.copy())
    assert np.abs(Ynl - Yd).max() <= 1e-13 * np.abs(Yd).max()
    Yloc = s.apply(s.cell_op(p.H), X0.copy())
    Yfused = s.apply(s.cell_op(p.H, nonlocal_part=nl), X0.copy())
    assert np.abs(Yfused - (Yloc + Yd)).max() <= 1e-13 * np.abs(Yfused).max()
    # symmetric: the projected operator is Hermitian
    G = Xp.T @ Ynl
    assert np.abs(G - G.T).max() <= 1e-13 * np.abs(G).max()


def test_oracle_assembly_reproduces_generator_enriched():
    """The oracle's cell-matrix assembly (reinit's B^T diag(w) B plus the
    kinetic part) reproduces the generator's enriched H: cells of two sizes
    and two quadrature rules."""
    import gbfe.enrichment as E

    p = E.enriched_problem(4, 2, 16.0, 1, 4.0, 0.5, 108, keep_quadrature=True)
    q = p.extra["quad_cells"]
    assert len(np.unique(q["nq"])) == 2 and len(np.unique(p.nd_per_cell)) == 2
    H = O.assemble_cells(p.nd_per_cell, q["nq"], q["B"], q["w"], p.K, 0.5)
    assert np.abs(H - p.H).max() <= 1e-13 * np.abs(p.H).max()
