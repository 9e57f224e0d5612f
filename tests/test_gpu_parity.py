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


@pytest.mark.parametrize("faithful", [True, False])
def test_ks_eigen_solve_fp64_matches_oracle(gpu_ctx, small_problem, faithful):
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
    solver = api.KohnShamEigenSolver(nw, 12, 40, 1e-9, bounds=bounds, faithful_passes=faithful)
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


def test_mixed_apply_fp32_simt(gpu_ctx, small_problem):
    """FP32 SIMT cell product: <= 2e-6 relative max-norm against FP64."""
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
    gpu_ctx.set_tensor_cores(0)
    try:
        H.apply(Xf, Yf)
    finally:
        gpu_ctx.set_tensor_cores(2)
    assert rel_maxnorm(Yf.numpy(), Y.numpy()) <= 2e-6


TC_TOL = 1e-4  # split-BF16 (3 products, FP32 accumulation): ~2^-18 per operand


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("n,p,m", [(3, 3, 32), (3, 4, 64), (2, 5, 40), (2, 4, 300), (2, 3, 7), (5, 4, 24)])
def test_mixed_apply_tensor_cores(gpu_ctx, n, p, m, mode):
    """tcgen05 split-BF16 cell product against the FP64 apply of the same X
    (cells of 64, 125 and 216 dofs; one and two 128-row M tiles; ragged and
    multi-tile vector counts)."""
    from gbfe import api

    prob = M.ks_box(n, p, 2.0 * n, 1, 4.0, 0.5, seed=30 + p)
    basis = api.FEBasisManager.from_problem(gpu_ctx, prob)
    H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=True)
    X0 = M.random_block(prob.n_dofs, m, 40 + m).astype(np.float32).astype(np.float64)
    X = api.MultiVector(basis, m, init=X0)
    Y = api.MultiVector(basis, m)
    H.apply(X, Y)
    Xf = api.MultiVector(basis, m, dtype=np.float32, init=X0.astype(np.float32))
    Yf = api.MultiVector(basis, m, dtype=np.float32)
    gpu_ctx.set_tensor_cores(mode)
    try:
        H.apply(Xf, Yf)
        gpu_ctx.check_status()
    finally:
        gpu_ctx.set_tensor_cores(2)
    err = rel_maxnorm(Yf.numpy(), Y.numpy())
    print(f"tc{mode} apply n={n} p={p} m={m}: rel max-norm err {err:.2e}")
    assert err <= TC_TOL


def test_tensor_core_kernels_agree_bitwise(gpu_ctx):
    """The persistent kernel (16-byte and 4-byte gathers) and the
    one-CTA-per-cell kernel issue the same MMAs on the same operands in the
    same order per cell, so their results are identical."""
    from gbfe import api

    prob = M.ks_box(4, 4, 8.0, 1, 4.0, 0.5, seed=44)
    basis = api.FEBasisManager.from_problem(gpu_ctx, prob)
    H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=True)
    X0 = M.random_block(prob.n_dofs, 48, 5).astype(np.float32)
    outs = []
    for mode in (1, 2, 2, 3):
        Xf = api.MultiVector(basis, 48, dtype=np.float32, init=X0)
        Yf = api.MultiVector(basis, 48, dtype=np.float32)
        gpu_ctx.set_tensor_cores(mode)
        H.apply(Xf, Yf)
        gpu_ctx.check_status()
        outs.append(Yf.numpy())
    gpu_ctx.set_tensor_cores(2)
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


def test_mixed_apply_tensor_cores_variable_nd(gpu_ctx):
    from gbfe import api

    rng = np.random.default_rng(17)
    C, N = 50, 700
    nd = np.concatenate([rng.integers(20, 41, size=C - 5), rng.integers(130, 160, size=5)]).astype(np.uint32)
    ids = np.concatenate([rng.choice(N, size=k, replace=False) for k in nd]).astype(np.uint32)
    mats = rng.standard_normal(int((nd.astype(np.int64) ** 2).sum()))
    basis = api.FEBasisManager(gpu_ctx, nd, ids, N)
    A = api.CellMatrixOperatorContext(basis, mats, mixed=True, use_constraints=False)
    X0 = M.random_block(N, 24, 3).astype(np.float32).astype(np.float64)
    X = api.MultiVector(basis, 24, init=X0)
    Y = api.MultiVector(basis, 24)
    A.apply(X, Y)
    Xf = api.MultiVector(basis, 24, dtype=np.float32, init=X0.astype(np.float32))
    Yf = api.MultiVector(basis, 24, dtype=np.float32)
    A.apply(Xf, Yf)
    gpu_ctx.check_status()
    assert rel_maxnorm(Yf.numpy(), Y.numpy()) <= TC_TOL


def test_mixed_residual_filter_close_to_fp64(gpu_ctx, small_problem):
    """Mixed filter (FP32 recurrence, split-BF16 products) vs the FP64 filter:
    the output is a filtered subspace, compared at 1e-3 relative max-norm."""
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p, mixed=True)
    m, deg = 8, 10
    b = s.lanczos_bounds(oH, oM, oMi)
    wl, wu, uu = b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10
    eig = np.linspace(-2, 1, m)
    X0 = M.random_block(p.n_dofs, m, 12)
    X = api.MultiVector(basis, m, init=X0)
    Y64 = api.MultiVector(basis, m)
    Y32 = api.MultiVector(basis, m)
    api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig, X, deg, wl, wu, uu, Y64)
    X.copy_from(X0)
    api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig, X, deg, wl, wu, uu, Y32, mixed=True)
    gpu_ctx.check_status()
    assert rel_maxnorm(Y32.numpy(), Y64.numpy()) <= 1e-3


def test_mixed_ks_solve_eigenvalues(gpu_ctx, small_problem):
    """Mixed ChFSI (FP64 ortho / RR / residual) reaches the FP64 eigenvalues
    within 1e-6 Ha."""
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p, mixed=True)
    m, nw = 10, 6
    X0 = M.random_block(p.n_dofs, m, 15)
    b = api.lanczos_bounds(H, Mo, Mi)
    bounds = (b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10)
    X = api.MultiVector(basis, m, init=X0)
    rc64, e64, r64, n64 = api.KohnShamEigenSolver(nw, 12, 60, 1e-8, bounds=bounds).solve(H, X, Mo, Mi)
    X.copy_from(X0)
    rc32, e32, r32, n32 = api.KohnShamEigenSolver(nw, 12, 60, 1e-8, mixed=True, bounds=bounds).solve(H, X, Mo, Mi)
    gpu_ctx.check_status()
    assert rc64 == 0 and rc32 == 0
    assert np.abs(e32[:nw] - e64[:nw]).max() <= 1e-6
    # the same solve again: its filter graph is the previous solve's, updated
    # in place with this solve's buffers -- the same bits
    Xa = X.numpy().copy()
    X.copy_from(X0)
    rc2, e2, r2, n2 = api.KohnShamEigenSolver(nw, 12, 60, 1e-8, mixed=True, bounds=bounds).solve(H, X, Mo, Mi)
    gpu_ctx.check_status()
    assert rc2 == 0 and n2 == n32
    assert np.array_equal(e2, e32) and np.array_equal(r2, r32) and np.array_equal(X.numpy(), Xa)


def test_graph_replayed_filter_matches_eager(gpu_ctx, small_problem):
    """KS solves with the Chebyshev recurrence captured into a CUDA graph
    (replayed from the second pass on) give bitwise the same eigenvalues as
    the eagerly launched recurrence, FP64 and mixed."""
    from gbfe import api

    p = small_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H, mixed=True)
    Mo = api.CFEOverlapOperatorContext(basis, p.M, mixed=True)
    Mi = api.CFEOverlapInverseOpContextGLL(basis, p.m_gll_diag)
    X0 = M.random_block(p.n_dofs, 8, 21)
    b = api.lanczos_bounds(H, Mo, Mi)
    bounds = (b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10)
    for mixed in (False, True):
        # one solve first: one-time setup launches (the fused filter's folded
        # tiles) do not enter the compared counts
        api.KohnShamEigenSolver(4, 10, 2, 1e-12, mixed=mixed, bounds=bounds, fixed_passes=True).solve(
            H, api.MultiVector(basis, 8, init=X0), Mo, Mi)
        out = []
        for graphs in (False, True):
            gpu_ctx.set_graphs(graphs)
            X = api.MultiVector(basis, 8, init=X0)
            l0 = gpu_ctx.kernel_launches()
            rc, eig, res, passes = api.KohnShamEigenSolver(4, 10, 6, 1e-12, mixed=mixed, bounds=bounds,
                                                           fixed_passes=True).solve(H, X, Mo, Mi)
            out.append((eig, X.numpy(), gpu_ctx.kernel_launches() - l0))
        gpu_ctx.set_graphs(True)
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
        assert out[0][2] == out[1][2]  # replays count the kernels they contain


def test_autotuned_tensor_core_shape(gpu_ctx, tmp_path, monkeypatch):
    """The autotuner picks a (vector tile, stages, CTAs per SM, TMEM buffers, prefetch, orientation) shape per
    cell-size group;
    every shape gives the split-BF16 result (TC_TOL against FP64), and the
    chosen shapes are written to and read back from the cache file."""
    from gbfe import api

    prob = M.ks_box(4, 4, 8.0, 1, 4.0, 0.5, seed=44)
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("GBFE_AUTOTUNE_CACHE", str(cache))
    ctx = api.LinAlgOpContext(0)
    try:
        basis = api.FEBasisManager.from_problem(ctx, prob)
        H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=True)
        X0 = M.random_block(prob.n_dofs, 40, 5)
        X = api.MultiVector(basis, 40, init=X0)
        Y = api.MultiVector(basis, 40)
        H.apply(X, Y)
        Xf = api.MultiVector(basis, 40, dtype=np.float32, init=X0.astype(np.float32))
        Yf = api.MultiVector(basis, 40, dtype=np.float32)
        lines = api.autotune(H, 40)
        # "tc2 nd_max tiles m N stages occupancy ms tmem_buffers prefetch swapped"
        assert lines and all(ln.split()[0] == "tc2" and len(ln.split()) == 11 for ln in lines)
        H.apply(Xf, Yf)
        ctx.check_status()
        assert rel_maxnorm(Yf.numpy(), Y.numpy()) <= TC_TOL
        assert cache.read_text().strip().splitlines() == lines
        tuned = Yf.numpy()
    finally:
        ctx.close()  # also frees the vectors and operators made on it
    ctx2 = api.LinAlgOpContext(0)  # loads the cache
    try:
        basis = api.FEBasisManager.from_problem(ctx2, prob)
        H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=True)
        Xf = api.MultiVector(basis, 40, dtype=np.float32, init=X0.astype(np.float32))
        Yf2 = api.MultiVector(basis, 40, dtype=np.float32)
        H.apply(Xf, Yf2)
        ctx2.check_status()
        assert np.array_equal(Yf2.numpy(), tuned)
        # the cached shapes are reported again, not re-timed or re-appended
        again = api.autotune(H, 40)
        drop_ms = lambda ln: ln.split()[:7] + ln.split()[8:]
        assert [drop_ms(ln) for ln in again] == [drop_ms(ln) for ln in lines]
        assert cache.read_text().strip().splitlines() == lines
    finally:
        ctx2.close()


def test_small_eigenproblem_host_and_cusolver_agree(gpu_ctx, small_problem):
    """Rayleigh-Ritz with the m x m eigenproblem on the host (default) and in
    cuSOLVER syevd: eigenvalues within 1e-12 Ha; fused KS solves within 1e-10 Ha."""
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p)
    X0 = M.random_block(p.n_dofs, 12, 7)
    out = {}
    for host in (True, False):
        gpu_ctx.set_small_eig(host)
        try:
            X = api.MultiVector(basis, 12, init=X0)
            Xo = api.MultiVector(basis, 12)
            Xr = api.MultiVector(basis, 12)
            api.OrthonormalizationFunctions.CholeskyGramSchmidt(X, Xo, Mo)
            eig = api.RayleighRitzEigenSolver.solve(H, Xo, Xr)
            X2 = api.MultiVector(basis, 12, init=X0)
            b = s.lanczos_bounds(oH, oM, oMi)
            bounds = (b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10)
            rc, eks, _, _ = api.KohnShamEigenSolver(8, 12, 40, 1e-9, bounds=bounds).solve(H, X2, Mo, Mi)
            assert rc == 0
            out[host] = (np.asarray(eig), eks)
        finally:
            gpu_ctx.set_small_eig(True)
    assert np.abs(out[True][0] - out[False][0]).max() <= 1e-12
    assert np.abs(out[True][1][:8] - out[False][1][:8]).max() <= 1e-10


def test_fused_mixed_filter_step_matches_separate_launches(gpu_ctx, small_problem):
    """The two-launch mixed filter step (B^-1 folded into the split-BF16
    tiles, the recurrence in the assembly) against the separate launches:
    the same filter up to the split-BF16 rounding of A diag(B^-1) versus A
    (filtered blocks within 1e-3 relative), KS eigenvalues within 1e-6 Ha of
    each other (both within 1e-6 Ha of FP64)."""
    from gbfe import api

    p = small_problem
    basis, H, Mo, Mi, s, oH, oM, oMi = _setup(gpu_ctx, p, mixed=True)
    X0 = M.random_block(p.n_dofs, 16, 9)
    eig0 = np.linspace(-3.0, 0.5, 16)
    b = s.lanczos_bounds(oH, oM, oMi)
    wl, wu, uu = b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10
    outs, eigs = {}, {}
    for fused in (True, False):
        gpu_ctx.set_fused_filter(fused)
        try:
            X = api.MultiVector(basis, 16, init=X0)
            Y = api.MultiVector(basis, 16)
            api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig0, X, 10, wl, wu, uu, Y, mixed=True)
            gpu_ctx.check_status()
            outs[fused] = Y.numpy()
            X2 = api.MultiVector(basis, 16, init=X0)
            rc, e, _, _ = api.KohnShamEigenSolver(10, 12, 40, 1e-7, mixed=True, bounds=(wl, wu, uu)).solve(
                H, X2, Mo, Mi)
            assert rc == 0
            eigs[fused] = e
        finally:
            gpu_ctx.set_fused_filter(True)
    err = rel_maxnorm(outs[True], outs[False])
    print(f"fused filter vs separate: rel max-norm {err:.2e}, bitwise {np.array_equal(outs[True], outs[False])}")
    assert err <= 1e-3
    assert np.abs(eigs[True][:10] - eigs[False][:10]).max() <= 1e-6
