"""GPU parity on the benchmark workloads themselves, against the oracle on
identical inputs (the oracle restates the reference's algorithm; it is pinned
to reference-built golden vectors in test_golden.py).

Tolerances:
  * FP64 applies: relative max-norm <= 1e-12 (the plain path's bar);
  * Lanczos bounds from the same start vector: <= 1e-10 relative;
  * FP64 KS solves: wanted eigenvalues within 1e-8 Ha of the oracle's solve
    (KohnShamEigenSolver.t.cpp:319-487), pass counts within one;
  * mixed-precision KS solve: wanted eigenvalues within 1e-6 Ha of the
    oracle's FP64 solve;
  * one ChFSI pass (ChebyshevFilteredEigenSolver.t.cpp:194-437): Ritz values
    <= 1e-10 relative of the largest magnitude.

Workloads (bench.py CONFIGS): cfg1 = 8^3 cells of degree 3, 24 vectors;
cfg2 = 12^3 cells of degree 4 with five orthogonalised enrichment functions
per atom (cells of 125-145 dofs), 64 vectors.
"""
import numpy as np
import pytest

import bench
import gbfe.mesh as M
from oracle import oracle as O
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg1():
    cfg = bench.CONFIGS["cfg1"]
    prob = bench.make_problem(cfg)
    s = O.OracleSystem.from_problem(prob)
    ops = (s.cell_op(prob.H), s.cell_op(prob.M), s.diag_op(1.0 / prob.m_gll_diag))
    start = bench.lanczos_start_for(prob, cfg)
    X0 = bench.random_block_for(prob, cfg)
    bounds, deg = bench.lanczos_setup(prob, cfg, lambda: s.lanczos_bounds(*ops, 20, start=start))
    st, eig, _, res, passes = s.ks_eigen_solve(*ops, X0, deg, cfg["max_passes"], cfg["n_wanted"], cfg["tol"],
                                               lanczos_start=start)
    assert st == 0
    return dict(cfg=cfg, prob=prob, s=s, ops=ops, start=start, X0=X0, deg=deg, eig=eig, passes=passes,
                bounds=bounds)


def _gpu_ops(ctx, prob, mixed=False, fp64_tensor=False):
    from gbfe import api

    basis = api.FEBasisManager.from_problem(ctx, prob)
    H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=mixed, fp64_tensor=fp64_tensor)
    Mo = api.CFEOverlapOperatorContext(basis, prob.M, mixed=mixed, fp64_tensor=fp64_tensor)
    if "enr_block_inv" in prob.extra:
        Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, prob.m_gll_diag, prob.extra["enr_begin"],
                                                    prob.extra["enr_block_inv"])
    else:
        Mi = api.CFEOverlapInverseOpContextGLL(basis, prob.m_gll_diag)
    return basis, H, Mo, Mi


def test_lanczos_bounds_match_oracle_from_same_start(gpu_ctx, cfg1):
    from gbfe import api

    prob = cfg1["prob"]
    basis, H, Mo, Mi = _gpu_ops(gpu_ctx, prob)
    b_gpu = api.lanczos_bounds(H, Mo, Mi, 20, start=cfg1["start"])
    b_ref = cfg1["s"].lanczos_bounds(*cfg1["ops"], 20, start=cfg1["start"])
    assert np.abs(b_gpu - b_ref).max() <= 1e-10 * np.abs(b_ref).max(), (b_gpu, b_ref)
    # a device-resident start vector gives the same bounds bit for bit
    sd = api.MultiVector(basis, 1, init=cfg1["start"][:, None])
    assert np.array_equal(api.lanczos_bounds(H, Mo, Mi, 20, start=sd), b_gpu)


@pytest.mark.parametrize("mode", ["fp64_fma", "fp64_sliced", "mixed"])
def test_cfg1_ks_solve_matches_oracle(gpu_ctx, cfg1, mode):
    """The whole solve of the cfg1 workload (Lanczos inside, from the same
    start vector) against the oracle's FP64 solve."""
    from gbfe import api

    cfg, prob = cfg1["cfg"], cfg1["prob"]
    mixed = mode == "mixed"
    fp64_tensor = 0 if mode == "fp64_fma" else 1
    basis, H, Mo, Mi = _gpu_ops(gpu_ctx, prob, mixed=mixed, fp64_tensor=bool(fp64_tensor))
    X = api.MultiVector(basis, cfg["m"], init=cfg1["X0"])
    solver = api.KohnShamEigenSolver(cfg["n_wanted"], cfg1["deg"], cfg["max_passes"], cfg["tol"], mixed=mixed,
                                     fp64_tensor=fp64_tensor, lanczos_start=cfg1["start"])
    rc, eig, res, passes = solver.solve(H, X, Mo, Mi)
    nw = cfg["n_wanted"]
    assert rc == 0
    assert np.all(res[:nw] <= cfg["tol"])
    err = np.abs(eig[:nw] - cfg1["eig"][:nw]).max()
    assert err <= (1e-6 if mixed else 1e-8), err
    if not mixed:
        assert abs(passes - cfg1["passes"]) <= 1, (passes, cfg1["passes"])


@pytest.fixture(scope="module")
def cfg2():
    cfg = bench.CONFIGS["cfg2"]
    prob = bench.make_problem(cfg)
    s = O.OracleSystem.from_problem(prob)
    ops = (s.cell_op(prob.H), s.cell_op(prob.M),
           s.diag_block_op(1.0 / prob.m_gll_diag, prob.extra["enr_begin"], prob.extra["enr_block_inv"]))
    return dict(cfg=cfg, prob=prob, s=s, ops=ops)


@pytest.mark.parametrize("fp64_tensor", [False, True], ids=["fma", "sliced"])
def test_cfg2_fp64_applies_match_oracle(gpu_ctx, cfg2, fp64_tensor):
    """H, M and the OrthoEFE inverse overlap of the enriched workload, with all
    64 vectors, against the oracle at the FP64 apply bar."""
    from gbfe import api

    prob, m = cfg2["prob"], cfg2["cfg"]["m"]
    basis, H, Mo, Mi = _gpu_ops(gpu_ctx, prob, fp64_tensor=fp64_tensor)
    gpu_ctx.set_fp64_apply(2 if fp64_tensor else 0)
    try:
        X0 = M.random_block(prob.n_dofs, m, 404)
        for gop, oop in zip((H, Mo, Mi), cfg2["ops"]):
            X = api.MultiVector(basis, m, init=X0)
            Y = api.MultiVector(basis, m)
            gop.apply(X, Y)
            Xo = X0.copy()
            Yo = cfg2["s"].apply(oop, Xo)
            assert rel_maxnorm(Y.numpy(), Yo) <= 1e-12
            assert rel_maxnorm(X.numpy(), Xo) == 0.0
    finally:
        gpu_ctx.set_fp64_apply(0)


def test_cfg2_chfsi_pass_matches_oracle(gpu_ctx, cfg2):
    """One reference-sequence ChFSI pass (residual filter, Cholesky-GS,
    Rayleigh-Ritz) of the enriched workload from the seeded block."""
    from gbfe import api

    cfg, prob = cfg2["cfg"], cfg2["prob"]
    start = bench.lanczos_start_for(prob, cfg)
    bounds, deg = bench.lanczos_setup(prob, cfg, lambda: cfg2["s"].lanczos_bounds(*cfg2["ops"], 20, start=start))
    X0 = bench.random_block_for(prob, cfg)
    eig0 = np.zeros(cfg["m"])
    ev_ref, _ = cfg2["s"].chfsi_pass(*cfg2["ops"], X0.copy(), eig0, deg, *bounds)
    basis, H, Mo, Mi = _gpu_ops(gpu_ctx, prob)
    X = api.MultiVector(basis, cfg["m"], init=X0)
    ev = api.ChebyshevFilteredEigenSolver(*bounds, deg).solve(H, eig0, X, Mo, Mi)
    assert np.abs(ev - ev_ref).max() <= 1e-10 * np.abs(ev_ref).max(), np.abs(ev - ev_ref).max()


def test_cg_residual_divergence_matches_oracle(gpu_ctx, small_problem):
    """CGLinearSolver's RESIDUAL_DIVERGENCE (CGLinearSolver.t.cpp:260-294): a
    residual norm above divergenceTol stops the solve with that status, on
    the GPU as in the oracle, at the same iteration."""
    from gbfe import api

    p = small_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    K = api.LaplaceOperatorContextFE(basis, p.K)
    diag = np.zeros(p.n_dofs)
    off = p.mat_offsets()
    for c in range(p.n_cells):
        nd = int(p.nd_per_cell[c])
        blk = p.K[off[c]: off[c + 1]].reshape(nd, nd)
        np.add.at(diag, p.cell_dof_ids[c * nd:(c + 1) * nd].astype(np.int64), np.diag(blk))
    diag[p.constraints.row_ids] = 1.0
    J = api.PreconditionerJacobi(basis, diag)
    rng = np.random.default_rng(3)
    b0 = rng.standard_normal((p.n_dofs, 1))
    b0[p.constraints.row_ids] = 0.0
    bn = float(np.linalg.norm(b0))
    div_tol = 0.5 * bn  # the initial residual (x0 = 0) already exceeds it
    b = api.MultiVector(basis, 1, init=b0)
    x = api.MultiVector(basis, 1)
    rc, it, rn = api.CGLinearSolver(100, 1e-14, 1e-10, div_tol).solve(K, J, b, x)
    s = O.OracleSystem.from_problem(p)
    rc_o, _, it_o, rn_o = s.cg(s.cell_op(p.K), s.jacobi_op(diag), b0, np.zeros_like(b0), 100, 1e-14, 1e-10, div_tol)
    assert rc == 7 and rc_o == 7  # GBFE_ERR_DIVERGED / the oracle's divergence code
    assert it == it_o
    assert abs(rn[0] - rn_o[0]) <= 1e-12 * rn_o[0]


def test_bounded_wait_gives_up_with_timeout_status(gpu_ctx, small_problem):
    """A bounded device wait on a barrier nothing completes gives up after its
    limit, leaves GBFE_ERR_TIMEOUT in the status word (read once), and the
    context keeps working."""
    from gbfe import api

    lib = gpu_ctx.lib
    assert gpu_ctx.lib.gbfe_ctx_check_status(gpu_ctx.h) == 0
    assert lib.gbfe_ctx_check_wait_timeout(gpu_ctx.h, 0.05) == 0
    assert lib.gbfe_ctx_check_status(gpu_ctx.h) == 8  # GBFE_ERR_TIMEOUT
    assert lib.gbfe_ctx_check_status(gpu_ctx.h) == 0  # cleared by the read
    assert lib.gbfe_ctx_check_wait_timeout(gpu_ctx.h, 2.0) == 1  # limit above one second: rejected
    p = small_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H)
    X0 = M.random_block(p.n_dofs, 4, 8)
    X = api.MultiVector(basis, 4, init=X0)
    Y = api.MultiVector(basis, 4)
    H.apply(X, Y)
    s = O.OracleSystem.from_problem(p)
    assert rel_maxnorm(Y.numpy(), s.apply(s.cell_op(p.H), X0.copy())) <= 1e-12
