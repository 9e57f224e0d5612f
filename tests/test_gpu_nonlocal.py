"""GPU parity of the nonlocal pseudopotential part (C^T V C) against the oracle.

Tolerances: FP64 standalone and fused applies <= 1e-12 relative max-norm
(the plain path's bar); FP32 / split-BF16 fused apply <= 1e-4 against FP64;
eigenvalues of a solve with the nonlocal part <= 1e-8 Ha.
"""
import numpy as np
import pytest

import gbfe.mesh as M
from gbfe import nonlocal_psp as NL
from oracle import oracle as O
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu
TC_TOL = 1e-4


def _problem(seed=31, hanging=False):
    p = M.ks_box(3, 3, 8.0, 2, 4.0, 0.5, seed=seed)
    if hanging:
        p.constraints = M.add_synthetic_hanging(p.constraints, 3, 3, np.random.default_rng(4), 0.15,
                                                inhomogeneous=True)
    return p, NL.projectors(p)


@pytest.mark.parametrize("m", [1, 7, 24, 64])
def test_standalone_nonlocal_apply(gpu_ctx, m):
    from gbfe import api

    p, d = _problem()
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    V = api.AtomCenterNonLocalOpContextFE(basis, d)
    s = O.OracleSystem.from_problem(p)
    X0 = M.random_block(p.n_dofs, m, 5)
    X, Y = api.MultiVector(basis, m, init=X0), api.MultiVector(basis, m)
    V.apply(X, Y)
    Xo = X0.copy()
    Yo = s.apply(s.nonlocal_op(s.nonlocal_part(d)), Xo)
    err = rel_maxnorm(Y.numpy(), Yo)
    print(f"nonlocal standalone m={m}: rel max-norm err {err:.2e}")
    assert err <= 1e-12
    assert rel_maxnorm(X.numpy(), Xo) <= 1e-14


@pytest.mark.parametrize("hanging", [False, True])
@pytest.mark.parametrize("fp64_tensor", [False, True])
def test_fused_ks_apply_with_nonlocal(gpu_ctx, hanging, fp64_tensor):
    from gbfe import api

    p, d = _problem(hanging=hanging)
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    nl = api.AtomCenterNonLocalOpContextFE(basis, d)
    H = api.KohnShamOperatorContextFE(basis, p.H, fp64_tensor=fp64_tensor, nonlocal_part=nl)
    s = O.OracleSystem.from_problem(p)
    X0 = M.random_block(p.n_dofs, 24, 6)
    X, Y = api.MultiVector(basis, 24, init=X0), api.MultiVector(basis, 24)
    gpu_ctx.set_fp64_apply(1 if fp64_tensor else 0)
    try:
        H.apply(X, Y)
    finally:
        gpu_ctx.set_fp64_apply(0)
    Yo = s.apply(s.cell_op(p.H, nonlocal_part=s.nonlocal_part(d)), X0.copy())
    err = rel_maxnorm(Y.numpy(), Yo)
    print(f"fused KS+nonlocal hanging={hanging} fp64_tensor={fp64_tensor}: rel max-norm err {err:.2e}")
    assert err <= 1e-12
    # detaching gives back the local operator
    H.attach_nonlocal(None)
    Y2 = api.MultiVector(basis, 24)
    X2 = api.MultiVector(basis, 24, init=X0)
    H.apply(X2, Y2)
    assert rel_maxnorm(Y2.numpy(), s.apply(s.cell_op(p.H), X0.copy())) <= 1e-12


@pytest.mark.parametrize("mode", [0, 2])
def test_fused_mixed_apply_with_nonlocal(gpu_ctx, mode):
    """FP32 cell buffer path (SIMT = 0, persistent tensor-core kernel = 2)."""
    from gbfe import api

    p, d = _problem()
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    nl = api.AtomCenterNonLocalOpContextFE(basis, d)
    H = api.KohnShamOperatorContextFE(basis, p.H, mixed=True, nonlocal_part=nl)
    s = O.OracleSystem.from_problem(p)
    X0 = M.random_block(p.n_dofs, 40, 8).astype(np.float32)
    Xf = api.MultiVector(basis, 40, dtype=np.float32, init=X0)
    Yf = api.MultiVector(basis, 40, dtype=np.float32)
    gpu_ctx.set_tensor_cores(mode)
    try:
        H.apply(Xf, Yf)
        gpu_ctx.check_status()
    finally:
        gpu_ctx.set_tensor_cores(2)
    Yo = s.apply(s.cell_op(p.H, nonlocal_part=s.nonlocal_part(d)), X0.astype(np.float64))
    err = rel_maxnorm(Yf.numpy(), Yo)
    print(f"mixed KS+nonlocal mode={mode}: rel max-norm err {err:.2e}")
    assert err <= TC_TOL


def test_ks_solve_with_nonlocal_matches_oracle(gpu_ctx):
    from gbfe import api

    p, d = _problem(seed=33)
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    nl = api.AtomCenterNonLocalOpContextFE(basis, d)
    H = api.KohnShamOperatorContextFE(basis, p.H, nonlocal_part=nl)
    Mo = api.CFEOverlapOperatorContext(basis, p.M)
    Mi = api.CFEOverlapInverseOpContextGLL(basis, p.m_gll_diag)
    s = O.OracleSystem.from_problem(p)
    oH = s.cell_op(p.H, nonlocal_part=s.nonlocal_part(d))
    oM, oMi = s.cell_op(p.M), s.diag_op(1.0 / p.m_gll_diag)
    m, nw = 10, 6
    X0 = M.random_block(p.n_dofs, m, 15)
    b = s.lanczos_bounds(oH, oM, oMi)
    res = b[2] / 10
    bounds = (b[0], (b[1] + res - b[0]) * (m * 200.0 / p.n_dofs) + b[0], b[1] + res)
    if bounds[1] >= bounds[2]:
        bounds = (b[0], (bounds[2] + b[0]) * 0.5, bounds[2])
    st, eig_ref, _, _, passes_ref = s.ks_eigen_solve(oH, oM, oMi, X0, 12, 40, nw, 1e-9, bounds=bounds)
    X = api.MultiVector(basis, m, init=X0)
    rc, eig, resid, passes = api.KohnShamEigenSolver(nw, 12, 40, 1e-9, bounds=bounds).solve(H, X, Mo, Mi)
    assert rc == 0 and st == 0
    assert np.abs(eig[:nw] - eig_ref[:nw]).max() <= 1e-8
    # the nonlocal part changes the spectrum (a real term, not a no-op)
    st0, eig_loc, _, _, _ = s.ks_eigen_solve(s.cell_op(p.H), oM, oMi, X0, 12, 40, nw, 1e-9, bounds=bounds)
    assert np.abs(eig_loc[:nw] - eig_ref[:nw]).max() > 1e-4
