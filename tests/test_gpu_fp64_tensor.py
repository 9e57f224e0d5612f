"""FP64-accurate sliced tensor-core cell product (eight 7-bit slices per
operand, exact FP32 accumulation per level) against the FP64 FMA product and
the reference-built golden vectors.  Tolerance: 1e-12 relative max-norm, the
bar of the plain FP64 path."""
from pathlib import Path

import numpy as np
import pytest

import gbfe.enrichment as E
import gbfe.mesh as M
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu


def _both(ctx, basis, mats, X0):
    from gbfe import api

    op = api.CellMatrixOperatorContext(basis, mats, fp64_tensor=True)
    out = []
    for mode in (0, 1):
        X = api.MultiVector(basis, X0.shape[1], init=X0)
        Y = api.MultiVector(basis, X0.shape[1])
        ctx.set_fp64_apply(mode)
        try:
            op.apply(X, Y)
            ctx.check_status()
        finally:
            ctx.set_fp64_apply(0)
        out.append(Y.numpy())
    return out


@pytest.mark.parametrize("n,p,m", [(3, 3, 24), (3, 4, 64), (2, 5, 40), (2, 4, 100), (2, 3, 1), (3, 2, 7)])
def test_fp64_tensor_apply_matches_fma(gpu_ctx, n, p, m):
    from gbfe import api

    prob = M.ks_box(n, p, 2.0 * n, 1, 4.0, 0.5, seed=80 + p)
    basis = api.FEBasisManager.from_problem(gpu_ctx, prob)
    X0 = M.random_block(prob.n_dofs, m, 90 + m)
    y_fma, y_tc = _both(gpu_ctx, basis, prob.H, X0)
    err = rel_maxnorm(y_tc, y_fma)
    print(f"fp64 tensor apply n={n} p={p} m={m}: rel max-norm err {err:.2e}")
    assert err <= 1e-12


def test_fp64_tensor_apply_enriched(gpu_ctx):
    from gbfe import api

    prob = E.enriched_problem(4, 3, 12.0, 2, 6.0, 0.4, seed=3)
    basis = api.FEBasisManager.from_problem(gpu_ctx, prob)
    X0 = M.random_block(prob.n_dofs, 16, 7)
    y_fma, y_tc = _both(gpu_ctx, basis, prob.H, X0)
    assert rel_maxnorm(y_tc, y_fma) <= 1e-12


@pytest.mark.parametrize("path", sorted((Path(__file__).resolve().parent / "golden").glob("case_*.npz"))[:3],
                         ids=lambda p: p.stem)
def test_fp64_tensor_apply_golden(gpu_ctx, path):
    from gbfe import api

    z = dict(np.load(path))
    cons = M.Constraints(z["cons_rows"], z["cons_sizes"], z["cons_cols"], z["cons_acc"], z["cons_vals"],
                         z["cons_inh"])
    basis = api.FEBasisManager(gpu_ctx, z["nd"], z["ids"], int(z["n_dofs"]), cons)
    H = api.CellMatrixOperatorContext(basis, z["H"], fp64_tensor=True)
    X = api.MultiVector(basis, z["X"].shape[1], init=z["X"])
    Y = api.MultiVector(basis, z["X"].shape[1])
    gpu_ctx.set_fp64_apply(1)
    try:
        H.apply(X, Y)
    finally:
        gpu_ctx.set_fp64_apply(0)
    assert rel_maxnorm(Y.numpy(), z["Y_H"]) <= 1e-12


def test_ks_solve_with_fp64_tensor_products(gpu_ctx, small_problem):
    """FP64 solve whose FP64 applies all use the sliced tensor-core product,
    and the mixed solve that uses it for its FP64 stages: eigenvalues within
    1e-8 Ha / 1e-6 Ha of the FP64 FMA solve."""
    from gbfe import api

    p = small_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H, mixed=True, fp64_tensor=True)
    Mo = api.CFEOverlapOperatorContext(basis, p.M, mixed=True, fp64_tensor=True)
    Mi = api.CFEOverlapInverseOpContextGLL(basis, p.m_gll_diag)
    X0 = M.random_block(p.n_dofs, 10, 15)
    b = api.lanczos_bounds(H, Mo, Mi)
    bounds = (b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10)
    res = {}
    for key, mixed, tensor in (("fma", False, 0), ("tensor", False, 1), ("tensor_cells", False, 2),
                               ("mixed_tensor", True, 1)):
        X = api.MultiVector(basis, 10, init=X0)
        rc, eig, r, n = api.KohnShamEigenSolver(6, 12, 60, 1e-8, mixed=mixed, bounds=bounds,
                                                fp64_tensor=tensor).solve(H, X, Mo, Mi)
        gpu_ctx.check_status()
        assert rc == 0
        res[key] = eig
        # the residual norms the solver returns (with the sliced products: R
        # straight from [HY | MY] [T; -T diag(eps)]) against plain FP64 applies
        # on the returned block: 1e-11 absolute (the tolerance is 1e-8)
        rr = api.eigen_residual_norms(H, Mo, X, eig)
        assert np.abs(rr - r).max() <= 1e-11, (key, rr, r)
    assert np.abs(res["tensor"][:6] - res["fma"][:6]).max() <= 1e-8
    assert np.abs(res["tensor_cells"][:6] - res["fma"][:6]).max() <= 1e-8
    assert np.abs(res["mixed_tensor"][:6] - res["fma"][:6]).max() <= 1e-6


def _flat_basis(ctx, N):
    """N one-dof cells: a mesh whose block vectors are plain N x m arrays."""
    from gbfe import api

    return api.FEBasisManager(ctx, np.ones(N, np.uint32), np.arange(N, dtype=np.uint32), N)


def _block(rng, N, m, spread):
    """N x m normal entries, rows scaled over `spread` decades (exponent handling)."""
    X = rng.standard_normal((N, m))
    if spread:
        X *= 10.0 ** rng.uniform(-spread, spread, size=(N, 1))
    return X


@pytest.mark.parametrize("N,mx,my,spread", [(1000, 10, 10, 0), (5000, 64, 64, 6), (20000, 128, 64, 0),
                                            (3000, 200, 136, 3), (130000, 64, 64, 0), (40000, 512, 512, 2),
                                            (7, 3, 5, 0)])
def test_sliced_gram_matches_fp64(gpu_ctx, N, mx, my, spread):
    """S = X^T Y by the sliced tensor-core product: error below 1e-13 of
    max(|X|^T |Y|), the scale of an FP64 dot-product error bound."""
    from gbfe import api

    rng = np.random.default_rng(N + mx)
    X0, Y0 = _block(rng, N, mx, spread), _block(rng, N, my, spread)
    basis = _flat_basis(gpu_ctx, N)
    X, Y = api.MultiVector(basis, mx, init=X0), api.MultiVector(basis, my, init=Y0)
    ref = X0.T @ Y0
    scale = (np.abs(X0).T @ np.abs(Y0)).max()
    out = {}
    for mode in (0, 1):
        gpu_ctx.set_fp64_apply(mode)
        try:
            out[mode] = api.gram(X, Y)
            gpu_ctx.check_status()
        finally:
            gpu_ctx.set_fp64_apply(0)
    err = np.abs(out[1] - ref).max() / scale
    print(f"sliced gram N={N} {mx}x{my} spread={spread}: err {err:.2e} (dgemm {np.abs(out[0] - ref).max() / scale:.2e})")
    assert err <= 1e-13


@pytest.mark.parametrize("N,m,mo,spread", [(1000, 10, 10, 0), (5000, 64, 64, 6), (20000, 128, 100, 0),
                                           (3000, 200, 200, 3), (117689, 64, 64, 0), (20000, 512, 512, 2),
                                           (5, 3, 4, 0)])
def test_sliced_rotation_matches_fp64(gpu_ctx, N, m, mo, spread):
    """Y = X T by the sliced tensor-core product (one exponent per row of X,
    one per column of T): error below 1e-14 of max_i |X_ki| sum_i |T_ij|, the
    normwise bound of a 55-bit block floating-point product."""
    from gbfe import api

    rng = np.random.default_rng(N + m + 1)
    X0 = _block(rng, N, m, spread)
    T = rng.standard_normal((m, mo)) * 10.0 ** rng.uniform(-2, 2, size=(1, mo))
    basis = _flat_basis(gpu_ctx, N)
    X, Y = api.MultiVector(basis, m, init=X0), api.MultiVector(basis, mo)
    gpu_ctx.set_fp64_apply(1)
    try:
        api.rotate(X, T, Y)
        gpu_ctx.check_status()
    finally:
        gpu_ctx.set_fp64_apply(0)
    ref = X0 @ T
    scale = np.abs(X0).max(axis=1, keepdims=True) * np.abs(T).sum(axis=0, keepdims=True)
    err = (np.abs(Y.numpy() - ref) / np.maximum(scale, 1e-300)).max()
    print(f"sliced rotation N={N} {m}->{mo} spread={spread}: err {err:.2e}")
    assert err <= 1e-14
