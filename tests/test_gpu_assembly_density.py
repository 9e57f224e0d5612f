"""Device assembly of the Hamiltonian cell matrices (reinit path) and the
electron density from wavefunctions, against the host generator / numpy.
Tolerances: matrices 1e-13 relative max-norm, density 1e-12."""
import numpy as np
import pytest

import gbfe.mesh as M
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def quad_problem():
    return M.build_problem(3, 3, 9.0, np.array([[4.0, 4.5, 5.0]]), np.array([4.0]), 0.5, keep_quadrature=True)


def test_assemble_local_matches_host(gpu_ctx, quad_problem):
    from gbfe import api

    p = quad_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, np.zeros_like(p.H), mixed=True, fp64_tensor=True)
    api.assemble_local(H, p.extra["quad_B"], p.extra["quad_w"], np.tile(p.extra["K_cell"], p.n_cells), 0.5)
    # the operator now applies the host-built H
    Href = api.KohnShamOperatorContextFE(basis, p.H)
    X0 = M.random_block(p.n_dofs, 9, 3)
    Y1, Y2 = api.MultiVector(basis, 9), api.MultiVector(basis, 9)
    H.apply(api.MultiVector(basis, 9, init=X0), Y1)
    Href.apply(api.MultiVector(basis, 9, init=X0), Y2)
    assert rel_maxnorm(Y1.numpy(), Y2.numpy()) <= 1e-13
    # derived copies were rebuilt: the mixed and sliced-FP64 applies follow
    gpu_ctx.set_fp64_apply(1)
    try:
        Y3 = api.MultiVector(basis, 9)
        H.apply(api.MultiVector(basis, 9, init=X0), Y3)
    finally:
        gpu_ctx.set_fp64_apply(0)
    assert rel_maxnorm(Y3.numpy(), Y2.numpy()) <= 1e-12
    Yf = api.MultiVector(basis, 9, dtype=np.float32)
    H.apply(api.MultiVector(basis, 9, dtype=np.float32, init=X0.astype(np.float32)), Yf)
    assert rel_maxnorm(Yf.numpy(), Y2.numpy()) <= 1e-4


def test_density_matches_numpy(gpu_ctx, quad_problem):
    from gbfe import api

    p = quad_problem
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    m = 12
    Psi0 = M.random_block(p.n_dofs, m, 4)
    Psi0[p.constraints.row_ids] = 0.0
    occ = np.linspace(1.0, 0.0, m)
    rho = api.density(api.MultiVector(basis, m, init=Psi0), occ, p.extra["quad_B"])
    B = p.extra["quad_B"]
    ids = p.cell_dof_ids.reshape(p.n_cells, p.nd).astype(np.int64)
    ref = np.stack([((B @ Psi0[ids[c]]) ** 2 * (2.0 * occ)[None, :]).sum(axis=1) for c in range(p.n_cells)])
    assert rel_maxnorm(rho, ref) <= 1e-12


@pytest.fixture(scope="module")
def enriched_quad():
    import gbfe.enrichment as E

    # 20 enriched cells (32 dofs, 216-point rule) beside 44 classical ones (27 dofs, 27 points)
    return E.enriched_problem(4, 2, 16.0, 1, 4.0, 0.5, 108, keep_quadrature=True)


def test_assemble_cells_uneven_matches_oracle(gpu_ctx, enriched_quad):
    """Cells of two sizes and two quadrature rules: the device assembly
    applies like the oracle's assembled matrices (1e-13 relative)."""
    from gbfe import api
    from oracle import oracle as O

    p = enriched_quad
    q = p.extra["quad_cells"]
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, np.zeros_like(p.H), mixed=True)
    api.assemble_cells(H, q["nq"], q["B"], q["w"], p.K, 0.5)
    Href = api.KohnShamOperatorContextFE(basis, O.assemble_cells(p.nd_per_cell, q["nq"], q["B"], q["w"], p.K, 0.5))
    X0 = M.random_block(p.n_dofs, 7, 5)
    Y1, Y2 = api.MultiVector(basis, 7), api.MultiVector(basis, 7)
    H.apply(api.MultiVector(basis, 7, init=X0), Y1)
    Href.apply(api.MultiVector(basis, 7, init=X0), Y2)
    assert rel_maxnorm(Y1.numpy(), Y2.numpy()) <= 1e-13
    # the split-BF16 copies follow the new matrices
    Yf = api.MultiVector(basis, 7, dtype=np.float32)
    H.apply(api.MultiVector(basis, 7, dtype=np.float32, init=X0.astype(np.float32)), Yf)
    assert rel_maxnorm(Yf.numpy(), Y2.numpy()) <= 1e-4


@pytest.mark.parametrize("m", [5, 80])
def test_density_cells_uneven_matches_oracle(gpu_ctx, enriched_quad, m):
    """Density at every cell's own quadrature points (27 or 216 per cell),
    one and two 64-vector tiles (1e-12 relative)."""
    from gbfe import api
    from oracle import oracle as O

    p = enriched_quad
    q = p.extra["quad_cells"]
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    Psi0 = M.random_block(p.n_dofs, m, 6)
    occ = np.linspace(1.0, 0.1, m)
    rho = api.density_cells(api.MultiVector(basis, m, init=Psi0), occ, q["nq"], q["B"])
    ref = O.density_cells(p.nd_per_cell, p.cell_dof_ids, Psi0, occ, q["nq"], q["B"])
    assert rho.shape == ref.shape
    assert rel_maxnorm(rho, ref) <= 1e-12


@pytest.mark.parametrize("fp64_mode", [0, 2], ids=["fma", "sliced_tensor"])
def test_density_through_cell_product(gpu_ctx, quad_problem, fp64_mode):
    """The interpolation as a cell product with the basis values as each
    cell's matrix (Gauss points = dofs per cell), FP64 FMA or the sliced
    FP64-accurate tensor-core kernel; 300 vectors (1e-12 relative)."""
    from gbfe import api
    from oracle import oracle as O

    p = quad_problem
    B = p.extra["quad_B"]
    assert B.shape[0] == B.shape[1]
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    Bop = api.CellMatrixOperatorContext(basis, np.tile(B.ravel(), p.n_cells), use_constraints=False,
                                        fp64_tensor=True)
    m = 300
    Psi0 = M.random_block(p.n_dofs, m, 7)
    occ = np.linspace(1.0, 0.0, m)
    gpu_ctx.set_fp64_apply(fp64_mode)
    try:
        rho = api.density_op(Bop, api.MultiVector(basis, m, init=Psi0), occ)
    finally:
        gpu_ctx.set_fp64_apply(0)
    nq = np.full(p.n_cells, B.shape[0], np.uint32)
    ref = O.density_cells(p.nd_per_cell, p.cell_dof_ids, Psi0, occ, nq, np.tile(B.ravel(), p.n_cells))
    assert rel_maxnorm(rho, ref) <= 1e-12
