"""Launch shapes of the persistent split-BF16 cell product, forced through the
autotune cache file: the X-row gather into registers and the cp.async
prefetch of 1-3 chunks ahead hand the same operands to the same MMAs, so for
one vector tile and orientation (cell rows on the MMA's M extent, or the
vectors) the results are bitwise equal; every shape is within TC_TOL
(1e-4 relative max-norm, split-BF16) of the FP64 apply.  Cells of 125 dofs
(one 128-row tile), 216 dofs (two tiles, the A stage trimmed to 216 rows) and
the enriched fused filter step (rows substituted from the inverse overlap's
enrichment block) are covered."""
import numpy as np
import pytest

import gbfe.mesh as M
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu

TC_TOL = 1e-4

# (vector tile, ring stages, CTAs per SM asked (1: with 16 gather warps), TMEM buffers flag, prefetch chunks,
#  swapped)
SHAPES = [
    (32, 2, 2, 0, 0, 0), (32, 2, 2, 0, 1, 0), (32, 3, 2, 0, 3, 0),
    (64, 2, 2, 0, 0, 0), (64, 2, 2, 0, 2, 0), (64, 2, 2, 1, 3, 0), (64, 4, 2, 0, 1, 0),
    (128, 2, 2, 0, 0, 1), (128, 2, 2, 1, 0, 1), (128, 3, 2, 0, 2, 1), (128, 4, 2, 0, 0, 1),
    # one CTA per SM with 16 gather warps
    (32, 4, 1, 0, 0, 0), (64, 4, 1, 0, 1, 0), (128, 4, 1, 0, 0, 1), (128, 3, 1, 0, 1, 1),
]


def _groups(nd_per_cell):
    """(128-row tiles -> largest cell) of the launch groups."""
    nd = np.asarray(nd_per_cell, dtype=np.int64)
    return {mt: int(nd[(nd + 127) // 128 == mt].max()) for mt in (1, 2) if np.any((nd + 127) // 128 == mt)}


def _ctx_with_shape(monkeypatch, tmp_path, nd_per_cell, m, shape):
    from gbfe import api

    N, st, occ, nbuf, pf, sw = shape
    cache = tmp_path / ("tune_" + "_".join(map(str, shape)) + f"_{m}.txt")
    cache.write_text("".join(f"tc2 {nd} {mt} {m} {N} {st} {occ} 1.0 {nbuf} {pf} {sw}\n"
                             for mt, nd in _groups(nd_per_cell).items()))
    monkeypatch.setenv("GBFE_AUTOTUNE_CACHE", str(cache))
    return api.LinAlgOpContext(0)


@pytest.mark.parametrize("degree", [4, 5])
def test_gather_modes_bitwise_equal(gpu_ctx, tmp_path, monkeypatch, degree):
    from gbfe import api

    prob = M.ks_box(3 if degree == 4 else 2, degree, 8.0, 1, 4.0, 0.5, seed=45)
    m = 64
    X0 = M.random_block(prob.n_dofs, m, 9)
    basis = api.FEBasisManager.from_problem(gpu_ctx, prob)
    H = api.KohnShamOperatorContextFE(basis, prob.H)
    Y = api.MultiVector(basis, m)
    H.apply(api.MultiVector(basis, m, init=X0), Y)
    ref = Y.numpy()
    out = {}
    for shape in SHAPES:
        ctx = _ctx_with_shape(monkeypatch, tmp_path, prob.nd_per_cell, m, shape)
        try:
            b = api.FEBasisManager.from_problem(ctx, prob)
            Hm = api.KohnShamOperatorContextFE(b, prob.H, mixed=True)
            Yf = api.MultiVector(b, m, dtype=np.float32)
            Hm.apply(api.MultiVector(b, m, dtype=np.float32, init=X0.astype(np.float32)), Yf)
            ctx.check_status()
            out[shape] = Yf.numpy()
        finally:
            ctx.close()
        assert rel_maxnorm(out[shape], ref) <= TC_TOL, shape
    for shape, y in out.items():
        base = next(s for s in SHAPES if s[0] == shape[0] and s[5] == shape[5] and s[4] == 0)
        assert np.array_equal(y, out[base]), (shape, base)


def test_enriched_fused_filter_prefetch_bitwise(gpu_ctx, tmp_path, monkeypatch):
    """The fused mixed filter step on uneven enriched cells: the prefetched
    gather takes the substituted enrichment rows like the register gather."""
    import gbfe.enrichment as E
    from gbfe import api
    from oracle import oracle as O

    p = E.enriched_problem(4, 3, 12.0, 2, 6.0, 0.4, seed=3)
    m = 16
    X0 = M.random_block(p.n_dofs, m, 8)
    eig0 = np.linspace(-2.0, 0.5, m)
    s = O.OracleSystem.from_problem(p)
    b = s.lanczos_bounds(s.cell_op(p.H), s.cell_op(p.M),
                         s.diag_block_op(1.0 / p.m_gll_diag, p.extra["enr_begin"], p.extra["enr_block_inv"]))
    wl, wu, uu = b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10
    out = {}
    for shape in [(16, 2, 2, 0, 0, 0), (16, 2, 2, 0, 2, 0), (16, 3, 2, 0, 3, 0),
                  (128, 2, 2, 0, 0, 1), (128, 3, 2, 0, 2, 1)]:
        ctx = _ctx_with_shape(monkeypatch, tmp_path, p.nd_per_cell, m, shape)
        try:
            basis = api.FEBasisManager.from_problem(ctx, p)
            H = api.KohnShamOperatorContextFE(basis, p.H, mixed=True)
            Mo = api.CFEOverlapOperatorContext(basis, p.M, mixed=True)
            Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, p.m_gll_diag, p.extra["enr_begin"],
                                                        p.extra["enr_block_inv"])
            X = api.MultiVector(basis, m, init=X0)
            Y = api.MultiVector(basis, m)
            api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig0, X, 9, wl, wu, uu, Y, mixed=True)
            ctx.check_status()
            out[shape] = Y.numpy()
        finally:
            ctx.close()
    for shape, y in out.items():
        assert np.all(np.isfinite(y)), shape
        assert np.array_equal(y, out[(16, 2, 2, 0, 0, 0) if shape[5] == 0 else (128, 2, 2, 0, 0, 1)]), shape
    # the two orientations: the same products, possibly summed in another order
    assert rel_maxnorm(out[(128, 2, 2, 0, 0, 1)], out[(16, 2, 2, 0, 0, 0)]) <= TC_TOL
