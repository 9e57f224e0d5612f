"""Batched Poisson CG (block-diagonal independent instances, per-instance
scalars on the device, CUDA-graph replay) against the oracle's
CGLinearSolver restatement run on each instance alone.

Tolerances: solution 1e-9 relative max-norm (both reach relative residual
1e-10 from the same start along the same recurrence); iteration counts equal
within 1 (reductions sum in a different order).
"""
import numpy as np
import pytest

import gbfe.mesh as M
import gbfe.poisson as P
from oracle import oracle as O
from conftest import rel_maxnorm


def test_poisson_batch_generator_shapes():
    pb = P.batch(count=4, seed=5, n_range=(2, 3), degrees=(2, 3))
    assert pb.inst_dof_off[-1] == pb.n_dofs and pb.b.shape == (pb.n_dofs,)
    for i in range(pb.n_inst):
        v = P.instance_view(pb, i)
        n, p = pb.sizes[i]
        assert v["N"] == (n * p + 1) ** 3 and v["nd"].size == n ** 3
        assert np.all(v["b"][v["cons"].row_ids] == 0.0) and np.all(v["diag"][v["cons"].row_ids] == 1.0)
    # total charge ~ 0: the rhs of the pure-Neumann part sums to ~0 (Dirichlet rows removed, so only roughly)
    assert np.isfinite(pb.b).all()


def test_oracle_cg_on_one_instance_converges():
    pb = P.batch(count=2, seed=6, n_range=(3, 3), degrees=(2,))
    v = P.instance_view(pb, 0)
    s = O.OracleSystem(v["nd"], v["ids"], v["N"], v["cons"])
    rc, x, it, rn = s.cg(s.cell_op(v["K"]), s.jacobi_op(v["diag"]), v["b"][:, None], np.zeros((v["N"], 1)),
                         2000, 1e-14, 1e-10, 1e10)
    assert rc == 0 and it > 3


@pytest.mark.gpu
def test_indexed_operator_matches_expanded(gpu_ctx):
    from gbfe import api

    pb = P.batch(count=3, seed=7, n_range=(2, 4), degrees=(2, 3))
    basis = api.FEBasisManager(gpu_ctx, pb.nd_per_cell, pb.cell_dof_ids, pb.n_dofs, pb.constraints)
    Ki = api.IndexedCellMatrixOperatorContext(basis, pb.mats, pb.cell_to_mat)
    # expand to one matrix per cell
    offs, o = [], 0
    for u in range(int(pb.cell_to_mat.max()) + 1):
        nd_u = int(pb.nd_per_cell[np.argmax(pb.cell_to_mat == u)])
        offs.append((o, nd_u))
        o += nd_u * nd_u
    full = np.concatenate([pb.mats[offs[u][0]:offs[u][0] + offs[u][1] ** 2] for u in pb.cell_to_mat])
    Kf = api.LaplaceOperatorContextFE(basis, full)
    X0 = M.random_block(pb.n_dofs, 3, 9)
    Y1, Y2 = api.MultiVector(basis, 3), api.MultiVector(basis, 3)
    Ki.apply(api.MultiVector(basis, 3, init=X0), Y1)
    Kf.apply(api.MultiVector(basis, 3, init=X0), Y2)
    assert np.array_equal(Y1.numpy(), Y2.numpy())


@pytest.mark.gpu
def test_batched_pcg_matches_oracle_per_instance(gpu_ctx):
    from gbfe import api

    pb = P.batch(count=6, seed=8, n_range=(3, 5), degrees=(2, 3))
    basis = api.FEBasisManager(gpu_ctx, pb.nd_per_cell, pb.cell_dof_ids, pb.n_dofs, pb.constraints)
    K = api.IndexedCellMatrixOperatorContext(basis, pb.mats, pb.cell_to_mat)
    J = api.PreconditionerJacobi(basis, pb.jacobi_diag)
    b = api.MultiVector(basis, 1, init=pb.b[:, None])
    x = api.MultiVector(basis, 1)
    iters, status, rn = api.pcg_solve_batched(K, J, b, x, pb.inst_dof_off, 3000, 1e-14, 1e-10, 1e10, iters_chunk=8)
    xs = x.numpy()[:, 0]
    for i in range(pb.n_inst):
        v = P.instance_view(pb, i)
        s = O.OracleSystem(v["nd"], v["ids"], v["N"], v["cons"])
        rc, xo, it, rno = s.cg(s.cell_op(v["K"]), s.jacobi_op(v["diag"]), v["b"][:, None], np.zeros((v["N"], 1)),
                               3000, 1e-14, 1e-10, 1e10)
        d0, d1 = int(pb.inst_dof_off[i]), int(pb.inst_dof_off[i + 1])
        assert rc == 0 and status[i] == 0
        assert abs(int(iters[i]) - it) <= 1, (i, iters[i], it)
        assert rel_maxnorm(xs[d0:d1], xo[:, 0]) <= 1e-9
