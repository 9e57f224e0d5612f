"""Batched electrostatic Poisson inputs: independent solves on their own cube
meshes, concatenated into one block-diagonal system for a single batched
Jacobi-preconditioned CG.

Each instance: a uniform hex mesh of n^3 cells (h = 1 bohr) of degree p,
homogeneous Dirichlet boundary, right-hand side b = 4 pi int rho N_i with
rho = (sum of g normalised Gaussian charges) - (their compensating uniform
neutralising density), assembled with Gauss quadrature (p+1 points per axis),
Dirichlet rows zero.  The Jacobi diagonal is the assembled cell diagonal with
constrained rows set to 1, as PoissonLinearSolverFunctionFE builds it
(electrostatics/PoissonLinearSolverFunctionFE.t.cpp:38-100, 231-256).

Cells of one uniform mesh share one Laplace matrix, so the batch stores one
matrix per degree (``cell_to_mat``) instead of one per cell.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import mesh as M


@dataclass
class PoissonBatch:
    n_inst: int
    n_dofs: int
    nd_per_cell: np.ndarray
    cell_dof_ids: np.ndarray
    constraints: M.Constraints
    mats: np.ndarray  # distinct Laplace cell matrices, concatenated
    cell_to_mat: np.ndarray
    b: np.ndarray  # [N] right-hand side
    jacobi_diag: np.ndarray  # [N]
    inst_dof_off: np.ndarray  # [n_inst+1] uint64
    inst_cell_off: np.ndarray
    sizes: list  # (n, p) per instance


def _instance(n: int, p: int, rng: np.random.Generator, h: float = 1.0):
    L = n * h
    nq = p + 1
    n1 = n * p + 1
    N = n1 ** 3
    nd = (p + 1) ** 3
    xg, _ = M.gll_points(p)
    xq, wq = M.gauss_points(nq)
    phi, dphi = M.lagrange_tables(xg, xq)
    M1 = (phi * wq[:, None]).T @ phi
    K1 = (dphi * wq[:, None]).T @ dphi
    jac = h / 2.0
    Kc = (np.kron(np.kron(M1, M1), K1) + np.kron(np.kron(M1, K1), M1) + np.kron(np.kron(K1, M1), M1)) * jac
    Kc = 0.5 * (Kc + Kc.T)
    ids = M._cell_dof_ids(n, p)
    cons = M.dirichlet_constraints(n, p)
    # charges
    g = int(rng.integers(2, 17))
    centers = rng.uniform(0.25 * L, 0.75 * L, size=(g, 3))
    sig = rng.uniform(0.5, 1.5, size=g)
    B = np.einsum("ka,jb,ic->kjicba", phi, phi, phi).reshape(nq ** 3, nd)
    wq3 = np.einsum("k,j,i->kji", wq, wq, wq).ravel() * jac ** 3
    qz, qy, qx = np.meshgrid(xq, xq, xq, indexing="ij")
    qloc = np.stack([qx.ravel(), qy.ravel(), qz.ravel()], axis=1)
    cz, cy, cx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    corner = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], axis=1) * h
    pts = corner[:, None, :] + (qloc[None, :, :] + 1.0) * jac  # [C, Q, 3]
    rho = np.full(pts.shape[:2], -g / L ** 3)
    for c, s in zip(centers, sig):
        r2 = ((pts - c) ** 2).sum(axis=-1)
        rho += np.exp(-0.5 * r2 / (s * s)) / ((2.0 * np.pi * s * s) ** 1.5)
    bc = (4.0 * np.pi) * (rho * wq3[None, :]) @ B  # [C, nd]
    b = np.bincount(ids.astype(np.int64), weights=bc.ravel(), minlength=N)
    b[cons.row_ids] = 0.0
    diag = np.bincount(ids.astype(np.int64), weights=np.tile(np.diag(Kc), n ** 3), minlength=N)
    diag[cons.row_ids] = 1.0
    return dict(N=N, C=n ** 3, nd=nd, ids=ids, cons=cons, K=Kc, b=b, diag=diag)


def batch(count: int = 64, seed: int = 12349, n_range=(6, 20), degrees=(3, 4)) -> PoissonBatch:
    rng = np.random.default_rng(seed)
    sizes = [(int(rng.integers(n_range[0], n_range[1] + 1)), int(rng.choice(degrees))) for _ in range(count)]
    insts = [_instance(n, p, rng) for n, p in sizes]
    deg_index = {p: i for i, p in enumerate(sorted(set(p for _, p in sizes)))}
    mats = [None] * len(deg_index)
    dof_off = np.zeros(count + 1, np.uint64)
    cell_off = np.zeros(count + 1, np.uint64)
    ids, nd, c2m, b, diag = [], [], [], [], []
    rows, inh = [], []
    for i, ((n, p), d) in enumerate(zip(sizes, insts)):
        k = deg_index[p]
        if mats[k] is None:
            mats[k] = d["K"].T.ravel()
        ids.append(d["ids"].astype(np.uint64) + dof_off[i])
        nd.append(np.full(d["C"], d["nd"], np.uint32))
        c2m.append(np.full(d["C"], k, np.uint32))
        b.append(d["b"])
        diag.append(d["diag"])
        rows.append(d["cons"].row_ids.astype(np.uint64) + dof_off[i])
        dof_off[i + 1] = dof_off[i] + d["N"]
        cell_off[i + 1] = cell_off[i] + d["C"]
    N = int(dof_off[-1])
    if N >= 2 ** 32:
        raise ValueError("batch too large for 32-bit dof ids")
    r = np.concatenate(rows).astype(np.uint32)
    cons = M.Constraints(r, np.zeros(r.size, np.uint32), np.zeros(0, np.uint32), np.zeros(r.size, np.uint32),
                         np.zeros(0), np.zeros(r.size))
    return PoissonBatch(count, N, np.concatenate(nd), np.concatenate(ids).astype(np.uint32), cons,
                        np.concatenate(mats), np.concatenate(c2m), np.concatenate(b), np.concatenate(diag), dof_off,
                        cell_off, sizes)


def instance_view(pb: PoissonBatch, i: int):
    """Mesh / constraints / rhs of instance i alone (for per-instance checks)."""
    d0, d1 = int(pb.inst_dof_off[i]), int(pb.inst_dof_off[i + 1])
    c0, c1 = int(pb.inst_cell_off[i]), int(pb.inst_cell_off[i + 1])
    nd = pb.nd_per_cell[c0:c1]
    coff = np.zeros(pb.nd_per_cell.size + 1, np.int64)
    np.cumsum(pb.nd_per_cell.astype(np.int64), out=coff[1:])
    ids = pb.cell_dof_ids[coff[c0]:coff[c1]].astype(np.int64) - d0
    rows = pb.constraints.row_ids[(pb.constraints.row_ids >= d0) & (pb.constraints.row_ids < d1)].astype(np.int64) - d0
    cons = M.Constraints(rows.astype(np.uint32), np.zeros(rows.size, np.uint32), np.zeros(0, np.uint32),
                         np.zeros(rows.size, np.uint32), np.zeros(0), np.zeros(rows.size))
    k = int(pb.cell_to_mat[c0])
    nd0 = int(nd[0])
    moff = 0
    for u in range(k):
        # matrices are stored in degree order; each has its own nd
        nd_u = int(pb.nd_per_cell[np.argmax(pb.cell_to_mat == u)])
        moff += nd_u * nd_u
    K = pb.mats[moff:moff + nd0 * nd0]
    return dict(N=d1 - d0, nd=nd, ids=ids.astype(np.uint32), cons=cons, K=np.tile(K, c1 - c0),
                b=pb.b[d0:d1].copy(), diag=pb.jacobi_diag[d0:d1].copy())
