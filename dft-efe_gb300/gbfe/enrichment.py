"""Orthogonalised enriched FE inputs (uneven cell sizes).

Each atom carries enrichment functions phi(x) = exp(-zeta r) Y_lm(r^) c(r)
with real spherical harmonics Y_lm and the smooth cutoff of
atoms/SmoothCutoffFunctions.cpp (c(r) = f2(1 - d (r - r0) / r0),
f2(y) = f1(y) / (f1(y) + f1(1 - y)), f1(y) = exp(-1/y) for y > 0, else 0):
c = 1 for r <= r0 and 0 for r >= r0 (1 + 1/d).  With r0 = 3, d = 3 the
support ends at 4 bohr.

Orthogonalisation follows the idea of
basis/EnrichmentClassicalInterfaceSpherical.t.cpp:350-405 (enrichment minus
its L2 projection onto the classical space): phi~ = phi - sum_i a_i N_i with
a = M^-1 int N phi.  Here M is the GLL-lumped classical mass (diagonal), a
documented simplification of the reference's CG solve on the consistent mass;
inputs are synthetic and the same arrays feed the oracle and the GPU path.

A cell whose box meets an atom's support carries, after its (p+1)^3 classical
dofs, the atom's enrichment dofs (global ids N_classical + 5 a + k), as
EFEBasisDofHandlerDealii.t.cpp:944-949 lays out cell dofs.  Cell matrices of
enriched cells (H, M, K) are assembled with a finer Gauss rule over the
extended basis [N | phi~].  The OrthoEFE inverse overlap
(basis/OrthoEFEOverlapInverseOpContextGLL.t.cpp:1182-1270) is the GLL
diagonal inverse on classical dofs plus the dense inverse of the assembled
enrichment-enrichment overlap block.
"""
from __future__ import annotations

import math

import numpy as np

from . import mesh as M

SQRT3_4PI = math.sqrt(3.0 / (4.0 * math.pi))
Y00 = 0.5 / math.sqrt(math.pi)
# (l, m, zeta) per atom
DEFAULT_SPECS = [(0, 0, 5.5), (0, 0, 1.6), (1, -1, 1.6), (1, 0, 1.6), (1, 1, 1.6)]


def _f1(y):
    out = np.zeros_like(y)
    pos = y > 0
    out[pos] = np.exp(-1.0 / y[pos])
    return out


def _f1d(y):
    out = np.zeros_like(y)
    pos = y > 0
    out[pos] = np.exp(-1.0 / y[pos]) / (y[pos] * y[pos])
    return out


def cutoff(r, r0=3.0, d=3.0):
    y = 1.0 - d * (r - r0) / r0
    a, b = _f1(y), _f1(1.0 - y)
    return a / (a + b)


def cutoff_deriv(r, r0=3.0, d=3.0):
    y = 1.0 - d * (r - r0) / r0
    a, b = _f1(y), _f1(1.0 - y)
    ad, bd = _f1d(y), _f1d(1.0 - y)
    den = (a + b) ** 2
    return (ad * b + a * bd) / den * (-d / r0)


def enrichment_values(pts, center, l, mm, zeta, r0=3.0, d=3.0):
    """phi and grad phi at points [P, 3]."""
    x = pts - center
    r = np.sqrt((x * x).sum(axis=1))
    rs = np.maximum(r, 1e-12)
    c = cutoff(r, r0, d)
    cd = cutoff_deriv(r, r0, d)
    e = np.exp(-zeta * r)
    if l == 0:
        g = e * c
        gd = -zeta * e * c + e * cd
        phi = Y00 * g
        grad = (Y00 * gd / rs)[:, None] * x
        return phi, grad
    # l = 1: Y = C x_i / r -> phi = C x_i g(r) / r
    comp = {-1: 1, 0: 2, 1: 0}[mm]
    g = e * c / rs
    gd = (-zeta * e * c + e * cd) / rs - e * c / (rs * rs)
    xi = x[:, comp]
    phi = SQRT3_4PI * xi * g
    grad = (SQRT3_4PI * xi * gd / rs)[:, None] * x
    grad[:, comp] += SQRT3_4PI * g
    return phi, grad


def enriched_problem(n=12, p=4, L=24.0, n_atoms=8, Z=6.0, rc=0.4, seed=12347, specs=DEFAULT_SPECS, r0=3.0, d=3.0,
                     nq_enr=None, keep_quadrature=False):
    """keep_quadrature: also keep, per cell, the basis values at its
    quadrature points (classical cells: the (p+1)^3 Gauss rule; enriched
    cells: the finer rule over [N | phi~]) and the weights JxW V_loc, so that
    H_c = 0.5 K_c + B_c^T diag(w_c) B_c (extra["quad_cells"])."""
    rng = np.random.default_rng(seed)
    atoms = rng.uniform(0.25 * L, 0.75 * L, size=(n_atoms, 3))
    charges = np.full(n_atoms, Z)
    base = M.build_problem(n, p, L, atoms, charges, rc, keep_quadrature=keep_quadrature)
    q_nq, q_B, q_w = [], [], []
    nq = p + 1
    nq_e = nq_enr or (p + 4)
    h = L / n
    jac = h / 2.0
    nd0 = (p + 1) ** 3
    C = n ** 3
    Ncl = base.n_dofs
    n_per = len(specs)
    nE = n_atoms * n_per
    support = r0 * (1.0 + 1.0 / d)
    xg, wgll = M.gll_points(p)
    # cell boxes
    cz, cy, cx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    lo = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], axis=1) * h
    # atom -> cells whose box is within the support radius
    cells_of = []
    for a in range(n_atoms):
        q = np.clip(atoms[a], lo, lo + h)
        dist = np.sqrt(((q - atoms[a]) ** 2).sum(axis=1))
        cells_of.append(np.nonzero(dist < support)[0])
    enr_of_cell = [[] for _ in range(C)]
    for a in range(n_atoms):
        for c in cells_of[a]:
            enr_of_cell[c].append(a)
    # fine Gauss rule for enriched cells
    xq, wq = M.gauss_points(nq_e)
    phi1, dphi1 = M.lagrange_tables(xg, xq)
    B = np.einsum("ka,jb,ic->kjicba", phi1, phi1, phi1).reshape(nq_e ** 3, nd0)
    Gx = np.einsum("ka,jb,ic->kjicba", phi1, phi1, dphi1).reshape(nq_e ** 3, nd0) / jac
    Gy = np.einsum("ka,jb,ic->kjicba", phi1, dphi1, phi1).reshape(nq_e ** 3, nd0) / jac
    Gz = np.einsum("ka,jb,ic->kjicba", dphi1, phi1, phi1).reshape(nq_e ** 3, nd0) / jac
    w3 = np.einsum("k,j,i->kji", wq, wq, wq).ravel() * jac ** 3
    qz, qy, qx = np.meshgrid(xq, xq, xq, indexing="ij")
    qloc = np.stack([qx.ravel(), qy.ravel(), qz.ravel()], axis=1)
    ids0 = base.cell_dof_ids.reshape(C, nd0).astype(np.int64)
    # projection coefficients a_e = M_GLL^-1 int N phi_e (support cells only)
    coef = np.zeros((nE, Ncl))
    cache = {}
    for a in range(n_atoms):
        for c in cells_of[a]:
            pts = lo[c] + (qloc + 1.0) * jac
            vals = [enrichment_values(pts, atoms[a], l, mm, z, r0, d) for (l, mm, z) in specs]
            cache[(a, c)] = (pts, vals)
            for k, (ph, _) in enumerate(vals):
                coef[a * n_per + k] += np.bincount(ids0[c], weights=B.T @ (w3 * ph), minlength=Ncl)
    coef /= base.m_gll_diag[None, :]
    # per-cell matrices
    nd_list, ids_list, H_list, M_list, K_list = [], [], [], [], []
    Mee = np.zeros((nE, nE))
    nd2 = nd0 * nd0
    for c in range(C):
        if not enr_of_cell[c]:
            nd_list.append(nd0)
            ids_list.append(ids0[c])
            sl = slice(c * nd2, (c + 1) * nd2)
            H_list.append(base.H[sl])
            M_list.append(base.M[sl])
            K_list.append(base.K[sl])
            if keep_quadrature:
                q_nq.append(base.extra["quad_B"].shape[0])
                q_B.append(base.extra["quad_B"].ravel())
                q_w.append(base.extra["quad_w"][c])
            continue
        pts = lo[c] + (qloc + 1.0) * jac
        vq = M.local_potential(pts, atoms, charges, rc)
        cols, gcols, eids = [], [], []
        for a in enr_of_cell[c]:
            vals = cache.get((a, c))[1]
            for k, (ph, gr) in enumerate(vals):
                e = a * n_per + k
                ce = coef[e, ids0[c]]
                cols.append(ph - B @ ce)
                gcols.append(gr - np.stack([Gx @ ce, Gy @ ce, Gz @ ce], axis=1))
                eids.append(e)
        Bx = np.concatenate([B, np.stack(cols, axis=1)], axis=1)
        Gxx = np.concatenate([Gx, np.stack([g[:, 0] for g in gcols], axis=1)], axis=1)
        Gyy = np.concatenate([Gy, np.stack([g[:, 1] for g in gcols], axis=1)], axis=1)
        Gzz = np.concatenate([Gz, np.stack([g[:, 2] for g in gcols], axis=1)], axis=1)
        Mc = Bx.T @ (w3[:, None] * Bx)
        Kc = Gxx.T @ (w3[:, None] * Gxx) + Gyy.T @ (w3[:, None] * Gyy) + Gzz.T @ (w3[:, None] * Gzz)
        Vc = Bx.T @ ((w3 * vq)[:, None] * Bx)
        Mc, Kc, Vc = [0.5 * (A + A.T) for A in (Mc, Kc, Vc)]
        Hc = 0.5 * Kc + Vc
        if keep_quadrature:
            q_nq.append(Bx.shape[0])
            q_B.append(np.ascontiguousarray(Bx).ravel())
            q_w.append(w3 * vq)
        ndc = nd0 + len(eids)
        nd_list.append(ndc)
        ids_list.append(np.concatenate([ids0[c], Ncl + np.array(eids, np.int64)]))
        H_list.append(Hc.T.ravel())
        M_list.append(Mc.T.ravel())
        K_list.append(Kc.T.ravel())
        ee = np.array(eids)
        Mee[np.ix_(ee, ee)] += Mc[nd0:, nd0:]
    prob = M.FEProblem(n_side=n, degree=p, length=L, n_dofs=Ncl + nE, n_cells=C,
                       nd_per_cell=np.array(nd_list, np.uint32),
                       cell_dof_ids=np.concatenate(ids_list).astype(np.uint32),
                       constraints=base.constraints, atoms=atoms, charges=charges, rc=rc,
                       K=np.concatenate(K_list), M=np.concatenate(M_list), H=np.concatenate(H_list))
    diag = np.ones(Ncl + nE)
    diag[:Ncl] = base.m_gll_diag
    prob.m_gll_diag = diag
    prob.extra.update(n_classical=Ncl, n_enrichment=nE, enr_begin=Ncl,
                      enr_block_inv=np.linalg.inv(0.5 * (Mee + Mee.T)),
                      enriched_cells=int(sum(1 for e in enr_of_cell if e)), seed=seed)
    if keep_quadrature:
        prob.extra["quad_cells"] = dict(nq=np.array(q_nq, np.uint32), B=np.concatenate(q_B), w=np.concatenate(q_w))
    return prob


def config2(seed: int = 12347, **kw):
    """12^3 cells of degree 4 on a 24 bohr cube, 8 atoms (Z=6, rc=0.4), five
    enrichment functions per atom (zeta of the l=1 functions: 1.6)."""
    return enriched_problem(12, 4, 24.0, 8, 6.0, 0.4, seed, **kw)
