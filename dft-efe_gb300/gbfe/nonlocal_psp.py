"""Synthetic separable (ONCV-style) nonlocal projectors on a uniform hex problem.

Projector (l, p, m) of an atom is beta_lp(r) Y_lm(r^) with the radial part
beta_lp(r) = r^l exp(-(r / s_lp)^2) c(r), real spherical harmonics (l <= 1)
and the smooth cutoff c(r) of atoms/SmoothCutoffFunctions.cpp (the one the
enrichment functions use), so the support ends at r0 (1 + 1/d).  Per atom the
projectors run over (l, p) ascending with m fastest, the order
basis/AtomCenterNonLocalOpContextFE.t.cpp:556-593 assumes; the coupling is
diagonal, V = D[beta index of (l, p)] (:595-619).

A cell whose box meets an atom's support carries all of that atom's
projectors, atoms ascending.  Its block is
C_c(b, i) = sum_q p_b(x_q) JxW_q N_i(x_q) over the cell's Gauss points
(:438-499), stored column-major with the projector index fastest, cells
concatenated -- the reference's d_cellWiseC.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import enrichment as E
from . import mesh as M

# (l, p, width s, coupling D in Ha)
DEFAULT_PROJECTORS = [(0, 0, 0.6, 2.5), (0, 1, 1.1, -0.8), (1, 0, 0.7, 1.2), (1, 1, 1.2, -0.4)]
SQRT3_4PI = math.sqrt(3.0 / (4.0 * math.pi))
Y00 = 0.5 / math.sqrt(math.pi)


@dataclass
class NonLocalData:
    n_proj: int
    proj_per_cell: np.ndarray  # uint32 [C]
    proj_ids: np.ndarray       # uint32 [sum np_c]
    cell_c: np.ndarray         # float64 [sum np_c * nd_c]
    coupling: np.ndarray       # float64 [n_proj]
    per_atom: int = 0

    def dense(self, nd_per_cell: np.ndarray, cell_dof_ids: np.ndarray, n_dofs: int) -> np.ndarray:
        """The assembled projector matrix [n_proj, n_dofs] (test helper)."""
        Cg = np.zeros((self.n_proj, n_dofs))
        so = co = do = 0
        for c, np_c in enumerate(self.proj_per_cell):
            nd = int(nd_per_cell[c])
            if np_c:
                blk = self.cell_c[co:co + np_c * nd].reshape(nd, np_c).T  # [np_c, nd]
                ids = cell_dof_ids[do:do + nd].astype(np.int64)
                pid = self.proj_ids[so:so + np_c].astype(np.int64)
                np.add.at(Cg, (pid[:, None], ids[None, :]), blk)
            so += np_c
            co += np_c * nd
            do += nd
        return Cg


def _projector_values(x: np.ndarray, specs, r0: float, d: float) -> np.ndarray:
    """Values [P, n_atom_proj] at offsets x [P, 3] from the atom."""
    r = np.sqrt((x * x).sum(axis=1))
    c = E.cutoff(r, r0, d)
    cols = []
    for (l, p, s, _) in specs:
        g = np.exp(-(r / s) ** 2) * c
        if l == 0:
            cols.append(Y00 * g)
        elif l == 1:
            for comp in (1, 2, 0):  # m = -1, 0, 1 -> y, z, x
                cols.append(SQRT3_4PI * x[:, comp] * g)
        else:
            raise ValueError("l <= 1 only")
    return np.stack(cols, axis=1)


def beta_index(specs) -> list:
    """Coupling index of each projector (m fastest within (l, p))."""
    out = []
    for k, (l, p, s, D) in enumerate(specs):
        out += [k] * (2 * l + 1)
    return out


def projectors(prob: M.FEProblem, specs=DEFAULT_PROJECTORS, r0: float = 2.0, d: float = 4.0,
               nq: int | None = None) -> NonLocalData:
    """Projector data for a uniform classical problem of `mesh.build_problem`."""
    n, p, L = prob.n_side, prob.degree, prob.length
    C = prob.n_cells
    nd = (p + 1) ** 3
    assert np.all(prob.nd_per_cell == nd), "uniform classical meshes only"
    nq = nq or (p + 2)
    h = L / n
    jac = h / 2.0
    xg, _ = M.gll_points(p)
    xq, wq = M.gauss_points(nq)
    phi, _ = M.lagrange_tables(xg, xq)
    B = np.einsum("ka,jb,ic->kjicba", phi, phi, phi).reshape(nq ** 3, nd)
    w3 = np.einsum("k,j,i->kji", wq, wq, wq).ravel() * jac ** 3
    qz, qy, qx = np.meshgrid(xq, xq, xq, indexing="ij")
    qloc = np.stack([qx.ravel(), qy.ravel(), qz.ravel()], axis=1)
    cz, cy, cx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    lo = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], axis=1) * h
    support = r0 * (1.0 + 1.0 / d)
    atoms = prob.atoms
    per_atom = sum(2 * l + 1 for (l, _, _, _) in specs)
    bidx = beta_index(specs)
    coupling = np.tile(np.array([specs[k][3] for k in bidx]), len(atoms))
    blocks = [[] for _ in range(C)]  # per cell: (atom, block [per_atom, nd])
    for a, pos in enumerate(atoms):
        q = np.clip(pos, lo, lo + h)
        cells = np.nonzero(np.sqrt(((q - pos) ** 2).sum(axis=1)) < support)[0]
        for c0 in range(0, len(cells), 512):
            cs = cells[c0:c0 + 512]
            pts = lo[cs][:, None, :] + (qloc[None, :, :] + 1.0) * jac  # [nc, Q, 3]
            vals = _projector_values((pts - pos).reshape(-1, 3), specs, r0, d).reshape(len(cs), -1, per_atom)
            Cc = np.einsum("cqb,q,qi->cbi", vals, w3, B)  # [nc, per_atom, nd]
            for k, c in enumerate(cs):
                blocks[c].append((a, Cc[k]))
    ppc = np.zeros(C, np.uint32)
    pids, cmat = [], []
    for c in range(C):
        if not blocks[c]:
            continue
        blocks[c].sort(key=lambda t: t[0])
        blk = np.concatenate([b for (_, b) in blocks[c]], axis=0)  # [np_c, nd]
        ppc[c] = blk.shape[0]
        pids.append(np.concatenate([a * per_atom + np.arange(per_atom) for (a, _) in blocks[c]]))
        cmat.append(blk.T.ravel())  # column-major: projector index fastest
    return NonLocalData(n_proj=len(atoms) * per_atom, proj_per_cell=ppc,
                        proj_ids=(np.concatenate(pids) if pids else np.zeros(0)).astype(np.uint32),
                        cell_c=np.concatenate(cmat) if cmat else np.zeros(0), coupling=coupling,
                        per_atom=per_atom)
