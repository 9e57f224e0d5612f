"""Finite-element input generator for the cellwise operator apply.

The reference builds its mesh, dof numbering, quadrature and cell matrices
through deal.II (``basis/FEBasisOperations.t.cpp:2201-2268``,
``ksdft/KineticFE.t.cpp:90-97``, ``ksdft/ElectrostaticLocalFE.t.cpp:1625-1660``,
``basis/CFEConstraintsLocalDealii.t.cpp:360-460``).  deal.II is not part of
this project, so this module produces the same *kinds* of arrays itself and in
the reference's layouts, so that the same inputs feed the CPU oracle and the
GPU path:

* uniform hexahedral mesh of ``n`` cells per side on ``[0, L]^3``;
* Lagrange elements of degree ``p`` with nodes at the Gauss-Lobatto-Legendre
  (GLL) points; global nodes numbered lexicographically (x fastest);
* per-cell local node order (i, j, k) with i fastest;
* cell-to-global dof ids flattened cell-major (``size_type`` = uint32);
* dense per-cell matrices, column-major, cells concatenated (offset
  ``sum nd_c^2``), as ``KohnShamOperatorContextFE::d_hamiltonianInAllCells``;
* homogeneous Dirichlet constraints on the boundary as CSR rows with zero
  columns (``ConstraintsInternal`` arrays: rowIds, rowSizes, colIds,
  rowSizesAccumulated, colValues, inhomogeneities);
* the GLL-lumped diagonal mass used by ``CFEOverlapInverseOpContextGLL``.

Matrices: ``K_c = int grad N_i . grad N_j``, ``M_c = int N_i N_j`` (Gauss
quadrature), ``V_c = int N_i V_loc N_j`` and ``H_c = 0.5 K_c + V_c`` with
``V_loc(r) = sum_a -Z erf(r / rc) / r``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

try:  # scipy is present on both machines; math.erf is the fallback
    from scipy.special import erf as _erf
except Exception:  # pragma: no cover
    _erf = np.vectorize(math.erf)


# ----------------------------------------------------------------------------
# 1-D building blocks
# ----------------------------------------------------------------------------
def gll_points(p: int) -> tuple[np.ndarray, np.ndarray]:
    """GLL nodes and weights on [-1, 1] for polynomial degree ``p`` (p+1 points)."""
    if p < 1:
        raise ValueError("degree must be >= 1")
    from numpy.polynomial import legendre as L

    cp = np.zeros(p + 1)
    cp[p] = 1.0
    interior = np.sort(np.real(L.legroots(L.legder(cp)))) if p > 1 else np.zeros(0)
    x = np.concatenate([[-1.0], interior, [1.0]])
    Pp = L.legval(x, cp)
    w = 2.0 / (p * (p + 1) * Pp * Pp)
    return x, w


def gauss_points(q: int) -> tuple[np.ndarray, np.ndarray]:
    """Gauss-Legendre nodes and weights on [-1, 1]."""
    return np.polynomial.legendre.leggauss(q)


def lagrange_tables(nodes: np.ndarray, x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Values ``phi[q, i]`` and derivatives ``dphi[q, i]`` of the Lagrange
    polynomials through ``nodes`` at the points ``x``."""
    n = len(nodes)
    phi = np.ones((len(x), n))
    dphi = np.zeros((len(x), n))
    for i in range(n):
        others = [j for j in range(n) if j != i]
        denom = np.prod([nodes[i] - nodes[j] for j in others])
        for qi, xq in enumerate(x):
            terms = np.array([xq - nodes[j] for j in others])
            phi[qi, i] = np.prod(terms) / denom
            s = 0.0
            for a in range(len(others)):
                s += np.prod(np.delete(terms, a))
            dphi[qi, i] = s / denom
    return phi, dphi


# ----------------------------------------------------------------------------
# problem container
# ----------------------------------------------------------------------------
@dataclass
class Constraints:
    """CSR constraints in the layout of ``basis/ConstraintsInternal.h``.

    Row ``r`` means ``x[row_ids[r]] = inhomogeneities[r] +
    sum_j col_values[acc[r]+j] * x[col_ids[acc[r]+j]]``; Dirichlet rows have
    zero columns.
    """

    row_ids: np.ndarray  # uint32 [nrows]
    row_sizes: np.ndarray  # uint32 [nrows]
    col_ids: np.ndarray  # uint32 [nnz]
    row_acc: np.ndarray  # uint32 [nrows]
    col_values: np.ndarray  # float64 [nnz]
    inhomogeneities: np.ndarray  # float64 [nrows]

    @property
    def nrows(self) -> int:
        return int(self.row_ids.size)


@dataclass
class FEProblem:
    n_side: int
    degree: int
    length: float
    n_dofs: int
    n_cells: int
    nd_per_cell: np.ndarray  # uint32 [C]
    cell_dof_ids: np.ndarray  # uint32 [sum nd]
    constraints: Constraints
    atoms: np.ndarray  # [A, 3]
    charges: np.ndarray  # [A]
    rc: float
    K: Optional[np.ndarray] = None  # float64 [sum nd^2]  (col-major per cell)
    M: Optional[np.ndarray] = None
    V: Optional[np.ndarray] = None
    H: Optional[np.ndarray] = None
    m_gll_diag: Optional[np.ndarray] = None  # float64 [N]
    node_xyz: Optional[np.ndarray] = None  # [N, 3]
    extra: dict = field(default_factory=dict)

    @property
    def nd(self) -> int:
        return int(self.nd_per_cell[0])

    def cell_offsets(self) -> np.ndarray:
        off = np.zeros(self.n_cells + 1, dtype=np.int64)
        np.cumsum(self.nd_per_cell.astype(np.int64), out=off[1:])
        return off

    def mat_offsets(self) -> np.ndarray:
        off = np.zeros(self.n_cells + 1, dtype=np.int64)
        np.cumsum(self.nd_per_cell.astype(np.int64) ** 2, out=off[1:])
        return off


def local_potential(points: np.ndarray, atoms: np.ndarray, charges: np.ndarray, rc: float) -> np.ndarray:
    """``V_loc(r) = sum_a -Z_a erf(|r - R_a| / rc) / |r - R_a|`` (finite at r=0)."""
    v = np.zeros(points.shape[0])
    for a in range(atoms.shape[0]):
        r = np.sqrt(((points - atoms[a]) ** 2).sum(axis=1))
        small = r < 1e-12
        rs = np.where(small, 1.0, r)
        val = -charges[a] * _erf(rs / rc) / rs
        val = np.where(small, -charges[a] * 2.0 / (math.sqrt(math.pi) * rc), val)
        v += val
    return v


def _cell_dof_ids(n: int, p: int) -> np.ndarray:
    n1 = n * p + 1
    loc = np.arange(p + 1)
    k, j, i = np.meshgrid(loc, loc, loc, indexing="ij")  # local order i fastest
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    cz, cy, cx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    cx, cy, cz = cx.ravel(), cy.ravel(), cz.ravel()
    gx = cx[:, None] * p + i[None, :]
    gy = cy[:, None] * p + j[None, :]
    gz = cz[:, None] * p + k[None, :]
    return ((gz * n1 + gy) * n1 + gx).astype(np.uint32).ravel()


def dirichlet_constraints(n: int, p: int) -> Constraints:
    n1 = n * p + 1
    z, y, x = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    bnd = (x == 0) | (y == 0) | (z == 0) | (x == n1 - 1) | (y == n1 - 1) | (z == n1 - 1)
    rows = np.nonzero(bnd.ravel())[0].astype(np.uint32)
    nr = rows.size
    return Constraints(
        row_ids=rows,
        row_sizes=np.zeros(nr, np.uint32),
        col_ids=np.zeros(0, np.uint32),
        row_acc=np.zeros(nr, np.uint32),
        col_values=np.zeros(0, np.float64),
        inhomogeneities=np.zeros(nr, np.float64),
    )


def add_synthetic_hanging(cons: Constraints, n: int, p: int, rng: np.random.Generator,
                          fraction: float = 0.05, inhomogeneous: bool = False) -> Constraints:
    """Append hanging-node-like rows: a fraction of interior nodes, each tied to
    2-4 unconstrained interior neighbours with random weights summing to 1.
    Columns are never constrained rows (the constraint set stays closed), as
    deal.II guarantees for the reference's ``AffineConstraints``."""
    n1 = n * p + 1
    N = n1 ** 3
    constrained = np.zeros(N, bool)
    constrained[cons.row_ids] = True
    z, y, x = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    interior = ~constrained.reshape(n1, n1, n1)
    cand = np.nonzero(interior.ravel())[0]
    pick = np.sort(rng.choice(cand, size=max(1, int(fraction * cand.size)), replace=False))
    is_row = constrained.copy()
    is_row[pick] = True
    rows, sizes, cols, vals, inh = [], [], [], [], []
    offs = [1, -1, n1, -n1, n1 * n1, -n1 * n1]
    for r in pick:
        nb = [r + o for o in offs if 0 <= r + o < N and not is_row[r + o]]
        if len(nb) < 2:
            is_row[r] = False
            continue
        k = int(rng.integers(2, min(4, len(nb)) + 1))
        sel = rng.choice(nb, size=k, replace=False)
        w = rng.random(k) + 0.5
        w /= w.sum()
        rows.append(r)
        sizes.append(k)
        cols.extend(sel.tolist())
        vals.extend(w.tolist())
        inh.append(rng.normal() * 0.1 if inhomogeneous else 0.0)
    all_rows = np.concatenate([cons.row_ids, np.array(rows, np.uint32)])
    all_sizes = np.concatenate([cons.row_sizes, np.array(sizes, np.uint32)])
    all_cols = np.concatenate([cons.col_ids, np.array(cols, np.uint32)])
    all_vals = np.concatenate([cons.col_values, np.array(vals, np.float64)])
    all_inh = np.concatenate([cons.inhomogeneities, np.array(inh, np.float64)])
    acc = np.zeros(all_rows.size, np.uint32)
    if all_rows.size:
        acc[1:] = np.cumsum(all_sizes[:-1])
    return Constraints(all_rows, all_sizes, all_cols.astype(np.uint32), acc, all_vals, all_inh)


def build_problem(n: int, p: int, length: float, atoms: np.ndarray, charges: np.ndarray, rc: float,
                  nq: Optional[int] = None, matrices: tuple = ("K", "M", "V", "H"),
                  cell_chunk: int = 2048, keep_quadrature: bool = False) -> FEProblem:
    """Assemble a uniform-hex FE problem (see module docstring)."""
    nq = nq or (p + 1)
    n1 = n * p + 1
    N = n1 ** 3
    C = n ** 3
    nd = (p + 1) ** 3
    h = length / n
    xg, wg = gll_points(p)
    xq, wq = gauss_points(nq)
    phi, dphi = lagrange_tables(xg, xq)  # [nq, p+1]

    # 1-D reference mass / stiffness on [-1, 1]
    M1 = (phi * wq[:, None]).T @ phi
    K1 = (dphi * wq[:, None]).T @ dphi
    jac = h / 2.0
    # local order i fastest: index a = (k*(p+1)+j)*(p+1)+i -> kron(z, y, x)
    Mc = np.kron(np.kron(M1, M1), M1) * jac ** 3
    Kc = (np.kron(np.kron(M1, M1), K1) + np.kron(np.kron(M1, K1), M1) + np.kron(np.kron(K1, M1), M1)) * jac

    ids = _cell_dof_ids(n, p)
    cons = dirichlet_constraints(n, p)
    prob = FEProblem(n_side=n, degree=p, length=length, n_dofs=N, n_cells=C,
                     nd_per_cell=np.full(C, nd, np.uint32), cell_dof_ids=ids, constraints=cons,
                     atoms=np.asarray(atoms, np.float64).reshape(-1, 3),
                     charges=np.asarray(charges, np.float64), rc=rc)

    # node coordinates (GLL positions)
    g1 = np.concatenate([c * h + (xg[:-1] + 1.0) * jac for c in range(n)] + [np.array([length])])
    prob.extra["grid_1d"] = g1

    if "K" in matrices:
        prob.K = np.tile(Kc.T.ravel(), C)  # column-major per cell
    if "M" in matrices:
        prob.M = np.tile(Mc.T.ravel(), C)

    need_v = ("V" in matrices) or ("H" in matrices)
    if need_v:
        # basis at the 3-D quadrature points, local order i fastest
        B = np.einsum("ka,jb,ic->kjicba", phi, phi, phi).reshape(nq ** 3, nd)  # B[q, a]
        wq3 = np.einsum("k,j,i->kji", wq, wq, wq).ravel() * jac ** 3
        qz, qy, qx = np.meshgrid(xq, xq, xq, indexing="ij")
        qloc = np.stack([qx.ravel(), qy.ravel(), qz.ravel()], axis=1)  # local coords
        cz, cy, cx = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        corner = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], axis=1) * h
        V = np.empty(C * nd * nd) if "V" in matrices else None
        H = np.empty(C * nd * nd) if "H" in matrices else None
        halfK = 0.5 * Kc
        quad_w = np.empty((C, nq ** 3)) if keep_quadrature else None
        for c0 in range(0, C, cell_chunk):
            c1 = min(C, c0 + cell_chunk)
            pts = corner[c0:c1, None, :] + (qloc[None, :, :] + 1.0) * jac
            vq = local_potential(pts.reshape(-1, 3), prob.atoms, prob.charges, rc).reshape(c1 - c0, -1)
            wv = vq * wq3[None, :]
            if quad_w is not None:
                quad_w[c0:c1] = wv
            Vc = np.matmul(B.T[None, :, :] * wv[:, None, :], B[None, :, :])  # [c, nd, nd] symmetric
            Vc = 0.5 * (Vc + np.transpose(Vc, (0, 2, 1)))
            seg = slice(c0 * nd * nd, c1 * nd * nd)
            if V is not None:
                V[seg] = np.transpose(Vc, (0, 2, 1)).ravel()
            if H is not None:
                H[seg] = np.transpose(Vc + halfK[None], (0, 2, 1)).ravel()
        prob.V, prob.H = V, H
        if keep_quadrature:
            # B[q][a] and w[c][q] = JxW * V_loc: H_c = 0.5 K_c + B^T diag(w_c) B
            prob.extra.update(quad_B=np.ascontiguousarray(B), quad_w=quad_w, quad_JxW=wq3.copy(),
                              K_cell=Kc.T.ravel().copy())

    # GLL-lumped mass diagonal: w_i w_j w_k jac^3 assembled over cells
    wl = np.einsum("k,j,i->kji", wg, wg, wg).ravel() * jac ** 3
    diag = np.zeros(N)
    np.add.at(diag, ids.astype(np.int64), np.tile(wl, C))
    prob.m_gll_diag = diag
    return prob


# ----------------------------------------------------------------------------
# the named workloads
# ----------------------------------------------------------------------------
def seeded_atoms(kind: str, rng: np.random.Generator, length: float, count: int) -> np.ndarray:
    if kind == "uniform_inner_half":
        return rng.uniform(0.25 * length, 0.75 * length, size=(count, 3))
    if kind == "jittered_cubic":
        s = round(count ** (1.0 / 3.0))
        a = length / s
        g = (np.arange(s) + 0.5) * a
        z, y, x = np.meshgrid(g, g, g, indexing="ij")
        pos = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
        return pos + rng.uniform(-0.1 * a, 0.1 * a, size=pos.shape)
    raise ValueError(kind)


def ks_box(n: int, p: int, length: float, n_atoms: int, Z: float, rc: float, seed: int,
           atom_layout: str = "uniform_inner_half", **kw) -> FEProblem:
    rng = np.random.default_rng(seed)
    atoms = seeded_atoms(atom_layout, rng, length, n_atoms) if n_atoms else np.zeros((0, 3))
    prob = build_problem(n, p, length, atoms, np.full(len(atoms), Z), rc, **kw)
    prob.extra["seed"] = seed
    return prob


def config1(seed: int = 12346) -> FEProblem:
    """Plain FP64 ChFSI case: 8^3 cells, p=3, side 20 bohr, 4 atoms (Z=4, rc=0.5)
    uniform in the inner half, 4 Gauss points per axis."""
    return ks_box(8, 3, 20.0, 4, 4.0, 0.5, seed, nq=4)


def config3(seed: int = 12348, **kw) -> FEProblem:
    """Mixed-precision case at scale: 24^3 cells, p=5, side 40 bohr, 64 atoms on
    a jittered 4x4x4 lattice (Z=4, rc=0.5)."""
    return ks_box(24, 5, 40.0, 64, 4.0, 0.5, seed, atom_layout="jittered_cubic", **kw)


def lanczos_start_vector(n_dofs: int, seed: int) -> np.ndarray:
    """Seeded uniform [0, 1) Lanczos start vector (the reference draws
    std::rand() / RAND_MAX per entry, LanczosExtremeEigenSolver.t.cpp:40-52,
    from an unseeded generator; a seeded one makes runs repeatable)."""
    return np.random.Generator(np.random.MT19937(seed)).random(n_dofs)


def random_block(n_dofs: int, m: int, seed: int, dtype=np.float64) -> np.ndarray:
    """Seeded N(0,1) initial block, row-major [N][m] (vector index fastest)."""
    return np.random.default_rng(seed).standard_normal((n_dofs, m)).astype(dtype)
