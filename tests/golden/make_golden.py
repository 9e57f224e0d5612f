"""Generate the golden vectors in this folder by running the reference's own
CPU implementation (oracle/_ref/ref_driver, built by oracle/build_ref.sh from
the reference sources) on small seeded inputs.

Each case_*.npz holds the inputs (mesh, constraints, cell matrices, X, b, ...)
and the reference outputs:
  Y_H, X_after   KohnShamOperatorContextFE::apply on H and X after constraints
  Y_M            the same apply on the overlap matrices
  Y_Minv         the GLL-diagonal inverse overlap apply
  Y_rfilter      ResidualChebyshevFilterGEP(H, M, M^-1)
  Y_filter       ChebyshevFilter(H, M^-1)
  x_cg, cg_ok    Jacobi-preconditioned CGLinearSolver on K
  Y_nl, Y_Hnl    (nonlocal cases) AtomCenterNonLocalOpContextFE::apply alone,
                 and the KS apply of H with the nonlocal part fused in
  Y_Minv_efe     (enriched cases) OrthoEFEOverlapInverseOpContextGLL::apply:
                 GLL diagonal inverse plus the dense inverse enrichment block
                 (inputs enr_begin, enr_blk)

Run (in a checkout where the reference sources exist):
    bash oracle/build_ref.sh && python tests/golden/make_golden.py [case names]
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "dft-efe_gb300"))
import gbfe.mesh as M  # noqa: E402

DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"
HERE = Path(__file__).resolve().parent


def run_case(name, nd, ids, N, cons, H, Mm, K, minv, jacdiag, X, eig, b, degree, wl, wu, uu,
             max_iter=3000, abs_tol=1e-14, rel_tol=1e-11, div_tol=1e8, nl=None, efe=None):
    m = X.shape[1]
    nrhs = b.shape[1]
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        (d / "meta.txt").write_text(f"{N} {nd.size} {m} {degree} {wl!r} {wu!r} {uu!r} {max_iter} {abs_tol!r} "
                                    f"{rel_tol!r} {div_tol!r} {nrhs}\n")
        for fname, arr, dt in [("nd.u32", nd, np.uint32), ("ids.u32", ids, np.uint32), ("H.f64", H, np.float64),
                               ("M.f64", Mm, np.float64), ("K.f64", K, np.float64), ("minv.f64", minv, np.float64),
                               ("jacdiag.f64", jacdiag, np.float64), ("cons_rows.u32", cons.row_ids, np.uint32),
                               ("cons_sizes.u32", cons.row_sizes, np.uint32),
                               ("cons_cols.u32", cons.col_ids, np.uint32), ("cons_acc.u32", cons.row_acc, np.uint32),
                               ("cons_vals.f64", cons.col_values, np.float64),
                               ("cons_inh.f64", cons.inhomogeneities, np.float64), ("X.f64", X, np.float64),
                               ("eig.f64", eig, np.float64), ("b.f64", b, np.float64)]:
            np.ascontiguousarray(arr, dtype=dt).tofile(d / fname)
        extra = {}
        if nl is not None:
            (d / "nl_meta.txt").write_text(f"{nl.n_proj}\n")
            for fname, arr, dt in [("nl_np.u32", nl.proj_per_cell, np.uint32), ("nl_pids.u32", nl.proj_ids, np.uint32),
                                   ("nl_c.f64", nl.cell_c, np.float64), ("nl_v.f64", nl.coupling, np.float64)]:
                np.ascontiguousarray(arr, dtype=dt).tofile(d / fname)
            extra = dict(nl_n_proj=np.array(nl.n_proj), nl_np=nl.proj_per_cell, nl_pids=nl.proj_ids,
                         nl_c=nl.cell_c, nl_v=nl.coupling)
        if efe is not None:
            enr_begin, blk = efe  # blk: the inverse enrichment overlap block, row-major
            (d / "efe_meta.txt").write_text(f"{enr_begin} {blk.shape[0]}\n")
            np.ascontiguousarray(blk.T, dtype=np.float64).tofile(d / "efe_blk.f64")  # column-major
            extra.update(enr_begin=np.array(enr_begin), enr_blk=blk)
        subprocess.run([str(DRIVER), str(d)], check=True)
        rd = lambda f, shape: np.fromfile(d / f, dtype=np.float64).reshape(shape)  # noqa: E731
        out = dict(Y_H=rd("Y_H.f64", (N, m)), X_after=rd("X_after.f64", (N, m)), Y_M=rd("Y_M.f64", (N, m)),
                   Y_Minv=rd("Y_Minv.f64", (N, m)), Y_rfilter=rd("Y_rfilter.f64", (N, m)),
                   Y_filter=rd("Y_filter.f64", (N, m)), x_cg=rd("x_cg.f64", (N, nrhs)),
                   cg_ok=np.array(int((d / "cg.txt").read_text().split()[0]) == 0))
        if nl is not None:
            if not (d / "Y_nl.f64").exists():
                sys.exit("ref_driver was built without the nonlocal part (see oracle/build_ref.sh)")
            out.update(Y_nl=rd("Y_nl.f64", (N, m)), Y_Hnl=rd("Y_Hnl.f64", (N, m)))
        if efe is not None:
            if not (d / "Y_Minv_efe.f64").exists():
                sys.exit("ref_driver was built without the OrthoEFE inverse (see oracle/build_ref.sh)")
            out.update(Y_Minv_efe=rd("Y_Minv_efe.f64", (N, m)))
    np.savez_compressed(HERE / f"{name}.npz", nd=nd.astype(np.uint32), ids=ids.astype(np.uint32), n_dofs=np.array(N),
                        cons_rows=cons.row_ids, cons_sizes=cons.row_sizes, cons_cols=cons.col_ids,
                        cons_acc=cons.row_acc, cons_vals=cons.col_values, cons_inh=cons.inhomogeneities,
                        H=H, M=Mm, K=K, minv=minv, jacdiag=jacdiag, X=X, eig=eig, b=b,
                        params=np.array([degree, wl, wu, uu, max_iter, abs_tol, rel_tol, div_tol]), **out, **extra)
    print(f"{name}: N={N} cells={nd.size} m={m} -> {HERE / (name + '.npz')}")


def jacobi_diag(nd, ids, K, N, cons):
    diag = np.zeros(N)
    off = 0
    p = 0
    for k in nd.astype(np.int64):
        A = K[off:off + k * k].reshape(k, k)
        np.add.at(diag, ids[p:p + k].astype(np.int64), np.diag(A))
        off += k * k
        p += k
    diag[cons.row_ids] = 1.0  # c2p then setConstrainedNodes(1.0) for Dirichlet rows
    return diag


def fe_case(name, n, p, L, atoms, seed, m, degree, hanging=False, nonlocal_part=False):
    prob = M.ks_box(n, p, L, atoms, 4.0, 0.5, seed=seed)
    if hanging:
        prob.constraints = M.add_synthetic_hanging(prob.constraints, n, p, np.random.default_rng(seed), 0.1,
                                                   inhomogeneous=True)
    rng = np.random.default_rng(seed + 1)
    X = rng.standard_normal((prob.n_dofs, m))
    eig = np.sort(rng.uniform(-3.0, 0.5, m))
    b = rng.standard_normal((prob.n_dofs, 2))
    b[prob.constraints.row_ids] = 0.0
    # bounds from the spectrum of M_GLL^-1 H estimated with a dense solve (small case)
    wl, wu, uu = -4.0, 1.0, 40.0 * p * p / (L / n) ** 2
    nl = None
    if nonlocal_part:
        from gbfe import nonlocal_psp

        nl = nonlocal_psp.projectors(prob)
    run_case(name, prob.nd_per_cell, prob.cell_dof_ids, prob.n_dofs, prob.constraints, prob.H, prob.M, prob.K,
             1.0 / prob.m_gll_diag, jacobi_diag(prob.nd_per_cell, prob.cell_dof_ids, prob.K, prob.n_dofs,
                                                prob.constraints), X, eig, b, degree, wl, wu, uu, nl=nl)


def enriched_case(name, n, p, L, atoms, seed, m, degree):
    """Orthogonalised enrichment (gbfe/enrichment.py): uneven cells, the
    enrichment ids after the classical ones, the OrthoEFE inverse overlap."""
    from gbfe import enrichment

    prob = enrichment.enriched_problem(n, p, L, atoms, 4.0, 0.5, seed)
    rng = np.random.default_rng(seed + 1)
    X = rng.standard_normal((prob.n_dofs, m))
    eig = np.sort(rng.uniform(-3.0, 0.5, m))
    b = rng.standard_normal((prob.n_dofs, 2))
    b[prob.constraints.row_ids] = 0.0
    wl, wu, uu = -4.0, 1.0, 40.0 * p * p / (L / n) ** 2
    run_case(name, prob.nd_per_cell, prob.cell_dof_ids, prob.n_dofs, prob.constraints, prob.H, prob.M, prob.K,
             1.0 / prob.m_gll_diag, jacobi_diag(prob.nd_per_cell, prob.cell_dof_ids, prob.K, prob.n_dofs,
                                                prob.constraints), X, eig, b, degree, wl, wu, uu,
             efe=(int(prob.extra["enr_begin"]), prob.extra["enr_block_inv"]))


def variable_case(name, seed):
    """Uneven cell sizes (as enriched cells have) with SPD cell matrices."""
    rng = np.random.default_rng(seed)
    C, N = 24, 260
    nd = rng.integers(8, 19, size=C).astype(np.uint32)
    ids = np.concatenate([np.sort(rng.choice(N, size=k, replace=False)) for k in nd]).astype(np.uint32)
    used = np.unique(ids)
    mats = []
    for k in nd.astype(int):
        B = rng.standard_normal((k, k))
        mats.append((B @ B.T / k + np.eye(k)).T.ravel())
    H = np.concatenate(mats)
    Mm = np.concatenate([(0.1 * np.eye(k) + 0.01).T.ravel() for k in nd.astype(int)])
    K = H.copy()
    rows = np.sort(rng.choice(used, size=6, replace=False)).astype(np.uint32)
    cons = M.Constraints(rows, np.zeros(6, np.uint32), np.zeros(0, np.uint32), np.zeros(6, np.uint32), np.zeros(0),
                         np.zeros(6))
    unused = np.setdiff1d(np.arange(N), used)
    minv = np.ones(N) * 5.0
    jd = jacobi_diag(nd, ids, K, N, cons)
    jd[unused] = 1.0
    X = rng.standard_normal((N, 3))
    b = rng.standard_normal((N, 1))
    b[rows] = 0.0
    b[unused] = 0.0
    run_case(name, nd, ids, N, cons, H, Mm, K, minv, jd, X, np.array([0.5, 1.0, 1.5]), b, 5, 0.0, 2.0, 30.0)


if __name__ == "__main__":
    if not DRIVER.exists():
        sys.exit("build oracle/_ref first: bash oracle/build_ref.sh")
    cases = {
        "case_dirichlet_p2": lambda n: fe_case(n, 2, 2, 6.0, 1, 101, 4, 6),
        "case_dirichlet_p3": lambda n: fe_case(n, 2, 3, 8.0, 2, 102, 5, 8),
        "case_hanging_p2": lambda n: fe_case(n, 3, 2, 6.0, 2, 103, 3, 5, hanging=True),
        "case_variable_nd": lambda n: variable_case(n, 104),
        "case_nonlocal_p3": lambda n: fe_case(n, 2, 3, 8.0, 2, 105, 5, 6, nonlocal_part=True),
        "case_nonlocal_hanging_p2": lambda n: fe_case(n, 3, 2, 6.0, 2, 106, 4, 5, hanging=True,
                                                      nonlocal_part=True),
        "case_enriched_p2": lambda n: enriched_case(n, 3, 2, 8.0, 2, 107, 5, 6),
    }
    for name in (sys.argv[1:] or list(cases)):
        cases[name](name)
