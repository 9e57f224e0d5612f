"""Time one FE operator apply (the Hamiltonian on a block of vectors).

    python -m gbfe.apply_bench --config cfg2c --precision mixed --reps 20

Prints one JSON line: device time per apply (CUDA events on the library's
stream via the per-kernel statistics), algorithmic GFLOP/s (2 m sum nd_c^2)
and GB/s (2 N m s_x + sum nd_c^2 s_A) of the cell-product kernel, and the
whole apply.  The workloads are the seeded synthetic meshes of gbfe.mesh.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api
from . import mesh as M

WORKLOADS = {
    "cfg1": dict(n=8, p=3, L=20.0, atoms=4, Z=4.0, rc=0.5, layout="uniform_inner_half", nq=4, m=24, seed=12346),
    "cfg2c": dict(n=12, p=4, L=24.0, atoms=8, Z=6.0, rc=0.4, layout="uniform_inner_half", nq=None, m=64,
                  seed=12347),
    "cfg3": dict(n=24, p=5, L=40.0, atoms=64, Z=4.0, rc=0.5, layout="jittered_cubic", nq=None, m=512, seed=12348),
    # the same cells (degree 5, 216 dofs) and block width on an 8^3 mesh: a
    # case small enough for a full profiler capture (X 141 MB, tiles 95 MB)
    "cfg3s": dict(n=8, p=5, L=40.0 / 3.0, atoms=8, Z=4.0, rc=0.5, layout="jittered_cubic", nq=None, m=512,
                  seed=12348),
    "cfg2": dict(enriched=True, m=64),  # gbfe.enrichment.config2(): 12^3 cells of degree 4 + 40 enrichment dofs
}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="cfg2c", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["f64", "f64_tensor", "mixed", "mixed_v1", "simt"])
    ap.add_argument("--m", type=int, default=0, help="vectors (0: the workload's)")
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--filter", type=int, default=0,
                    help="time the mixed residual Chebyshev filter of this degree instead of one apply")
    ap.add_argument("--tune", action="store_true", help="autotune the split-BF16 launch shape first (as bench.py)")
    ap.add_argument("--passes", type=int, default=0,
                    help="time this many fused mixed ChFSI passes (degree 16, sliced FP64 stages) instead")
    args = ap.parse_args()
    w = WORKLOADS[args.config]
    m = args.m or w["m"]
    if w.get("enriched"):
        from . import enrichment

        prob = enrichment.config2()
    else:
        prob = M.ks_box(w["n"], w["p"], w["L"], w["atoms"], w["Z"], w["rc"], w["seed"], atom_layout=w["layout"],
                        nq=w["nq"], matrices=("H",))
    ctx = api.LinAlgOpContext(0)
    basis = api.FEBasisManager.from_problem(ctx, prob)
    if args.filter:
        return filter_bench(args, prob, ctx, basis, m)
    if args.passes:
        return passes_bench(args, prob, ctx, basis, m)
    mixed = args.precision not in ("f64", "f64_tensor")
    H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=mixed, fp64_tensor=args.precision == "f64_tensor")
    if args.precision == "f64_tensor":
        ctx.set_fp64_apply(1)
    dt = np.float32 if mixed else np.float64
    X = api.MultiVector(basis, m, dtype=dt, init=M.random_block(prob.n_dofs, m, 1).astype(dt))
    Y = api.MultiVector(basis, m, dtype=dt)
    if args.precision == "simt":
        ctx.set_tensor_cores(0)
    elif args.precision == "mixed_v1":
        ctx.set_tensor_cores(1)
    tuned = api.autotune(H, m) if (args.tune and args.precision == "mixed") else None
    for _ in range(3):
        H.apply(X, Y)
    ctx.synchronize()
    ctx.set_profiling(True)
    ctx.reset_kernel_stats()
    t0 = time.perf_counter()
    for _ in range(args.reps):
        H.apply(X, Y)
    ctx.synchronize()
    wall = (time.perf_counter() - t0) / args.reps
    st = ctx.kernel_stats({"f64": "cell_apply_f64", "f64_tensor": "cell_apply_f64_oz"}.get(args.precision,
                                                                                         "cell_apply_mixed"))
    ctx.check_status()
    sx = 4 if mixed else 8
    flops = 2.0 * m * float((prob.nd_per_cell.astype(np.float64) ** 2).sum())
    bytes_ = 2.0 * prob.n_dofs * m * sx + float((prob.nd_per_cell.astype(np.float64) ** 2).sum()) * (4 if mixed else 8)
    k_ms = st["ms"] / max(1, st["launches"]) * max(1, st["launches"] // args.reps)
    print(json.dumps({
        "config": args.config, "precision": args.precision, "m": m, "n_dofs": prob.n_dofs, "cells": prob.n_cells,
        "nd": int(prob.nd_per_cell.max()), "cell_kernel_ms": k_ms, "apply_wall_ms": wall * 1e3,
        "cell_kernel_tflops": flops / (k_ms * 1e-3) / 1e12, "cell_kernel_gbs": bytes_ / (k_ms * 1e-3) / 1e9,
        "algorithmic_gflop": flops / 1e9, "algorithmic_mb": bytes_ / 1e6, "tuned": tuned,
    }))


def filter_bench(args, prob, ctx, basis, m) -> None:
    """Mixed residual Chebyshev filter (FP32 recurrence, split-BF16 products)
    of the workload's Hamiltonian, overlap and inverse overlap."""
    H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=True)
    Mo = api.CFEOverlapOperatorContext(basis, prob.M, mixed=True)
    if "enr_block_inv" in prob.extra:
        Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, prob.m_gll_diag, prob.extra["enr_begin"],
                                                    prob.extra["enr_block_inv"])
    else:
        Mi = api.CFEOverlapInverseOpContextGLL(basis, prob.m_gll_diag)
    b = api.lanczos_bounds(H, Mo, Mi, 20, 7)
    wl, wu, uu = b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10
    eig = np.linspace(wl, wu, m)
    X = api.MultiVector(basis, m, init=M.random_block(prob.n_dofs, m, 1))
    Y = api.MultiVector(basis, m)
    for _ in range(3):
        api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig, X, args.filter, wl, wu, uu, Y, mixed=True)
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.reps):
        api.ResidualChebyshevFilterGEP(H, Mo, Mi, eig, X, args.filter, wl, wu, uu, Y, mixed=True)
    ctx.synchronize()
    ctx.check_status()
    print(json.dumps({"config": args.config, "filter_degree": args.filter, "m": m, "n_dofs": prob.n_dofs,
                      "filter_ms": (time.perf_counter() - t0) / args.reps * 1e3}))


def passes_bench(args, prob, ctx, basis, m) -> None:
    """A fixed number of fused mixed ChFSI passes (the bench's solve, cut
    short): mixed filter of degree 16, sliced FP64 applies, Gram products and
    the rotation with the residual."""
    H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=True, fp64_tensor=True)
    Mo = api.CFEOverlapOperatorContext(basis, prob.M, mixed=True, fp64_tensor=True)
    if "enr_block_inv" in prob.extra:
        Mi = api.OrthoEFEOverlapInverseOpContextGLL(basis, prob.m_gll_diag, prob.extra["enr_begin"],
                                                    prob.extra["enr_block_inv"])
    else:
        Mi = api.CFEOverlapInverseOpContextGLL(basis, prob.m_gll_diag)
    b = api.lanczos_bounds(H, Mo, Mi, 20, 7)
    bounds = (b[0], b[0] + 0.1 * (b[1] - b[0]), b[1] + b[2] / 10)
    X0 = M.random_block(prob.n_dofs, m, 1)
    solver = api.KohnShamEigenSolver(max(1, 3 * m // 4), 16, args.passes, 1e-6, mixed=True, bounds=bounds,
                                     fixed_passes=True, fp64_tensor=True)
    ts = []
    for _ in range(max(1, args.reps)):
        X = api.MultiVector(basis, m, init=X0)
        ctx.synchronize()
        t0 = time.perf_counter()
        solver.solve(H, X, Mo, Mi)
        ctx.synchronize()
        ts.append(time.perf_counter() - t0)
    ctx.check_status()
    print(json.dumps({"config": args.config, "passes": args.passes, "m": m, "n_dofs": prob.n_dofs,
                      "ms_per_pass": min(ts) / args.passes * 1e3}))


if __name__ == "__main__":
    main()
