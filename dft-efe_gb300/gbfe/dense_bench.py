"""Time the dense FP64 stages of a ChFSI pass: the Gram matrix X^T Y and the
rotation X T of N x m blocks, DGEMM against the sliced tensor-core products.

    python -m gbfe.dense_bench --n 117689 --m 64 --reps 20

Prints one JSON line per shape: milliseconds per call (wall clock around
`reps` synchronised calls, and the CUDA-event time of the sliced kernel),
algorithmic FP64 TFLOP/s (2 N m^2 per call) and the error of the sliced
result against the DGEMM result (Gram: relative to ||x_i|| ||y_j||; rotation:
relative to max_i |X_ki| sum_i |T_ij|).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api


def _flat_basis(ctx, N):
    return api.FEBasisManager(ctx, np.ones(N, np.uint32), np.arange(N, dtype=np.uint32), N)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=117689)
    ap.add_argument("--m", type=int, default=64)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--only", choices=["gram", "rotate", "both"], default="both")
    args = ap.parse_args()
    N, m = args.n, args.m
    rng = np.random.default_rng(5)
    ctx = api.LinAlgOpContext(0)
    basis = _flat_basis(ctx, N)
    X0, Y0 = rng.standard_normal((N, m)), rng.standard_normal((N, m))
    T = rng.standard_normal((m, m))
    X, Y, Z = api.MultiVector(basis, m, init=X0), api.MultiVector(basis, m, init=Y0), api.MultiVector(basis, m)
    flops = 2.0 * N * m * m
    out = {"n": N, "m": m, "reps": args.reps}
    for what in (("gram", "rotate") if args.only == "both" else (args.only,)):
        res = {}
        for mode in (0, 1):
            ctx.set_fp64_apply(mode)

            def call():
                if what == "gram":
                    return api.gram(X, Y)
                api.rotate(X, T, Z)
                return None

            for _ in range(3):
                call()
            ctx.synchronize()
            ctx.set_profiling(True)
            ctx.reset_kernel_stats()
            t0 = time.perf_counter()
            for _ in range(args.reps):
                r = call()
            ctx.synchronize()
            ms = (time.perf_counter() - t0) / args.reps * 1e3
            st = ctx.kernel_stats("gram_f64_oz" if what == "gram" else "rotate_f64_oz")
            ctx.set_profiling(False)
            ctx.check_status()
            res[mode] = (ms, st, r if what == "gram" else Z.numpy())
        ctx.set_fp64_apply(0)
        if what == "gram":  # relative to ||x_i|| ||y_j|| (Cauchy-Schwarz bound of each entry)
            scale = np.sqrt((X0 * X0).sum(axis=0))[:, None] * np.sqrt((Y0 * Y0).sum(axis=0))[None, :]
            err = float((np.abs(res[1][2] - res[0][2]) / scale).max())
        else:
            scale = np.abs(X0).max(axis=1, keepdims=True) * np.abs(T).sum(axis=0, keepdims=True)
            err = float((np.abs(res[1][2] - res[0][2]) / scale).max())
        k_ms = res[1][1]["ms"] / max(1, res[1][1]["launches"])
        out[what] = {"dgemm_ms": res[0][0], "sliced_ms": res[1][0], "sliced_kernel_ms": k_ms,
                     "dgemm_tflops": flops / (res[0][0] * 1e-3) / 1e12,
                     "sliced_tflops": flops / (res[1][0] * 1e-3) / 1e12,
                     "sliced_kernel_tflops": flops / (k_ms * 1e-3) / 1e12 if k_ms > 0 else None,
                     "speedup": res[0][0] / res[1][0], "rel_err_vs_dgemm": err}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
