#!/usr/bin/env python
"""ChFSI solves/s on one GB300: mixed precision vs FP64, with p50/p99 latency.

One step = one Kohn-Sham ChFSI eigen solve (Lanczos bounds, then filter ->
Cholesky-GS -> Rayleigh-Ritz passes until the residuals of the wanted pairs
reach the tolerance) of a fixed workload from the same seeded random block.
A mixed solve counts only if its wanted eigenvalues agree with the FP64 solve
of the same inputs within 1e-6 Ha.

Workloads (synthetic, seeded; see gbfe/mesh.py):
  cfg2c  12^3 hex cells of degree 4 on a 24 bohr cube, 8 atoms (Z=6, rc=0.4),
         64 vectors -- the classical part of the enriched configuration
         (enrichment functions are not generated yet); default
  cfg1   8^3 cells of degree 3, 20 bohr, 4 atoms (Z=4, rc=0.5), 24 vectors,
         degree 20
  cfg3   24^3 cells of degree 5, 40 bohr, 64 atoms, 512 vectors, degree 30

--impl reference times the reference's CPU implementation of the same solve
(the oracle port in oracle/, per-cell dgemm through OpenBLAS as the reference
does) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "dft-efe_gb300", ROOT):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

# reference Chebyshev degree lookup (ksdft/Defaults.cpp CHEBY_ORDER_LOOKUP)
CHEBY_ORDER_LOOKUP = [(10, 6), (50, 9), (100, 12), (200, 16), (300, 19), (500, 24), (750, 30), (1000, 39),
                      (1500, 50), (2000, 53), (3000, 57), (4000, 62), (5000, 69), (9000, 77), (14000, 104),
                      (20000, 119), (30000, 162), (50000, 300), (80000, 450), (100000, 550), (200000, 700),
                      (500000, 1000)]

CONFIGS = {
    "cfg1": dict(n=8, p=3, L=20.0, atoms=4, Z=4.0, rc=0.5, layout="uniform_inner_half", nq=4, m=24, n_wanted=16,
                 degree=20, max_passes=30, tol=1e-6, seed=12346),
    "cfg2c": dict(n=12, p=4, L=24.0, atoms=8, Z=6.0, rc=0.4, layout="uniform_inner_half", nq=None, m=64,
                  n_wanted=48, degree=None, max_passes=40, tol=1e-6, seed=12347),
    "cfg3": dict(n=24, p=5, L=40.0, atoms=64, Z=4.0, rc=0.5, layout="jittered_cubic", nq=None, m=512, n_wanted=384,
                 degree=30, max_passes=40, tol=1e-6, seed=12348),
}
EIG_TOL = 1e-6  # Ha


def cheby_degree(unwanted_upper: float) -> int:
    v = int(unwanted_upper)
    for k, d in CHEBY_ORDER_LOOKUP:
        if k >= v:
            return d
    return 1250


def make_problem(cfg):
    import gbfe.mesh as M

    return M.ks_box(cfg["n"], cfg["p"], cfg["L"], cfg["atoms"], cfg["Z"], cfg["rc"], cfg["seed"],
                    atom_layout=cfg["layout"], nq=cfg["nq"])


def lanczos_setup(prob, cfg, bounds_from):
    """Bounds as KohnShamEigenSolver.t.cpp:262-300 derives them from Lanczos."""
    b = bounds_from()
    res = b[2] / 10.0
    m = cfg["m"]
    wl, uu = b[0], b[1] + res
    wu = (b[1] + res - b[0]) * (m * 200.0 / prob.n_dofs) + b[0]
    if wu >= uu:
        wu = (uu + b[0]) * 0.5
    deg = cfg["degree"] or cheby_degree(uu)
    return (wl, wu, uu), deg


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, out_path: Path | None):
        self.proc = None
        self.path = out_path

    def __enter__(self):
        try:
            self.f = open(self.path, "w") if self.path else subprocess.DEVNULL
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [ln for ln in out.splitlines() if ln.strip()]
            if self.path:
                Path(self.path).write_text("\n".join(self.lines) + "\n")

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- CPU side
def _cpu_worker(args):
    """One oracle process: a bounded sample of FP64 ChFSI passes on the workload."""
    cfg_name, passes, m_override = args
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    sys.path.insert(0, str(ROOT / "dft-efe_gb300"))
    sys.path.insert(0, str(ROOT))
    import gbfe.mesh as M
    from oracle import oracle as O

    cfg = dict(CONFIGS[cfg_name])
    if m_override:
        cfg["m"] = m_override
    prob = make_problem(cfg)
    s = O.OracleSystem.from_problem(prob)
    H, Mo, Mi = s.cell_op(prob.H), s.cell_op(prob.M), s.diag_op(1.0 / prob.m_gll_diag)
    (wl, wu, uu), deg = lanczos_setup(prob, cfg, lambda: s.lanczos_bounds(H, Mo, Mi, 20, 7))
    X = M.random_block(prob.n_dofs, cfg["m"], cfg["seed"] + 1)
    eig = np.zeros(cfg["m"])
    t0 = time.perf_counter()
    for _ in range(passes):
        eig, X = s.chfsi_pass(H, Mo, Mi, X, eig, deg, wl, wu, uu)
        s.eigen_residual_norms(H, Mo, X, eig)
        wl, wu = eig[0], eig[-1]
    return time.perf_counter() - t0


def cpu_baseline(cfg_name: str, passes_per_solve: float, procs: int, sample_passes: int = 1):
    """Time `sample_passes` FP64 ChFSI passes in `procs` concurrent oracle
    processes; solves/s = procs / (time per pass * passes per solve)."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        t0 = time.perf_counter()
        times = pool.map(_cpu_worker, [(cfg_name, sample_passes, None)] * procs)
        wall = time.perf_counter() - t0
    per_pass = max(times) / sample_passes
    return {"value": procs / (per_pass * passes_per_solve), "unit": "solves/s", "cores": procs, "kind": "port",
            "sample": f"{sample_passes} FP64 ChFSI pass(es) + residual check of {cfg_name} in each of {procs} "
                      f"single-threaded oracle processes ({per_pass:.2f} s/pass), extrapolated to "
                      f"{passes_per_solve:g} passes per solve; wall {wall:.1f} s"}


# ----------------------------------------------------------------------------- GPU side
def run_gpu(args, cfg_name, rank, world):
    import gbfe.mesh as M
    from gbfe import api

    cfg = CONFIGS[cfg_name]
    prob = make_problem(cfg)
    ctx = api.LinAlgOpContext(0)
    basis = api.FEBasisManager.from_problem(ctx, prob)
    H = api.KohnShamOperatorContextFE(basis, prob.H, mixed=True)
    Mo = api.CFEOverlapOperatorContext(basis, prob.M, mixed=True)
    Mi = api.CFEOverlapInverseOpContextGLL(basis, prob.m_gll_diag)
    m, nw = cfg["m"], cfg["n_wanted"]
    (wl, wu, uu), deg = lanczos_setup(prob, cfg, lambda: api.lanczos_bounds(H, Mo, Mi, 20, 7))
    X0 = M.random_block(prob.n_dofs, m, cfg["seed"] + 1)
    X0dev = api.MultiVector(basis, m, init=X0)
    X = api.MultiVector(basis, m)

    def solver(mixed):
        return api.KohnShamEigenSolver(nw, deg, cfg["max_passes"], cfg["tol"], mixed=mixed, bounds=(wl, wu, uu))

    def solve(mixed):
        X0dev.copy_to(X)
        return solver(mixed).solve(H, X, Mo, Mi)

    # FP64 solve of the same inputs: the accuracy reference and the FP64 arm
    t0 = time.perf_counter()
    rc64, eig64, res64, passes64 = solve(False)
    t_fp64 = time.perf_counter() - t0
    fp64_times = [t_fp64]
    for _ in range(max(0, args.fp64_repeats - 1)):
        t0 = time.perf_counter()
        solve(False)
        fp64_times.append(time.perf_counter() - t0)

    import torch

    torch.cuda.set_device(0)
    dist = world > 1

    def barrier():
        if dist:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        solve(True)
    ctx.synchronize()
    ctx.set_profiling(True)
    ctx.reset_kernel_stats()
    launches0 = ctx.kernel_launches()
    lat, errs, passes, ok, eigs, rcs = [], [], [], 0, [], []
    clocks = ClockSampler(ROOT / "gpurun_out" / "bench_clocks.csv" if (ROOT / "gpurun_out").is_dir() else None)
    with clocks:  # sampler runs across the timed region, started and stopped outside it
        time.sleep(0.5)
        barrier()
        ctx.synchronize()
        t_start = time.perf_counter()
        for _ in range(args.steps):
            ts = time.perf_counter()
            rc, eig, res, npass = solve(True)
            ctx.synchronize()
            lat.append(time.perf_counter() - ts)
            eigs.append(eig)
            passes.append(npass)
            rcs.append(rc)
        ctx.synchronize()
        barrier()
        t_total = time.perf_counter() - t_start
    for rc, eig in zip(rcs, eigs):
        err = float(np.abs(eig[:nw] - eig64[:nw]).max())
        errs.append(err)
        ok += int(rc == 0 and err <= EIG_TOL)
    launches = ctx.kernel_launches() - launches0
    st_mixed = ctx.kernel_stats("cell_apply_mixed")
    st_f64 = ctx.kernel_stats("cell_apply_f64")
    ctx.set_profiling(False)

    # e2e: the same solve through the C ABI with host buffers each step
    pinned = torch.empty((prob.n_dofs, m), dtype=torch.float64, pin_memory=True)
    pinned.numpy()[:] = X0
    out_host = torch.empty((prob.n_dofs, m), dtype=torch.float64, pin_memory=True)
    lib = ctx.lib
    e2e_lat = []
    for _ in range(args.steps):
        ctx.synchronize()
        ts = time.perf_counter()
        lib.gbfe_mv_copy_in(X.h, api.C.c_void_p(pinned.data_ptr()))
        rc, eig, res, npass = solver(True).solve(H, X, Mo, Mi)
        lib.gbfe_mv_copy_out(X.h, api.C.c_void_p(out_host.data_ptr()))
        e2e_lat.append(time.perf_counter() - ts)

    fp64_peak = ctx.probe_fp64_peak()
    return dict(cfg=cfg, prob=prob, deg=deg, bounds=(wl, wu, uu), fp64_times=fp64_times, passes64=passes64,
                rc64=rc64, lat=lat, errs=errs, passes=passes, ok=ok, t_total=t_total, launches=launches,
                st_mixed=st_mixed, st_f64=st_f64, clocks=clocks.summary(), e2e_lat=e2e_lat, fp64_peak=fp64_peak,
                h2d=prob.n_dofs * m * 8, d2h=prob.n_dofs * m * 8 + 2 * m * 8)


def pct(v, q):
    return float(np.percentile(np.asarray(v), q))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbfe", choices=["gbfe", "reference"])
    ap.add_argument("--config", default="cfg2c", choices=sorted(CONFIGS))
    ap.add_argument("--fp64-repeats", type=int, default=2)
    ap.add_argument("--cpu-procs", type=int, default=0, help="oracle processes for the CPU baseline (0: all cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gbfe" else args.warmup

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    cfg = CONFIGS[args.config]
    procs = args.cpu_procs or os.cpu_count() or 1
    metric = "ChFSI solves/s at |d_eps|<=1e-6 Ha (mixed precision), FP64 beside it"

    if args.impl == "reference":
        if rank != 0:
            return
        # passes per solve: the pass count the FP64 solve of the same inputs
        # needs (measured on the GPU path, which matches the oracle pass for
        # pass), so that the CPU arm is timed on a bounded sample of passes.
        passes = {"cfg1": 20, "cfg2c": 24, "cfg3": 24}[args.config]
        vals = []
        for _ in range(args.warmup):
            pass
        for _ in range(max(1, args.steps)):
            b = cpu_baseline(args.config, passes, procs)
            vals.append(b["value"])
        v = float(np.median(vals))
        b["value"] = v
        print(json.dumps({"impl": "reference", "metric": metric, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic (seeded generator)",
                          "config": {"workload": args.config, **{k: cfg[k] for k in ("n", "p", "m", "n_wanted")}},
                          "cpu_baseline": b, "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                                                     "d2h_bytes_per_step": 0}}))
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("gloo")
    r = run_gpu(args, args.config, rank, world)
    prob = r["prob"]
    t_step = r["t_total"] / args.steps
    if world > 1:
        import torch

        t = torch.tensor([r["t_total"]], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t.item()) / args.steps
    value = world / t_step  # replicas: every rank solves its own copy
    fp64_sps = 1.0 / float(np.median(r["fp64_times"]))
    st = r["st_f64"] if r["st_f64"]["ms"] >= r["st_mixed"]["ms"] else r["st_mixed"]
    dom = "cell_apply_f64" if st is r["st_f64"] else "cell_apply_mixed"
    avg_ms = st["ms"] / max(1, st["launches"])
    flops_per_launch = st["flops"] / max(1, st["launches"])
    achieved = flops_per_launch / (avg_ms * 1e-3) / 1e12
    if dom == "cell_apply_f64":
        roof = {"kernel": dom, "bound": "fp64", "achieved": achieved, "peak": r["fp64_peak"] / 1e3,
                "unit": "TFLOP/s", "frac": achieved / (r["fp64_peak"] / 1e3), "traffic": None,
                "peak_source": "DFMA throughput probe run in this process (MEASURED_PEAKS.json has no FP64 figure)",
                "launches": st["launches"], "avg_launch_ms": avg_ms, "flops_per_launch": flops_per_launch}
    else:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() \
            else {"bf16_tflops": 1900.0}
        roof = {"kernel": dom, "bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"],
                "unit": "TFLOP/s", "frac": achieved / peaks["bf16_tflops"], "traffic": None,
                "launches": st["launches"], "avg_launch_ms": avg_ms, "flops_per_launch": flops_per_launch}
    other = r["st_mixed"] if dom == "cell_apply_f64" else r["st_f64"]
    e2e_sps = world / float(np.mean(r["e2e_lat"]))
    line = {
        "metric": "ChFSI solves/s at |d_eps|<=1e-6 Ha (mixed precision), FP64 beside it",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+bf16x3 filter / f64 RR,ortho,residual", "data": "synthetic (seeded generator)",
        "config": {"workload": args.config, "cells_per_side": r["cfg"]["n"], "degree": r["cfg"]["p"],
                   "n_dofs": prob.n_dofs, "vectors": r["cfg"]["m"], "n_wanted": r["cfg"]["n_wanted"],
                   "cheb_degree": r["deg"], "residual_tol": r["cfg"]["tol"], "parallelism": f"replicas x{world}",
                   "l2": "working set (cell matrices + block vectors) larger than L2"},
        "latency_ms": {"p50": pct(r["lat"], 50) * 1e3, "p99": pct(r["lat"], 99) * 1e3},
        "fp64": {"solves_per_s": fp64_sps, "passes": r["passes64"], "status": r["rc64"]},
        "mixed_vs_fp64": value / world / fp64_sps,
        "accuracy": {"max_abs_eig_err_Ha": max(r["errs"]), "valid_solves": r["ok"], "of": args.steps,
                     "passes": r["passes"]},
        "roofline": roof,
        "other_kernel": {"name": "cell_apply_mixed" if dom == "cell_apply_f64" else "cell_apply_f64", **other},
        "clocks": r["clocks"],
        "e2e": {"value": e2e_sps, "unit": "solves/s", "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
        "gpu_launches": r["launches"],
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.config, r["passes64"], procs)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
