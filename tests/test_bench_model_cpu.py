"""The arithmetic behind bench.py's line, checked on synthetic inputs: the
roofline entries (algorithmic bytes or flops per launch over the average
launch time, against the measured peaks; 36 BF16 products per FP64 product
for the sliced kernels, 3 for the split-BF16 tensor fraction) and the
operation counts of one FP64 pass that the CPU-baseline model multiplies
out (ChebyshevFilter.t.cpp:242-444, OrthonormalizationFunctions.t.cpp:
356-415, RayleighRitzEigenSolver.t.cpp:233-301, KohnShamEigenSolver.t.cpp:
574-684)."""
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

import bench  # noqa: E402
from oracle import cpu_baseline as CB  # noqa: E402


def test_pass_counts_follow_the_reference_sequence():
    c = CB.pass_counts(30)
    # filter: B and A for the initial residual + 29 A; Cholesky-GS: B; RR: A;
    # residual: A and B -> 35 cell applies; 29 B^-1 in the steps + 1 final
    assert c == {"cell": 35, "diag": 30, "sweep": 93, "gram": 2, "rot": 2, "chol": 1, "eig": 1}
    assert CB.pass_counts(2)["cell"] == 2 + 1 + 1 + 1 + 2


def test_roofline_hbm_kernel():
    peaks, _ = bench._peaks()
    st = {"launches": 2, "ms": 4.0, "flops": 2e12, "bytes": 2e10}
    r = bench.roofline("cell_apply_mixed", st, 1250.0)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["avg_launch_ms"] == pytest.approx(2.0)
    assert r["achieved"] == pytest.approx(1e10 / 2e-3 / 1e9)  # 5000 GB/s
    assert r["frac"] == pytest.approx(r["achieved"] / peaks["hbm_gbs"])
    sustained = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
    assert r["tensor_frac"] == pytest.approx(1e12 / 2e-3 / 1e12 * bench.SPLIT_PRODUCTS / sustained)


def test_roofline_sliced_kernel_counts_every_bf16_product():
    peaks, _ = bench._peaks()
    st = {"launches": 1, "ms": 10.0, "flops": 1e12, "bytes": 1e9}
    r = bench.roofline("gram_f64_oz", st, 1250.0)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert r["fp64_equivalent_tflops"] == pytest.approx(100.0)
    assert r["achieved"] == pytest.approx(100.0 * bench.SLICED_PRODUCTS)
    sustained = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))
    assert r["frac"] == pytest.approx(r["achieved"] / sustained)


def test_roofline_fp64_kernel_uses_the_fp64_peak():
    st = {"launches": 4, "ms": 8.0, "flops": 4e9 * 1e3, "bytes": 0.0}
    r = bench.roofline("cell_apply_f64", st, 1250.0)
    assert r["bound"] == "fp64"
    assert r["achieved"] == pytest.approx(1e12 / 2e-3 / 1e12)  # 500 TFLOP/s of a 1.25 TFLOP/s peak
    assert r["frac"] == pytest.approx(r["achieved"] / 1.25)
