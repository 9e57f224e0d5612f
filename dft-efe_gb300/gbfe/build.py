"""Build libgbfe.so (CUDA, sm_103a) in-tree, next to this file.

Each translation unit under ``csrc/`` is compiled by its own ``nvcc`` process
in parallel, then linked once.  Only one ``-gencode`` (compute_103a / sm_103a)
is emitted: the library runs on GB300 and nothing else.  The same recipe runs
in the x86 build container (cross-compilation without a GPU) and on the Arm
GPU host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
LIB = PKG / "libgbfe.so"
OBJDIR = PKG.parent / "_build"

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-v"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OBJDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    srcs = sources()
    objs = [OBJDIR / (s.name.replace(".", "_") + ".o") for s in srcs]
    nv = nvcc()

    def compile_one(pair):
        src, obj = pair
        if not force and not _stale(obj, [src, *headers]):
            return obj, ""
        cmd = [nv, *GENCODE, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose:
        for obj, log in results:
            if log:
                print(f"--- {obj.name}\n{log}", file=sys.stderr)
    if force or _stale(LIB, objs):
        cmd = [nv, *GENCODE, "-shared", "-o", str(LIB), *map(str, objs), "-lcublas", "-lcusolver", "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
