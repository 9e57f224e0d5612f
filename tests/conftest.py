"""Test configuration: the `gpu` marker, import paths and shared fixtures."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "dft-efe_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbfe.so")


def gpu_available() -> bool:
    try:
        import torch  # noqa: F401  (only used to ask whether a GPU is visible)

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx():
    if not gpu_available():
        pytest.skip("no GPU visible")
    from gbfe.build import build

    build()
    from gbfe import api

    ctx = api.LinAlgOpContext(0)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def small_problem():
    import gbfe.mesh as M

    return M.ks_box(3, 3, 8.0, 2, 4.0, 0.5, seed=11)


def rel_maxnorm(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
