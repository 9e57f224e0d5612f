"""The FP64 apply that allocates nothing (gbfe_apply_f64_noalloc).

It serves callers that cannot call cudaMalloc while applying an operator:
a process whose device memory is owned by another component's pool, or a
latency-critical loop that must not pay the device-wide synchronisation a
cudaMalloc can trigger.  Its cell-wise intermediate lives in a fixed
64 MiB library array instead of a buffer grown per operator.

This file is collected last.  The tests call the entry point through the C ABI
twice in a row on caller-owned device buffers and check both results against
gbfe_apply (relative max-norm <= 1e-12, the FP64 apply tolerance): once on a
mesh with homogeneous Dirichlet rows only, once on the reference-built
hanging-node fixture (constraint rows with parents and inhomogeneities, an odd
number of vectors), where the result is also checked against the reference's
own output.  An oversize request must be rejected.  The file must pass alone
in a fresh process and after the rest of the suite.
"""
from pathlib import Path

import ctypes as C

import numpy as np
import pytest

import gbfe.mesh as M
from conftest import rel_maxnorm

pytestmark = pytest.mark.gpu


def test_noalloc_apply_matches_apply_twice(gpu_ctx):
    from gbfe import api

    p = M.ks_box(3, 3, 8.0, 2, 4.0, 0.5, seed=77)
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H)
    lib = gpu_ctx.lib
    for call, m in enumerate((12, 12)):
        X0 = M.random_block(p.n_dofs, m, 900 + call)
        # reference result through the allocating entry point
        Xa = api.MultiVector(basis, m, init=X0)
        Ya = api.MultiVector(basis, m)
        H.apply(Xa, Ya)
        # caller-owned device buffers (allocated here, during set-up)
        Xd = api.MultiVector(basis, m, init=X0)
        Yd = api.MultiVector(basis, m)
        Yd.setValue(np.nan)  # the entry point must overwrite every output element
        rc = lib.gbfe_apply_f64_noalloc(H.h, C.c_void_p(Xd.device_ptr()), C.c_void_p(Yd.device_ptr()), m)
        assert rc == 0, rc
        gpu_ctx.synchronize()
        assert rel_maxnorm(Yd.numpy(), Ya.numpy()) <= 1e-12
        assert rel_maxnorm(Xd.numpy(), Xa.numpy()) == 0.0


def test_noalloc_apply_hanging_constraints_twice(gpu_ctx):
    """Parent-to-child distribution and the parent-weighted assembly (the
    constraint branch Dirichlet-only meshes never reach), with m = 3 and m = 5
    (odd widths: the scalar paths of the kernels)."""
    from gbfe import api

    z = np.load(Path(__file__).resolve().parent / "golden" / "case_hanging_p2.npz")
    cons = M.Constraints(z["cons_rows"], z["cons_sizes"], z["cons_cols"], z["cons_acc"], z["cons_vals"],
                         z["cons_inh"])
    assert cons.row_sizes.max() > 0 and np.abs(cons.inhomogeneities).max() > 0
    basis = api.FEBasisManager(gpu_ctx, z["nd"], z["ids"], int(z["n_dofs"]), cons)
    H = api.KohnShamOperatorContextFE(basis, z["H"])
    lib = gpu_ctx.lib
    for call, X0 in enumerate((z["X"], M.random_block(int(z["n_dofs"]), 5, 901))):
        m = X0.shape[1]
        Xa = api.MultiVector(basis, m, init=X0)
        Ya = api.MultiVector(basis, m)
        H.apply(Xa, Ya)
        Xd = api.MultiVector(basis, m, init=X0)
        Yd = api.MultiVector(basis, m)
        Yd.setValue(np.nan)
        rc = lib.gbfe_apply_f64_noalloc(H.h, C.c_void_p(Xd.device_ptr()), C.c_void_p(Yd.device_ptr()), m)
        assert rc == 0, rc
        gpu_ctx.synchronize()
        assert rel_maxnorm(Yd.numpy(), Ya.numpy()) <= 1e-12
        assert rel_maxnorm(Xd.numpy(), Xa.numpy()) == 0.0
        if call == 0:  # the reference's own output on this fixture
            assert rel_maxnorm(Yd.numpy(), z["Y_H"]) <= 1e-12
            assert rel_maxnorm(Xd.numpy(), z["X_after"]) <= 1e-15


def test_noalloc_apply_rejects_oversize(gpu_ctx):
    from gbfe import api

    p = M.ks_box(2, 3, 6.0, 0, 4.0, 0.5, seed=78)
    basis = api.FEBasisManager.from_problem(gpu_ctx, p)
    H = api.KohnShamOperatorContextFE(basis, p.H)
    m = (8 << 20) // (p.n_cells * p.nd) + 1  # one vector past the fixed scratch
    X = api.MultiVector(basis, 1)  # the size check comes before any device access
    rc = gpu_ctx.lib.gbfe_apply_f64_noalloc(H.h, C.c_void_p(X.device_ptr()), C.c_void_p(X.device_ptr() + 8), m)
    assert rc == 1  # GBFE_ERR_ARG, before any device work
