"""Host-side mirror of the reference operator / solver interface on top of the
C ABI.  Class and method names follow dft-efe so that calling code reads like
the reference's own:

=============================================  ==========================================================
this module                                    reference
=============================================  ==========================================================
``LinAlgOpContext``                            ``linearAlgebra/LinAlgOpContext.h:148-176``
``FEBasisManager``                             ``basis/FEBasisManager.h`` (cell->dof map + constraints)
``MultiVector``                                ``linearAlgebra/MultiVector.h:133`` ([N][m], vector fastest)
``KohnShamOperatorContextFE.apply``            ``ksdft/KohnShamOperatorContextFE.t.cpp:1326-1443``
``CFEOverlapOperatorContext.apply``            ``basis/CFEOverlapOperatorContext.t.cpp:539-641``
``CFEOverlapInverseOpContextGLL.apply``        ``basis/CFEOverlapInverseOpContextGLL.t.cpp:499-560``
``LaplaceOperatorContextFE.apply``             ``electrostatics/LaplaceOperatorContextFE.t.cpp:397-467``
``PreconditionerJacobi.apply``                 ``linearAlgebra/PreconditionerJacobi.t.cpp:56-80``
``ResidualChebyshevFilterGEP``                 ``linearAlgebra/ChebyshevFilter.t.cpp:242-444``
``ChebyshevFilter``                            ``linearAlgebra/ChebyshevFilter.t.cpp:39-135``
``OrthonormalizationFunctions``                ``linearAlgebra/OrthonormalizationFunctions.t.cpp:153-431``
``RayleighRitzEigenSolver``                    ``linearAlgebra/RayleighRitzEigenSolver.t.cpp:67-302``
``ChebyshevFilteredEigenSolver``               ``linearAlgebra/ChebyshevFilteredEigenSolver.t.cpp:194-437``
``KohnShamEigenSolver``                        ``ksdft/KohnShamEigenSolver.t.cpp:214-684``
``CGLinearSolver``                             ``linearAlgebra/CGLinearSolver.t.cpp:68-313``
=============================================  ==========================================================

Every compute call goes to libgbfe.so on the GPU; nothing here computes on the
CPU.
"""
from __future__ import annotations

import ctypes as C
import weakref
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import (GBFE_F32, GBFE_F64, GBFE_PREC_FP64, GBFE_PREC_FP64_TENSOR, GBFE_PREC_MIXED, GBFEError, KSParams,
                   check)


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class LinAlgOpContext:
    """One CUDA device, one stream, cuBLAS/cuSOLVER handles."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.gbfe_ctx_create(device, C.byref(h))
        if rc != 0:
            raise GBFEError(rc, f"gbfe_ctx_create(device={device}) failed")
        self.h = h
        self._dependents = weakref.WeakSet()  # vectors / operators to free before the context

    def _track(self, obj) -> None:
        self._dependents.add(obj)

    def synchronize(self) -> None:
        check(self.lib.gbfe_ctx_synchronize(self.h), self.h, "synchronize")

    def kernel_launches(self) -> int:
        n = C.c_uint64()
        check(self.lib.gbfe_ctx_kernel_launches(self.h, C.byref(n)), self.h, "launch count")
        return int(n.value)

    def check_status(self) -> None:
        check(self.lib.gbfe_ctx_check_status(self.h), self.h, "device status")

    def set_tensor_cores(self, mode: int) -> None:
        """2: persistent tcgen05 kernel (default), 3: the same with scalar gathers,
        1: one-CTA-per-cell tcgen05, 0: FP32 SIMT."""
        check(self.lib.gbfe_ctx_set_tensor_cores(self.h, int(mode)), self.h, "set_tensor_cores")

    def set_split_groups(self, on: bool) -> None:
        """Size groups of a split-BF16 cell product on two streams (default) or one."""
        check(self.lib.gbfe_ctx_set_split_groups(self.h, 1 if on else 0), self.h, "set_split_groups")

    def set_graphs(self, on: bool) -> None:
        check(self.lib.gbfe_ctx_set_graphs(self.h, 1 if on else 0), self.h, "set_graphs")

    def set_fused_filter(self, on: bool) -> None:
        """Mixed filter steps as two fused launches (default) or as separate applies."""
        check(self.lib.gbfe_ctx_set_fused_filter(self.h, 1 if on else 0), self.h, "set_fused_filter")

    def set_profile_filter(self, names: Sequence[str] = ()) -> None:
        """Profile only these scopes (empty: all)."""
        check(self.lib.gbfe_ctx_set_profile_filter(self.h, ",".join(names).encode() if names else None), self.h,
              "set_profile_filter")

    def set_small_eig(self, on_host: bool) -> None:
        """Rayleigh-Ritz m x m eigenproblems on the host (m <= 128, default) or in cuSOLVER."""
        check(self.lib.gbfe_ctx_set_small_eig(self.h, 1 if on_host else 0), self.h, "set_small_eig")

    def set_fp64_apply(self, mode: int) -> None:
        """0: FP64 FMA / DGEMM; 1: sliced tensor-core products for cell applies, Gram matrices and
        rotations; 2: sliced cell products only."""
        check(self.lib.gbfe_ctx_set_fp64_apply(self.h, int(mode)), self.h, "set_fp64_apply")

    def set_profiling(self, on: bool) -> None:
        check(self.lib.gbfe_ctx_set_profiling(self.h, 1 if on else 0), self.h, "set_profiling")

    def kernel_stats(self, name: str) -> dict:
        n, ms, fl, by = C.c_uint64(), C.c_double(), C.c_double(), C.c_double()
        check(self.lib.gbfe_ctx_kernel_stats(self.h, name.encode(), C.byref(n), C.byref(ms), C.byref(fl),
                                             C.byref(by)), self.h, "kernel_stats")
        return {"launches": int(n.value), "ms": ms.value, "flops": fl.value, "bytes": by.value}

    def reset_kernel_stats(self) -> None:
        check(self.lib.gbfe_ctx_reset_kernel_stats(self.h), self.h, "reset_kernel_stats")

    def probe_fp64_peak(self) -> float:
        g = C.c_double()
        check(self.lib.gbfe_probe_fp64_peak(self.h, C.byref(g)), self.h, "probe_fp64_peak")
        return g.value

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self.lib.gbfe_ctx_set_stream(self.h, C.c_void_p(stream_ptr or 0)), self.h, "set_stream")

    def close(self) -> None:
        if getattr(self, "h", None):
            for obj in list(getattr(self, "_dependents", ())):
                try:
                    obj.close()
                except Exception:
                    pass
            self.lib.gbfe_ctx_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class FEBasisManager:
    """Cell->dof map and constraints on the device."""

    def __init__(self, ctx: LinAlgOpContext, nd_per_cell: np.ndarray, cell_dof_ids: np.ndarray, n_dofs: int,
                 constraints=None):
        self.ctx = ctx
        lib = ctx.lib
        self._nd = np.ascontiguousarray(nd_per_cell, dtype=np.uint32)
        self._ids = np.ascontiguousarray(cell_dof_ids, dtype=np.uint32)
        self.n_dofs = int(n_dofs)
        self.n_cells = int(self._nd.size)
        h = C.c_void_p()
        check(lib.gbfe_mesh_upload(ctx.h, self.n_cells, _ptr(self._nd), _ptr(self._ids), self.n_dofs, C.byref(h)),
              ctx.h, "mesh_upload")
        self.h = h
        self.cons_h = None
        if constraints is not None:
            self.set_constraints(constraints)

    @classmethod
    def from_problem(cls, ctx: LinAlgOpContext, prob) -> "FEBasisManager":
        return cls(ctx, prob.nd_per_cell, prob.cell_dof_ids, prob.n_dofs, prob.constraints)

    def set_constraints(self, cons) -> None:
        lib = self.ctx.lib
        arrs = [np.ascontiguousarray(a, dtype=t) for a, t in (
            (cons.row_ids, np.uint32), (cons.row_sizes, np.uint32), (cons.col_ids, np.uint32),
            (cons.row_acc, np.uint32), (cons.col_values, np.float64), (cons.inhomogeneities, np.float64))]
        self._cons_arrays = arrs
        h = C.c_void_p()
        check(lib.gbfe_constraints_upload(self.h, int(arrs[0].size), *[_ptr(a) for a in arrs], C.byref(h)),
              self.ctx.h, "constraints_upload")
        self.cons_h = h

    def distributeParentToChild(self, X: "MultiVector") -> None:
        check(self.ctx.lib.gbfe_constraints_distribute_parent_to_child(self.cons_h, X.h), self.ctx.h, "p2c")

    def distributeChildToParent(self, X: "MultiVector") -> None:
        check(self.ctx.lib.gbfe_constraints_distribute_child_to_parent(self.cons_h, X.h), self.ctx.h, "c2p")


class MultiVector:
    """Device block vector, row-major [n_dofs][m] (vector index fastest)."""

    def __init__(self, basis: FEBasisManager, num_vectors: int, dtype=np.float64, init: Optional[np.ndarray] = None):
        self.basis = basis
        self.ctx = basis.ctx
        self.m = int(num_vectors)
        self.dtype = np.dtype(dtype)
        code = GBFE_F64 if self.dtype == np.float64 else GBFE_F32
        if self.dtype not in (np.float64, np.float32):
            raise ValueError("MultiVector dtype must be float64 or float32")
        h = C.c_void_p()
        check(self.ctx.lib.gbfe_mv_create(basis.h, self.m, code, C.byref(h)), self.ctx.h, "mv_create")
        self.h = h
        self.ctx._track(self)
        if init is not None:
            self.copy_from(init)

    @property
    def shape(self):
        return (self.basis.n_dofs, self.m)

    def copy_from(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self.dtype).reshape(self.shape)
        check(self.ctx.lib.gbfe_mv_copy_in(self.h, _ptr(a)), self.ctx.h, "mv_copy_in")

    def numpy(self) -> np.ndarray:
        out = np.empty(self.shape, dtype=self.dtype)
        check(self.ctx.lib.gbfe_mv_copy_out(self.h, _ptr(out)), self.ctx.h, "mv_copy_out")
        return out

    def copy_to(self, other: "MultiVector") -> None:
        check(self.ctx.lib.gbfe_mv_copy(self.h, other.h), self.ctx.h, "mv_copy")

    def setValue(self, v: float) -> None:
        check(self.ctx.lib.gbfe_mv_set_value(self.h, float(v)), self.ctx.h, "mv_set_value")

    def l2Norms(self) -> np.ndarray:
        out = np.empty(self.m)
        check(self.ctx.lib.gbfe_mv_l2_norms(self.h, _ptr(out)), self.ctx.h, "l2Norms")
        return out

    def dot(self, other: "MultiVector") -> np.ndarray:
        out = np.empty(self.m)
        check(self.ctx.lib.gbfe_mv_dots(self.h, other.h, _ptr(out)), self.ctx.h, "dots")
        return out

    def device_ptr(self) -> int:
        v = C.c_void_p()
        check(self.ctx.lib.gbfe_mv_device_ptr(self.h, C.byref(v)), self.ctx.h, "device_ptr")
        return int(v.value or 0)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.ctx.lib.gbfe_mv_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class OperatorContext:
    """``apply(X, Y, updateGhostX=False, updateGhostY=False)``; ghosts are no-ops on one GPU."""

    h = None
    ctx: LinAlgOpContext

    def apply(self, X: MultiVector, Y: MultiVector, updateGhostX: bool = False, updateGhostY: bool = False) -> None:
        check(self.ctx.lib.gbfe_apply(self.h, X.h, Y.h), self.ctx.h, "apply")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.ctx.lib.gbfe_op_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class CellMatrixOperatorContext(OperatorContext):
    def __init__(self, basis: FEBasisManager, cell_matrices: np.ndarray, mixed: bool = False,
                 use_constraints: bool = True, fp64_tensor: bool = False,
                 nonlocal_part: Optional["AtomCenterNonLocalOpContextFE"] = None):
        self.basis, self.ctx = basis, basis.ctx
        mats = np.ascontiguousarray(cell_matrices, dtype=np.float64)
        h = C.c_void_p()
        flags = GBFE_PREC_FP64 | (GBFE_PREC_MIXED if mixed else 0) | (GBFE_PREC_FP64_TENSOR if fp64_tensor else 0)
        cons = basis.cons_h if use_constraints else None
        check(self.ctx.lib.gbfe_cellmat_upload(basis.h, cons, _ptr(mats), flags, C.byref(h)), self.ctx.h,
              "cellmat_upload")
        self.h = h
        self.ctx._track(self)
        self.mixed = mixed
        self.nonlocal_part = None
        if nonlocal_part is not None:
            self.attach_nonlocal(nonlocal_part)

    def attach_nonlocal(self, nl: Optional["AtomCenterNonLocalOpContextFE"]) -> None:
        """Fuse C^T V C into this operator's apply (None detaches)."""
        check(self.ctx.lib.gbfe_op_attach_nonlocal(self.h, nl.h if nl is not None else None), self.ctx.h,
              "attach_nonlocal")
        self.nonlocal_part = nl  # keeps the projector data alive while attached


class AtomCenterNonLocalOpContextFE(OperatorContext):
    """Separable nonlocal pseudopotential part, Y = sum_atoms C^T V C X
    (basis/AtomCenterNonLocalOpContextFE.h); `data` carries the per-cell
    projector blocks (gbfe.nonlocal_psp.NonLocalData)."""

    def __init__(self, basis: FEBasisManager, data, use_constraints: bool = True):
        self.basis, self.ctx = basis, basis.ctx
        self._keep = [np.ascontiguousarray(data.proj_per_cell, dtype=np.uint32),
                      np.ascontiguousarray(data.proj_ids, dtype=np.uint32),
                      np.ascontiguousarray(data.cell_c, dtype=np.float64),
                      np.ascontiguousarray(data.coupling, dtype=np.float64)]
        ppc, pid, cc, v = self._keep
        h = C.c_void_p()
        check(self.ctx.lib.gbfe_nonlocal_upload(basis.h, int(data.n_proj), _ptr(ppc), _ptr(pid), _ptr(cc), _ptr(v),
                                                C.byref(h)), self.ctx.h, "nonlocal_upload")
        self.h = h
        self.ctx._track(self)
        self._keep = None
        self.cons_h = basis.cons_h if use_constraints else None

    def apply(self, X: MultiVector, Y: MultiVector, updateGhostX: bool = False, updateGhostY: bool = False) -> None:
        check(self.ctx.lib.gbfe_nonlocal_apply(self.h, self.cons_h, X.h, Y.h), self.ctx.h, "nonlocal_apply")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.ctx.lib.gbfe_nonlocal_destroy(self.h)
            self.h = None


def gram(X: "MultiVector", Y: "MultiVector") -> np.ndarray:
    """S = X^T Y (mx x my) on the device (DGEMM, or the sliced FP64 product in FP64 mode 1)."""
    S = np.empty((Y.m, X.m))  # column-major mx x my == row-major my x mx
    check(X.ctx.lib.gbfe_mv_gram(X.h, Y.h, _ptr(S)), X.ctx.h, "gram")
    return S.T.copy()


def rotate(X: "MultiVector", T: np.ndarray, Y: "MultiVector") -> None:
    """Y = X T on the device, T of shape (X.m, Y.m)."""
    Tc = np.asfortranarray(np.asarray(T, dtype=np.float64))
    check(X.ctx.lib.gbfe_mv_rotate(X.h, C.c_void_p(Tc.ctypes.data), Y.h), X.ctx.h, "rotate")


def autotune(op: "OperatorContext", m: int) -> list:
    """Tune the tensor-core kernel's launch shape for `op` with m vectors."""
    buf = C.create_string_buffer(4096)
    check(op.ctx.lib.gbfe_autotune(op.h, int(m), buf, 4096), op.ctx.h, "autotune")
    return [ln for ln in buf.value.decode().splitlines() if ln.strip()]


def assemble_local(op: "OperatorContext", basis_values: np.ndarray, weights: np.ndarray,
                   fixed_mats: Optional[np.ndarray] = None, alpha: float = 1.0) -> None:
    """A_c = alpha F_c + B^T diag(w_c) B on the device (KohnShamOperatorContextFE::reinit)."""
    B = np.ascontiguousarray(basis_values, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    F = None if fixed_mats is None else np.ascontiguousarray(fixed_mats, dtype=np.float64)
    check(op.ctx.lib.gbfe_op_assemble_local(op.h, B.shape[0], _ptr(B), _ptr(w), _ptr(F) if F is not None else None,
                                            float(alpha)), op.ctx.h, "assemble_local")


def assemble_cells(op: "OperatorContext", nq_per_cell, basis_values: np.ndarray, weights: np.ndarray,
                   fixed_mats: Optional[np.ndarray] = None, alpha: float = 1.0) -> None:
    """A_c = alpha F_c + B_c^T diag(w_c) B_c for cells of any size and rule: B_c nq_c x nd_c row-major and
    w_c (nq_c) per cell, cells concatenated."""
    nq = np.ascontiguousarray(nq_per_cell, dtype=np.uint32)
    B = np.ascontiguousarray(basis_values, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64)
    F = None if fixed_mats is None else np.ascontiguousarray(fixed_mats, dtype=np.float64)
    check(op.ctx.lib.gbfe_op_assemble_cells(op.h, _ptr(nq), _ptr(B), _ptr(w), _ptr(F) if F is not None else None,
                                            float(alpha)), op.ctx.h, "assemble_cells")


def density_cells(Psi: "MultiVector", occupation, nq_per_cell, basis_values: np.ndarray) -> np.ndarray:
    """rho at each cell's quadrature points (cells concatenated) for cells of any size and rule."""
    nq = np.ascontiguousarray(nq_per_cell, dtype=np.uint32)
    B = np.ascontiguousarray(basis_values, dtype=np.float64)
    f = np.ascontiguousarray(occupation, dtype=np.float64)
    out = np.empty(int(nq.astype(np.int64).sum()))
    check(Psi.ctx.lib.gbfe_density_cells(Psi.h, _ptr(f), _ptr(nq), _ptr(B), _ptr(out)), Psi.ctx.h, "density_cells")
    return out


def density_op(basis_op: "OperatorContext", Psi: "MultiVector", occupation) -> np.ndarray:
    """rho at nd_c points per cell with the interpolation run as the cell product of `basis_op` (a
    CellMatrixOperatorContext built from each cell's basis values, use_constraints=False)."""
    f = np.ascontiguousarray(occupation, dtype=np.float64)
    out = np.empty(int(np.asarray(Psi.basis._nd, dtype=np.int64).sum()))
    check(Psi.ctx.lib.gbfe_density_op(basis_op.h, Psi.h, _ptr(f), _ptr(out)), Psi.ctx.h, "density_op")
    return out


def density(Psi: "MultiVector", occupation, basis_values: np.ndarray) -> np.ndarray:
    """rho[c][q] = sum_i 2 f_i psi_i(x_cq)^2 (DensityCalculator::computeRho)."""
    B = np.ascontiguousarray(basis_values, dtype=np.float64)
    f = np.ascontiguousarray(occupation, dtype=np.float64)
    out = np.empty((Psi.basis.n_cells, B.shape[0]))
    check(Psi.ctx.lib.gbfe_density(Psi.h, _ptr(f), B.shape[0], _ptr(B), _ptr(out)), Psi.ctx.h, "density")
    return out


class IndexedCellMatrixOperatorContext(OperatorContext):
    """Cell operator whose cells name one of a few stored matrices."""

    def __init__(self, basis: FEBasisManager, mats: np.ndarray, cell_to_mat: np.ndarray, mixed: bool = False,
                 use_constraints: bool = True):
        self.basis, self.ctx = basis, basis.ctx
        mats = np.ascontiguousarray(mats, dtype=np.float64)
        idx = np.ascontiguousarray(cell_to_mat, dtype=np.uint32)
        n_mats = int(idx.max()) + 1 if idx.size else 0
        h = C.c_void_p()
        flags = GBFE_PREC_FP64 | (GBFE_PREC_MIXED if mixed else 0)
        cons = basis.cons_h if use_constraints else None
        check(self.ctx.lib.gbfe_cellmat_upload_indexed(basis.h, cons, n_mats, _ptr(mats), _ptr(idx), flags,
                                                       C.byref(h)), self.ctx.h, "cellmat_upload_indexed")
        self.h = h
        self.ctx._track(self)


class KohnShamOperatorContextFE(CellMatrixOperatorContext):
    """H = sum over cells of the Hamiltonian cell matrices (local part)."""


class CFEOverlapOperatorContext(CellMatrixOperatorContext):
    """Consistent (Gauss) overlap M."""


class LaplaceOperatorContextFE(CellMatrixOperatorContext):
    """K = int grad N_i . grad N_j."""


class CFEOverlapInverseOpContextGLL(OperatorContext):
    """Y = M_GLL^{-1} X with constraints; takes the assembled GLL-lumped diagonal."""

    def __init__(self, basis: FEBasisManager, m_gll_diagonal: np.ndarray):
        self.basis, self.ctx = basis, basis.ctx
        inv = np.ascontiguousarray(1.0 / np.asarray(m_gll_diagonal, dtype=np.float64))
        h = C.c_void_p()
        check(self.ctx.lib.gbfe_diag_upload(basis.h, basis.cons_h, _ptr(inv), C.byref(h)), self.ctx.h, "diag_upload")
        self.h = h
        self.ctx._track(self)


class OrthoEFEOverlapInverseOpContextGLL(OperatorContext):
    """GLL diagonal inverse on classical dofs + dense inverse of the enrichment
    overlap block on the enrichment dofs [enr_begin, enr_begin + n)."""

    def __init__(self, basis: FEBasisManager, m_gll_diagonal: np.ndarray, enr_begin: int, enr_block_inv: np.ndarray):
        self.basis, self.ctx = basis, basis.ctx
        inv = np.ascontiguousarray(1.0 / np.asarray(m_gll_diagonal, dtype=np.float64))
        blk = np.ascontiguousarray(np.asarray(enr_block_inv, dtype=np.float64).T)  # column-major
        h = C.c_void_p()
        check(self.ctx.lib.gbfe_diag_block_upload(basis.h, basis.cons_h, _ptr(inv), int(enr_begin), int(blk.shape[0]),
                                                  _ptr(blk), C.byref(h)), self.ctx.h, "diag_block_upload")
        self.h = h
        self.ctx._track(self)


class DiagonalOperatorContext(OperatorContext):
    """Y = d o X with constraints (lumped overlap or any diagonal operator)."""

    def __init__(self, basis: FEBasisManager, diagonal: np.ndarray, use_constraints: bool = True):
        self.basis, self.ctx = basis, basis.ctx
        d = np.ascontiguousarray(diagonal, dtype=np.float64)
        h = C.c_void_p()
        check(self.ctx.lib.gbfe_diag_upload(basis.h, basis.cons_h if use_constraints else None, _ptr(d), C.byref(h)),
              self.ctx.h, "diag_upload")
        self.h = h
        self.ctx._track(self)


class PreconditionerJacobi(OperatorContext):
    """Y = diag^{-1} o X (no constraints), reciprocal taken from ``diagonal``."""

    def __init__(self, basis: FEBasisManager, diagonal: np.ndarray):
        self.basis, self.ctx = basis, basis.ctx
        d = np.ascontiguousarray(diagonal, dtype=np.float64)
        h = C.c_void_p()
        check(self.ctx.lib.gbfe_jacobi_upload(basis.h, _ptr(d), C.byref(h)), self.ctx.h, "jacobi_upload")
        self.h = h
        self.ctx._track(self)


def ResidualChebyshevFilterGEP(A, B, BInv, eigenvalues: Sequence[float], X: MultiVector, polynomialDegree: int,
                               wantedSpectrumLowerBound: float, wantedSpectrumUpperBound: float,
                               unWantedSpectrumUpperBound: float, Y: MultiVector, mixed: bool = False) -> None:
    ev = np.ascontiguousarray(eigenvalues, dtype=np.float64)
    check(A.ctx.lib.gbfe_residual_chebyshev_filter(A.h, B.h, BInv.h, _ptr(ev), X.h, int(polynomialDegree),
                                                   float(wantedSpectrumLowerBound), float(wantedSpectrumUpperBound),
                                                   float(unWantedSpectrumUpperBound),
                                                   GBFE_F32 if mixed else GBFE_F64, Y.h), A.ctx.h, "residual filter")


def ChebyshevFilter(A, BInv, eigenSubspaceGuess: MultiVector, polynomialDegree: int, wantedSpectrumLowerBound: float,
                    wantedSpectrumUpperBound: float, unWantedSpectrumUpperBound: float,
                    filteredSubspace: MultiVector) -> None:
    check(A.ctx.lib.gbfe_chebyshev_filter(A.h, BInv.h, eigenSubspaceGuess.h, int(polynomialDegree),
                                          float(wantedSpectrumLowerBound), float(wantedSpectrumUpperBound),
                                          float(unWantedSpectrumUpperBound), filteredSubspace.h), A.ctx.h, "filter")


class OrthonormalizationFunctions:
    @staticmethod
    def CholeskyGramSchmidt(X: MultiVector, orthogonalizedX: MultiVector, B) -> None:
        check(B.ctx.lib.gbfe_cholesky_gram_schmidt(B.h, X.h, orthogonalizedX.h), B.ctx.h, "CholeskyGramSchmidt")


class RayleighRitzEigenSolver:
    @staticmethod
    def solve(A, X: MultiVector, eigenVectors: MultiVector) -> np.ndarray:
        ev = np.empty(X.m)
        check(A.ctx.lib.gbfe_rayleigh_ritz(A.h, X.h, _ptr(ev), eigenVectors.h), A.ctx.h, "RayleighRitz")
        return ev


def eigen_residual_norms(A, B, X: MultiVector, eigenvalues) -> np.ndarray:
    ev = np.ascontiguousarray(eigenvalues, dtype=np.float64)
    out = np.empty(X.m)
    check(A.ctx.lib.gbfe_eigen_residual_norms(A.h, B.h, X.h, _ptr(ev), _ptr(out)), A.ctx.h, "residual norms")
    return out


class ChebyshevFilteredEigenSolver:
    def __init__(self, wantedSpectrumLowerBound: float, wantedSpectrumUpperBound: float,
                 unWantedSpectrumUpperBound: float, polynomialDegree: int, mixed: bool = False):
        self.wl, self.wu, self.uu = wantedSpectrumLowerBound, wantedSpectrumUpperBound, unWantedSpectrumUpperBound
        self.degree, self.mixed = int(polynomialDegree), mixed

    def solve(self, A, eigenValues: np.ndarray, eigenVectors: MultiVector, B, BInv) -> np.ndarray:
        ev = np.ascontiguousarray(eigenValues, dtype=np.float64).copy()
        check(A.ctx.lib.gbfe_chfsi_pass(A.h, B.h, BInv.h, eigenVectors.h, _ptr(ev), self.degree, self.wl, self.wu,
                                        self.uu, GBFE_F32 if self.mixed else GBFE_F64), A.ctx.h, "chfsi pass")
        return ev


def lanczos_bounds(A, B, BInv, steps: int = 20, seed: int = 7, start=None) -> np.ndarray:
    """[smallest, largest Ritz value, last beta] of B^-1 A after `steps` Lanczos steps, from `start` (a one-column
    MultiVector or a host array of n_dofs values) or a seeded uniform start vector."""
    out = np.empty(3)
    if start is None:
        check(A.ctx.lib.gbfe_lanczos_bounds(A.h, B.h, BInv.h, int(steps), int(seed), _ptr(out)), A.ctx.h, "lanczos")
        return out
    if isinstance(start, MultiVector):
        ptr = C.c_void_p(start.device_ptr())
    else:
        start = np.ascontiguousarray(start, dtype=np.float64).ravel()
        ptr = _ptr(start)
    check(A.ctx.lib.gbfe_lanczos_bounds_from(A.h, B.h, BInv.h, int(steps), ptr, _ptr(out)), A.ctx.h, "lanczos")
    return out


class KohnShamEigenSolver:
    def __init__(self, n_wanted: int, degree: int, max_passes: int, residual_tol: float = 1e-6, mixed: bool = False,
                 bounds: Optional[Sequence[float]] = None, lanczos_steps: int = 20, lanczos_seed: int = 7,
                 fixed_passes: bool = False, faithful_passes: bool = False, fp64_tensor: bool = False,
                 lanczos_start=None):
        """lanczos_start (with bounds=None): the Lanczos start vector, a MultiVector with one column (device
        resident) or a host array of n_dofs values; None draws a seeded uniform vector (lanczos_seed)."""
        self.p = KSParams()
        self.p.degree, self.p.max_passes, self.p.n_wanted = int(degree), int(max_passes), int(n_wanted)
        self.p.filter_precision = GBFE_F32 if mixed else GBFE_F64
        self.p.residual_tol = float(residual_tol)
        if bounds is not None:
            self.p.use_lanczos = 0
            self.p.wanted_lower, self.p.wanted_upper, self.p.unwanted_upper = map(float, bounds)
        else:
            self.p.use_lanczos = 1
        self.p.lanczos_steps, self.p.lanczos_seed = int(lanczos_steps), int(lanczos_seed)
        self.p.fixed_passes = 1 if fixed_passes else 0
        self.p.faithful_passes = 1 if faithful_passes else 0
        self.p.fp64_apply = int(fp64_tensor)  # True / 1: sliced products everywhere; 2: cell products only
        self._start = None
        if lanczos_start is not None:
            if isinstance(lanczos_start, MultiVector):
                if lanczos_start.m != 1 or lanczos_start.dtype != np.float64:
                    raise ValueError("lanczos_start must be one FP64 column")
                self._start = lanczos_start
                self.p.lanczos_start = lanczos_start.device_ptr()
            else:
                self._start = np.ascontiguousarray(lanczos_start, dtype=np.float64).ravel()
                self.p.lanczos_start = self._start.ctypes.data

    def solve(self, H, X: MultiVector, M, MInv, eigenvalues: Optional[np.ndarray] = None):
        ev = np.zeros(X.m) if eigenvalues is None else np.ascontiguousarray(eigenvalues, dtype=np.float64).copy()
        res = np.empty(X.m)
        passes = C.c_uint32()
        rc = H.ctx.lib.gbfe_ks_eigen_solve(H.h, M.h, MInv.h, X.h, C.byref(self.p), _ptr(ev), _ptr(res),
                                           C.byref(passes))
        return rc, ev, res, int(passes.value)


class CGLinearSolver:
    def __init__(self, maxIter: int, absoluteTol: float, relativeTol: float, divergenceTol: float):
        self.maxIter, self.absTol, self.relTol, self.divTol = int(maxIter), absoluteTol, relativeTol, divergenceTol

    def solve(self, A, PC, b: MultiVector, x: MultiVector):
        iters = C.c_uint32()
        rn = np.empty(b.m)
        rc = A.ctx.lib.gbfe_cg_solve(A.h, PC.h, b.h, x.h, self.maxIter, float(self.absTol), float(self.relTol),
                                     float(self.divTol), C.byref(iters), _ptr(rn))
        return rc, int(iters.value), rn


def pcg_solve_batched(A, PC, b: MultiVector, x: MultiVector, inst_dof_off: np.ndarray, maxIter: int,
                      absoluteTol: float, relativeTol: float, divergenceTol: float, iters_chunk: int = 16):
    """Batched CGLinearSolver over block-diagonal independent instances.
    Returns (iterations, status, residual norms) per instance."""
    off = np.ascontiguousarray(inst_dof_off, dtype=np.uint64)
    n = off.size - 1
    iters = np.zeros(n, np.uint32)
    status = np.zeros(n, np.int32)
    rn = np.zeros(n)
    check(A.ctx.lib.gbfe_pcg_solve_batched(A.h, PC.h, b.h, x.h, n, _ptr(off), int(maxIter), float(absoluteTol),
                                           float(relativeTol), float(divergenceTol), int(iters_chunk), _ptr(iters),
                                           _ptr(status), _ptr(rn)), A.ctx.h, "pcg_solve_batched")
    return iters, status, rn
