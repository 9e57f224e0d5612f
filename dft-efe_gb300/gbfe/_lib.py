"""ctypes binding of libgbfe.so (the C ABI declared in include/gbfe.h).

There is no fallback: if the CUDA library is missing or cannot be loaded the
import of the compute API fails with a clear error.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgbfe.so"

GBFE_OK = 0
STATUS_NAMES = {
    0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_ALLOC", 4: "ERR_NOT_ORTHONORMALIZABLE",
    5: "ERR_LAPACK", 6: "ERR_NOT_CONVERGED", 7: "ERR_DIVERGED", 8: "ERR_TIMEOUT", 9: "ERR_CANCELLED",
}
GBFE_F64, GBFE_F32 = 0, 1
GBFE_PREC_FP64, GBFE_PREC_MIXED, GBFE_PREC_FP64_TENSOR = 1, 2, 4

p = C.c_void_p
u32, u64, i32, f64 = C.c_uint32, C.c_uint64, C.c_int, C.c_double
pu32, pf64 = C.POINTER(C.c_uint32), C.POINTER(C.c_double)


class KSParams(C.Structure):
    _fields_ = [
        ("degree", u32), ("max_passes", u32), ("n_wanted", u32), ("filter_precision", i32),
        ("residual_tol", f64), ("wanted_lower", f64), ("wanted_upper", f64), ("unwanted_upper", f64),
        ("use_lanczos", i32), ("lanczos_steps", u32), ("lanczos_seed", u64), ("fixed_passes", i32),
        ("fp64_apply", i32), ("faithful_passes", i32), ("lanczos_start", p),
    ]


class MeshDesc(C.Structure):
    _fields_ = [("n_cells", u32), ("nd_per_cell", p), ("cell_dof_ids", p), ("n_dofs", u64), ("n_cons_rows", u32),
                ("row_ids", p), ("row_sizes", p), ("col_ids", p), ("row_acc", p), ("col_values", p),
                ("inhomogeneities", p)]


class RequestInfo(C.Structure):
    _fields_ = [("status", i32), ("t_submit", f64), ("t_admit", f64), ("t_done", f64), ("passes_or_iters", u32),
                ("footprint_bytes", u64), ("message", C.c_char * 256)]


# name -> (restype, argtypes)
SIGNATURES = {
    "gbfe_ctx_create": (i32, [i32, C.POINTER(p)]),
    "gbfe_ctx_destroy": (i32, [p]),
    "gbfe_last_error": (i32, [p, C.c_char_p, C.c_size_t]),
    "gbfe_ctx_set_stream": (i32, [p, p]),
    "gbfe_ctx_synchronize": (i32, [p]),
    "gbfe_ctx_kernel_launches": (i32, [p, C.POINTER(u64)]),
    "gbfe_ctx_check_status": (i32, [p]),
    "gbfe_ctx_check_wait_timeout": (i32, [p, f64]),
    "gbfe_ctx_set_tensor_cores": (i32, [p, i32]),
    "gbfe_ctx_set_split_groups": (i32, [p, i32]),
    "gbfe_ctx_set_sm_budget": (i32, [p, i32]),
    "gbfe_ctx_set_profiling": (i32, [p, i32]),
    "gbfe_ctx_set_fp64_apply": (i32, [p, i32]),
    "gbfe_ctx_set_graphs": (i32, [p, i32]),
    "gbfe_autotune": (i32, [p, u32, C.c_char_p, C.c_size_t]),
    "gbfe_ctx_set_small_eig": (i32, [p, i32]),
    "gbfe_ctx_set_profile_filter": (i32, [p, C.c_char_p]),
    "gbfe_ctx_set_fused_filter": (i32, [p, i32]),
    "gbfe_nonlocal_upload": (i32, [p, u32, p, p, p, p, C.POINTER(p)]),
    "gbfe_mv_gram": (i32, [p, p, p]),
    "gbfe_mv_rotate": (i32, [p, p, p]),
    "gbfe_nonlocal_destroy": (i32, [p]),
    "gbfe_nonlocal_apply": (i32, [p, p, p, p]),
    "gbfe_op_attach_nonlocal": (i32, [p, p]),
    "gbfe_ctx_kernel_stats": (i32, [p, C.c_char_p, C.POINTER(u64), pf64, pf64, pf64]),
    "gbfe_ctx_reset_kernel_stats": (i32, [p]),
    "gbfe_probe_fp64_peak": (i32, [p, pf64]),
    "gbfe_mesh_upload": (i32, [p, u32, p, p, u64, C.POINTER(p)]),
    "gbfe_mesh_destroy": (i32, [p]),
    "gbfe_constraints_upload": (i32, [p, u32, p, p, p, p, p, p, C.POINTER(p)]),
    "gbfe_constraints_destroy": (i32, [p]),
    "gbfe_constraints_distribute_parent_to_child": (i32, [p, p]),
    "gbfe_constraints_distribute_child_to_parent": (i32, [p, p]),
    "gbfe_cellmat_upload": (i32, [p, p, p, i32, C.POINTER(p)]),
    "gbfe_cellmat_upload_indexed": (i32, [p, p, u32, p, p, i32, C.POINTER(p)]),
    "gbfe_diag_upload": (i32, [p, p, p, C.POINTER(p)]),
    "gbfe_diag_block_upload": (i32, [p, p, p, u64, u64, p, C.POINTER(p)]),
    "gbfe_jacobi_upload": (i32, [p, p, C.POINTER(p)]),
    "gbfe_op_destroy": (i32, [p]),
    "gbfe_op_assemble_local": (i32, [p, u32, p, p, p, f64]),
    "gbfe_density": (i32, [p, p, u32, p, p]),
    "gbfe_op_assemble_cells": (i32, [p, p, p, p, p, f64]),
    "gbfe_density_cells": (i32, [p, p, p, p, p]),
    "gbfe_density_op": (i32, [p, p, p, p]),
    "gbfe_mv_create": (i32, [p, u32, i32, C.POINTER(p)]),
    "gbfe_mv_wrap": (i32, [p, u32, i32, p, C.POINTER(p)]),
    "gbfe_mv_destroy": (i32, [p]),
    "gbfe_mv_copy_in": (i32, [p, p]),
    "gbfe_mv_copy_out": (i32, [p, p]),
    "gbfe_mv_copy": (i32, [p, p]),
    "gbfe_mv_set_value": (i32, [p, f64]),
    "gbfe_mv_device_ptr": (i32, [p, C.POINTER(p)]),
    "gbfe_mv_l2_norms": (i32, [p, p]),
    "gbfe_mv_dots": (i32, [p, p, p]),
    "gbfe_apply": (i32, [p, p, p]),
    "gbfe_apply_f64_noalloc": (i32, [p, p, p, u32]),
    "gbfe_residual_chebyshev_filter": (i32, [p, p, p, p, p, u32, f64, f64, f64, i32, p]),
    "gbfe_chebyshev_filter": (i32, [p, p, p, u32, f64, f64, f64, p]),
    "gbfe_cholesky_gram_schmidt": (i32, [p, p, p]),
    "gbfe_rayleigh_ritz": (i32, [p, p, p, p]),
    "gbfe_eigen_residual_norms": (i32, [p, p, p, p, p]),
    "gbfe_chfsi_pass": (i32, [p, p, p, p, p, u32, f64, f64, f64, i32]),
    "gbfe_ks_eigen_solve": (i32, [p, p, p, p, C.POINTER(KSParams), p, p, C.POINTER(u32)]),
    "gbfe_lanczos_bounds": (i32, [p, p, p, u32, u64, p]),
    "gbfe_lanczos_bounds_from": (i32, [p, p, p, u32, p, p]),
    "gbfe_cg_solve": (i32, [p, p, p, p, u32, f64, f64, f64, C.POINTER(u32), p]),
    "gbfe_pcg_solve_batched": (i32, [p, p, p, p, u32, p, u32, f64, f64, f64, u32, p, p, p]),
    "gbfe_server_create": (i32, [i32, u32, u64, C.POINTER(p)]),
    "gbfe_server_destroy": (i32, [p]),
    "gbfe_server_submit_ks": (i32, [p, C.POINTER(MeshDesc), p, p, p, u64, u64, p, p, u32, C.POINTER(KSParams),
                                    C.POINTER(u64)]),
    "gbfe_server_submit_poisson": (i32, [p, C.POINTER(MeshDesc), u32, p, p, p, p, u32, f64, f64, f64,
                                         C.POINTER(u64)]),
    "gbfe_server_cancel": (i32, [p, u64]),
    "gbfe_server_wait": (i32, [p, u64, f64, C.POINTER(RequestInfo)]),
    "gbfe_server_result": (i32, [p, u64, p, p]),
    "gbfe_server_release": (i32, [p, u64]),
    "gbfe_server_stats": (i32, [p, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64), C.POINTER(u64), C.POINTER(u32)]),
    "gbfe_server_inject_alloc_failures": (i32, [p, i32]),
    "gbfe_server_batch_stats": (i32, [p, C.POINTER(u64), C.POINTER(u64)]),
    "gbfe_server_set_max_batch": (i32, [p, u32]),
}

_lib = None


def exported_symbols() -> list[str]:
    return list(SIGNATURES)


def load(path: Path | None = None) -> C.CDLL:
    """Load libgbfe.so and declare every entry point.  Raises if it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    lp = Path(path) if path else LIB_PATH
    if not lp.exists():
        raise ImportError(f"libgbfe.so not built at {lp}; run gbfe.build.build() (no CPU fallback exists)")
    lib = C.CDLL(str(lp))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class GBFEError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code
        self.status = STATUS_NAMES.get(code, str(code))


def check(rc: int, ctx_handle=None, what: str = "") -> None:
    if rc == GBFE_OK:
        return
    msg = what
    if ctx_handle:
        buf = C.create_string_buffer(1024)
        load().gbfe_last_error(ctx_handle, buf, 1024)
        msg = f"{what}: {buf.value.decode(errors='replace')}"
    raise GBFEError(rc, msg)
