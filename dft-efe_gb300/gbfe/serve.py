"""Continuous-batching request loop for independent KS eigen solves and
Poisson solves (the C ABI gbfe_server_*).

    srv = Server(slots=4, hbm_budget_bytes=64 << 30)
    rid = srv.submit_ks(problem, X0, n_wanted=8, degree=20, max_passes=40)
    info = srv.wait(rid)            # status, t_submit / t_admit / t_done
    eig, res = srv.ks_result(rid, m)

Requests are admitted in arrival order as slots and HBM free up; admitted
requests run concurrently (one stream per slot) with their data resident on the
device until they finish.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import GBFE_F32, GBFE_F64, GBFEError, KSParams, MeshDesc, RequestInfo


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


@dataclass
class Info:
    status: int
    t_submit: float
    t_admit: float
    t_done: float
    passes_or_iters: int
    footprint_bytes: int
    message: str

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class Server:
    def __init__(self, device: int = 0, slots: int = 4, hbm_budget_bytes: int = 64 << 30):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.gbfe_server_create(device, slots, int(hbm_budget_bytes), C.byref(h))
        if rc:
            raise GBFEError(rc, "gbfe_server_create failed")
        self.h = h

    def _mesh(self, nd, ids, n_dofs, cons):
        keep = [np.ascontiguousarray(nd, np.uint32), np.ascontiguousarray(ids, np.uint32),
                np.ascontiguousarray(cons.row_ids, np.uint32), np.ascontiguousarray(cons.row_sizes, np.uint32),
                np.ascontiguousarray(cons.col_ids, np.uint32), np.ascontiguousarray(cons.row_acc, np.uint32),
                np.ascontiguousarray(cons.col_values, np.float64),
                np.ascontiguousarray(cons.inhomogeneities, np.float64)]
        d = MeshDesc(keep[0].size, _ptr(keep[0]), _ptr(keep[1]), int(n_dofs), keep[2].size, *[_ptr(k) for k in keep[2:]])
        return d, keep

    def submit_ks(self, prob, X0, n_wanted, degree, max_passes, residual_tol=1e-6, mixed=True, bounds=None,
                  lanczos_seed=7, fixed_passes=False) -> int:
        desc, keep = self._mesh(prob.nd_per_cell, prob.cell_dof_ids, prob.n_dofs, prob.constraints)
        m = X0.shape[1]
        prm = KSParams()
        prm.degree, prm.max_passes, prm.n_wanted = int(degree), int(max_passes), int(n_wanted)
        prm.filter_precision = GBFE_F32 if mixed else GBFE_F64
        prm.residual_tol = float(residual_tol)
        if bounds is None:
            prm.use_lanczos, prm.lanczos_steps, prm.lanczos_seed = 1, 20, int(lanczos_seed)
        else:
            prm.use_lanczos = 0
            prm.wanted_lower, prm.wanted_upper, prm.unwanted_upper = map(float, bounds)
        prm.fixed_passes = 1 if fixed_passes else 0
        H = np.ascontiguousarray(prob.H, np.float64)
        Mm = np.ascontiguousarray(prob.M, np.float64)
        minv = np.ascontiguousarray(1.0 / prob.m_gll_diag, np.float64)
        blk = prob.extra.get("enr_block_inv")
        blk_c = np.ascontiguousarray(np.asarray(blk).T) if blk is not None else None
        X = np.ascontiguousarray(X0, np.float64)
        rid = C.c_uint64()
        rc = self.lib.gbfe_server_submit_ks(self.h, C.byref(desc), _ptr(H), _ptr(Mm), _ptr(minv),
                                            int(prob.extra.get("enr_begin", 0)), int(blk_c.shape[0]) if blk_c is not None else 0,
                                            _ptr(blk_c), _ptr(X), m, C.byref(prm), C.byref(rid))
        if rc:
            raise GBFEError(rc, "submit_ks")
        return int(rid.value)

    def submit_poisson(self, inst: dict, max_iter=5000, abs_tol=1e-14, rel_tol=1e-10, div_tol=1e10) -> int:
        desc, keep = self._mesh(inst["nd"], inst["ids"], inst["N"], inst["cons"])
        mats = np.ascontiguousarray(inst["mats"], np.float64)
        c2m = np.ascontiguousarray(inst["cell_to_mat"], np.uint32)
        diag = np.ascontiguousarray(inst["diag"], np.float64)
        b = np.ascontiguousarray(inst["b"], np.float64)
        rid = C.c_uint64()
        rc = self.lib.gbfe_server_submit_poisson(self.h, C.byref(desc), int(c2m.max()) + 1, _ptr(mats), _ptr(c2m),
                                                 _ptr(diag), _ptr(b), int(max_iter), float(abs_tol), float(rel_tol),
                                                 float(div_tol), C.byref(rid))
        if rc:
            raise GBFEError(rc, "submit_poisson")
        return int(rid.value)

    def wait(self, rid: int, timeout_s: float = 600.0) -> Info:
        info = RequestInfo()
        rc = self.lib.gbfe_server_wait(self.h, rid, float(timeout_s), C.byref(info))
        if rc:
            raise GBFEError(rc, f"wait({rid})")
        return Info(info.status, info.t_submit, info.t_admit, info.t_done, info.passes_or_iters,
                    info.footprint_bytes, info.message.decode(errors="replace"))

    def ks_result(self, rid: int, m: int):
        eig, res = np.empty(m), np.empty(m)
        rc = self.lib.gbfe_server_result(self.h, rid, _ptr(eig), _ptr(res))
        if rc:
            raise GBFEError(rc, "result")
        return eig, res

    def poisson_result(self, rid: int, n_dofs: int):
        x = np.empty(n_dofs)
        rc = self.lib.gbfe_server_result(self.h, rid, _ptr(x), None)
        if rc:
            raise GBFEError(rc, "result")
        return x

    def cancel(self, rid: int) -> None:
        self.lib.gbfe_server_cancel(self.h, rid)

    def release(self, rid: int) -> None:
        self.lib.gbfe_server_release(self.h, rid)

    def inject_alloc_failures(self, count: int) -> None:
        self.lib.gbfe_server_inject_alloc_failures(self.h, int(count))

    def stats(self) -> dict:
        a, c, r, u = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        q = C.c_uint32()
        self.lib.gbfe_server_stats(self.h, C.byref(a), C.byref(c), C.byref(r), C.byref(u), C.byref(q))
        nb, nr = C.c_uint64(), C.c_uint64()
        self.lib.gbfe_server_batch_stats(self.h, C.byref(nb), C.byref(nr))
        return dict(admitted=a.value, completed=c.value, rejected=r.value, used_bytes=u.value, queued=q.value,
                    poisson_batches=nb.value, poisson_batched_requests=nr.value)

    def set_max_batch(self, n: int) -> None:
        """Largest batch of Poisson requests solved together (1: no batching)."""
        self.lib.gbfe_server_set_max_batch(self.h, int(n))

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gbfe_server_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def poisson_request_from_batch(pb, i: int) -> dict:
    """One instance of a PoissonBatch as a stand-alone request (indexed K)."""
    from . import poisson as P

    v = P.instance_view(pb, i)
    nd0 = int(v["nd"][0])
    return dict(nd=v["nd"], ids=v["ids"], N=v["N"], cons=v["cons"], mats=v["K"][: nd0 * nd0],
                cell_to_mat=np.zeros(v["nd"].size, np.uint32), diag=v["diag"], b=v["b"])
