"""Serving loop: continuous admission by HBM footprint, results independent
of the mix, and host-side failure handling (over-budget rejection,
cancellation, injected allocation failure).  No GPU fault is provoked."""
import numpy as np
import pytest

import gbfe.mesh as M
import gbfe.poisson as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload():
    ks = [M.ks_box(n, p, 2.0 * n, 1 + (n % 2), 4.0, 0.5, seed=50 + n) for n, p in ((2, 3), (3, 3), (2, 4), (3, 2))]
    pb = P.batch(count=4, seed=9, n_range=(3, 4), degrees=(2, 3))
    return ks, pb


def _submit_all(srv, ks, pb, mixed=True):
    from gbfe.serve import poisson_request_from_batch

    ids = []
    for j, prob in enumerate(ks):
        X0 = M.random_block(prob.n_dofs, 8, 60 + j)
        ids.append(("ks", srv.submit_ks(prob, X0, 4, 10, 60, 1e-8, mixed=mixed), 8))
        ids.append(("poisson", srv.submit_poisson(poisson_request_from_batch(pb, j)), P.instance_view(pb, j)["N"]))
    return ids


def test_results_same_alone_and_in_the_mix(gpu_ctx, workload):
    from gbfe.serve import Server

    ks, pb = workload
    # alone: one slot, each request submitted after the previous one finished
    # (so no Poisson batch forms)
    from gbfe.serve import poisson_request_from_batch

    srv1 = Server(slots=1, hbm_budget_bytes=8 << 30)
    alone = []
    for j, prob in enumerate(ks):
        X0 = M.random_block(prob.n_dofs, 8, 60 + j)
        rid = srv1.submit_ks(prob, X0, 4, 10, 60, 1e-8, mixed=True)
        assert srv1.wait(rid).status == 0
        alone.append(srv1.ks_result(rid, 8)[0])
        rid = srv1.submit_poisson(poisson_request_from_batch(pb, j))
        assert srv1.wait(rid).status == 0
        alone.append(srv1.poisson_result(rid, P.instance_view(pb, j)["N"]))
    assert srv1.stats()["poisson_batches"] == 0
    srv1.close()
    # mixed: four slots, everything in flight together
    srv4 = Server(slots=4, hbm_budget_bytes=8 << 30)
    ids = _submit_all(srv4, ks, pb)
    mixed = []
    for kind, rid, n in ids:
        info = srv4.wait(rid)
        assert info.status == 0, info.message
        mixed.append(srv4.ks_result(rid, n)[0] if kind == "ks" else srv4.poisson_result(rid, n))
    st = srv4.stats()
    srv4.close()
    assert st["completed"] == len(ids)
    for a, b in zip(alone, mixed):
        assert np.array_equal(a, b)  # private buffers + deterministic kernels: bitwise equal


def test_poisson_requests_batched_bitwise_as_alone(gpu_ctx, workload):
    """Poisson requests queued together run as one batched solve (continuous
    batching); each result is bitwise the result of its solve alone."""
    from gbfe.serve import Server, poisson_request_from_batch

    _, pb = workload
    srv = Server(slots=1, hbm_budget_bytes=8 << 30)
    alone = []
    for j in range(pb.n_inst):
        rid = srv.submit_poisson(poisson_request_from_batch(pb, j))
        assert srv.wait(rid).status == 0
        alone.append(srv.poisson_result(rid, P.instance_view(pb, j)["N"]))
    assert srv.stats()["poisson_batches"] == 0
    # a KS request holds the slot while the Poisson requests queue behind it
    ks = M.ks_box(3, 3, 6.0, 1, 4.0, 0.5, seed=71)
    srv.submit_ks(ks, M.random_block(ks.n_dofs, 8, 72), 4, 10, 60, 1e-8, mixed=True)
    rids = [srv.submit_poisson(poisson_request_from_batch(pb, j)) for j in range(pb.n_inst)]
    batched = []
    for j, rid in enumerate(rids):
        info = srv.wait(rid)
        assert info.status == 0, info.message
        batched.append(srv.poisson_result(rid, P.instance_view(pb, j)["N"]))
    st = srv.stats()
    srv.close()
    assert st["poisson_batches"] >= 1 and st["poisson_batched_requests"] >= 2
    for a, b in zip(alone, batched):
        assert np.array_equal(a, b)


def test_admission_respects_budget_and_rejects_oversize(gpu_ctx, workload):
    from gbfe.serve import Server

    ks, pb = workload
    srv = Server(slots=4, hbm_budget_bytes=256 << 20)
    big = M.ks_box(3, 3, 6.0, 1, 4.0, 0.5, seed=1)
    # the estimated footprint of a 4096-vector block (~410 MB) exceeds a 256 MiB budget: rejected, never admitted
    rid_big = srv.submit_ks(big, M.random_block(big.n_dofs, 4096, 1), 4, 6, 2)
    info = srv.wait(rid_big)
    assert info.status == 3  # GBFE_ERR_ALLOC
    # a budget that fits one small request at a time still completes them all, in order
    srv.close()
    srv = Server(slots=4, hbm_budget_bytes=30 << 20)  # one small request (~17.5 MB estimate) at a time
    prob = ks[0]
    rids = [srv.submit_ks(prob, M.random_block(prob.n_dofs, 8, 70 + k), 4, 8, 30, 1e-6) for k in range(3)]
    infos = [srv.wait(r) for r in rids]
    assert all(i.status in (0, 6) for i in infos)
    assert infos[1].t_admit >= infos[0].t_done - 1e-6 and infos[2].t_admit >= infos[1].t_done - 1e-6
    srv.close()


def test_cancel_and_injected_allocation_failure(gpu_ctx, workload):
    from gbfe.serve import Server

    ks, pb = workload
    srv = Server(slots=1, hbm_budget_bytes=8 << 30)
    srv.inject_alloc_failures(1)
    prob = ks[1]
    r1 = srv.submit_ks(prob, M.random_block(prob.n_dofs, 8, 1), 4, 10, 60, 1e-8)
    r2 = srv.submit_ks(prob, M.random_block(prob.n_dofs, 8, 2), 4, 10, 60, 1e-8)
    r3 = srv.submit_ks(prob, M.random_block(prob.n_dofs, 8, 3), 4, 10, 60, 1e-8)
    srv.cancel(r3)
    i1, i2, i3 = srv.wait(r1), srv.wait(r2), srv.wait(r3)
    assert i1.status == 3 and "injected" in i1.message
    assert i2.status == 0
    assert i3.status == 9  # GBFE_ERR_CANCELLED
    srv.close()
