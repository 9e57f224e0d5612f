"""The multi-GPU mode of bench.py is replicas only: each rank runs its own
solves and the ranks share nothing but the timing reduction.  Checked here with
two gloo ranks on the CPU: the job time is the slowest rank's and the value
counts every rank's steps."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import sys
    from pathlib import Path

    import torch.distributed as dist

    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    value, t_step = bench.aggregate_replicas(times[rank], 4, world)
    out[rank] = (value, t_step)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    times = [2.0, 3.0]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        value, t_step = out[r]
        assert abs(t_step - 0.75) < 1e-12  # max(2, 3) / 4 steps
        assert abs(value - 2 / 0.75) < 1e-12
