"""World-size-2 gloo run of the replica aggregation used by bench.py --gpus N."""
import os
import socket

import torch
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from ves2dpy_gb300.replicas import aggregate, barrier
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    barrier()
    # rank r "ran" 100*(r+1) vesicle-steps in 1000*(r+1) ms
    tmax, rate = aggregate(1000.0 * (rank + 1), 100.0 * (rank + 1))
    out[rank] = torch.tensor([tmax, rate])
    barrier()
    dist.destroy_process_group()


def test_aggregate_two_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        tmax, rate = out[r].tolist()
        assert tmax == 2000.0
        assert abs(rate - 300.0 / 2.0) < 1e-9


def test_aggregate_single_process():
    from ves2dpy_gb300.replicas import aggregate
    tmax, rate = aggregate(500.0, 1000.0)
    assert tmax == 500.0 and rate == 2000.0
