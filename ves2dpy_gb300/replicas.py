"""Multi-GPU runs of the step: independent replicas, one process per GPU.

The implicit step has no data exchange between suspensions, so N GPUs run N
independent suspensions (weak scaling).  Ranks only meet at barriers around
the timed region and in one max-reduction of the elapsed time; there is no
collective on the data path.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def aggregate(elapsed_ms: float, vesicle_steps: float, device=None) -> tuple[float, float]:
    """Whole-job throughput: (max elapsed ms over ranks, total vesicle-steps/s).

    Every rank contributes its own vesicle-steps; the job time is the slowest
    rank's time.  Works with the nccl (GPU) and gloo (CPU) backends.
    """
    if not dist.is_available() or not dist.is_initialized():
        return elapsed_ms, vesicle_steps / (elapsed_ms * 1e-3)
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([elapsed_ms], dtype=torch.float64, device=dev)
    w = torch.tensor([vesicle_steps], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    tmax = float(t.item())
    return tmax, float(w.item()) / (tmax * 1e-3)


def barrier():
    if dist.is_available() and dist.is_initialized():
        dist.barrier()
