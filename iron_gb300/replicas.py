"""Replica bookkeeping of the benchmark when it runs one process per GPU.

The assembly path shards naturally: every rank assembles its own mesh (a replica, no data-path
collective), so the only cross-rank steps are a barrier before each timed region and the maximum
of the per-rank step times after it (the slowest replica sets the job's pace).  Whole-job
throughput is world_size x units per replica / that maximum.  The functions work with any
torch.distributed backend (NCCL on GPUs, gloo on CPUs) and degrade to no-ops without a process
group.
"""
from __future__ import annotations

import torch


class ReplicaLost(RuntimeError):
    """A collective of the replica bookkeeping failed: another rank left the job (exited, was
    killed, or stopped answering within the process group's timeout)."""


def _active() -> bool:
    return torch.distributed.is_available() and torch.distributed.is_initialized()


def world_size() -> int:
    return torch.distributed.get_world_size() if _active() else 1


def barrier() -> None:
    if _active():
        try:
            torch.distributed.barrier()
        except Exception as e:  # gloo / NCCL report a lost peer as various RuntimeErrors
            raise ReplicaLost(f"barrier failed: {e}") from e


def max_over_replicas(value: float, device: torch.device | None = None) -> float:
    """The maximum of `value` over all ranks (the value itself without a process group).  `device`
    is where the reduction tensor lives: a CUDA device for NCCL, None (CPU) for gloo."""
    if not _active():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    try:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    except Exception as e:
        raise ReplicaLost(f"maximum over replicas failed: {e}") from e
    return float(t.item())


def job_throughput(units_per_replica: float, ms_max: float, replicas: int | None = None) -> float:
    """Units per second of the whole job: every replica processed `units_per_replica` in the time
    of the slowest one."""
    n = world_size() if replicas is None else replicas
    return n * units_per_replica / (ms_max * 1e-3)
