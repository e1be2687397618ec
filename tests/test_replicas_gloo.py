"""The benchmark's multi-replica bookkeeping on CPUs: two gloo ranks (one per process, rendezvous
on 127.0.0.1) each report their own step time; both must see the maximum and the same whole-job
throughput, world_size x units / max_ms.  The same functions run under NCCL on GPUs."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from iron_gb300 import replicas

        replicas.barrier()
        local_ms = [2.5, 3.75][rank]
        ms = replicas.max_over_replicas(local_ms)
        out[rank] = (ms, replicas.world_size(), replicas.job_throughput(1_000_000, ms))
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_replicas_agree_on_the_slowest_step():
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed unavailable")
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms, world, thr = res[0]
    assert ms == 3.75 and world == 2
    assert thr == pytest.approx(2 * 1_000_000 / 3.75e-3)


def test_without_a_process_group_everything_is_local():
    from iron_gb300 import replicas

    assert replicas.world_size() == 1
    assert replicas.max_over_replicas(1.25) == 1.25
    assert replicas.job_throughput(10, 2.0) == pytest.approx(5000.0)


def _rank_leaves(rank, port, q):
    import datetime

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=2,
                                         timeout=datetime.timedelta(seconds=5))
    from iron_gb300 import replicas

    replicas.barrier()
    ms = replicas.max_over_replicas([1.0, 2.0][rank])
    if rank == 1:
        # leaves the job between steps: nothing of its own in flight
        q.put((1, "left", ms))
        q.close()
        q.join_thread()  # the message is out before the process ends
        os._exit(0)
    try:
        replicas.max_over_replicas(1.5)
        q.put((0, "no error", None))
    except replicas.ReplicaLost as e:
        q.put((0, "ReplicaLost", str(e)[:200]))
    except Exception as e:  # anything else is a failure of the test
        q.put((0, type(e).__name__, str(e)[:200]))


def test_survivor_fails_cleanly_when_a_replica_leaves():
    """Rank 1 exits between steps; rank 0's next maximum over replicas raises ReplicaLost within
    the process group's timeout instead of hanging."""
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed unavailable")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_leaves, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(2):
        r, what, detail = q.get(timeout=60)
        got[r] = (what, detail)
    for p in procs:
        p.join(timeout=60)
    assert got[1][0] == "left" and got[1][1] == 2.0
    assert got[0][0] == "ReplicaLost", got[0]
