"""The multi-GPU path is independent replicas: each rank steps its own filter and the
job reports total weights / slowest rank's time.  The reductions bench.py uses for
that (barrier, max of the times, sum of the weights) run here as two gloo ranks on
the CPU; a rank that fails raises on the host and the other rank sees the failure
through the collective's timeout instead of hanging."""

import datetime
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q, fail_rank):
    import sys

    import torch
    import torch.distributed as dist

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    try:
        if rank == fail_rank:
            raise RuntimeError("injected failure before the timed region")
        bench.barrier(world)
        dev = torch.device("cpu")
        t_max = bench.allreduce_max(1.5 + rank, world, dev)
        w_sum = bench.allreduce_sum(1000 * (rank + 1), world, dev)
        q.put((rank, "ok", t_max, w_sum))
    except Exception as e:  # reported to the parent, never a GPU fault
        q.put((rank, "error", type(e).__name__, str(e)[:80]))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, fail_rank=-1):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q, fail_rank)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
    return sorted(out)


def test_replica_reductions_two_ranks():
    out = _run(2)
    assert [o[1] for o in out] == ["ok", "ok"]
    for rank, _, t_max, w_sum in out:
        assert t_max == 2.5  # slowest rank's time
        assert w_sum == 3000  # weights of both replicas
    # value = total weights / slowest time
    assert out[0][3] / out[0][2] == pytest.approx(1200.0)


def test_failed_rank_surfaces_on_the_host():
    out = _run(2, fail_rank=1)
    status = {o[0]: o[1] for o in out}
    assert status[1] == "error"
    assert status[0] == "error"  # the barrier gives up (timeout / peer gone) instead of hanging
