"""The multi-replica path of bench.py on the CPU (gloo, world size 2): the
max-over-ranks timing, and a rank that fails before the barrier ends the
other rank's wait with an error after the process-group timeout instead of
hanging."""
import datetime
import multiprocessing as mp
import os
import socket

import pytest


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, mode, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    try:
        if mode == "fail" and rank == 1:
            raise RuntimeError("replica failed")
        dist.barrier()
        q.put((rank, "max", bench.reduce_max(dist, 10.0 + rank)))
    except Exception as e:  # the survivor sees the failed rank as an error
        q.put((rank, "error", type(e).__name__))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(mode):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, mode, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = {}
    for _ in range(2):
        r, kind, val = q.get(timeout=120)
        out[r] = (kind, val)
    for p in ps:
        p.join(timeout=60)
    return out


def test_max_over_ranks():
    out = _run("ok")
    assert out[0] == ("max", 11.0) and out[1] == ("max", 11.0)


def test_failed_rank_is_seen_by_the_other():
    out = _run("fail")
    assert out[1][0] == "error"
    assert out[0][0] == "error"
