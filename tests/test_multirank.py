"""The replica path of bench.py with two ranks over gloo on the CPU: barrier, max over ranks
of the timed region, and the whole-job aggregation (no GPU, no collective on the data)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        dev = torch.device("cpu")
        bench.dist_barrier(ws, dev)
        local_t = 1.0 + rank  # rank 1 is the slow replica
        t = bench.dist_max(local_t, ws, dev)
        v = bench.aggregate_builds_per_s(ws, 4, t)
        q.put((rank, t, v, bench.dist_env()))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_over_gloo():
    ws = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v, env in out:
        assert t == 2.0                  # the slowest rank's time
        assert abs(v - 2 * 4 / 2.0) < 1e-12
        assert env[0] == 2 and env[1] == rank
