"""The N-GPU path of bench.py on the CPU: N independent replicas, one rank per
process, timed as one job (max over ranks) with the whole-job rate summed
over ranks.  World size 2 over gloo (127.0.0.1)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        local_ms = 100.0 + 25.0 * rank          # rank 1 is the slower replica
        t = bench.replica_max(local_ms, ws, device="cpu")
        v = bench.replica_value(ws, 1000, 4, t * 1e-3)
        dist.barrier()
        out.put((r, ws, local, t, v))
    finally:
        dist.destroy_process_group()


def test_two_replicas_over_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, ws, local, t, v) in enumerate(res):
        assert (rank, ws, local) == (r, 2, r)
        assert t == 125.0                         # both ranks see the slowest rank's time
        assert v == pytest.approx(2 * 1000 * 4 / 0.125 / 1e9)


def test_one_replica_is_the_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_max(3.5, 1) == 3.5
    assert bench.replica_value(1, 10, 2, 4.0) == pytest.approx(5e-9)
