"""The N > 1 path of bench.py on CPU: two ranks over gloo (127.0.0.1), replicas with no
data-path collective. Checks the max / sum reductions of the timing bookkeeping, the
whole-job time per solve of the weak-scaling line, and that the reference arm works on
rank 0 only (other ranks exit without work)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    r = bench.Ranks(world, rank, "cpu")
    r.barrier()
    t = 1.0 + rank  # rank 1 is the slower replica
    res = {"max": r.max(t), "sum": r.sum(float(rank + 1)),
           "value": bench.whole_job_seconds_per_solve(r.max(t), 5, world), "env": bench.dist_env()}
    # the reference arm returns at once on ranks other than 0
    if rank != 0:

        class A:
            steps, warmup, gpus = 1, 0, world

        bench.run_reference(A())
    r.barrier()
    dist.destroy_process_group()
    out.put((rank, res))


def test_two_replicas_over_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(world):
        res = got[rank]
        assert res["max"] == 2.0 and res["sum"] == 3.0
        assert res["value"] == pytest.approx(2.0 / (5 * world))
        assert res["env"] == (world, rank, rank)

