"""The N > 1 path of bench.py on the CPU: world_size 2 over gloo (no GPU).  The path does not shard — every rank
solves its own replica of the workload with no collective on the data path — so what N > 1 adds is the timing
aggregation (the slowest rank's time) and the guarantee that replicas compute the same result."""
import os
import socket
import sys

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle
        from ikarus_gb300 import problems
        t = bench.max_over_ranks(1.5 + rank, world, device="cpu")
        # a replica: every rank solves the same small load path with the oracle
        p = problems.cantilever(4, 2, 2, load_steps=2, traction=(0.0, 0.0, -1.0))
        r = oracle.from_problem(p).load_control(2, tol=1e-10)
        checksum = float(np.abs(r["u"]).sum())
        sums = [None] * world
        dist.all_gather_object(sums, checksum)
        out.put((rank, t, sums, r["success"]))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_over_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, sums, ok in results:
        assert ok
        assert t == 2.5  # the slowest rank's value on every rank
        assert sums[0] == sums[1]  # replicas agree bit for bit
