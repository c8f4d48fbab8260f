"""The N > 1 paths of bench.py on CPU: two ranks over gloo (127.0.0.1). The per-rank numbers are
combined as a multi-GPU run reports them (max of the times, sum of the paths), and under torchrun
only rank 0 runs the reference arm: the other ranks join the rendezvous and exit 0 without work."""
import multiprocessing as mp
import os
import socket
from types import SimpleNamespace


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as dist

    import bench

    args = SimpleNamespace(impl="reference", gpus=world, steps=1, warmup=1)
    if rank == 1:
        # Joins the group, then returns at once (rank 0 alone times the reference).
        got = bench.run_reference(args)
        q.put(("reference", rank, got))
        bench.barrier(world)
        mx = bench.allmax(world, 1.5 + rank)
        sm = bench.allsum(world, 1.0 + rank)
    else:
        r, w = bench.dist_init(args)
        q.put(("init", r, w))
        bench.barrier(world)
        mx = bench.allmax(world, 1.5 + rank)
        sm = bench.allsum(world, 1.0 + rank)
    q.put(("reduce", rank, (mx, sm)))
    dist.destroy_process_group()


def test_two_gloo_ranks_combine_and_only_rank0_runs_the_reference():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    msgs = []
    try:
        for _ in range(4):  # each rank sends two messages; read them before joining
            msgs.append(q.get(timeout=120))
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.exitcode is None:
                p.kill()
    codes = [p.exitcode for p in procs]
    assert codes == [0, 0], (codes, msgs)
    assert ("init", 0, 2) in msgs
    assert ("reference", 1, 0) in msgs
    reduces = {m[1]: m[2] for m in msgs if m[0] == "reduce"}
    assert reduces == {0: (2.5, 3.0), 1: (2.5, 3.0)}
