"""The N > 1 paths of bench.py on CPU: two ranks over gloo (127.0.0.1). The per-rank numbers are
combined as a multi-GPU run reports them (max of the times, sum of the paths), under torchrun
only rank 0 runs the reference arm (the other ranks join the rendezvous and exit 0 without work),
and each rank of the CUDA arm selects GPU LOCAL_RANK for torch and for the backend's context."""
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


class _FakeContext:
    def __init__(self, device=None):
        self.device = device


def _device_rank(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import torch.distributed as dist

    import bench

    chosen = []
    args = SimpleNamespace(impl="cuda", gpus=world, steps=1, warmup=1)
    r, w, dev, ctx = bench.open_device(args, set_device=chosen.append, make_context=_FakeContext, backend="gloo")
    q.put(("device", rank, (r, w, dev, chosen, ctx.device)))
    dist.destroy_process_group()


def test_each_rank_opens_its_local_gpu():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_device_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    msgs = []
    try:
        for _ in range(2):
            msgs.append(q.get(timeout=120))
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.exitcode is None:
                p.kill()
    assert [p.exitcode for p in procs] == [0, 0], msgs
    got = {m[1]: m[2] for m in msgs}
    # rank, world, the ordinal given to torch.cuda.set_device, and the one the context was opened on
    assert got == {0: (0, 2, 0, [0], 0), 1: (1, 2, 1, [1], 1)}
