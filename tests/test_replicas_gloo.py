"""The multi-process path of bench.py (`--gpus N` under torchrun): replicas
only, joined by barriers and one max-reduction of the timings over the ranks.
Here two gloo ranks on the CPU check that reduction."""
import os
import socket

import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out = bench.max_over_ranks(dist, 1.0 + rank, 10.0 * (world - rank))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


def test_max_over_ranks_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: (2.0, 20.0), 1: (2.0, 20.0)}


def test_single_process_is_unchanged():
    import bench
    assert bench.max_over_ranks(None, 3.0, 4.0) == (3.0, 4.0)
