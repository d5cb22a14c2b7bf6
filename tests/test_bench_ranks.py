"""bench.py's multi-rank path on CPU: two gloo ranks meet at the timing
barriers and report the slowest rank's step time with the outputs of both
ranks (replicas: no collective on the data path)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        import bench

        bench.barrier()
        res = bench.combine_ranks({"ms_per_step": 2.0 + rank, "outputs_per_step": 1e9}, world)
        bench.barrier()
        q.put((rank, res["ms_per_step"], res["value"]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(world))
    for rank, ms, value in got:
        assert ms == 3.0  # the slower rank's 3 ms
        assert value == pytest.approx(2e9 / 3e-3)


def test_single_rank_helpers_are_identity():
    sys.path.insert(0, ROOT)
    import bench

    bench.barrier()
    assert bench.rank_max(4.5) == 4.5
    res = bench.combine_ranks({"ms_per_step": 2.0, "outputs_per_step": 1e9}, 1)
    assert res["value"] == pytest.approx(5e11)
