"""The multi-GPU form of the bench is N independent replicas (views are
independent; no collective on the data path): the only cross-rank step is
the barrier and the max over ranks of the step time.  Covered here with two
gloo ranks on the CPU (no GPU)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        assert (r, w, local) == (rank, world, rank)
        dist.barrier()
        got = bench.max_over_ranks(1.5 + rank * 0.25, world)  # rank-dependent step times
        out[rank] = got
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 1.75, 1: 1.75}


def test_single_rank_is_identity():
    import bench

    assert bench.max_over_ranks(3.25, 1) == 3.25
