"""The multi-rank path of bench.py (replicas: a barrier and a max over
ranks of the timed region, no collective on the data path) with two gloo
ranks on the CPU, launched the way torchrun would set the environment."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local, dist = bench.dist_setup()
    assert (ws, r, local) == (world, rank, rank) and dist is not None
    bench.barrier(dist)
    out[rank] = bench.max_over_ranks(dist, 1.5 + rank)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_take_the_max_of_the_timed_region():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(100)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert dict(out) == {0: 2.5, 1: 2.5}
