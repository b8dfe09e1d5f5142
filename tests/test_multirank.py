"""The benchmark's multi-rank host logic on CPU ranks (gloo, world size 2):
each rank unbinds its own batch (weak scaling: a seed per rank), the job's
time is the slowest rank's and its bound particles are the sum over ranks,
and the reference arm runs on rank 0 alone.  No GPU is involved."""
import os
import socket
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import argparse

    import numpy as np
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        import bench
        r, w, local = bench.dist_env()
        assert (r, w, local) == (rank, world, rank)
        # weak scaling: every rank draws its own batch (seed + rank)
        inp, _ = bench.workload(20_000, 7 + rank, "batched")
        first = np.asarray(inp.pos[:4], np.float64).ravel()
        firsts = [None] * world
        dist.all_gather_object(firsts, first.tolist())
        ms = bench._max_over_ranks(10.0 + rank)
        bound = bench._sum_over_ranks(100 * (rank + 1))
        # the reference arm: rank 0 alone runs (and prints); the others return at once
        args = argparse.Namespace(total=20_000, seed=0, workload="batched", ref_sample=2000, warmup=0, steps=1)
        rc = bench.bench_reference(args) if rank != 0 else None
        out[rank] = dict(ms=ms, bound=bound, differ=firsts[0] != firsts[1], rc=rc)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_weak_scaling_reductions():
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        assert res[rank]["ms"] == pytest.approx(11.0)      # the slowest rank's time
        assert res[rank]["bound"] == pytest.approx(300.0)  # every rank's particles
        assert res[rank]["differ"]                         # each rank has its own batch
    assert res[1]["rc"] == 0                               # a non-zero rank skips the reference arm
