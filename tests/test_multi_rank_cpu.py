"""Multi-rank host logic of the bench on CPU (gloo, world size 2).

The overlap path shards by reads with no data-path collective: every rank
takes a length-balanced share of the reads against the index of all of
them, and ranks meet only to agree on the timed region (barrier) and to
combine their results (sum of bases, max of times)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, results):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    # rank r processed (r + 1) * 1000 bases in (r + 1) * 0.5 s
    bases = bench.reduce_sum(w, float((r + 1) * 1000))
    slowest = bench.reduce_max(w, (r + 1) * 0.5)
    results[rank] = (bases, slowest, bases / slowest)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_combine_like_the_bench():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        results = m.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, world, port, results))
                 for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        got = dict(results)
    # all bases over the slowest rank's time, the same on every rank
    for r in range(world):
        assert got[r] == (3000.0, 1.0, 3000.0)


def test_single_rank_needs_no_process_group(monkeypatch):
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    assert bench.dist_setup() == (1, 0, 0)
    assert bench.reduce_max(1, 2.5) == 2.5
    assert bench.reduce_sum(1, 7.0) == 7.0


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_read_shards_are_disjoint_complete_and_balanced(world):
    import numpy as np
    import bench
    rng = np.random.default_rng(world)
    lengths = np.clip(rng.lognormal(np.log(15_000), 0.2, size=1_000).astype(np.int64), 1_000,
                      100_000)
    shards = bench.shard_reads(lengths, world)
    assert len(shards) == world
    allidx = np.sort(np.concatenate(shards))
    assert np.array_equal(allidx, np.arange(len(lengths)))  # each read exactly once
    for s in shards:
        assert np.all(np.diff(s) > 0)  # input order within a shard
    loads = np.array([lengths[s].sum() for s in shards])
    # greedy longest-first: no rank exceeds another by more than the longest read
    assert loads.max() - loads.min() <= lengths.max()
