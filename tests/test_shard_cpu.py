"""The N > 1 host path: contiguous shards, max-over-ranks timing and result assembly, run as two
gloo ranks on CPU (the per-rank compute here is the oracle: the GPU path is covered by the gpu
tests; no device collective exists on this path)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from bwacuda import shard


def test_shard_ranges_partition():
    for n in (0, 1, 7, 32, 1000, 8388608):
        for world in (1, 2, 3, 4, 8):
            spans = [shard.shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, results):
    import sys

    import torch.distributed as dist

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, ".."))
    sys.path.insert(0, os.path.join(here, "..", "bwa-mem4_gb300"))
    import bwacuda as B
    import oracle
    from bwacuda import shard as S

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        js = B.synth_ext(2, 3001, seed=17)  # every rank builds the same batch
        a, b = S.shard_range(len(js), rank, world)
        part, _ = oracle.extend_batch(js.take(np.arange(a, b)), nthreads=1)
        t = S.max_over_ranks(0.5 + rank)  # the slowest rank's time
        full = S.gather_results(part, len(js))
        if rank == 0:
            want, _ = oracle.extend_batch(js, nthreads=1)
            results.put(("ok", bool(np.array_equal(full, want)), t))
        else:
            results.put(("rank", full is None, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_gather():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    (k0, same, t0), (k1, none_on_rank1, t1) = got
    assert (k0, k1) == ("ok", "rank")
    assert same and none_on_rank1
    assert t0 == t1 == 1.5
