"""CPU: the multi-GPU form (replicas sharing nothing): the largest-first shard of streams over ranks,
and the same shard and the max-over-ranks timing across two real ranks (gloo, 127.0.0.1)."""
import os
import random

import pytest

from gpuzip_gb300 import shard


def test_shard_is_a_balanced_partition():
    rng = random.Random(3)
    sizes = [int(2 ** rng.uniform(10, 26)) for _ in range(1000)]
    for ws in (1, 2, 3, 8):
        shares = shard.shard_streams(sizes, ws)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in s) for s in shares]
        # greedy largest-first: no rank exceeds the mean by more than the largest stream
        assert max(loads) - sum(loads) / ws <= max(sizes)
        assert all(s == sorted(s) for s in shares)


def test_shard_is_deterministic_and_edge_cases():
    sizes = [5, 5, 5, 5]
    assert shard.shard_streams(sizes, 2) == [[0, 2], [1, 3]]
    assert shard.shard_streams([], 3) == [[], [], []]
    assert shard.shard_streams([7], 4) == [[0], [], [], []]
    with pytest.raises(ValueError):
        shard.shard_streams(sizes, 0)


def _rank(rank, world, port, sizes, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.shard_streams(sizes, world)[rank]
    seconds = 0.25 + rank  # a slower second rank
    slowest = shard.max_over_ranks(seconds)
    got = [None] * world
    dist.all_gather_object(got, mine)
    dist.destroy_process_group()
    q.put((rank, mine, slowest, got))


def test_two_gloo_ranks_share_the_streams():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    sizes = [int(1.7 ** k) % 100_000 + 1 for k in range(200)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    expect = shard.shard_streams(sizes, 2)
    for rank, mine, slowest, got in out:
        assert mine == expect[rank]
        assert slowest == pytest.approx(1.25)  # the max over ranks
        assert got == expect
    assert sorted(out[0][1] + out[1][1]) == list(range(len(sizes)))
