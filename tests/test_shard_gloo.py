"""Multi-rank sharding of a case range, world_size 2 over gloo on CPU; the
counting is the oracle (no GPU), the host logic is the product's."""
import os
import socket

import pytest

from map_folding_gb300.shard import combine, shard_range


def test_shard_range_covers_exactly():
    for count in [0, 1, 7, 100, 50001]:
        for world in [1, 2, 3, 8]:
            seen = []
            for r in range(world):
                first, n = shard_range(10, count, r, world)
                seen.extend(range(first, first + n))
            assert seen == list(range(10, 10 + count))
    with pytest.raises(ValueError):
        shard_range(0, 10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from map_folding_gb300.shard import run_rank
    from oracle import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)

    def count_chunk(first, n):
        ans, _ = oracle.sym_solve(7, 2, max_cases=n, start_case=first, expanded_n=28)
        return ans

    def gather(part):
        parts = [None] * world
        dist.all_gather_object(parts, part)
        return parts

    total = run_rank(count_chunk, 0, 600, rank, world, gather)
    out[rank] = total
    dist.destroy_process_group()


def test_two_ranks_gloo_match_single(orc, golden):
    import torch.multiprocessing as mp

    port = _free_port()
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    single, _ = orc.sym_solve(7, 2, max_cases=600, start_case=0, expanded_n=28)
    assert out[0] == out[1] == single
    assert combine(["1", 2, "3"]) == 6
