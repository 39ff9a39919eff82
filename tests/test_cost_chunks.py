"""Cost-weighted chunking: shallow estimate_work scores per block of cases
(SymPlan.block_costs, on the GPU), contiguous chunks of about equal
estimated cost (chunks.partition_by_cost), and coverage checks for sweeps
whose chunks differ in size."""
import json
import os

import numpy as np
import pytest


def test_partition_tiles_the_range():
    from map_folding_gb300.chunks import partition_by_cost

    rng = np.random.Generator(np.random.PCG64(3))
    for trial in range(50):
        blocks = int(rng.integers(1, 200))
        block = int(rng.integers(1, 50))
        count = (blocks - 1) * block + int(rng.integers(1, block + 1))
        costs = rng.integers(0, 1000, blocks) ** 2
        k = int(rng.integers(1, 60))
        start = int(rng.integers(0, 10**6))
        chunks = partition_by_cost(costs, block, start, count, k)
        assert 1 <= len(chunks) <= k
        pos = start
        for s, m in chunks:
            assert s == pos and m > 0
            assert (s - start) % block == 0
            pos = s + m
        assert pos == start + count


def test_partition_balances_cost():
    from map_folding_gb300.chunks import partition_by_cost

    costs = np.ones(1000)
    costs[100:120] = 50  # a heavy band
    chunks = partition_by_cost(costs, 10, 0, 10000, 10)
    per = [costs[s // 10:(s + m) // 10].sum() for s, m in chunks]
    total = costs.sum()
    # no chunk exceeds its share by more than one block's cost
    assert max(per) <= total / len(chunks) + costs.max()
    # the heavy band is cut finer than the light range
    sizes = [m for s, m in chunks]
    assert min(sizes) < max(sizes)


def test_variable_chunk_coverage(tmp_path):
    from map_folding_gb300.chunks import summarize_jsonl

    def write(rows):
        p = tmp_path / "s.jsonl"
        p.write_text("".join(json.dumps({"start_case": s, "max_cases": m, "count": str(c)}) + "\n"
                             for s, m, c in rows))
        return p

    ok = summarize_jsonl(write([(0, 30, 1), (30, 5, 2), (35, 65, 3)]), 100, 0)
    assert ok["complete"] and ok["unique_sum"] == "6"
    gap = summarize_jsonl(write([(0, 30, 1), (40, 60, 2)]), 100, 0)
    assert not gap["complete"] and gap["missing_starts"] == [30]
    short = summarize_jsonl(write([(0, 30, 1), (30, 60, 2)]), 100, 0)
    assert not short["complete"] and short["missing_starts"] == [90]
    overlap = summarize_jsonl(write([(0, 30, 1), (20, 80, 2)]), 100, 0)
    assert not overlap["complete"] and overlap["extra_starts"] == [20]
    dup = summarize_jsonl(write([(0, 50, 1), (0, 50, 1), (50, 50, 2)]), 100, 0)
    assert not dup["complete"] and dup["duplicate_count"] == 1


@pytest.mark.gpu
def test_block_costs_match_oracle(engine, orc, cuda):
    cyc, _ = orc.sym_expand(7, 24, 1000, 5000)
    plan = engine.SymPlan(7, 24)
    try:
        for depth in (0, 2, 4):
            got = plan.block_costs(1000, 5000, depth, 64)
            scores = orc.sym_estimate_cases(7, 24, depth, cyc, os.cpu_count() or 1) + 1
            want = [int(scores[k:k + 64].sum()) for k in range(0, 5000, 64)]
            assert got.tolist() == want, depth
    finally:
        plan.close()


@pytest.mark.gpu
def test_cost_chunks_sum_to_the_range(engine, cuda, golden):
    from map_folding_gb300.chunks import ChunkRunner, plan_cost_chunks

    chunks = plan_cost_chunks(7, 24, 6, cost_depth=3, start_case=0, total_cases=2000, block=50)
    assert chunks[0][0] == 0 and sum(m for _, m in chunks) == 2000
    runner = ChunkRunner(7, 24)
    total = sum(int(runner.run(s, m)["count"]) for s, m in chunks)
    assert total == golden["sym"]["7x7_d24_first2000"]
