"""MF_COST_DEPTH / MF_SORT_CASES (sym_fold.cpp:267-314): cases scored by
estimate_work and, when asked, reordered by score with the reference's
unstable std::sort; start_case / max_cases then index the sorted order.

The golden vectors were printed by the reference's own sym_fold
(tests/golden/make_golden.py --cost).  Shallow depths give many equal
(score, multiplier) keys, so they also pin where the unstable sort puts
equal keys."""
import os
import subprocess

import numpy as np
import pytest

N2_START = {6: 16, 7: 24}


def _vectors(golden):
    for key, v in sorted(golden["sym_cost"].items()):
        n, _threads, max_cases, start = (int(a) for a in v["args"])
        env = v["env"]
        depth = int(env["MF_COST_DEPTH"])
        sort = env.get("MF_SORT_CASES")
        order = None if not sort or sort == "0" else ("asc" if sort == "asc" else "desc")
        yield key, n, max_cases, start, depth, order, v


def test_oracle_scores_and_sorted_chunks_match_reference(golden, orc, engine):
    threads = os.cpu_count() or 1
    cases = {}
    for key, n, max_cases, start, depth, order, v in _vectors(golden):
        if n not in cases:
            cases[n] = orc.sym_expand(n, 24 if n >= 7 else 16, 0, 0)
        cyc, mult = cases[n]
        start_i = N2_START[n]
        scores = orc.sym_estimate_cases(n, start_i, depth, cyc, threads)
        assert int(scores.min()) == v["min_score"], key
        assert int(scores.max()) == v["max_score"], key
        assert int(scores.sum()) == v["total_score"], key
        if order is None:
            idx = np.arange(len(cyc))
        else:
            idx = engine.sym_sort_order(scores, mult, ascending=order == "asc").astype(np.int64)
        sel = idx[start:start + max_cases]
        total, _, _ = orc.sym_count_cases(n, start_i, cyc[sel], mult[sel], threads)
        assert total * n * n == v["count"], key


def test_sort_order_ties_by_multiplier(engine):
    scores = np.array([5, 1, 5, 3, 5], np.uint64)
    mults = np.array([8, 1, 2, 4, 1], np.uint64)
    desc = engine.sym_sort_order(scores, mults).tolist()
    assert [int(scores[k]) for k in desc] == [5, 5, 5, 3, 1]
    assert [int(mults[k]) for k in desc[:3]] == [1, 2, 8]
    asc = engine.sym_sort_order(scores, mults, ascending=True).tolist()
    assert [int(scores[k]) for k in asc] == [1, 3, 5, 5, 5]


@pytest.mark.gpu
def test_plan_score_and_sorted_chunks(golden, engine, cuda):
    for key, n, max_cases, start, depth, order, v in _vectors(golden):
        plan = engine.SymPlan(n, 24 if n >= 7 else 0)
        try:
            lo, hi, tot = plan.score(depth, order)
            assert (lo, hi, tot) == (v["min_score"], v["max_score"], v["total_score"]), key
            ans, _ = plan.solve(max_cases, start)
            assert ans == v["count"], key
        finally:
            plan.close()


@pytest.mark.gpu
def test_sym_fold_cli_cost_order(golden, engine, cuda):
    from map_folding_gb300 import build as mfbuild

    for key, n, max_cases, start, depth, order, v in _vectors(golden):
        env = dict(os.environ)
        env.update(v["env"])
        res = subprocess.run([str(mfbuild.BIN / "sym_fold"), str(n), "8", str(max_cases), str(start)],
                             capture_output=True, text=True, env=env, check=True)
        assert res.stdout.strip() == str(v["count"]), key
        line = next(ln for ln in res.stderr.splitlines() if ln.startswith("cost_depth="))
        kv = dict(tok.split("=", 1) for tok in line.split())
        assert int(kv["min_score"]) == v["min_score"] and int(kv["max_score"]) == v["max_score"]
        assert int(kv["total_score"]) == v["total_score"], key
        if order:
            assert f"sorted_cases={order}" in res.stderr, key
