"""The CPU oracle pinned against the reference's own outputs (golden file
made by the reference binaries, published values, and vectors from the
reference's Python counter).  CPU only."""
import json
import os
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
THREADS = os.cpu_count() or 4

FAST_SHAPES = ["2x2", "2x3", "2x4", "2x5", "2x6", "3x3", "3x4", "3x5", "3x6", "4x4", "4x5", "4x6",
               "5x5", "1x8", "1x9", "1x10", "1x11", "1x12", "1x13", "1x14", "1x15", "1x16",
               "2x2x1", "2x2x2", "2x2x3", "2x2x4", "2x2x5", "1x1", "2x3x4",
               "2x2x6", "3x3x3", "2x2x2x2", "2x2x2x3", "2x2x2x2x2"]


@pytest.mark.parametrize("key", FAST_SHAPES)
def test_lunnon_counts(orc, golden, key):
    dims = tuple(int(x) for x in key.split("x"))
    got, _ = orc.lunnon_count(dims)
    assert got == golden["lunnon"][key]


def test_transposed_shapes_agree(orc):
    for dims in [(2, 3), (3, 4), (2, 5), (2, 2, 3)]:
        assert orc.lunnon_count(dims)[0] == orc.lunnon_count(tuple(reversed(dims)))[0]


def test_res_mod_split_sums_to_total(orc, golden):
    # mf.c:100 and run_parallel.sh:15-30: residues of one modulus partition the count
    mod = 7
    parts = [orc.lunnon_count((4, 4), res, mod)[0] for res in range(mod)]
    assert sum(parts) == golden["lunnon"]["4x4"]


def test_prefix_states(orc, golden):
    for key, want in golden["prefix_states"].items():
        shape, depth = key.split("@")
        grid = int(shape.split("x")[0])
        if grid >= 7:
            continue
        a, b, g = orc.lunnon_collect((grid, grid), int(depth))
        assert len(b) == want, key


def test_resume_sums_to_whole_count(orc, golden):
    a, b, g = orc.lunnon_collect((4, 5), 8)
    total, per, w = orc.lunnon_resume_many((4, 5), 9, a, b, threads=THREADS)
    assert total == golden["lunnon"]["4x5"]
    assert per.sum() == total


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6])
def test_sym_squares(orc, golden, n):
    got, _ = orc.sym_solve(n, THREADS)
    assert got == golden["sym"][f"n{n}"]
    assert got == golden["published"]["squares"][str(n)]


def test_sym_setup_counts(orc, golden):
    cyc, mult, centers = orc.sym_reps(8)
    assert centers == 9394 and len(cyc) == 1225
    cyc, mult, centers = orc.sym_reps(7)
    assert centers == 76 and len(cyc) == 11
    c24, _ = orc.sym_expand(7, 24)
    assert len(c24) == golden["sym_setup"]["7x7_d24"]
    c24, _ = orc.sym_expand(8, 24)
    assert len(c24) == golden["sym_setup"]["8x8_d24"]
    assert len(c24) == golden["published"]["sym_8x8_expanded_cases"]["24"]


def test_sym_chunks(orc, golden):
    got, _ = orc.sym_solve(8, THREADS, max_cases=200, start_case=0, expanded_n=36)
    assert got == golden["sym"]["8x8_d36_first200"]
    got, _ = orc.sym_solve(7, THREADS, max_cases=2000, start_case=0, expanded_n=28)
    assert got == golden["sym"]["7x7_d28_first2000"]
    got, _ = orc.sym_solve(8, THREADS, max_cases=100, start_case=0, expanded_n=32)
    assert got == golden["sym"]["8x8_d32_first100"]


def test_wasm_vectors(orc):
    vecs = json.loads((ROOT / "tests" / "golden" / "wasm_vectors.json").read_text())
    for v in vecs["cases"]:
        total = 0
        for cyc in v["prefix_bytes"]:
            c, _ = orc.sym_count_to(v["n"], np.array(cyc, np.uint8), v["depth"], v["stopDepth"])
            total += c
        assert total == v["expected"]


def test_mfah_campaign_total(orc, golden):
    """mfah/README.md:59-68: the bounded 7x7 campaign -- every raw prefix at
    14 cells grown from the 3-cell cycle, counted to 28 cells -- totals
    35044546."""
    prefixes = orc.sym_raw_prefixes(7, 14)
    per = orc.sym_estimate_cases(7, 14, 14, prefixes, threads=THREADS)
    assert int(per.sum()) == golden["published"]["mfah_7x7_d14_s28"]
    # its first unit of 64 prefixes is the WASM test's 7x7 payload
    vecs = json.loads((ROOT / "tests" / "golden" / "wasm_vectors.json").read_text())
    first = next(v for v in vecs["cases"] if v["n"] == 7)
    assert (prefixes[:64] == np.array(first["prefix_bytes"], np.uint8)).all()
    assert int(per[:64].sum()) == first["expected"]


def test_sym_node_counts_are_consistent(orc):
    # nodes of a whole count equal the sum over its cases' subtrees plus the
    # nodes above the case depth
    cyc, mult = orc.sym_expand(7, 20, 0, 50)
    t1, per, w = orc.sym_count_cases(7, 20, cyc, None, threads=2)
    w2 = 0
    for c in cyc:
        _, w1 = orc.sym_count_to(7, c, 20, 49)
        w2 += w1.nodes
    # count_to also counts the calls at the stop level (one per completion)
    assert w2 == w.nodes + t1


def test_work_counts_fixture_is_consistent(golden):
    """The oracle's whole-7x7 work totals (tests/golden/work_counts.json)
    belong to the published 7x7 answer."""
    import json
    from pathlib import Path

    w = json.loads((Path(__file__).parent / "golden" / "work_counts.json").read_text())["7x7_d24_all"]
    assert w["answer"] == golden["published"]["squares"]["7"]
    assert w["cases"] == 433131 and w["steps"] > w["nodes"] > 0
