"""GPU parity of the sym_fold kernels: per-case counts and node counts
against the oracle, chunk sums against the reference's own sym_fold output
(golden), and the WASM solve_cases contract against mfah/folding.py."""
import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_small_squares(engine, cuda, golden, n, mode):
    assert engine.sym_fold(n, mode=mode) == golden["sym"][f"n{n}"]


CHUNKS = [
    # (golden key, n, expanded_n, max_cases, start_case)
    ("7x7_d24_first2000", 7, 24, 2000, 0),
    ("7x7_d24_300000+500", 7, 24, 500, 300000),
    ("7x7_d28_first2000", 7, 28, 2000, 0),
    ("8x8_d36_first200", 8, 36, 200, 0),
    ("8x8_d36_120000000+200", 8, 36, 200, 120000000),
    ("8x8_d36_240192700+500", 8, 36, 500, 240192700),
    ("8x8_d24_case400000", 8, 24, 1, 400000),
    ("8x8_d32_first100", 8, 32, 100, 0),
]


# The plain kernel runs one case per thread, so a chunk takes as long as its
# heaviest case alone (a single 8x8 depth-24 case: ~80 s); it is checked on
# the chunks whose heaviest case is light, and on partial depths and per-case
# counts below.
PLAIN_CHUNKS = {"7x7_d24_300000+500", "7x7_d28_first2000"}


@pytest.mark.parametrize("key,n,e,count,start", CHUNKS)
@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_chunks_match_reference(engine, cuda, golden, key, n, e, count, start, mode):
    if mode == "plain" and key not in PLAIN_CHUNKS:
        pytest.skip("plain kernel: chunk bound by one heavy case; covered by partial-depth tests")
    assert engine.sym_fold(n, count, start, expanded_n=e, mode=mode) == golden["sym"][key]


# The reference's published 8x8 partial sums (EXPERIMENTS.md:77-81, kept in
# reference_counts.json["published"]): each is what `sym_fold 8 ...` printed
# for that chunk with MF_EXPANDED_N set.  The depth-36 100,000-case chunk is
# twice the serving benchmark's chunk size.
PUBLISHED_8X8 = [
    # (published key, expanded_n, max_cases, start_case)
    ("d36_first100000", 36, 100000, 0),
    ("d32_first1000", 32, 1000, 0),
    ("d24_case100000", 24, 1, 100000),
    ("d24_case400000", 24, 1, 400000),
]


@pytest.mark.parametrize("key,e,count,start", PUBLISHED_8X8)
def test_published_8x8_partial_sums(engine, cuda, golden, key, e, count, start):
    want = golden["published"]["sym_8x8_partial_sums"][key]
    assert engine.sym_fold(8, count, start, expanded_n=e, mode="batched") == want


SERVING_GOLDEN = json.loads((ROOT / "tests" / "golden" / "reference_counts.json").read_text()
                            ).get("sym_serving", {})


@pytest.mark.parametrize("key", sorted(SERVING_GOLDEN))
def test_serving_chunks_match_reference(engine, cuda, golden, key):
    """The serving benchmark's 50,000-case 8x8 chunks (serving_stream(seed=5)),
    against the reference's own sym_fold on the same chunk."""
    rec = golden["sym_serving"][key]
    got = engine.sym_fold(8, rec["max_cases"], rec["start_case"], expanded_n=rec["expanded_n"],
                          mode="batched")
    assert got == rec["count"]


def _device_counts(engine, torch, n, start_i, stop_i, cycles, mode):
    d_cyc = torch.from_numpy(np.ascontiguousarray(cycles)).cuda()
    counts = torch.zeros(len(cycles), dtype=torch.int64, device="cuda")
    nodes = torch.zeros(1, dtype=torch.int64, device="cuda")
    if mode == "plain":
        engine.count_cases_device(n, start_i, stop_i, d_cyc.data_ptr(), len(cycles),
                                  counts.data_ptr(), nodes.data_ptr())
    else:
        ws = torch.empty(engine.sym_workspace_bytes(), dtype=torch.uint8, device="cuda")
        engine.count_cases_batched_device(n, start_i, stop_i, d_cyc.data_ptr(), len(cycles),
                                          counts.data_ptr(), ws.data_ptr(), ws.numel(),
                                          nodes.data_ptr())
    torch.cuda.synchronize()
    return counts.cpu().numpy().view(np.uint64), int(nodes.item())


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_per_case_counts_and_nodes_7x7(engine, cuda, orc, mode):
    plan = engine.SymPlan(7, 24)
    rng = np.random.default_rng(7)
    pick = np.sort(rng.choice(plan.total_cases, 600, replace=False))
    cyc_all, mult_all = plan.cases()
    cycles = cyc_all[pick]
    got, nodes = _device_counts(engine, cuda, 7, 24, 49, cycles, mode)
    total, want, w = orc.sym_count_cases(7, 24, cycles, None, threads=os.cpu_count() or 4)
    assert (got == want).all()
    assert nodes == w.nodes  # recurse_count calls, sym_fold.cpp:219


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_partial_depth_counts_8x8(engine, cuda, orc, mode):
    # stop_i < n*n counts cycles reaching stop_i cells (the expansion index).
    plan = engine.SymPlan(8, 24)
    cycles, _ = plan.cases(1000, 300)
    got, _ = _device_counts(engine, cuda, 8, 24, 30, cycles, mode)
    want = [orc.sym_count_to(8, c, 24, 30)[0] for c in cycles]
    assert list(got) == want


def test_batched_equals_plain_on_skewed_cases(engine, cuda):
    # 1225 6x6 representatives of very uneven size force device-side splits.
    plan = engine.SymPlan(6)
    cycles, _ = plan.cases()
    plain, n1 = _device_counts(engine, cuda, 6, 16, 36, cycles, "plain")
    batched, n2 = _device_counts(engine, cuda, 6, 16, 36, cycles, "batched")
    assert (plain == batched).all()
    assert n1 == n2


def test_full_7x7(engine, cuda, golden):
    ans, st = engine.sym_fold(7, mode="batched", with_stats=True)
    assert ans == golden["published"]["squares"]["7"]
    assert st.splits > 0


def test_malformed_case_reported(engine, cuda):
    torch = cuda
    plan = engine.SymPlan(7, 24)
    cycles, _ = plan.cases(0, 8)
    cycles = cycles.copy()
    cycles[3, 0] = 60  # points outside the placed cells
    got, _ = _device_counts(engine, torch, 7, 24, 49, cycles, "plain")
    assert got[3] == np.uint64(2**64 - 1)
    assert (got[[0, 1, 2, 4]] != np.uint64(2**64 - 1)).all()


def _wasm_vectors():
    return json.loads((ROOT / "tests" / "golden" / "wasm_vectors.json").read_text())


@pytest.mark.parametrize("idx", range(3))
def test_solve_cases_contract(engine, cuda, orc, idx):
    vec = _wasm_vectors()["cases"][idx]
    n, depth, stop = vec["n"], vec["depth"], vec["stopDepth"]
    cycles = np.array(vec["prefix_bytes"], np.uint8)
    mults = [1] * len(cycles)
    buf = engine.pack_case_buffer(cycles, mults, n)
    count, nodes, status = engine.solve_cases(n, depth, stop, buf, len(cycles))
    assert status == 0
    assert count == vec["expected"]
    want_nodes = sum(orc.sym_count_to(n, c, depth, stop)[1].nodes for c in cycles)
    assert nodes == want_nodes


def test_solve_cases_multiplier(engine, cuda, orc):
    plan = engine.SymPlan(6)
    cycles, mults = plan.cases(0, 40)
    buf = engine.pack_case_buffer(cycles, mults, 6)
    count, nodes, status = engine.solve_cases(6, 16, 36, buf, 40)
    total, per, w = orc.sym_count_cases(6, 16, cycles, mults, threads=4)
    assert status == 0 and count == total


def test_solve_cases_mfah_campaign(engine, cuda, orc, golden):
    """The bounded 7x7 campaign of mfah/README.md:59-68 through solve_cases,
    as its coordinator hands it out: the raw 14-cell prefixes in units of 64
    (MFAH_PREFIXES_PER_UNIT), each counted to 28 cells; the units' counts
    total 35044546."""
    prefixes = orc.sym_raw_prefixes(7, 14)
    total = 0
    for k in range(0, len(prefixes), 64):
        unit = prefixes[k:k + 64]
        buf = engine.pack_case_buffer(unit, [1] * len(unit), 7)
        count, nodes, status = engine.solve_cases(7, 14, 28, buf, len(unit))
        assert status == 0
        total += count
    assert total == golden["published"]["mfah_7x7_d14_s28"]


def _cli(name, *args, env=None):
    from map_folding_gb300 import build

    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([str(build.BIN / name), *map(str, args)], capture_output=True,
                          text=True, env=e)


def test_sym_fold_cli_stream_chunk(engine, cuda, golden):
    r = _cli("sym_fold", 8, 16, 200, 0, env={"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "36"})
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == str(golden["sym"]["8x8_d36_first200"])
    assert "stream_seed_cases=1225 stream_from=16 stream_to=36" in r.stderr
    assert "completed=200" in r.stderr
    assert "n=8 threads=16 max_cases=200 start_case=0 total_s=" in r.stderr


def test_sym_fold_cli_progress_lines_7x7(engine, cuda, golden):
    """The whole 7x7 through the CLI: the answer (the chunk runs as pieces
    whose counts add up), and the reference's `progress=c/total rate=
    elapsed_s=` lines every 5 s while it runs (sym_fold.cpp:442-454)."""
    import re

    r = _cli("sym_fold", 7, 4)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == str(golden["published"]["squares"]["7"])
    lines = re.findall(r"^progress=(\d+)/(\d+) rate=[0-9.e+-]+/s elapsed_s=([0-9.e+-]+)$",
                       r.stderr, re.M)
    assert len(lines) >= 3, r.stderr  # two or more ticks, then the final line
    done = [int(c) for c, _, _ in lines]
    assert all(t == "433131" for _, t, _ in lines)
    assert done == sorted(done) and done[-1] == 433131
    assert float(lines[0][2]) >= 4.5


def test_sym_fold_cli_full_6(engine, cuda, golden):
    for mode in ("plain", "batched"):
        r = _cli("sym_fold", 6, 4, env={"MF_GPU_MODE": mode})
        assert r.returncode == 0, r.stderr
        assert r.stdout.strip() == str(golden["sym"]["n6"])
        assert "center_cases=9394" in r.stderr and "reduced_cases=1225" in r.stderr


def test_gpu_folding_cli(engine, cuda, golden):
    r = _cli("gpu_folding", 5, 15)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == ["Number of partial states at depth 15: 13416",
                                     f"Total number of ways: {golden['lunnon']['5x5']}"]
    r = _cli("gpu_folding", 4, 6, "plain", "3x6")
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines()[-1] == f"Total number of ways: {golden['lunnon']['3x6']}"


def test_concurrent_host_threads_match_sequential(engine, cuda, golden):
    """Host-buffer entry points called from several threads at once (ctypes
    releases the GIL) give the same counts as one after another."""
    from concurrent.futures import ThreadPoolExecutor

    plan7 = engine.SymPlan(7, 24)
    lplan = engine.LunnonPlan((4, 5))
    jobs = [lambda: plan7.solve(2000, 0)[0], lambda: plan7.solve(500, 300000)[0],
            lambda: lplan.count(-1)[0], lambda: engine.sym_fold(6)] * 3
    try:
        with ThreadPoolExecutor(max_workers=6) as ex:
            got = list(ex.map(lambda f: f(), jobs))
    finally:
        plan7.close()
        lplan.close()
    want = [golden["sym"]["7x7_d24_first2000"], golden["sym"]["7x7_d24_300000+500"],
            golden["lunnon"]["4x5"], golden["published"]["squares"]["6"]] * 3
    assert got == want


def test_empty_and_ragged_chunks(engine, cuda, golden):
    """Chunk edge cases (sym_fold.cpp:416-426, 536-545; modal_sym.py:166-172): a chunk
    at or past the last case counts 0, a chunk running past the end stops
    there, and chunks that tile the cases sum to the whole count."""
    plan = engine.SymPlan(6)
    try:
        total = plan.total_cases
        assert plan.solve(10, total)[0] == 0
        assert plan.solve(0, total + 5)[0] == 0
        head, _ = plan.solve(500, 0)
        tail, st = plan.solve(10 * total, 500)
        assert st.units == total - 500
        assert head + tail == golden["published"]["squares"]["6"]
        assert plan.solve(1000, total - 3)[0] == plan.solve(3, total - 3)[0]
    finally:
        plan.close()


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_lunnon_ranges_tile_the_count(engine, cuda, golden, mode):
    """Prefix-state ranges (gpu_folding_v2's max_states): a range past the
    last state counts 0 and consecutive ranges sum to the whole map."""
    plan = engine.LunnonPlan((4, 5))
    states = plan.count_prefixes(10)
    assert plan.count_range(10, states, 0, mode)[:2] == (0, 0)
    parts = [plan.count_range(10, s, 37, mode) for s in range(0, states, 37)]
    assert sum(p[1] for p in parts) == states
    assert sum(p[0] for p in parts) == golden["lunnon"]["4x5"]
