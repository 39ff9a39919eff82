"""CPU tests of the engine's host side: the C ABI library, prefix-state
generation, sym case setup and argument checking.  No kernel runs here."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "mapfold.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\S.*?\b(mf_\w+)\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol(engine):
    from map_folding_gb300 import _native

    lib = _native.load()
    names = declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"
    assert lib.mf_abi_version() == 1


def test_exports_match_nm(engine):
    from map_folding_gb300 import _native

    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (mf_\w+)", out))
    assert set(declared_symbols()) <= exported


@pytest.mark.parametrize("dims,depth", [
    ((5, 5), 15), ((4, 4), 8), ((2, 3), 3), ((1, 12), 6), ((2, 2, 3), 5), ((3, 5), 0),
    ((2, 2), 4), ((4, 6), 12), ((2, 2, 5), 9), ((1, 1), 1), ((3, 3), 9), ((1, 20), 10),
    # up to six dimensions and the 64-leaf limit
    ((2, 2, 2, 2), 10), ((2, 2, 2, 2, 2), 14), ((3, 3, 3), 14), ((4, 4, 4), 12), ((8, 8), 10),
    ((1, 64), 16), ((2, 2, 2, 2, 2, 2), 12),
])
def test_prefix_states_match_oracle(engine, orc, dims, depth):
    plan = engine.LunnonPlan(dims)
    got = plan.collect(depth)
    a, b, g = orc.lunnon_collect(dims, depth)
    assert len(got) == len(b)
    assert (got[:, :plan.n + 1] == b).all()
    assert (got[:, plan.n + 1:] == 0).all()
    assert plan.stride % 16 == 0


def test_prefix_counts_match_reference(engine, golden):
    for key, want in golden["prefix_states"].items():
        shape, depth = key.split("@")
        grid = int(shape.split("x")[0])
        if grid >= 7:
            continue  # covered by the published table below
        assert engine.LunnonPlan((grid, grid)).count_prefixes(int(depth)) == want, key
    pub = golden["published"]["prefix_states"]
    assert engine.LunnonPlan((7, 7)).count_prefixes(18) == pub["7x7@18"]
    assert engine.LunnonPlan((7, 7)).count_prefixes(20) == pub["7x7@20"]


def test_lunnon_plan_rejects_bad_shapes(engine):
    with pytest.raises(engine.EngineError):
        engine.LunnonPlan((9, 9))
    with pytest.raises(engine.EngineError):
        engine.LunnonPlan((0, 3))
    with pytest.raises(engine.EngineError):
        engine.LunnonPlan(())
    plan = engine.LunnonPlan((3, 3))
    with pytest.raises(engine.EngineError):
        plan.count_prefixes(10)


@pytest.mark.parametrize("n", range(1, 9))
def test_edge_pages_match_oracle(engine, orc, n):
    assert (engine.sym_edges(n) == orc.sym_edges(n)).all()


@pytest.mark.parametrize("n", [6, 7])
def test_sym_plan_matches_oracle_and_reference(engine, orc, golden, n):
    plan = engine.SymPlan(n)
    cyc, mult, centers = orc.sym_reps(n)
    assert plan.center_cases == centers
    assert plan.reduced_cases == len(cyc)
    cases, mults = plan.cases()
    oc, om = orc.sym_expand(n, plan.start_i)
    assert len(cases) == len(oc) == plan.total_cases
    assert (cases[:, :plan.start_i] == oc[:, :plan.start_i]).all()
    assert (mults == om).all()
    if n == 7:
        assert plan.total_cases == golden["sym_setup"]["7x7_d24"]


def test_sym_plan_slices(engine, orc):
    plan = engine.SymPlan(7, 20)
    full, fm = plan.cases()
    for start, count in [(0, 1), (5, 100), (len(full) - 3, 10), (len(full), 5), (17, 0)]:
        c, m = plan.cases(start, count)
        end = len(full) if count == 0 else min(len(full), start + count)
        assert len(c) == max(end - start, 0)
        assert (c[:, :20] == full[start:end, :20]).all()
        assert (m == fm[start:end]).all()


def test_sym_plan_rejects_bad_depth(engine):
    with pytest.raises(engine.EngineError):
        engine.SymPlan(7, 8)
    with pytest.raises(engine.EngineError):
        engine.SymPlan(7, 50)
    with pytest.raises(engine.EngineError):
        engine.SymPlan(5)


def test_solve_cases_status_codes(engine):
    # mfah/wasm/sym_kernel.c:252-260: status 1 (n / case_count), 2 (range)
    assert engine.solve_cases(1, 3, 9, b"", 0)[2] == 1
    assert engine.solve_cases(10, 3, 9, b"", 0)[2] == 1
    assert engine.solve_cases(5, 3, 9, b"", 300)[2] == 1
    assert engine.solve_cases(5, 10, 9, b"", 0)[2] == 2
    assert engine.solve_cases(5, 3, 26, b"", 0)[2] == 2


def _cli(name, *args, env=None):
    from map_folding_gb300 import build

    exe = build.BIN / name
    return subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, env=env)


def test_gpu_folding_cli_usage(engine):
    r = _cli("gpu_folding")
    assert r.returncode == 1
    assert r.stdout.splitlines() == ["Usage: ./gpu_folding grid_size partition_depth",
                                     "Example: ./gpu_folding 20 8"]
    r = _cli("gpu_folding", 9, 4)
    assert r.returncode == 1 and r.stdout.strip() == "Grid too large, max 8 (64 stamps)"


def test_sym_fold_cli_argument_errors(engine):
    r = _cli("sym_fold")
    assert r.returncode == 1 and "Usage:" in r.stderr
    r = _cli("sym_fold", "x7")
    assert r.returncode == 2 and "Invalid n: x7" in r.stderr
    r = _cli("sym_fold", 9)
    assert r.returncode == 1 and "n must be between 1 and 8" in r.stderr
    r = _cli("sym_fold", 7, 0)
    assert r.returncode == 1 and "threads must be positive" in r.stderr
    r = _cli("sym_fold", 7, 4, "abc")
    assert r.returncode == 2 and "Invalid max_cases: abc" in r.stderr
    r = _cli("sym_fold", 1)
    assert r.returncode == 0 and r.stdout.strip() == "1"
    r = _cli("sym_fold", 2)
    assert r.returncode == 0 and r.stdout.strip() == "8"
    import os
    env = dict(os.environ, MF_EXPANDED_N="5")
    r = _cli("sym_fold", 7, 4, env=env)
    assert r.returncode == 1 and "MF_EXPANDED_N must be between 9 and 49" in r.stderr


def test_sym_fold_cli_setup_only(engine, golden):
    import os
    env = dict(os.environ, MF_SETUP_ONLY="1", MF_EXPANDED_N="24")
    r = _cli("sym_fold", 7, 4, env=env)
    assert r.returncode == 0
    assert int(r.stdout.strip()) == golden["sym_setup"]["7x7_d24"]
    assert "center_cases=76" in r.stderr and "reduced_cases=11" in r.stderr
    assert "expanded_cases=433131" in r.stderr and "setup_only=1" in r.stderr


def test_sym_fold_cli_queue_size_checked_in_stream_mode(engine):
    """sym_fold.cpp:539-542: the streaming solver parses MF_QUEUE_SIZE after
    the setup lines and exits 2 on bad text (the reference binary prints the
    same four stderr lines)."""
    import os
    env = dict(os.environ, MF_STREAM_CASES="1", MF_QUEUE_SIZE="abc")
    r = _cli("sym_fold", 7, 1, 10, 0, env=env)
    assert r.returncode == 2
    assert r.stderr.splitlines() == ["center_cases=76", "reduced_cases=11",
                                     "stream_seed_cases=11 stream_from=9 stream_to=24",
                                     "Invalid MF_QUEUE_SIZE: abc"]
    env = dict(os.environ, MF_SETUP_ONLY="1", MF_QUEUE_SIZE="abc")  # not read before solving
    assert _cli("sym_fold", 7, 1, env=env).returncode == 0
