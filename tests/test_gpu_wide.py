"""Boards over 64 cells: experiments/9x9/sym_fold9.cpp's 128-bit search and
5x5 centre.  The golden vectors were printed by the reference's own
sym_fold9 (tests/golden/make_golden.py --sym9).  The 128-bit kernel is also
checked against the 64-bit one on 7x7 and 8x8 chunks (stack_mode 2 selects
it for any board)."""
import os
import subprocess

import pytest

WIDE = {"stack_mode": 2}


def _vectors(golden):
    for key, v in sorted(golden["sym9"].items()):
        n, _threads, max_cases, start = (int(a) for a in v["args"])
        env = v["env"]
        c = int(env.get("MF_CENTER_N", "5" if n >= 9 else ("4" if n % 2 == 0 else "3")))
        e = int(env.get("MF_EXPANDED_N", max(24, c * c)))
        seed = (int(env.get("MF_SEED_START", 0)), int(env.get("MF_SEED_COUNT", 0)))
        yield key, n, c, e, seed, max_cases, start, v


def test_centre_setup_matches_reference(golden, engine):
    """CPU only: the 9x9 5x5-centre enumeration and D4 x reversal dedup."""
    p = engine.SymPlan(9, 25)
    try:
        s = golden["sym9_setup"]
        assert (p.center_cases, p.reduced_cases) == (s["center_cases"], s["reduced_cases"])
        assert p.total_cases == s["reduced_cases"]
    finally:
        p.close()


def test_sym_fold9_cli_setup(golden, engine):
    from map_folding_gb300 import build as mfbuild

    env = dict(os.environ, MF_CENTER_N="5", MF_SETUP_ONLY="1")
    res = subprocess.run([str(mfbuild.BIN / "sym_fold9"), "9", "1"], capture_output=True,
                         text=True, env=env, check=True)
    assert res.stdout.strip() == str(golden["sym9_setup"]["reduced_cases"])
    assert "center_size=5 center_cases=3721732" in res.stderr
    bad = subprocess.run([str(mfbuild.BIN / "sym_fold9"), "9", "1"], capture_output=True,
                         text=True, env=dict(os.environ, MF_CENTER_N="4"))
    assert bad.returncode == 2 and "MF_CENTER_N" in bad.stderr
    ten = subprocess.run([str(mfbuild.BIN / "sym_fold9"), "10", "1"], capture_output=True, text=True)
    assert ten.returncode == 1


@pytest.mark.gpu
def test_chunks_match_reference(golden, engine, cuda):
    plans = {}
    try:
        for key, n, c, e, seed, max_cases, start, v in _vectors(golden):
            k = (n, c, e, seed)
            if k not in plans:
                plans[k] = engine.SymPlan(n, e, center_n=c, seed_start=seed[0], seed_count=seed[1])
            ans, st = plans[k].solve(max_cases, start)
            assert ans == v["count"], key
    finally:
        for p in plans.values():
            p.close()


@pytest.mark.gpu
@pytest.mark.parametrize("key,n,e,max_cases,start", [
    ("7x7_d24_first2000", 7, 24, 2000, 0),
    ("7x7_d24_300000+500", 7, 24, 500, 300000),
    ("8x8_d36_first200", 8, 36, 200, 0),
    ("8x8_d36_240192700+500", 8, 36, 500, 240192700),
])
def test_wide_kernel_matches_on_small_boards(golden, engine, cuda, key, n, e, max_cases, start):
    plan = engine.SymPlan(n, e)
    try:
        ans, st = plan.solve(max_cases, start, "batched", WIDE)
        ans64, st64 = plan.solve(max_cases, start, "batched")
    finally:
        plan.close()
    assert ans == golden["sym"][key] == ans64
    assert st.nodes == st64.nodes  # the same reference nodes, counted by both kernels


@pytest.mark.gpu
def test_sym_fold9_cli_chunk(golden, engine, cuda):
    from map_folding_gb300 import build as mfbuild

    v = golden["sym9"]["9x9_c5_d44_first300"]
    env = dict(os.environ)
    env.update(v["env"])
    res = subprocess.run([str(mfbuild.BIN / "sym_fold9"), *v["args"]], capture_output=True,
                         text=True, env=env, check=True)
    assert res.stdout.strip() == str(v["count"])
    assert "stream_seed_cases=465883 stream_from=25 stream_to=44" in res.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["9x9_c5_d66_first100", "9x9_c5_d80_first50"])
def test_sym_fold9_cli_past_64_cells(golden, engine, cuda, key):
    """MF_EXPANDED_N past 64 cells (sym_fold9.cpp:1094-1099): 96-byte cases
    streamed in emission order, counted on the 128-bit kernel."""
    from map_folding_gb300 import build as mfbuild

    v = golden["sym9"][key]
    env = dict(os.environ)
    env.update(v["env"])
    res = subprocess.run([str(mfbuild.BIN / "sym_fold9"), *v["args"]], capture_output=True,
                         text=True, env=env, check=True)
    assert res.stdout.strip() == str(v["count"])


@pytest.mark.gpu
def test_past_64_cells_need_a_chunk_size(engine, cuda):
    """A streamed plan has no total: asking for all its cases is refused."""
    from map_folding_gb300._native import EngineError

    plan = engine.SymPlan(9, 66, center_n=5)
    try:
        assert plan.case_bytes == 96 and plan.total_cases == 0
        with pytest.raises(EngineError):
            plan.solve(0, 0)
    finally:
        plan.close()
