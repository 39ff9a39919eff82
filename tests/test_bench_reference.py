"""bench.py's reference arm runs the reference's own CPU solver (sym_fold.cpp,
built from the copy oracle/Makefile stages) on the host cores, no GPU, and
prints one JSON line in the bench contract's shape; where that source is not
staged or does not build, it runs the oracle's restatement and says why."""
import importlib.util
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _bench_module():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_arm_line():
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         check=True, timeout=900)
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "nodes/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["metric"].startswith("7x7 sym_fold count")
    cpu = d["cpu_baseline"]
    assert cpu["kind"] in ("reference", "port") and cpu["cores"] >= 1
    assert cpu["value"] == d["value"]
    if cpu["kind"] == "port":
        assert d["reference_unavailable"]
    assert d["e2e"] == {"value": d["value"], "unit": "nodes/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_sample_fixture():
    """The sample's chunks lie inside the 433,131-case list, its nodes add up,
    and the lightest chunk's answer and nodes are the oracle's count of those
    cases."""
    import os

    bench = _bench_module()
    sample = bench.reference_sample()
    chunks = sample["chunks"]
    assert len(chunks) == 4
    assert all(0 <= c["start_case"] and c["start_case"] + c["max_cases"] <= 433131 for c in chunks)
    assert sample["nodes"] == sum(c["nodes"] for c in chunks)
    from oracle import oracle

    oracle.build()
    c = min(chunks, key=lambda c: c["nodes"])
    cyc, mult = oracle.sym_expand(7, 24, c["start_case"], c["max_cases"])
    total, _, w = oracle.sym_count_cases(7, 24, cyc, mult, os.cpu_count() or 1)
    assert total * 49 == c["answer"] and w.nodes == c["nodes"]


def test_reference_binary_missing_source(tmp_path):
    """Without the staged source the arm reports why instead of failing."""
    bench = _bench_module()
    bench.REF_SRC = tmp_path / "sym_fold.cpp"
    bench.REF_BIN = tmp_path / "bin" / "sym_fold"
    binary, why = bench.reference_sym_fold()
    assert binary is None and "not staged" in why


def test_reference_binary_build_failure(tmp_path):
    """A source that does not compile is reported, not raised."""
    bench = _bench_module()
    src = tmp_path / "sym_fold.cpp"
    src.write_text("this is not C++\n")
    bench.REF_SRC = src
    bench.REF_BIN = tmp_path / "bin" / "sym_fold"
    binary, why = bench.reference_sym_fold()
    assert binary is None and why.startswith("building sym_fold.cpp failed")
