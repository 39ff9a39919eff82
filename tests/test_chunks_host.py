"""The chunk driver's host logic without a GPU: result parsing, the JSONL row
(modal_sym.py:127-137), fixed-size coverage summaries (:36-77), failing
chunks (:120-124) and a resumed sweep that skips chunks already on file."""
import json

import pytest

from map_folding_gb300 import chunks


def test_parse_result_takes_first_all_digit_line():
    assert chunks.parse_result("noise\n  152870282240 \n99\n") == "152870282240"
    assert chunks.parse_result("Total: 12\n") == ""


def test_row_keys_and_completed_hint():
    stderr = "\n".join(["center_cases=9394", "stream selected=10 completed=4 rate=1/s",
                        "stream selected=10 completed=10 rate=2/s", "a", "b", "c", "d"])
    row = chunks._row(8, 16, 36, 100, 10, "42", 1.5, stderr)
    assert sorted(row) == ["completed_hint", "count", "expanded_n", "max_cases", "n",
                           "start_case", "stderr_tail", "threads", "wall_s"]
    assert row["completed_hint"] == 10 and row["count"] == "42"
    assert row["stderr_tail"] == "\n".join(stderr.splitlines()[-6:])
    assert chunks._row(8, 16, 36, 100, 10, "42", 1.5, "")["completed_hint"] == 10


def _write(path, starts, size=10):
    with path.open("w") as f:
        for s in starts:
            f.write(json.dumps({"start_case": s, "max_cases": size, "count": str(s + 1)}) + "\n")


def test_fixed_size_summary(tmp_path):
    p = tmp_path / "s.jsonl"
    _write(p, [0, 10, 20])
    ok = chunks.summarize_jsonl(p, 30, 10)
    assert ok["complete"] and ok["unique_sum"] == str(1 + 11 + 21)
    _write(p, [0, 10, 10, 25])
    bad = chunks.summarize_jsonl(p, 30, 10)
    assert not bad["complete"]
    assert bad["duplicate_starts"] == [10] and bad["missing_starts"] == [20]
    assert bad["extra_starts"] == [25]


def test_failing_chunk_raises(engine):
    # n = 9 is outside sym_fold's range: rc 1, no count on stdout
    with pytest.raises(RuntimeError, match="chunk failed"):
        chunks.run_chunk_cli(9, 1, 36, 0, 10)


def test_sweep_resumes_without_repeating_chunks(tmp_path, monkeypatch):
    calls = []

    def fake(n, threads, expanded_n, s, m, mode):
        calls.append(s)
        return chunks._row(n, threads, expanded_n, s, m, str(s), 0.1, f"completed={m}")

    monkeypatch.setattr(chunks, "run_chunk_cli", fake)
    out = tmp_path / "sweep.jsonl"
    chunks.sweep(n=8, threads=2, expanded_n=36, total_cases=50, chunk_size=10, chunk_count=2,
                 out=str(out), in_process=False)
    assert calls == [0, 10]
    chunks.sweep(n=8, threads=2, expanded_n=36, total_cases=50, chunk_size=10, out=str(out),
                 resume_existing=True, in_process=False)
    assert calls == [0, 10, 20, 30, 40]
    summary = chunks.validate(str(out), total_cases=50, chunk_size=10)
    assert summary["complete"] and summary["unique_sum"] == str(0 + 10 + 20 + 30 + 40)


def _fixture():
    from pathlib import Path

    return json.loads((Path(__file__).resolve().parent / "golden" /
                       "jsonl_summaries.json").read_text())


def test_summaries_match_the_reference_function(tmp_path):
    """summarize_jsonl against the reference's own modal_sym.py:36-77 run on
    the same files (tests/golden/make_jsonl_summaries.py)."""
    for case in _fixture()["summaries"]:
        p = tmp_path / f"{case['name']}.jsonl"
        if case["jsonl"] is not None:
            p.write_text(case["jsonl"], encoding="utf-8")
        got = chunks.summarize_jsonl(p, case["total_cases"], case["chunk_size"])
        got["path"] = p.name
        assert got == case["summary"], case["name"]


def test_parse_result_matches_the_reference_function():
    for case in _fixture()["parse_result"]:
        assert chunks.parse_result(case["stdout"]) == case["result"], case["stdout"]
