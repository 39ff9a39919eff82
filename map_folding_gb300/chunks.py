"""Chunked sym_fold sweeps with the reference's JSONL record format.

Mirrors modal_sym.py (run_chunk :88-137, sweep :152-236, validate
:239-250, summarize_jsonl :36-77) with the GPU engine doing the counting on
this machine instead of remote CPU containers.  Rows carry exactly the keys
modal_sym.py writes (sorted on write):

    completed_hint, count (decimal string), expanded_n, max_cases, n,
    start_case, stderr_tail (last 6 stderr lines), threads, wall_s

    python -m map_folding_gb300.chunks sweep --n 8 --expanded-n 36 \
        --chunk-size 50000 --chunk-count 4 --out results/8x8.jsonl
    python -m map_folding_gb300.chunks validate --out results/8x8.jsonl --chunk-size 50000

Cost-weighted chunks (the balancing docs/8x8-method.md:128 proposes and the
reference does not build): `plan_cost_chunks` scores every case with a
shallow estimate_work lookahead on the GPU and cuts the case range into
contiguous chunks of about equal estimated cost, so rows keep the
(start_case, max_cases) form; `sweep(chunk_plan=...)` runs such a plan and
`validate(..., chunk_size=0)` checks that the rows tile the case range.

    python -m map_folding_gb300.chunks sweep --n 8 --expanded-n 36 \
        --cost-depth 4 --chunk-count 4804 --out results/8x8-cost.jsonl
    python -m map_folding_gb300.chunks validate --out results/8x8-cost.jsonl --chunk-size 0
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import time
from datetime import datetime, timezone
from pathlib import Path

TOTAL_8X8_DEPTH36_CASES = 240_192_829  # modal_sym.py:13


def parse_result(stdout: str) -> str:
    """First all-digit stdout line (modal_sym.py:28-33)."""
    for line in stdout.splitlines():
        text = line.strip()
        if text.isdigit():
            return text
    return ""


def summarize_jsonl(path: Path, total_cases: int, chunk_size: int) -> dict:
    """Coverage and sum of a sweep file (modal_sym.py:36-77).  chunk_size <=
    0 means variable-size chunks: the rows must tile [0, total_cases)."""
    rows = []
    path = Path(path)
    if path.exists():
        with path.open("r", encoding="utf-8") as f:
            for line_no, line in enumerate(f, 1):
                text = line.strip()
                if not text:
                    continue
                row = json.loads(text)
                row["_line_no"] = line_no
                rows.append(row)
    seen: dict[int, dict] = {}
    duplicate_starts = []
    for row in rows:
        start = int(row["start_case"])
        if start in seen:
            duplicate_starts.append(start)
        else:
            seen[start] = row
    if chunk_size > 0:
        expected_starts = list(range(0, total_cases, chunk_size))
        expected_set = set(expected_starts)
        missing = [s for s in expected_starts if s not in seen]
        extra = sorted(s for s in seen if s not in expected_set)
    else:
        # Variable chunks: walk the rows in start order; a gap is missing
        # cases (reported by its first case), an overlap is extra.
        missing, extra, pos = [], [], 0
        for start in sorted(seen):
            size = int(seen[start]["max_cases"])
            if start > pos:
                missing.append(pos)
            elif start < pos:
                extra.append(start)
            pos = max(pos, start + size)
        if pos < total_cases:
            missing.append(pos)
        expected_starts = sorted(seen) if not missing else sorted(seen) + missing
    unique_sum = sum(int(r["count"]) for r in seen.values())
    all_sum = sum(int(r["count"]) for r in rows)
    return {
        "path": str(path),
        "rows": len(rows),
        "unique_chunks": len(seen),
        "expected_chunks": len(expected_starts),
        "duplicate_count": len(duplicate_starts),
        "duplicate_starts": duplicate_starts[:20],
        "missing_count": len(missing),
        "missing_starts": missing[:20],
        "extra_count": len(extra),
        "extra_starts": extra[:20],
        "unique_sum": str(unique_sum),
        "all_rows_sum": str(all_sum),
        "complete": (not missing and not duplicate_starts and not extra and
                     (chunk_size <= 0 or len(seen) == len(expected_starts))),
    }


def _row(n, threads, expanded_n, start_case, max_cases, count, wall_s, stderr):
    matches = re.findall(r"completed=(\d+)", stderr)
    completed = int(matches[-1]) if matches else max_cases
    return {
        "n": n,
        "threads": threads,
        "expanded_n": expanded_n,
        "start_case": start_case,
        "max_cases": max_cases,
        "count": count,
        "wall_s": wall_s,
        "completed_hint": completed,
        "stderr_tail": "\n".join(stderr.splitlines()[-6:]),
    }


def run_chunk_cli(n: int, threads: int, expanded_n: int, start_case: int, max_cases: int,
                  mode: str = "batched") -> dict:
    """One chunk through the drop-in `sym_fold` binary, parsed the way
    modal_sym.py:95-137 parses the reference's."""
    from .build import BIN

    env = dict(os.environ, MF_STREAM_CASES="1", MF_EXPANDED_N=str(expanded_n), MF_GPU_MODE=mode)
    cmd = [str(BIN / "sym_fold"), str(n), str(threads), str(max_cases), str(start_case)]
    t0 = time.perf_counter()
    res = subprocess.run(cmd, env=env, text=True, capture_output=True, check=False)
    wall_s = time.perf_counter() - t0
    count = parse_result(res.stdout)
    if res.returncode != 0 or not count:
        raise RuntimeError(
            f"chunk failed start={start_case} max={max_cases} rc={res.returncode}\n"
            f"stdout:\n{res.stdout}\nstderr:\n{res.stderr}")
    return _row(n, threads, expanded_n, start_case, max_cases, count, wall_s, res.stderr)


class ChunkRunner:
    """In-process chunks over one resident plan (no per-chunk process or
    setup cost); produces the same row as run_chunk_cli."""

    def __init__(self, n: int, expanded_n: int, mode: str = "batched", threads: int = 1):
        from .api import SymPlan

        self.n, self.expanded_n, self.mode, self.threads = n, expanded_n, mode, threads
        self.plan = SymPlan(n, expanded_n)

    def run(self, start_case: int, max_cases: int) -> dict:
        t0 = time.perf_counter()
        ans, st = self.plan.solve(max_cases, start_case, self.mode)
        wall_s = time.perf_counter() - t0
        p = self.plan
        stderr = "\n".join([
            f"center_cases={p.center_cases}",
            f"reduced_cases={p.reduced_cases}",
            f"stream_seed_cases={p.reduced_cases} stream_from={16 if self.n % 2 == 0 else 9} "
            f"stream_to={self.expanded_n}",
            f"stream selected={st.units} completed={st.units} producer_done=1 "
            f"rate={st.units / wall_s if wall_s else 0:g}/s elapsed_s={wall_s:g}",
            f"n={self.n} threads={self.threads} max_cases={max_cases} start_case={start_case} "
            f"total_s={wall_s:g}",
        ])
        return _row(self.n, self.threads, self.expanded_n, start_case, max_cases, str(ans),
                    wall_s, stderr)


def plan_cost_chunks(n: int, expanded_n: int, chunk_count: int, cost_depth: int = 4,
                     start_case: int = 0, total_cases: int = 0, block: int = 1000,
                     mode: str = "batched") -> list[tuple[int, int]]:
    """Contiguous chunks of about equal estimated cost over [start_case,
    total_cases): block costs from the GPU (SymPlan.block_costs), then
    boundaries where the cumulative cost crosses k / chunk_count of the total."""
    from .api import SymPlan

    plan = SymPlan(n, expanded_n)
    try:
        total_cases = total_cases or plan.total_cases
        count = total_cases - start_case
        costs = plan.block_costs(start_case, count, cost_depth, block, mode)
    finally:
        plan.close()
    return partition_by_cost(costs, block, start_case, count, chunk_count)


def partition_by_cost(costs, block: int, start_case: int, count: int,
                      chunk_count: int) -> list[tuple[int, int]]:
    """Cut [start_case, start_case + count) at block boundaries into at most
    chunk_count contiguous, non-empty chunks of about equal summed cost."""
    import numpy as np

    if count <= 0 or chunk_count <= 0:
        return []
    csum = np.cumsum(np.asarray(costs, dtype=np.float64))
    total = float(csum[-1]) if len(csum) else 0.0
    cuts = [0]
    for k in range(1, chunk_count):
        b = int(np.searchsorted(csum, total * k / chunk_count, side="left")) + 1
        b = min(b, len(csum))
        if b > cuts[-1]:
            cuts.append(b)
    cases = [min(c * block, count) for c in cuts] + [count]
    out = []
    for a, b in zip(cases, cases[1:]):
        if b > a:
            out.append((start_case + a, b - a))
    return out


def sweep(n: int = 8, threads: int = 16, expanded_n: int = 36,
          total_cases: int = TOTAL_8X8_DEPTH36_CASES, chunk_size: int = 100000,
          start_case: int = 0, chunk_count: int = 0, out: str = "",
          resume_existing: bool = False, mode: str = "batched", in_process: bool = True,
          chunk_plan: list[tuple[int, int]] | None = None, max_seconds: float = 0.0) -> dict:
    """modal_sym.py:152-236 on the local GPU.  With chunk_plan, the given
    (start_case, max_cases) chunks run instead of equal-size ones.  With
    max_seconds > 0 no new chunk starts once that much wall time has passed
    (the rows written so far are the checkpoint; --resume-existing carries
    on from them), so a long sweep can run as bounded sessions."""
    if chunk_plan is not None:
        inputs = [(int(s), int(m)) for s, m in chunk_plan]
        if chunk_count > 0:
            inputs = inputs[:chunk_count]
        chunk_size = 0
    else:
        if chunk_size <= 0:
            raise ValueError("chunk_size must be positive")
        starts = list(range(start_case, total_cases, chunk_size))
        if chunk_count > 0:
            starts = starts[:chunk_count]
        inputs = [(s, min(chunk_size, total_cases - s)) for s in starts]
    if not inputs:
        raise ValueError("No chunks selected")
    if not out:
        stamp = datetime.now(timezone.utc).strftime("%Y%m%dT%H%M%SZ")
        out = f"results/{n}x{n}-depth{expanded_n}-{stamp}.jsonl"
    out_path = Path(out)
    out_path.parent.mkdir(parents=True, exist_ok=True)
    if resume_existing:
        summary = summarize_jsonl(out_path, total_cases, chunk_size)
        existing = set()
        if out_path.exists():
            for line in out_path.read_text(encoding="utf-8").splitlines():
                if line.strip():
                    existing.add(int(json.loads(line)["start_case"]))
        before = len(inputs)
        inputs = [item for item in inputs if item[0] not in existing]
        print(f"resume_existing=1 skipped={before - len(inputs)} remaining={len(inputs)} "
              f"existing_rows={summary['rows']} unique_chunks={summary['unique_chunks']}",
              flush=True)
        if not inputs:
            print(json.dumps(summary, indent=2, sort_keys=True), flush=True)
            return summary
    runner = ChunkRunner(n, expanded_n, mode, threads) if in_process else None
    total = 0
    done = 0
    started = time.perf_counter()
    print(f"chunks={len(inputs)} chunk_size={chunk_size} out={out_path}", flush=True)
    with out_path.open("a", encoding="utf-8") as f:
        for s, m in inputs:
            if max_seconds > 0 and time.perf_counter() - started >= max_seconds:
                print(f"stopped: max_seconds={max_seconds} reached after {done} chunks", flush=True)
                break
            row = runner.run(s, m) if runner else run_chunk_cli(n, threads, expanded_n, s, m, mode)
            done += 1
            total += int(row["count"])
            f.write(json.dumps(row, sort_keys=True) + "\n")
            f.flush()
            print(f"completed={done}/{len(inputs)} start={row['start_case']} "
                  f"wall_s={row['wall_s']:.2f} elapsed_s={time.perf_counter() - started:.1f}",
                  flush=True)
    summary = {
        "chunks": done,
        "chunk_size": chunk_size,
        "start_case": start_case,
        "total_cases": total_cases,
        "expanded_n": expanded_n,
        "partial_sum": str(total),
        "elapsed_s": time.perf_counter() - started,
        "out": str(out_path),
    }
    summary_path = out_path.with_suffix(out_path.suffix + ".summary.json")
    summary_path.write_text(json.dumps(summary, indent=2, sort_keys=True) + "\n", encoding="utf-8")
    print(json.dumps(summary, indent=2, sort_keys=True), flush=True)
    return summary


def validate(out: str, total_cases: int = TOTAL_8X8_DEPTH36_CASES, chunk_size: int = 50000,
             expected: str = "") -> dict:
    """modal_sym.py:239-250."""
    summary = summarize_jsonl(Path(out), total_cases, chunk_size)
    if expected:
        summary["expected"] = expected
        summary["matches_expected"] = summary["unique_sum"] == expected
    print(json.dumps(summary, indent=2, sort_keys=True), flush=True)
    return summary


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m map_folding_gb300.chunks")
    sub = ap.add_subparsers(dest="cmd", required=True)
    s = sub.add_parser("sweep")
    s.add_argument("--n", type=int, default=8)
    s.add_argument("--threads", type=int, default=16)
    s.add_argument("--expanded-n", type=int, default=36)
    s.add_argument("--total-cases", type=int, default=TOTAL_8X8_DEPTH36_CASES)
    s.add_argument("--chunk-size", type=int, default=100000)
    s.add_argument("--start-case", type=int, default=0)
    s.add_argument("--chunk-count", type=int, default=0)
    s.add_argument("--out", default="")
    s.add_argument("--resume-existing", action="store_true")
    s.add_argument("--mode", default="batched", choices=["plain", "batched"])
    s.add_argument("--cli", action="store_true", help="run each chunk through bin/sym_fold")
    s.add_argument("--cost-depth", type=int, default=0,
                   help="> 0: cost-weighted chunks (--chunk-count of them) scored this deep")
    s.add_argument("--max-seconds", type=float, default=0.0,
                   help="> 0: start no new chunk after this much wall time")
    v = sub.add_parser("validate")
    v.add_argument("--out", required=True)
    v.add_argument("--total-cases", type=int, default=TOTAL_8X8_DEPTH36_CASES)
    v.add_argument("--chunk-size", type=int, default=50000)
    v.add_argument("--expected", default="")
    a = ap.parse_args(argv)
    if a.cmd == "sweep":
        chunk_plan = None
        chunk_count = a.chunk_count
        if a.cost_depth > 0:
            if a.chunk_count <= 0:
                ap.error("--cost-depth needs --chunk-count")
            chunk_plan = plan_cost_chunks(a.n, a.expanded_n, a.chunk_count, a.cost_depth,
                                          a.start_case, a.total_cases, mode=a.mode)
            chunk_count = 0
        sweep(a.n, a.threads, a.expanded_n, a.total_cases, a.chunk_size, a.start_case,
              chunk_count, a.out, a.resume_existing, a.mode, not a.cli, chunk_plan,
              a.max_seconds)
    else:
        validate(a.out, a.total_cases, a.chunk_size, a.expected)


if __name__ == "__main__":
    main()
