"""Generate tests/golden/work_counts.json: the algorithmic work of the bench
workload, counted by the CPU oracle (oracle/oracle.c).

    python tests/golden/make_work_counts.py               # ~35 min on 8 cores
    python tests/golden/make_work_counts.py --ref-sample  # ~30 s; adds the sample only

For the whole 7x7 count (all 433,131 cases at MF_EXPANDED_N=24) it records
the reference nodes (recurse_count calls, sym_fold.cpp:219) and the chain
steps (iterations of get_good's cycle walk, sym_fold.cpp:189-196).  These are
the per-step work figures bench.py quotes throughput in; the GPU kernel's own
node counter must equal `nodes` (bench.py checks the count and reports both).
Unlike reference_counts.json these numbers come from the oracle, not from a
reference binary; the oracle is pinned to the reference by the tests.

`7x7_d24_ref_sample` is the bounded sample bench.py's reference arm runs the
reference's own sym_fold binary on: four chunks of 2,000 consecutive cases
(`sym_fold 7 <threads> 2000 <start>`) at evenly spaced starts over the case
list.  The binary prints only the answer, so the sample's nodes (the rate's
numerator) and each chunk's answer (checked against the binary's) are
counted here.
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))


REF_SAMPLE_CHUNKS = 4
REF_SAMPLE_CASES = 2000


def ref_sample(oracle, cyc, mult, threads):
    n = len(cyc)
    chunks = []
    for k in range(REF_SAMPLE_CHUNKS):
        s = round(k * (n - REF_SAMPLE_CASES) / (REF_SAMPLE_CHUNKS - 1))
        total, _, w = oracle.sym_count_cases(7, 24, cyc[s:s + REF_SAMPLE_CASES].copy(),
                                             mult[s:s + REF_SAMPLE_CASES].copy(), threads)
        chunks.append({"start_case": s, "max_cases": REF_SAMPLE_CASES,
                       "answer": int(total) * 49, "nodes": int(w.nodes)})
    return {"chunks": chunks, "nodes": sum(c["nodes"] for c in chunks)}


def main():
    from oracle import oracle

    threads = os.cpu_count() or 1
    cyc, mult = oracle.sym_expand(7, 24, 0, 0)
    path = HERE / "work_counts.json"
    if "--ref-sample" in sys.argv[1:]:
        out = json.loads(path.read_text())
        out["7x7_d24_ref_sample"] = ref_sample(oracle, cyc, mult, threads)
        path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
        print(json.dumps(out["7x7_d24_ref_sample"], indent=1))
        return
    t0 = time.time()
    total, _, w = oracle.sym_count_cases(7, 24, cyc, mult, threads)
    out = {
        "generated_by": "tests/golden/make_work_counts.py (oracle/oracle.c work counters)",
        "7x7_d24_all": {
            "cases": int(len(cyc)),
            "answer": int(total) * 49,
            "nodes": int(w.nodes),
            "steps": int(w.steps),
            "cpu_s": round(time.time() - t0, 1),
            "cpu_threads": threads,
        },
        "7x7_d24_ref_sample": ref_sample(oracle, cyc, mult, threads),
    }
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
