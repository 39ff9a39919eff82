"""Generate tests/golden/reference_counts.json from the reference's own CPU
solvers, built from source by `make -C oracle ref` into oracle/_ref/.

    python tests/golden/make_golden.py          # needs oracle/_ref/{mf,mf_fast,sym_fold}
    python tests/golden/make_golden.py --cost   # refresh only the cost-order vectors
    python tests/golden/make_golden.py --sym9   # refresh only the sym_fold9 (9x9) vectors
    python tests/golden/make_golden.py --sym9-deep  # add the 9x9 chunks expanded past 64 cells
    python tests/golden/make_golden.py --high-dim  # refresh only the 3- to 5-D Lunnon maps
    python tests/golden/make_golden.py --published # rewrite only the published values
    python tests/golden/make_golden.py --serving   # the serving stream's 8x8 chunks (hours, resumable)

Every value in the output was printed by an unmodified reference binary on
this machine; published values quoted in the reference's documents are kept
in a separate section with their source lines.  The oracle restatement and
the GPU engine are both checked against this file.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF = ROOT / "oracle" / "_ref"


def run(cmd, env=None):
    e = dict(os.environ)
    e.update(env or {})
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, env=e, check=True)
    return res.stdout.strip().splitlines()[0].strip()


def run_with_stderr(cmd, env=None):
    e = dict(os.environ)
    e.update(env or {})
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, env=e, check=True)
    return res.stdout.strip().splitlines()[0].strip(), res.stderr


def cost_jobs():
    """Chunks of the materialized case list reordered by MF_COST_DEPTH /
    MF_SORT_CASES (sym_fold.cpp:267-314).  Shallow depths give many equal
    (score, multiplier) keys, so these pin the unstable sort's order too."""
    return [
        ("7x7_cost2_desc_300000+300", [REF / "sym_fold", 7, 8, 300, 300000],
         {"MF_COST_DEPTH": "2", "MF_SORT_CASES": "1"}),
        ("7x7_cost3_desc_200000+400", [REF / "sym_fold", 7, 8, 400, 200000],
         {"MF_COST_DEPTH": "3", "MF_SORT_CASES": "desc"}),
        ("7x7_cost1_desc_100000+300", [REF / "sym_fold", 7, 8, 300, 100000],
         {"MF_COST_DEPTH": "1", "MF_SORT_CASES": "1"}),
        ("7x7_cost4_asc_30000+300", [REF / "sym_fold", 7, 8, 300, 30000],
         {"MF_COST_DEPTH": "4", "MF_SORT_CASES": "asc"}),
        ("7x7_cost2_unsorted_first200", [REF / "sym_fold", 7, 8, 200, 0], {"MF_COST_DEPTH": "2"}),
        ("6x6_cost3_desc_10+30", [REF / "sym_fold", 6, 8, 30, 10],
         {"MF_COST_DEPTH": "3", "MF_SORT_CASES": "1"}),
    ]


def cost_result(cmd, env):
    count, err = run_with_stderr(cmd, env)
    line = next(ln for ln in err.splitlines() if ln.startswith("cost_depth="))
    kv = dict(tok.split("=", 1) for tok in line.split())
    return {"count": int(count), "min_score": int(kv["min_score"]),
            "max_score": int(kv["max_score"]), "total_score": int(kv["total_score"]),
            "env": env, "args": [str(c) for c in cmd[1:]]}


def main_cost():
    """Add (or refresh) only the cost-order vectors in reference_counts.json."""
    path = HERE / "reference_counts.json"
    out = json.loads(path.read_text())
    with ThreadPoolExecutor(max_workers=2) as ex:
        futs = {k: ex.submit(cost_result, cmd, env) for k, cmd, env in cost_jobs()}
        out["sym_cost"] = {k: f.result() for k, f in futs.items()}
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(json.dumps(out["sym_cost"], indent=1, sort_keys=True))


def sym9_jobs():
    """experiments/9x9/sym_fold9.cpp (128-bit masks, 5x5 centre): 9x9 chunks
    deep enough to finish in seconds, the 5x5 centre on 7x7, and the 128-bit
    path on 8x8 (which must agree with sym_fold)."""
    s9 = REF / "sym_fold9"
    c5 = {"MF_CENTER_N": "5", "MF_CENTER_STREAM_DEDUP": "1", "MF_STREAM_CASES": "1"}
    return [
        ("9x9_c5_d42_first100", [s9, 9, 8, 100, 0], dict(c5, MF_EXPANDED_N="42")),
        ("9x9_c5_d40_1000000+100", [s9, 9, 8, 100, 1000000], dict(c5, MF_EXPANDED_N="40")),
        ("9x9_c5_d44_first300", [s9, 9, 8, 300, 0], dict(c5, MF_EXPANDED_N="44")),
        ("9x9_c5_d48_5000+2000", [s9, 9, 8, 2000, 5000], dict(c5, MF_EXPANDED_N="48")),
        ("7x7_c5_d30_first2000", [s9, 7, 8, 2000, 0], dict(c5, MF_EXPANDED_N="30")),
        ("8x8_c4_d36_first200", [s9, 8, 8, 200, 0], {"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "36"}),
        ("9x9_c5_seed1000x10_d44_20+300", [s9, 9, 8, 300, 20],
         dict(c5, MF_EXPANDED_N="44", MF_SEED_START="1000", MF_SEED_COUNT="10")),
    ]


def sym9_deep_jobs():
    """sym_fold9 with MF_EXPANDED_N past 64 cells (sym_fold9.cpp:1094-1099
    allows up to n*n): streamed chunks of the 5x5-centre 9x9 cases."""
    s9 = REF / "sym_fold9"
    c5 = {"MF_CENTER_N": "5", "MF_CENTER_STREAM_DEDUP": "1", "MF_STREAM_CASES": "1"}
    return [
        ("9x9_c5_d66_first100", [s9, 9, 8, 100, 0], dict(c5, MF_EXPANDED_N="66")),
        ("9x9_c5_d72_first100", [s9, 9, 8, 100, 0], dict(c5, MF_EXPANDED_N="72")),
        ("9x9_c5_d66_3000+200", [s9, 9, 8, 200, 3000], dict(c5, MF_EXPANDED_N="66")),
        ("9x9_c5_d80_first50", [s9, 9, 8, 50, 0], dict(c5, MF_EXPANDED_N="80")),
    ]


def main_sym9_deep():
    """Add (or refresh) only the past-64-cell sym_fold9 chunks."""
    path = HERE / "reference_counts.json"
    with ThreadPoolExecutor(max_workers=2) as ex:
        futs = {k: ex.submit(run, cmd, env) for k, cmd, env in sym9_deep_jobs()}
        res = {k: {"count": int(futs[k].result()), "env": env, "args": [str(c) for c in cmd[1:]]}
               for k, cmd, env in sym9_deep_jobs()}
    out = json.loads(path.read_text())
    out.setdefault("sym9", {}).update(res)
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(json.dumps(res, indent=1, sort_keys=True))


def sym9_setup():
    """Centre statistics of the 9x9 5x5-centre setup (stderr key=value)."""
    _, err = run_with_stderr([REF / "sym_fold9", 9, 1],
                             {"MF_CENTER_N": "5", "MF_SETUP_ONLY": "1"})
    out = {}
    for line in err.splitlines():
        for tok in line.split():
            if "=" in tok:
                k, v = tok.split("=", 1)
                if k in ("center_size", "center_cases", "reduced_cases") and v.isdigit():
                    out[k] = int(v)
    return out


def main_sym9():
    """Add (or refresh) only the sym_fold9 vectors in reference_counts.json."""
    path = HERE / "reference_counts.json"
    out = json.loads(path.read_text())
    with ThreadPoolExecutor(max_workers=2) as ex:
        futs = {k: ex.submit(run, cmd, env) for k, cmd, env in sym9_jobs()}
        setup = ex.submit(sym9_setup)
        out["sym9"] = {k: {"count": int(f.result()), "env": env,
                           "args": [str(c) for c in cmd[1:]]}
                       for (k, cmd, env), f in zip(sym9_jobs(), futs.values())}
        out["sym9_setup"] = setup.result()
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(json.dumps({"sym9": out["sym9"], "sym9_setup": out["sym9_setup"]}, indent=1,
                     sort_keys=True))


def lunnon_jobs():
    jobs = []
    for p in range(2, 7):
        for q in range(p, 7):
            if (p, q) == (6, 6):
                continue  # ~15 min single-threaded; the published value is used
            jobs.append((f"{p}x{q}", [REF / "mf", p, q]))
    for k in range(8, 21):
        jobs.append((f"1x{k}", [REF / "mf", 1, k]))
    for k in range(1, 6):
        jobs.append((f"2x2x{k}", [REF / "mf", 2, 2, k]))
    jobs.append(("1x1", [REF / "mf", 1, 1]))
    jobs.append(("2x3x4", [REF / "mf", 2, 3, 4]))
    jobs.extend(high_dim_jobs())
    return jobs


# Maps of three to five dimensions beyond the 2x2xk family (mf.c takes any
# number of dimensions); each runs in a few seconds at most.
HIGH_DIM_SHAPES = [(2, 2, 6), (3, 3, 3), (2, 2, 2, 2), (2, 2, 2, 3), (2, 2, 2, 2, 2)]


def high_dim_jobs():
    return [("x".join(map(str, d)), [REF / "mf", *d]) for d in HIGH_DIM_SHAPES]


def main_high_dim():
    """Refresh only the higher-dimensional Lunnon counts in the golden file."""
    path = HERE / "reference_counts.json"
    out = json.loads(path.read_text())
    with ThreadPoolExecutor(max_workers=os.cpu_count()) as ex:
        futs = {k: ex.submit(run, cmd) for k, cmd in high_dim_jobs()}
        for k, f in futs.items():
            out["lunnon"][k] = int(f.result())
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(json.dumps({k: out["lunnon"][k] for k in futs}, indent=1, sort_keys=True))


def prefix_jobs():
    out = []
    for grid, depth in [(4, 8), (5, 12), (5, 15), (6, 12), (6, 18), (7, 18), (7, 23)]:
        out.append((f"{grid}x{grid}@{depth}", [REF / "mf_fast", grid, depth, 1]))
    return out


def sym_jobs():
    jobs = []
    for n in range(1, 7):
        jobs.append((f"n{n}", [REF / "sym_fold", n, 8], {}))
    jobs.append(("7x7_d24_first2000", [REF / "sym_fold", 7, 8, 2000, 0], {"MF_STREAM_CASES": "1"}))
    jobs.append(("7x7_d24_300000+500", [REF / "sym_fold", 7, 8, 500, 300000], {"MF_STREAM_CASES": "1"}))
    jobs.append(("7x7_d28_first2000", [REF / "sym_fold", 7, 8, 2000, 0],
                 {"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "28"}))
    jobs.append(("8x8_d36_first200", [REF / "sym_fold", 8, 8, 200, 0],
                 {"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "36"}))
    jobs.append(("8x8_d36_120000000+200", [REF / "sym_fold", 8, 8, 200, 120000000],
                 {"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "36"}))
    jobs.append(("8x8_d36_240192700+500", [REF / "sym_fold", 8, 8, 500, 240192700],
                 {"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "36"}))
    jobs.append(("8x8_d24_case400000", [REF / "sym_fold", 8, 8, 1, 400000], {"MF_EXPANDED_N": "24"}))
    jobs.append(("8x8_d32_first100", [REF / "sym_fold", 8, 8, 100, 0],
                 {"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "32"}))
    return jobs


def setup_jobs():
    jobs = []
    for n, e in [(7, 24), (8, 24), (8, 28), (8, 36)]:
        jobs.append((f"{n}x{n}_d{e}", [REF / "sym_fold", n, 1],
                     {"MF_EXPANDED_N": str(e), "MF_SETUP_ONLY": "1"}))
    return jobs


PUBLISHED = {
    "squares": {  # mfah/folding.py:8-17
        "1": 1, "2": 8, "3": 1368, "4": 300608, "5": 186086600, "6": 123912532224,
        "7": 129950723279272, "8": 162403827553180928,
    },
    "prefix_states": {  # EXPERIMENTS.md:35-47
        "7x7@18": 293428, "7x7@20": 751142, "7x7@22": 5917082, "7x7@23": 8783910,
        "8x8@20": 1428966, "8x8@22": 3658148, "8x8@24": 8377532,
    },
    "sym_8x8_expanded_cases": {  # EXPERIMENTS.md:65-71
        "24": 414992, "26": 2512120, "28": 5158056, "30": 9447816, "32": 66351430,
        "34": 125889268, "36": 240192829,
    },
    "sym_8x8_partial_sums": {  # EXPERIMENTS.md:77-81
        "d24_case100000": 961512726016, "d24_case400000": 39987229696,
        "d32_first1000": 4354325657600, "d36_first100000": 35390073426944,
    },
    # mfah/README.md:59-68: the bounded 7x7 volunteer campaign (raw prefixes
    # at 14 cells, counted to 28 cells) "currently totals 35044546"
    "mfah_7x7_d14_s28": 35044546,
    "sources": "mfah/folding.py:8-17, EXPERIMENTS.md:35-47,65-71,77-81, mfah/README.md:59-68",
}


def serving_chunks(seed=5, requests=12, rate=0.15):
    """The 8x8 chunk requests of the serving benchmark's default stream:
    50,000 consecutive depth-36 cases from seeded uniform starts."""
    sys.path.insert(0, str(ROOT))
    from map_folding_gb300.workloads import serving_stream

    return [(r.start_case, r.max_cases) for r in serving_stream(seed, requests, rate)
            if r.kind == "chunk"]


def main_serving():
    """Count every 8x8 chunk of the serving stream with the reference's own
    sym_fold (MF_STREAM_CASES=1 MF_EXPANDED_N=36, all host threads).  Each
    chunk takes minutes to an hour of CPU, so results are written into
    reference_counts.json["sym_serving"] one chunk at a time and chunks that
    are already there are skipped: the run can be stopped and resumed."""
    path = HERE / "reference_counts.json"
    threads = str(os.cpu_count())
    for start, cases in serving_chunks():
        key = f"8x8_d36_{start}+{cases}"
        out = json.loads(path.read_text())
        if key in out.get("sym_serving", {}):
            continue
        count = run([REF / "sym_fold", 8, threads, cases, start],
                    {"MF_STREAM_CASES": "1", "MF_EXPANDED_N": "36"})
        out = json.loads(path.read_text())
        out.setdefault("sym_serving", {})[key] = {"count": int(count), "start_case": start,
                                                  "max_cases": cases, "expanded_n": 36}
        path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
        print(key, count, flush=True)


def main_published():
    """Rewrite only the published section (values quoted from the reference's documents)."""
    path = HERE / "reference_counts.json"
    out = json.loads(path.read_text())
    out["published"] = PUBLISHED
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")


def main():
    for b in ("mf", "mf_fast", "sym_fold", "sym_fold9"):
        if not (REF / b).exists():
            sys.exit(f"missing {REF / b}: run `make -C oracle ref` first")
    out = {"generated_by": "tests/golden/make_golden.py from oracle/_ref binaries",
           "lunnon": {}, "prefix_states": {}, "sym": {}, "sym_setup": {},
           "published": PUBLISHED}
    with ThreadPoolExecutor(max_workers=os.cpu_count()) as ex:
        lf = {k: ex.submit(run, cmd) for k, cmd in lunnon_jobs()}
        pf = {k: ex.submit(run, cmd, {"MF_COLLECT_ONLY": "1"}) for k, cmd in prefix_jobs()}
        sf = {k: ex.submit(run, cmd, env) for k, cmd, env in sym_jobs()}
        uf = {k: ex.submit(run, cmd, env) for k, cmd, env in setup_jobs()}
        cf = {k: ex.submit(cost_result, cmd, env) for k, cmd, env in cost_jobs()}
        nf = {k: ex.submit(run, cmd, env) for k, cmd, env in sym9_jobs()}
        n9 = ex.submit(sym9_setup)
        for k, f in lf.items():
            out["lunnon"][k] = int(f.result())
        for k, f in pf.items():
            out["prefix_states"][k] = int(f.result())
        for k, f in sf.items():
            out["sym"][k] = int(f.result())
        for k, f in uf.items():
            out["sym_setup"][k] = int(f.result())
        out["sym_cost"] = {k: f.result() for k, f in cf.items()}
        out["sym9"] = {k: {"count": int(nf[k].result()), "env": env, "args": [str(c) for c in cmd[1:]]}
                       for k, cmd, env in sym9_jobs()}
        out["sym9_setup"] = n9.result()
    (HERE / "reference_counts.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    if "--cost" in sys.argv:
        main_cost()
    elif "--sym9-deep" in sys.argv:
        main_sym9_deep()
    elif "--sym9" in sys.argv:
        main_sym9()
    elif "--high-dim" in sys.argv:
        main_high_dim()
    elif "--published" in sys.argv:
        main_published()
    elif "--serving" in sys.argv:
        main_serving()
    else:
        main()
