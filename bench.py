#!/usr/bin/env python
"""Benchmark: the 7x7 symmetry-reduced full count on one GB300.

Workload (one "step"): count all 433,131 sym_fold cases of the 7x7 map
expanded to 24 cells (MF_EXPANDED_N=24, the reference default) to
completion, i.e. the whole 7x7 answer 129950723279272, with the batched
persistent work-stealing kernel.  Inputs are resident in HBM for `value`;
`e2e` runs the same count through the C ABI with host buffers (case
selection, host->device copy, kernel, device->host copy of per-case counts).
After the timed steps, on one GPU: the plain one-thread-per-case kernel
counts the same cases once (`batched_vs_plain`), and the serving stream's
8x8 chunks run through the request server (`serving`: chunk p50/p99, each
chunk checked against the reference's count).

Metric: reference DFS nodes per second -- recurse_count calls of
sym_fold.cpp:219, counted exactly by the kernel (and equal to the oracle's
count, which the GPU tests check) -- divided by device time.  ms_per_step is
the 7x7 wall time on the device.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N = 7
EXPANDED_N = 24
ANSWER_7X7 = 129950723279272
METRIC = "7x7 sym_fold count: reference DFS nodes/s (recurse_count calls), batched GPU"
UNIT = "nodes/s"


# DRAM bytes per case of the batched kernel: read + write of the ncu capture
# of the first 20,000 7x7 cases (2,174,208 + 1,430,784 bytes), per case.
TRAFFIC_PER_CASE = (2_174_208 + 1_430_784) / 20_000

# Issue profile of the batched kernel over one whole 7x7 count (one ncu pass
# over a full launch of this bench's workload,
# profiles/sym_batched_7x7_full_count.md): warp instructions executed per
# reference node (11,214,661,565,249 over 556,214,135,282 nodes), active
# lanes per warp instruction, and the issue-active share of SMSP cycles.  The
# bench scales the first by its own live node rate to get the kernel's
# warp-instruction issue rate against the SMs' issue ceiling.  The ALU-pipe
# share comes from the fuller capture of the first 20,000 cases
# (profiles/sym_batched_7x7_first20k.md).
ISSUE_PROFILE = {"warp_inst_per_node": 11_214_661_565_249 / 556_214_135_282,
                 "lanes_per_inst": 168_654_826_519_677 / 11_214_661_565_249,
                 "issue_active": 11_214_661_565_249 / 14_115_856_002_000,
                 "alu_pipe_first20k": 0.635,
                 "source": "profiles/sym_batched_7x7_full_count.md"}


def work_counts() -> dict:
    """The whole 7x7 count's reference nodes and chain steps, counted by the
    oracle (tests/golden/make_work_counts.py)."""
    p = ROOT / "tests" / "golden" / "work_counts.json"
    return json.loads(p.read_text()).get("7x7_d24_all", {}) if p.exists() else {}


def issue_figures(nodes_per_step: int, t_step: float, clock_summary: dict) -> dict:
    """Issue-slot view of the DFS kernel: chain steps (get_good walk
    iterations) per second and per SMSP issue slot at the sampled SM clock."""
    import torch

    work = work_counts()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = clock_summary.get("sm_mhz") or clock_summary.get("sm_max_mhz")
    out = {"sms": sms, "sm_mhz": mhz, "nodes_match_oracle": None}
    if work.get("steps"):
        out["nodes_match_oracle"] = work.get("nodes") == nodes_per_step
        steps_s = work["steps"] / t_step
        out["chain_steps_per_s"] = steps_s
        out["chain_steps_per_step"] = work["steps"]
        if mhz:
            out["chain_steps_per_issue_slot"] = steps_s / (sms * 4 * mhz * 1e6)
    return out


def issue_roofline(cases: int, nodes_per_step: int, t_step: float, clock_summary: dict) -> dict:
    """The batched DFS kernel is bound by instruction issue, not by memory
    (HBM carries only the 72-byte case records): achieved = warp instructions
    per second (the ncu-measured warp instructions per node times the live
    node rate), peak = one warp instruction per SMSP per cycle at the sampled
    SM clock.  `useful_lane_frac` discounts inactive lanes.  The HBM figures
    of the case loads are kept as a sub-record."""
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = clock_summary.get("sm_mhz") or clock_summary.get("sm_max_mhz") or 2070.0
    peak = sms * 4 * mhz * 1e6 / 1e9
    achieved = ISSUE_PROFILE["warp_inst_per_node"] * nodes_per_step / t_step / 1e9
    algo_bytes = cases * (64 + 8)
    hbm_peak, peak_kind = peaks()
    hbm_achieved = algo_bytes / t_step / 1e9
    return {
        "bound": "int-issue", "achieved": achieved, "peak": peak, "unit": "Gwarp-inst/s",
        "frac": achieved / peak, "peak_source": f"{sms} SMs x 4 SMSPs x 1 inst/clk at {mhz:.0f} MHz",
        "lanes_per_inst": ISSUE_PROFILE["lanes_per_inst"],
        "useful_lane_frac": achieved / peak * ISSUE_PROFILE["lanes_per_inst"] / 32,
        "profile": ISSUE_PROFILE,
        # ncu DRAM read + write of the first-20,000-case launch scaled by the
        # case count
        "traffic": TRAFFIC_PER_CASE * cases, "traffic_unit": "bytes per launch",
        "hbm": {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": hbm_achieved / hbm_peak, "peak_source": peak_kind,
                "algorithmic_bytes": algo_bytes},
        "issue": issue_figures(nodes_per_step, t_step, clock_summary),
    }


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int = 0):
        self.device = device_index
        self.rows = []
        self._stop = threading.Event()
        self._thread = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.rows.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._thread.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def all_cases_7x7():
    """The 7x7 depth-24 case list in emission order, from the oracle; the CPU
    legs time a bounded prefix of it (time_cpu)."""
    from oracle import oracle

    cyc, mult = oracle.sym_expand(N, EXPANDED_N, 0, 0)
    return cyc, mult


def strided_sample(cases, mults, count):
    """`count` cases spread evenly over the whole case list (node cost varies
    along the emission order, so a prefix would not represent the count)."""
    import numpy as np

    idx = np.unique(np.linspace(0, len(cases) - 1, count).round().astype(np.int64))
    return np.ascontiguousarray(cases[idx]), np.ascontiguousarray(mults[idx])


def time_cpu(cases, mults, threads, target_s=12.0):
    """Time the oracle (a restatement of sym_fold.cpp's solver) on growing
    strided samples of the case list until one run takes ~target_s; returns
    (nodes/s, sample description, seconds, sample size)."""
    from oracle import oracle

    count = 256
    while True:
        c, m = strided_sample(cases, mults, count)
        t0 = time.perf_counter()
        _, _, w = oracle.sym_count_cases(N, EXPANDED_N, c, m, threads)
        el = time.perf_counter() - t0
        if el >= target_s * 0.5 or count >= len(cases):
            return (w.nodes / el, f"{len(c)} cases evenly strided over all {len(cases)} 7x7 "
                    f"depth-24 cases", el, count)
        count = min(len(cases), int(count * max(2.0, target_s / max(el, 1e-3))))


REF_SRC = ROOT / "baseline" / "_ref" / "src" / "sym_fold.cpp"
REF_BIN = ROOT / "baseline" / "_ref" / "bin" / "sym_fold"


def _ref_env():
    """The environment for the reference binary: none of its MF_* switches
    (case sorting, streaming, expansion depth) leak in from the caller."""
    return {k: v for k, v in os.environ.items() if not k.startswith("MF_")}


def _ref_runs(binary) -> bool:
    try:
        res = subprocess.run([str(binary), "7", "1"], capture_output=True, text=True,
                             timeout=120, env={**_ref_env(), "MF_SETUP_ONLY": "1"})
    except (OSError, subprocess.SubprocessError):
        return False
    return res.returncode == 0 and res.stdout.strip().splitlines()[-1:] == ["433131"]


def reference_sym_fold():
    """The reference's own CPU solver: sym_fold.cpp, staged unmodified into
    baseline/_ref/src by oracle/Makefile (the GPU host has no reference
    checkout), built with g++ -O3 -std=c++20 -pthread for this host, as the
    reference's README builds it.  Returns (path, None) or (None, why)."""
    if not REF_SRC.exists():
        return None, ("baseline/_ref/src/sym_fold.cpp is not staged "
                      "(make -C oracle cpu_src needs the reference checkout)")
    if REF_BIN.exists() and REF_BIN.stat().st_mtime >= REF_SRC.stat().st_mtime \
            and _ref_runs(REF_BIN):
        return REF_BIN, None
    cxx = os.environ.get("CXX") or "g++"
    REF_BIN.parent.mkdir(parents=True, exist_ok=True)
    tmp = REF_BIN.with_suffix(".tmp")
    try:
        res = subprocess.run([cxx, "-O3", "-std=c++20", "-pthread", "-o", str(tmp), str(REF_SRC)],
                             capture_output=True, text=True, timeout=600)
    except (OSError, subprocess.SubprocessError) as e:
        return None, f"building sym_fold.cpp failed: {e}"
    if res.returncode != 0:
        return None, "building sym_fold.cpp failed: " + (res.stderr.strip().splitlines() or ["?"])[-1]
    tmp.replace(REF_BIN)
    if not _ref_runs(REF_BIN):
        return None, "the built sym_fold did not list the 433131 7x7 cases"
    return REF_BIN, None


def reference_sample() -> dict:
    """The reference arm's bounded sample: chunks of consecutive 7x7 cases
    with their answers and reference nodes, counted by the oracle
    (tests/golden/make_work_counts.py --ref-sample)."""
    p = ROOT / "tests" / "golden" / "work_counts.json"
    return json.loads(p.read_text()).get("7x7_d24_ref_sample", {}) if p.exists() else {}


def time_reference_sample(binary, sample, threads):
    """One pass of the reference binary over the sample, one
    `sym_fold 7 <threads> <max_cases> <start_case>` process per chunk, each
    chunk's answer checked; returns (seconds, nodes)."""
    el_total = 0.0
    for c in sample["chunks"]:
        t0 = time.perf_counter()
        res = subprocess.run([str(binary), "7", str(threads), str(c["max_cases"]),
                              str(c["start_case"])], capture_output=True, text=True,
                             timeout=1800, env=_ref_env())
        el_total += time.perf_counter() - t0
        got = res.stdout.strip().splitlines()[-1:] if res.returncode == 0 else []
        if got != [str(c["answer"])]:
            raise RuntimeError(f"sym_fold chunk at {c['start_case']}: rc={res.returncode} "
                               f"stdout={got} want {c['answer']}")
    return el_total, sample["nodes"]


def reference_sample_desc(sample) -> str:
    starts = ", ".join(str(c["start_case"]) for c in sample["chunks"])
    return (f"reference sym_fold.cpp (unmodified, g++ -O3) on {len(sample['chunks'])} chunks of "
            f"{sample['chunks'][0]['max_cases']} consecutive 7x7 depth-24 cases at starts {starts} "
            f"of 433131, one process per chunk (its case expansion, ~0.1 s, included)")


def run_reference(args):
    """The reference's own CPU solver (sym_fold.cpp built from the staged
    source, reference_sym_fold) on all host threads, a bounded sample of the
    7x7 count per step (reference_sample); if it cannot be built or run here,
    the oracle's restatement of it on a strided sample, saying why."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    binary, why = reference_sym_fold()
    sample = reference_sample()
    if binary is not None and not sample:
        binary, why = None, "tests/golden/work_counts.json has no 7x7_d24_ref_sample"
    if binary is not None:
        try:
            for _ in range(args.warmup):
                time_reference_sample(binary, sample, threads)
            times = []
            nodes = 0
            for _ in range(args.steps):
                el, nodes = time_reference_sample(binary, sample, threads)
                times.append(el)
        except (RuntimeError, OSError, subprocess.SubprocessError) as e:
            binary, why = None, f"running sym_fold failed: {e}"
    if binary is not None:
        value = nodes * len(times) / sum(times)
        desc = reference_sample_desc(sample)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic: the reference's own 7x7 case list (deterministic)",
            "config": {"workload": f"7x7 sym_fold depth-24 cases, CPU sample ({desc})",
                       "n": N, "expanded_n": EXPANDED_N, "threads": threads},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "reference",
                             "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
        return
    cases, mults = all_cases_7x7()
    rate, sample, el, count = time_cpu(cases, mults, threads, target_s=8.0)
    from oracle import oracle

    c, m = strided_sample(cases, mults, count)
    for _ in range(args.warmup):
        oracle.sym_count_cases(N, EXPANDED_N, c, m, threads)
    times = []
    nodes = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, w = oracle.sym_count_cases(N, EXPANDED_N, c, m, threads)
        times.append(time.perf_counter() - t0)
        nodes = w.nodes
    value = nodes * len(times) / sum(times)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic: the reference's own 7x7 case list (deterministic)",
        "config": {"workload": f"7x7 sym_fold depth-24 cases, CPU sample ({sample})",
                   "n": N, "expanded_n": EXPANDED_N, "threads": threads},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_unavailable": why,
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    import map_folding_gb300 as mf
    from map_folding_gb300 import build as mfbuild

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not mfbuild.LIB.exists():
        mfbuild.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    plan = mf.SymPlan(N, EXPANDED_N)
    cycles, mults = plan.cases()
    # replicas: every rank counts the whole map (the path shards only by
    # case ranges across boxes; see the chunk driver)
    d_cyc = torch.from_numpy(np.ascontiguousarray(cycles)).cuda()
    d_counts = torch.zeros(len(cycles), dtype=torch.int64, device="cuda")
    d_nodes = torch.zeros(1, dtype=torch.int64, device="cuda")
    cfg = None
    ws = torch.empty(mf.sym_workspace_bytes(cfg), dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    stream = torch.cuda.current_stream()
    mult_t = torch.from_numpy(mults.astype(np.int64))

    def step():
        d_nodes.zero_()
        mf.count_cases_batched_device(N, EXPANDED_N, N * N, d_cyc.data_ptr(), len(cycles),
                                      d_counts.data_ptr(), ws.data_ptr(), ws.numel(),
                                      d_nodes.data_ptr(), cfg, stream.cuda_stream)

    def check():
        c = d_counts.cpu().numpy().view(np.uint64)
        total = sum(int(m) * int(x) for m, x in zip(mults, c)) * N * N
        return total

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    assert check() == ANSWER_7X7, "warm-up count is not bit-exact"
    nodes_per_step = int(d_nodes.item())

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b) * 1e-3)
            assert int(d_nodes.item()) == nodes_per_step
    assert check() == ANSWER_7X7, "timed count is not bit-exact"
    t_step = sum(times) / len(times)
    t_max = torch.tensor([sum(times)], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
        dist.barrier()
    value = world * nodes_per_step * len(times) / float(t_max.item())

    # End to end through the C ABI with host buffers (a few repeats: every
    # repeat is a whole 7x7 count).
    e2e_times = []
    e2e_st = None
    for _ in range(max(1, min(args.steps, args.e2e_steps))):
        t0 = time.perf_counter()
        ans, st = plan.solve(0, 0, "batched")
        e2e_times.append(time.perf_counter() - t0)
        assert ans == ANSWER_7X7
        e2e_st = st
    e2e_value = world * nodes_per_step * len(e2e_times) / sum(e2e_times)

    # The plain one-thread-per-case kernel on the same cases, once (single
    # GPU only: its ~430 s would hold the other ranks at the final barrier).
    plain_s = None
    if args.plain and world == 1:
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        mf.count_cases_device(N, EXPANDED_N, N * N, d_cyc.data_ptr(), len(cycles),
                              d_counts.data_ptr(), 0, stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        plain_s = a.elapsed_time(b) * 1e-3
        assert check() == ANSWER_7X7

    clock_summary = clocks.summary()
    roofline = issue_roofline(len(cycles), nodes_per_step, t_step, clock_summary)

    # Config 5 in brief: the serving stream's 8x8 chunks through the resident
    # server, every chunk checked against the reference's own count.
    serving = None
    if args.serving and world == 1:
        serving = serving_summary(run_serving_stream(args.seed, args.requests, args.rate))

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        binary, why = reference_sym_fold()
        ref_sample = reference_sample()
        if binary is not None and ref_sample:
            try:
                el, nodes = time_reference_sample(binary, ref_sample, threads)
                cpu = {"value": nodes / el, "unit": UNIT, "cores": threads, "kind": "reference",
                       "sample": reference_sample_desc(ref_sample)}
            except (RuntimeError, OSError, subprocess.SubprocessError) as e:
                why = f"running sym_fold failed: {e}"
        if cpu is None:
            rate, sample, el, count = time_cpu(cycles, mults, threads, target_s=10.0)
            cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                   "reference_unavailable": why or "no reference sample"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic: the reference's own 7x7 case list (deterministic)",
            "config": {"workload": "7x7 full count, sym_fold cases at MF_EXPANDED_N=24 (433131)",
                       "n": N, "expanded_n": EXPANDED_N, "cases": len(cycles),
                       "nodes_per_step": nodes_per_step, "l2": "flushed between steps (256 MB write)",
                       "kernel": "batched persistent work-stealing", "parallelism": "replicas"},
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(e2e_st.h2d_bytes) if e2e_st else 0,
                    "d2h_bytes_per_step": int(e2e_st.d2h_bytes) if e2e_st else 0,
                    "ms_per_step": 1e3 * sum(e2e_times) / len(e2e_times)},
            # per step: the split-ring reset kernel and the persistent kernel
            "gpu_launches": 2 * args.steps,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clock_summary,
            "plain_ms_per_step": None if plain_s is None else 1e3 * plain_s,
            "batched_vs_plain": None if plain_s is None else plain_s / t_step,
            "splits_per_step": int(e2e_st.splits) if e2e_st else None,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def _golden_lunnon() -> dict:
    g = json.loads((ROOT / "tests" / "golden" / "reference_counts.json").read_text())
    counts = {k: int(v) for k, v in g["lunnon"].items()}
    counts["6x6"] = 123912532224  # mfah/folding.py:8-17 (squares n = 1..8)
    return counts


def _gpu_common(args, clocks):
    return {"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "vs_baseline": None,
            "dtype": "u64", "clocks": clocks.summary()}


def run_lunnon(args):
    """Configs 1 and 2: 5x5 at depth 15, 6x6 at depth 18, every p x q map
    with 2 <= p <= q <= 6 and the strips of 8..20 stamps; batched kernel
    timed over `steps` runs per map (after `warmup`), the plain kernel once
    per map; every count checked against the reference's counts."""
    import map_folding_gb300 as mf

    golden = _golden_lunnon()
    shapes = [((5, 5), 15), ((6, 6), 18)]
    shapes += [((p, q), -1) for p in range(2, 7) for q in range(p, 7) if (p, q) not in ((5, 5), (6, 6))]
    shapes += [((1, n), -1) for n in range(8, 21)]
    rows = []
    tot_nodes = tot_b = tot_p = 0.0
    with ClockSampler(0) as clocks:
        for dims, depth in shapes:
            key = "x".join(map(str, dims))
            plan = mf.LunnonPlan(dims)
            try:
                for _ in range(args.warmup):
                    plan.count(depth, "batched")
                bt = []
                for _ in range(args.steps):
                    c, states, st = plan.count(depth, "batched")
                    assert c == golden[key], (key, c)
                    bt.append(st.kernel_s)
                nodes = st.nodes
                c, _, sp = plan.count(depth, "plain")
                assert c == golden[key], (key, c)
            finally:
                plan.close()
            b = sum(bt) / len(bt)
            rows.append({"map": key, "depth": depth, "states": int(states), "nodes": int(nodes),
                         "plain_nodes": int(sp.nodes),
                         "batched_ms": 1e3 * b, "plain_ms": 1e3 * sp.kernel_s,
                         "batched_vs_plain": sp.kernel_s / b})
            tot_nodes += nodes
            tot_b += b
            tot_p += sp.kernel_s
    # CPU baseline: the oracle's restatement of mf_fast.cpp's threaded resume
    # (mf_fast <n> <depth> $(nproc)) on 6x6 at depth 18, all host threads.
    cpu = None
    if not args.no_cpu:
        from oracle import oracle

        threads = os.cpu_count() or 1
        a, b, _ = oracle.lunnon_collect((6, 6), 18)
        count = 512
        while True:  # grow a prefix of the states until one run takes ~10 s
            t0 = time.perf_counter()
            _, _, w = oracle.lunnon_resume_many((6, 6), 19, a[:count], b[:count], threads)
            el = time.perf_counter() - t0
            if el >= 5.0 or count >= len(a):
                break
            count = min(len(a), int(count * max(2.0, 10.0 / max(el, 1e-3))))
        cpu = {"value": w.nodes / el, "unit": "nodes/s", "cores": threads, "kind": "port",
               "sample": f"first {count} of {len(a)} 6x6 depth-18 prefix states ({el:.2f} s)"}
        # mf.c single-threaded, as the reference runs rectangles, strips and
        # 3-D maps: the oracle's restatement on one shape of each kind.
        single_nodes, single_s = 0, 0.0
        for dims in ((4, 6), (1, 20), (2, 2, 5)):
            t0 = time.perf_counter()
            c, w1 = oracle.lunnon_count(dims)
            single_s += time.perf_counter() - t0
            single_nodes += w1.nodes
            assert c == golden["x".join(map(str, dims))], dims
        cpu["single_thread"] = {"value": single_nodes / single_s, "unit": "nodes/s", "cores": 1,
                                "kind": "port", "sample": f"4x6, 1x20, 2x2x5 whole ({single_s:.2f} s)"}
    line = {"metric": "Lunnon DFS nodes/s over configs 1-2 (5x5@15, 6x6@18, 20 rectangles, strips 8..20)",
            "cpu_baseline": cpu,
            "value": tot_nodes / tot_b, "unit": "nodes/s", "ms_per_step": 1e3 * tot_b,
            "higher_is_better": True, "scaling": "weak", "data": "synthetic: exhaustive map counts",
            "config": {"workload": "lunnon maps", "maps": len(rows)},
            "plain_ms_per_step": 1e3 * tot_p, "batched_vs_plain": tot_p / tot_b,
            "maps": rows, "gpu_launches": 2 * len(rows) * args.steps}
    line.update(_gpu_common(args, clocks))
    print(json.dumps(line), flush=True)


def run_uneven(args, seed: int = 2026):
    """Config 3: 64 maps drawn from a seed, all their prefix states in one
    persistent launch replayed from a CUDA graph, with depths and launch
    knobs from the autotuner; compared with the plain kernel map by map."""
    import map_folding_gb300 as mf
    from map_folding_gb300 import autotune
    from map_folding_gb300.workloads import uneven_instances

    shapes = uneven_instances(seed, 64)
    tuned = autotune.tune_lunnon_batch(shapes)
    batch = mf.LunnonBatch(shapes, tuned["depths"], autotune.as_config(tuned))
    try:
        for _ in range(args.warmup):
            batch.run()
        times = []
        with ClockSampler(0) as clocks:
            for _ in range(args.steps):
                counts, st = batch.run()
                times.append(st.kernel_s)
        nodes = st.nodes
    finally:
        batch.close()
    plain = []
    plain_s = 0.0
    for dims, depth in zip(shapes, tuned["depths"]):
        plan = mf.LunnonPlan(dims)
        try:
            c, _, sp = plan.count(depth, "plain")
        finally:
            plan.close()
        plain.append(c)
        plain_s += sp.kernel_s
    assert counts == plain, "batched counts differ from the plain kernel"
    golden = _golden_lunnon()
    for dims, c in zip(shapes, counts):
        key = "x".join(map(str, dims))
        if key in golden:
            assert c == golden[key], (key, c)
    t = sum(times) / len(times)
    line = {"metric": "64-map uneven batch: DFS nodes/s, one graph replay of the batched kernel",
            "value": nodes / t, "unit": "nodes/s", "ms_per_step": 1e3 * t,
            "higher_is_better": True, "scaling": "weak", "data": f"synthetic: uneven_instances(seed={seed})",
            "config": {"workload": "64 uneven maps", "seed": seed,
                       "block_threads": tuned["block_threads"], "node_budget": tuned["node_budget"],
                       "depths": tuned["depths"]},
            "plain_ms_per_step": 1e3 * plain_s, "batched_vs_plain": plain_s / t,
            "gpu_launches": 2 * args.steps}
    line.update(_gpu_common(args, clocks))
    print(json.dumps(line), flush=True)


def run_serving_stream(seed: int, requests: int, rate: float) -> dict:
    """The serving stream through one resident server: every chunk checked
    against the reference's own sym_fold count of the same chunk (golden,
    where tests/golden/make_golden.py --serving has made it) and every map
    against the reference's count."""
    from map_folding_gb300.serving import Server, run_stream
    from map_folding_gb300.workloads import serving_stream

    reqs = serving_stream(seed=seed, requests=requests, rate_per_s=rate, chunk_cases=50_000)
    golden = _golden_lunnon()
    served = json.loads((ROOT / "tests" / "golden" / "reference_counts.json").read_text()
                        ).get("sym_serving", {})
    with Server() as srv:
        # warm-up: the 8x8 expansion index and one small request of each kind
        srv.wait(srv.submit_sym(8, 36, 0, 100))
        srv.wait(srv.submit_lunnon((3, 4)))
        with ClockSampler(0) as clocks:
            out = run_stream(srv, reqs)
    for r, q in zip(out["results"], reqs):
        r["arrival_s"] = q.arrival_s
        if r["kind"] == "chunk":
            rec = served.get(f"8x8_d36_{r['start_case']}+{r['max_cases']}")
            r["golden"] = rec is not None
            if rec is not None:
                assert r["answer"] == rec["count"], ("chunk differs from the reference", r["rid"])
        else:
            key = "x".join(map(str, sorted(r["dims"])))  # p x q and q x p fold alike
            assert r["answer"] == golden[key], (key, r["answer"])
            r["golden"] = True
    out["clocks"] = clocks.summary()
    out["seed"], out["rate_per_s"] = seed, rate
    return out


def serving_summary(out: dict) -> dict:
    chunks = [r for r in out["results"] if r["kind"] == "chunk"]
    return {"workload": "serving_stream: 8x8 MF_EXPANDED_N=36 50,000-case chunks + maps <= 5x6",
            "seed": out["seed"], "requests": out["requests"], "rate_per_s": out["rate_per_s"],
            "chunks": len(chunks), "chunks_golden": sum(r["golden"] for r in chunks),
            "chunk_p50_s": out["chunk_p50_s"], "chunk_p99_s": out["chunk_p99_s"],
            "all_p50_s": out["all_p50_s"], "all_p99_s": out["all_p99_s"],
            "cases_per_s": out["cases_per_s"], "nodes_per_s": out["nodes_per_s"],
            "wall_s": out["wall_s"], "clocks": out["clocks"],
            "note": (f"p99 over {len(chunks)} chunks is their maximum" if len(chunks) < 100
                     else "")}


def run_serving(args):
    """Config 5: 8x8 chunk requests (MF_EXPANDED_N=36, 50,000 consecutive
    cases from a seeded uniform start) arriving as a Poisson stream,
    interleaved with whole maps up to 5x6, through one resident server.
    Latency is submit -> result; every chunk is checked against the
    reference's count (golden) and recounted alone afterwards (which also
    gives the alone capacity), every map against the reference's count."""
    import map_folding_gb300 as mf

    out = run_serving_stream(args.seed, args.requests, args.rate)
    plan = mf.SymPlan(8, 36)
    alone_s = 0.0
    cases = 0
    for r in out["results"]:
        if r["kind"] == "chunk":
            ans, st = plan.solve(r["max_cases"], r["start_case"], "batched")
            assert ans == r["answer"], ("chunk differs from the chunk counted alone", r["rid"])
            alone_s += st.kernel_s
            r["alone_s"] = st.kernel_s
            cases += r["max_cases"]
    plan.close()
    summary = serving_summary(out)
    line = {"metric": "8x8 chunk serving: chunk p99 latency (s) under a Poisson stream",
            "value": out["chunk_p99_s"], "unit": "s", "higher_is_better": False,
            "chunk_p50_s": out["chunk_p50_s"], "all_p50_s": out["all_p50_s"],
            "all_p99_s": out["all_p99_s"], "cases_per_s": out["cases_per_s"],
            "nodes_per_s": out["nodes_per_s"], "wall_s": out["wall_s"],
            "alone_cases_per_s": cases / alone_s if alone_s else None,
            "chunks_golden": summary["chunks_golden"],
            "ms_per_step": 1e3 * out["wall_s"], "scaling": "weak",
            "data": f"synthetic: serving_stream(seed={args.seed})",
            "config": {"workload": "8x8 MF_EXPANDED_N=36 50,000-case chunks + maps <= 5x6",
                       "requests": args.requests, "rate_per_s": args.rate,
                       "chunks": summary["chunks"]},
            "requests": [{k: r.get(k) for k in ("rid", "kind", "latency_s", "queue_s", "units",
                                                "arrival_s", "alone_s", "golden")}
                         for r in out["results"]],
            "gpu_launches": None, "n_gpus": 1, "steps": 1, "warmup": args.warmup,
            "vs_baseline": None, "dtype": "u64", "clocks": out["clocks"], "note": summary["note"]}
    print(json.dumps(line), flush=True)


def run_chunk_plan(args):
    """Equal-size chunks vs cost-weighted chunks (shallow estimate_work
    lookahead): the whole 7x7 count in 40 chunks, and the 8x8 band of
    1,000,000 cases at 50,000,000 (where the reference's slowest chunk
    started) in 20 chunks; every chunk timed alone on the GPU, and each
    plan's chunk sum checked against the other's."""
    import numpy as np

    import map_folding_gb300 as mf
    from map_folding_gb300.chunks import plan_cost_chunks

    def stats(times):
        t = np.sort(np.asarray(times))
        return {"chunks": len(t), "max_s": float(t[-1]), "p90_s": float(np.percentile(t, 90)),
                "median_s": float(np.median(t)), "mean_s": float(t.mean()),
                "max_over_mean": float(t[-1] / t.mean()), "sum_s": float(t.sum())}

    out = {}
    with ClockSampler(0) as clocks:
        for name, n, e, start, count, k, depth in [("7x7_all", 7, 24, 0, 0, 40, args.cost_depth),
                                                  ("8x8_d36_50M+1M", 8, 36, 50_000_000, 1_000_000,
                                                   20, args.cost_depth)]:
            plan = mf.SymPlan(n, e)
            count = count or plan.total_cases
            size = -(-count // k)
            equal = [(s, min(size, start + count - s)) for s in range(start, start + count, size)]
            t0 = time.perf_counter()
            cost = plan_cost_chunks(n, e, k, depth, start, start + count, block=500)
            plan_s = time.perf_counter() - t0
            res = {}
            for label, chunks in (("equal", equal), ("cost", cost)):
                times, total = [], 0
                for s, m in chunks:
                    ans, st = plan.solve(m, s, "batched")
                    times.append(st.kernel_s)
                    total += ans
                res[label] = dict(stats(times), answer=str(total),
                                  sizes=[m for _, m in chunks])
            plan.close()
            assert res["equal"]["answer"] == res["cost"]["answer"], name
            res["cost_depth"] = depth
            res["plan_s"] = plan_s
            out[name] = res
    line = {"metric": "chunk time spread: max/mean of per-chunk GPU time, equal vs cost-weighted",
            "value": out["8x8_d36_50M+1M"]["cost"]["max_over_mean"], "unit": "ratio",
            "higher_is_better": False, "scaling": "weak", "data": "synthetic: exhaustive case ranges",
            "config": {"workload": "7x7 all cases in 40 chunks; 8x8 d36 [50M, 51M) in 20 chunks",
                       "cost_depth": args.cost_depth},
            "results": out, "gpu_launches": None}
    line.update(_gpu_common(args, clocks))
    print(json.dumps(line), flush=True)


def run_nine(args):
    """9x9 chunks of experiments/9x9/sym_fold9.cpp (5x5 centre, streamed
    cases at MF_EXPANDED_N = 40..48) on the 128-bit kernel, each checked
    against the reference's count; plan setup (centre enumeration, dedup,
    expansion index) timed apart from the chunk's own count."""
    import map_folding_gb300 as mf

    golden = json.loads((ROOT / "tests" / "golden" / "reference_counts.json").read_text())["sym9"]
    chunks = [("9x9_c5_d42_first100", 42, 100, 0), ("9x9_c5_d40_1000000+100", 40, 100, 1000000),
              ("9x9_c5_d44_first300", 44, 300, 0), ("9x9_c5_d48_5000+2000", 48, 2000, 5000),
              ("9x9_d42_first5000", 42, 5000, 0)]
    plans, rows = {}, []
    nodes = kernel = 0.0
    with ClockSampler(0) as clocks:
        for key, e, m, s in chunks:
            if e not in plans:
                t0 = time.perf_counter()
                plans[e] = mf.SymPlan(9, e, center_n=5)
                plans[e].setup_s = time.perf_counter() - t0
            t0 = time.perf_counter()
            ans, st = plans[e].solve(m, s)
            wall = time.perf_counter() - t0
            if key in golden:
                assert ans == golden[key]["count"], key
            rows.append({"chunk": key, "cases": m, "kernel_s": st.kernel_s, "call_s": wall,
                         "plan_setup_s": plans[e].setup_s, "nodes": int(st.nodes),
                         "nodes_per_s": st.nodes / st.kernel_s, "answer": str(ans)})
            nodes += st.nodes
            kernel += st.kernel_s
    for p in plans.values():
        p.close()
    line = {"metric": "9x9 sym chunks (5x5 centre): reference DFS nodes/s on the 128-bit kernel",
            "value": nodes / kernel, "unit": "nodes/s", "higher_is_better": True,
            "ms_per_step": 1e3 * kernel, "scaling": "weak", "data": "synthetic: exhaustive case ranges",
            "config": {"workload": "9x9 MF_CENTER_N=5 streamed chunks, MF_EXPANDED_N 40..48"},
            "chunks": rows, "gpu_launches": None}
    line.update(_gpu_common(args, clocks))
    print(json.dumps(line), flush=True)


def _timed_run(cmd, timeout_s=900):
    t0 = time.perf_counter()
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, timeout=timeout_s)
    return time.perf_counter() - t0, res


def run_reference_gpu(args):
    """The reference's own GPU drivers on this GPU next to the engine: the
    unmodified gpu_folding.cu (one thread per prefix state) and
    gpu_folding_v2.cu (batched producer/worker solve_kernel), built here with
    nvcc for sm_103a from the copies oracle/Makefile stages into
    baseline/_ref/src/, run through their own CLIs on 5x5 at depth 15 and
    6x6 at depth 18 (each generates its own prefix states), wall-timed as
    processes; the engine's drop-in bin/gpu_folding on the same arguments,
    wall-timed the same way, and its kernel time through the C ABI.  Every
    count is checked against the reference's count."""
    import map_folding_gb300 as mf
    from map_folding_gb300 import build as mfbuild

    src = ROOT / "baseline" / "_ref" / "src"
    if not (src / "gpu_folding.cu").exists():
        print(json.dumps({"impl": "reference-gpu", "unavailable":
                          "baseline/_ref/src has no staged reference CUDA sources "
                          "(make -C oracle gpu_src needs the reference checkout)"}), flush=True)
        return
    out_dir = ROOT / "baseline" / "_ref" / "bin"
    out_dir.mkdir(parents=True, exist_ok=True)
    for name in ("gpu_folding", "gpu_folding_v2"):
        subprocess.run(["nvcc", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-o",
                        str(out_dir / name), str(src / f"{name}.cu")], check=True,
                       capture_output=True)
    if not mfbuild.LIB.exists():
        mfbuild.build()
    ours = mfbuild.BIN / "gpu_folding"
    golden = _golden_lunnon()
    rows = []
    with ClockSampler(0) as clocks:
        for grid, depth in ((5, 15), (6, 18)):
            want = golden[f"{grid}x{grid}"]
            row = {"map": f"{grid}x{grid}", "depth": depth}
            el, res = _timed_run([out_dir / "gpu_folding", grid, depth])
            got = int(res.stdout.strip().splitlines()[-1].split(":")[-1])
            assert res.returncode == 0 and got == want, ("gpu_folding", grid, got)
            row["reference_gpu_folding_s"] = el
            el, res = _timed_run([out_dir / "gpu_folding_v2", grid, depth, 5000, 128, 8, 1])
            got = int(res.stdout.strip().splitlines()[-1])
            assert res.returncode == 0 and got == want, ("gpu_folding_v2", grid, got)
            kv = dict(tok.split("=", 1) for tok in res.stderr.split() if "=" in tok)
            row["reference_gpu_folding_v2_s"] = el
            row["reference_gpu_folding_v2_solve_s"] = float(kv.get("solve_s", "nan"))
            for mode in ("batched", "plain"):
                best = None
                for _ in range(max(1, args.steps)):
                    el, res = _timed_run([ours, grid, depth, mode])
                    got = int(res.stdout.strip().splitlines()[-1].split(":")[-1])
                    assert res.returncode == 0 and got == want, ("ours", mode, grid, got)
                    best = el if best is None else min(best, el)
                row[f"ours_{mode}_process_s"] = best
                plan = mf.LunnonPlan((grid, grid))
                c, _, st = plan.count(depth, mode)
                plan.close()
                assert c == want
                row[f"ours_{mode}_kernel_s"] = st.kernel_s
            row["process_speedup_vs_gpu_folding"] = (row["reference_gpu_folding_s"] /
                                                     row["ours_batched_process_s"])
            row["process_speedup_vs_gpu_folding_v2"] = (row["reference_gpu_folding_v2_s"] /
                                                        row["ours_batched_process_s"])
            rows.append(row)
    line = {"metric": "Lunnon whole-map wall time: the reference's own GPU drivers vs the engine, same GPU",
            "value": rows[-1]["process_speedup_vs_gpu_folding_v2"], "unit": "x (gpu_folding_v2 / ours, 6x6@18)",
            "higher_is_better": True, "data": "synthetic: exhaustive map counts",
            "config": {"workload": "gpu_folding / gpu_folding_v2 (reference, unmodified, nvcc sm_103a) "
                                   "vs bin/gpu_folding on 5x5@15 and 6x6@18",
                       "v2_args": "batch_size 5000, threads_per_block 128, blocks_per_sm 8, max_gpus 1"},
            "maps": rows, "n_gpus": 1, "steps": args.steps, "warmup": 0, "vs_baseline": None,
            "dtype": "u64", "clocks": clocks.summary(), "gpu_launches": None}
    print(json.dumps(line), flush=True)


def run_profile_case(case: str):
    """One launch of each kernel on a small case, for ncu (a few seconds of
    GPU work, inputs ~28 MB): `sym-partial` counts the 433,131 7x7 cases from
    24 to 30 cells (plain kernel, then batched); `sym-steady` the first 20,000
    7x7 cases to completion (batched); `lunnon` counts the 6x6 map from its
    18-leaf prefix states (plain, then batched); `wide` 300 9x9 cases on the
    128-bit kernel; `serve` a 2,000-case 8x8 chunk and two maps through the
    request server."""
    import numpy as np
    import torch

    import map_folding_gb300 as mf
    from map_folding_gb300 import build as mfbuild

    if not mfbuild.LIB.exists():
        mfbuild.build()
    if case == "sym-partial":
        plan = mf.SymPlan(N, EXPANDED_N)
        cycles, _ = plan.cases()
        d_cyc = torch.from_numpy(np.ascontiguousarray(cycles)).cuda()
        d_counts = torch.zeros(len(cycles), dtype=torch.int64, device="cuda")
        ws = torch.empty(mf.sym_workspace_bytes(), dtype=torch.uint8, device="cuda")
        mf.count_cases_device(N, EXPANDED_N, 30, d_cyc.data_ptr(), len(cycles), d_counts.data_ptr())
        mf.count_cases_batched_device(N, EXPANDED_N, 30, d_cyc.data_ptr(), len(cycles),
                                      d_counts.data_ptr(), ws.data_ptr(), ws.numel())
    elif case == "sym-steady":
        # the bench's batched kernel on the first 20,000 7x7 cases, searched
        # to completion (~2.6e10 nodes, under a second per launch)
        plan = mf.SymPlan(N, EXPANDED_N)
        cycles, _ = plan.cases(0, 20000)
        d_cyc = torch.from_numpy(np.ascontiguousarray(cycles)).cuda()
        d_counts = torch.zeros(len(cycles), dtype=torch.int64, device="cuda")
        ws = torch.empty(mf.sym_workspace_bytes(), dtype=torch.uint8, device="cuda")
        mf.count_cases_batched_device(N, EXPANDED_N, N * N, d_cyc.data_ptr(), len(cycles),
                                      d_counts.data_ptr(), ws.data_ptr(), ws.numel())
    elif case == "lunnon":
        plan = mf.LunnonPlan((6, 6))
        for mode in ("plain", "batched"):
            count, _, _ = plan.count(18, mode)
            assert count == 123912532224
    elif case == "wide":
        # the 128-bit kernel on the first 300 9x9 5x5-centre cases at 44 cells
        plan = mf.SymPlan(9, 44, center_n=5)
        golden = json.loads((ROOT / "tests" / "golden" / "reference_counts.json").read_text())
        ans, _ = plan.solve(300, 0, "batched")
        assert ans == golden["sym9"]["9x9_c5_d44_first300"]["count"]
    elif case == "serve":
        # the request server on one 8x8 chunk of 2,000 depth-36 cases and two maps
        from map_folding_gb300.serving import Server

        with Server() as srv:
            ids = [srv.submit_sym(8, 36, 0, 2000), srv.submit_lunnon((4, 5)),
                   srv.submit_lunnon((3, 6))]
            got = [srv.wait(r)[0] for r in ids]
        golden = json.loads((ROOT / "tests" / "golden" / "reference_counts.json").read_text())
        assert got[1] == golden["lunnon"]["4x5"] and got[2] == golden["lunnon"]["3x6"]
    else:
        raise SystemExit(f"unknown profile case {case}")
    torch.cuda.synchronize()
    print(f"profile case {case} done")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # The plain one-thread-per-case kernel needs ~430 s for the 7x7 count (its
    # heaviest case runs on one thread); it runs once, after the timed steps.
    ap.add_argument("--plain", action="store_true", default=True)
    ap.add_argument("--no-plain", dest="plain", action="store_false")
    ap.add_argument("--no-serving", dest="serving", action="store_false", default=True,
                    help="7x7: skip the short serving-stream sub-record")
    ap.add_argument("--e2e-steps", type=int, default=3, help="7x7: end-to-end repeats")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-case", default="", help="run one small case for ncu and exit")
    # Supplementary workloads, one JSON line each; the default is the 7x7 count.
    ap.add_argument("--workload", default="7x7",
                    choices=["7x7", "lunnon", "uneven", "serving", "chunk-plan", "9x9",
                             "reference-gpu"])
    ap.add_argument("--cost-depth", type=int, default=6, help="chunk-plan: lookahead depth")
    ap.add_argument("--requests", type=int, default=12, help="serving: requests in the stream")
    ap.add_argument("--rate", type=float, default=0.15, help="serving: Poisson arrivals per second")
    ap.add_argument("--seed", type=int, default=5, help="serving: stream seed")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args.profile_case)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "lunnon":
        run_lunnon(args)
    elif args.workload == "uneven":
        run_uneven(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "chunk-plan":
        run_chunk_plan(args)
    elif args.workload == "9x9":
        run_nine(args)
    elif args.workload == "reference-gpu":
        run_reference_gpu(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
