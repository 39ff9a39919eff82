"""Python mirror of the reference's counting interfaces, over the C ABI.

    gpu_folding(grid_size, partition_depth)   -> (states, total)
        what `gpu_folding <n> <depth>` prints (gpu_folding.cu:209-311)
    sym_fold(n, max_cases=0, start_case=0, expanded_n=24)  -> int
        what `sym_fold n threads max_cases start_case` prints
        (sym_fold.cpp:649-774, MF_EXPANDED_N semantics)
    solve_cases(n, start_i, stop_i, case_buffer, case_count) -> (count, nodes, status)
        the WASM kernel's contract (mfah/wasm/sym_kernel.c:251-276)
    LunnonPlan / SymPlan                      -> the lower-level pieces
    lunnon_batch_count(shapes, depths)        -> per-map counts, one launch

Arguments are checked the way the reference checks them and raise
ValueError where the reference exits with rc 1.
"""
from __future__ import annotations

import ctypes
from typing import Iterable, Sequence

import numpy as np

from . import _native
from ._native import BatchConfig, EngineError, RunStats, check

MODES = {"plain": 0, "batched": 1}


def _mode(mode: str | int) -> int:
    if isinstance(mode, int):
        return mode
    if mode not in MODES:
        raise ValueError(f"mode must be one of {sorted(MODES)}")
    return MODES[mode]


def _cfg(cfg: BatchConfig | dict | None):
    if cfg is None:
        return None
    if isinstance(cfg, dict):
        c = BatchConfig()
        for k, v in cfg.items():
            setattr(c, k, int(v))
        cfg = c
    return ctypes.byref(cfg)


def _u128(words) -> int:
    return (int(words[1]) << 64) | int(words[0])


class LunnonPlan:
    """Tables of one p1 x p2 x ... map (mf.c:29-75)."""

    def __init__(self, dims: Sequence[int]):
        lib = _native.load()
        self.dims = tuple(int(d) for d in dims)
        arr = (ctypes.c_int32 * len(self.dims))(*self.dims)
        h = ctypes.c_void_p()
        check(lib.mf_lunnon_plan_create(arr, len(self.dims), ctypes.byref(h)))
        self._h = h
        self.n = lib.mf_lunnon_leaves(h)
        self.stride = lib.mf_lunnon_state_stride(h)

    def close(self):
        if getattr(self, "_h", None):
            _native.load().mf_lunnon_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def count_prefixes(self, depth: int) -> int:
        out = ctypes.c_uint64()
        check(_native.load().mf_lunnon_collect(self._h, depth, None, 0, ctypes.byref(out)))
        return out.value

    def collect(self, depth: int) -> np.ndarray:
        """Prefix states as a [S, stride] uint8 array of b[0..n] records."""
        total = self.count_prefixes(depth)
        buf = np.zeros((max(total, 1), self.stride), np.uint8)
        out = ctypes.c_uint64()
        check(_native.load().mf_lunnon_collect(self._h, depth, buf.ctypes.data, total,
                                               ctypes.byref(out)))
        return buf[:total]

    def count_states_device(self, start_leaf: int, d_states: int, num: int, d_per_state=0,
                            d_total=0, d_nodes=0, stream=0) -> None:
        """Plain kernel on device buffers (raw pointers)."""
        check(_native.load().mf_lunnon_count_states(self._h, start_leaf, d_states or None, num,
                                                    d_per_state or None, d_total or None,
                                                    d_nodes or None, stream or None))

    def count(self, depth: int = -1, mode: str | int = "batched", cfg=None):
        """(count, states, RunStats) for the whole map."""
        total = ctypes.c_uint64()
        states = ctypes.c_uint64()
        st = RunStats()
        check(_native.load().mf_lunnon_count(self._h, depth, _mode(mode), _cfg(cfg),
                                             ctypes.byref(total), ctypes.byref(states),
                                             ctypes.byref(st)))
        return total.value, states.value, st

    def count_range(self, depth: int, first_state: int = 0, max_states: int = 0,
                    mode: str | int = "batched", cfg=None):
        """(partial count, states counted, RunStats) over a range of the
        prefix states' emission order."""
        total = ctypes.c_uint64()
        states = ctypes.c_uint64()
        st = RunStats()
        check(_native.load().mf_lunnon_count_range(self._h, depth, first_state, max_states,
                                                   _mode(mode), _cfg(cfg), ctypes.byref(total),
                                                   ctypes.byref(states), ctypes.byref(st)))
        return total.value, states.value, st


def gpu_folding(grid_size: int, partition_depth: int, mode: str | int = "batched",
                dims: Sequence[int] | None = None):
    """(prefix states, total ways) as `gpu_folding <grid> <depth>` prints them."""
    dims = tuple(dims) if dims else (grid_size, grid_size)
    n = int(np.prod(dims))
    if grid_size * grid_size > 64 or n > 64:
        raise ValueError("Grid too large, max 8 (64 stamps)")
    depth = min(max(partition_depth, 0), n)
    plan = LunnonPlan(dims)
    try:
        total, states, _ = plan.count(depth, mode)
    finally:
        plan.close()
    return states, total


def lunnon_batch_count(shapes: Iterable[Sequence[int]], depths: Sequence[int] | None = None,
                       cfg=None):
    """Per-map counts of many maps in one persistent launch, plus RunStats."""
    plans = [LunnonPlan(s) for s in shapes]
    try:
        handles = (ctypes.c_void_p * len(plans))(*[p.handle for p in plans])
        d = None
        if depths is not None:
            d = (ctypes.c_int32 * len(plans))(*[int(x) for x in depths])
        out = (ctypes.c_uint64 * len(plans))()
        st = RunStats()
        check(_native.load().mf_lunnon_batch_count(handles, len(plans), d, _cfg(cfg), out,
                                                   ctypes.byref(st)))
        return [int(v) for v in out], st
    finally:
        for p in plans:
            p.close()


class LunnonBatch:
    """Many maps prepared once on the device and counted by replaying a
    recorded CUDA graph of the batched launch (mf_lunnon_batch_*)."""

    def __init__(self, shapes: Iterable[Sequence[int]], depths: Sequence[int] | None = None,
                 cfg=None):
        lib = _native.load()
        self.shapes = [tuple(s) for s in shapes]
        plans = [LunnonPlan(s) for s in self.shapes]
        try:
            handles = (ctypes.c_void_p * len(plans))(*[p.handle for p in plans])
            d = None
            if depths is not None:
                d = (ctypes.c_int32 * len(plans))(*[int(x) for x in depths])
            h = ctypes.c_void_p()
            check(lib.mf_lunnon_batch_create(handles, len(plans), d, _cfg(cfg), ctypes.byref(h)))
            self._h = h
        finally:
            for p in plans:
                p.close()

    def run(self):
        """(per-map counts, RunStats) -- one graph replay."""
        out = (ctypes.c_uint64 * len(self.shapes))()
        st = RunStats()
        check(_native.load().mf_lunnon_batch_run(self._h, out, ctypes.byref(st)))
        return [int(v) for v in out], st

    def close(self):
        if getattr(self, "_h", None):
            _native.load().mf_lunnon_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SymGraph:
    """A batched sym count on fixed device buffers, recorded once as a CUDA
    graph and replayed with launch() (mf_sym_graph_*)."""

    def __init__(self, n: int, start_i: int, stop_i: int, d_cycles: int, num: int,
                 d_counts: int, d_workspace: int, workspace_bytes: int, d_nodes: int = 0,
                 cfg=None):
        h = ctypes.c_void_p()
        check(_native.load().mf_sym_graph_create(n, start_i, stop_i, d_cycles or None, num,
                                                 d_counts or None, d_nodes or None,
                                                 d_workspace or None, workspace_bytes,
                                                 _cfg(cfg), ctypes.byref(h)))
        self._h = h

    def launch(self, stream: int = 0) -> None:
        check(_native.load().mf_graph_launch(self._h, stream or None))

    def close(self):
        if getattr(self, "_h", None):
            _native.load().mf_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sym_edges(n: int) -> np.ndarray:
    out = np.zeros((4, 64), np.uint8)
    check(_native.load().mf_sym_edges(n, out.ctypes.data))
    return out


class SymPlan:
    """Centre representatives and the expansion index (sym_fold.cpp:703-745)."""

    def __init__(self, n: int, expanded_n: int = 0, center_n: int = 0, seed_start: int = 0,
                 seed_count: int = 0):
        lib = _native.load()
        h = ctypes.c_void_p()
        opts = _native.SymPlanOptions(expanded_n, center_n, seed_start, seed_count)
        check(lib.mf_sym_plan_create_ex(n, ctypes.byref(opts), ctypes.byref(h)))
        self._h = h
        n_ = ctypes.c_int32()
        si = ctypes.c_int32()
        cc = ctypes.c_uint64()
        rc = ctypes.c_uint64()
        tc = ctypes.c_uint64()
        check(lib.mf_sym_plan_info(h, ctypes.byref(n_), ctypes.byref(si), ctypes.byref(cc),
                                   ctypes.byref(rc), ctypes.byref(tc)))
        self.n = n_.value
        self.start_i = si.value
        self.center_cases = cc.value
        self.reduced_cases = rc.value
        self.total_cases = tc.value

    def close(self):
        if getattr(self, "_h", None):
            _native.load().mf_sym_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def case_bytes(self) -> int:
        """Bytes per case record: 64, or 96 for cases expanded past 64 cells."""
        return int(_native.load().mf_sym_plan_case_bytes(self._h))

    def cases(self, start_case: int = 0, max_cases: int = 0):
        """(cycles [k, case_bytes] uint8, multipliers [k] uint64).  Plans
        whose cases go past 64 cells are streamed (no total): max_cases is
        then required."""
        lib = _native.load()
        if self.case_bytes > 64:
            want = max_cases
        else:
            avail = max(self.total_cases - start_case, 0)
            want = avail if max_cases == 0 else min(avail, max_cases)
        cyc = np.zeros((max(want, 1), self.case_bytes), np.uint8)
        mult = np.zeros(max(want, 1), np.uint64)
        out = ctypes.c_uint64()
        check(lib.mf_sym_cases(self._h, start_case, max_cases, cyc.ctypes.data, mult.ctypes.data,
                               want, ctypes.byref(out)))
        k = out.value
        return cyc[:k], mult[:k]

    def score(self, cost_depth: int, order: str | None = None, mode: str | int = "batched",
              cfg=None):
        """MF_COST_DEPTH / MF_SORT_CASES (sym_fold.cpp:267-314): score every
        case by its completions `cost_depth` cells further and, with order
        "desc" or "asc", hold the cases in that order for later chunks.
        Returns (min_score, max_score, total_score)."""
        o = {None: 0, "desc": 1, "asc": 2}[order]
        lo = ctypes.c_uint64()
        hi = ctypes.c_uint64()
        tot = (ctypes.c_uint64 * 2)()
        check(_native.load().mf_sym_plan_score(self._h, cost_depth, o, _mode(mode), _cfg(cfg),
                                               ctypes.byref(lo), ctypes.byref(hi), tot, None))
        return lo.value, hi.value, _u128(tot)

    def block_costs(self, start_case: int, count: int, cost_depth: int = 4, block: int = 1000,
                    mode: str | int = "batched", cfg=None) -> np.ndarray:
        """Estimated cost per block of `block` consecutive cases of
        [start_case, start_case + count): each case's estimate_work score at
        `cost_depth` cells further, plus one (mf_sym_plan_block_costs)."""
        out = np.zeros(max((count + block - 1) // block, 1), np.uint64)
        check(_native.load().mf_sym_plan_block_costs(self._h, start_case, count, cost_depth, block,
                                                     _mode(mode), _cfg(cfg), out.ctypes.data))
        return out[:(count + block - 1) // block]

    def solve(self, max_cases: int = 0, start_case: int = 0, mode: str | int = "batched",
              cfg=None):
        """(answer, RunStats) for the chunk, as `sym_fold` prints it."""
        ans = (ctypes.c_uint64 * 2)()
        st = RunStats()
        check(_native.load().mf_sym_plan_solve(self._h, max_cases, start_case, _mode(mode),
                                               _cfg(cfg), ans, ctypes.byref(st)))
        return _u128(ans), st


def sym_sort_order(scores, mults, ascending: bool = False) -> np.ndarray:
    """The reference's cost order (sym_fold.cpp:297-310) on the host:
    indices of the cases sorted by score, ties by multiplier."""
    s = np.ascontiguousarray(scores, dtype=np.uint64)
    m = np.ascontiguousarray(mults, dtype=np.uint64)
    perm = np.zeros(max(len(s), 1), np.uint64)
    check(_native.load().mf_sym_sort_order(s.ctypes.data, m.ctypes.data, len(s), int(ascending),
                                           perm.ctypes.data))
    return perm[:len(s)]


def sym_fold(n: int, max_cases: int = 0, start_case: int = 0, expanded_n: int = 24,
             mode: str | int = "batched", cfg=None, with_stats: bool = False):
    """The number `sym_fold n threads max_cases start_case` prints."""
    if n < 1 or n > 8:
        raise ValueError("n must be between 1 and 8")
    ans = (ctypes.c_uint64 * 2)()
    st = RunStats()
    check(_native.load().mf_sym_solve(n, max_cases, start_case, expanded_n, _mode(mode), _cfg(cfg),
                                      ans, ctypes.byref(st)))
    return (_u128(ans), st) if with_stats else _u128(ans)


def count_cases_device(n: int, start_i: int, stop_i: int, d_cycles: int, num: int, d_counts: int,
                       d_nodes: int = 0, stream: int = 0) -> None:
    """Plain per-case kernel on device buffers (raw pointers)."""
    check(_native.load().mf_sym_count_cases(n, start_i, stop_i, d_cycles or None, num,
                                            d_counts or None, d_nodes or None, stream or None))


def sym_workspace_bytes(cfg=None) -> int:
    return int(_native.load().mf_sym_workspace_bytes(_cfg(cfg)))


def count_cases_batched_device(n: int, start_i: int, stop_i: int, d_cycles: int, num: int,
                               d_counts: int, d_workspace: int, workspace_bytes: int,
                               d_nodes: int = 0, cfg=None, stream: int = 0) -> None:
    check(_native.load().mf_sym_count_cases_batched(
        n, start_i, stop_i, d_cycles or None, num, d_counts or None, d_nodes or None,
        d_workspace or None, workspace_bytes, _cfg(cfg), stream or None))


CASE_STRIDE = 112
MAX_CASES = 256


def pack_case_buffer(cycles: np.ndarray, mults: Sequence[int], n: int) -> bytes:
    """112-byte records as mfah/wasm/sym_kernel.c reads them."""
    n2 = n * n
    buf = bytearray(CASE_STRIDE * len(cycles))
    for k, (cy, m) in enumerate(zip(cycles, mults)):
        off = k * CASE_STRIDE
        buf[off:off + n2] = bytes(np.asarray(cy, np.uint8)[:n2])
        buf[off + 100:off + 108] = int(m).to_bytes(8, "little")
    return bytes(buf)


def solve_cases(n: int, start_i: int, stop_i: int, case_buffer: bytes, case_count: int):
    """(count, nodes, status) with the WASM kernel's output words."""
    out = (ctypes.c_uint32 * 8)()
    buf = ctypes.create_string_buffer(bytes(case_buffer), max(len(case_buffer), 1))
    status = _native.load().mf_solve_cases(n, start_i, stop_i, buf, case_count, out)
    count = out[0] | (out[1] << 32) | (out[2] << 64) | (out[3] << 96)
    nodes = out[4] | (out[5] << 32)
    return count, nodes, int(status)


__all__ = [
    "BatchConfig", "EngineError", "RunStats", "LunnonPlan", "LunnonBatch", "SymPlan", "SymGraph",
    "gpu_folding",
    "lunnon_batch_count", "sym_edges", "sym_fold", "count_cases_device", "sym_workspace_bytes",
    "count_cases_batched_device", "pack_case_buffer", "solve_cases",
]
