"""Request serving: a continuous-batching server and a Poisson load driver.

`Server` wraps mf_server_* (include/mapfold.h): one persistent kernel that
keeps running while requests arrive; a request (an 8x8 sym_fold chunk, a
whole small map) is admitted as soon as a slot and unit-arena memory are
free and then shares the GPU with the requests already running.

`run_stream` replays a timed request list (workloads.serving_stream) in real
time, submitting each request at its arrival time, and reports per-request
latency (submit -> result seen by the server), p50/p99 and throughput.
"""
from __future__ import annotations

import ctypes
import statistics
import time
from typing import Sequence

from . import _native
from ._native import RequestInfo, ServerConfig, check
from .workloads import Request


def _u128(words) -> int:
    return (int(words[1]) << 64) | int(words[0])


class Server:
    def __init__(self, unit_capacity: int = 0, max_requests: int = 0, table_bytes: int = 0,
                 node_budget: int = 0, queue_capacity: int = 0):
        cfg = ServerConfig()
        cfg.unit_capacity = unit_capacity
        cfg.max_requests = max_requests
        cfg.table_bytes = table_bytes
        cfg.node_budget = node_budget
        cfg.queue_capacity = queue_capacity
        h = ctypes.c_void_p()
        check(_native.load().mf_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def submit_sym(self, n: int, expanded_n: int, start_case: int, max_cases: int) -> int:
        rid = ctypes.c_uint64()
        check(_native.load().mf_server_submit_sym(self._h, n, expanded_n, start_case, max_cases,
                                                  ctypes.byref(rid)))
        return rid.value

    def submit_lunnon(self, dims: Sequence[int], depth: int = -1) -> int:
        arr = (ctypes.c_int32 * len(dims))(*[int(d) for d in dims])
        rid = ctypes.c_uint64()
        check(_native.load().mf_server_submit_lunnon(self._h, arr, len(dims), depth,
                                                     ctypes.byref(rid)))
        return rid.value

    def poll(self, rid: int):
        """(done, answer, RequestInfo)."""
        done = ctypes.c_int32()
        ans = (ctypes.c_uint64 * 2)()
        info = RequestInfo()
        check(_native.load().mf_server_poll(self._h, rid, ctypes.byref(done), ans,
                                            ctypes.byref(info)))
        return bool(done.value), _u128(ans), info

    def wait(self, rid: int, timeout_s: float = 600.0):
        """(answer, RequestInfo); raises EngineError on timeout."""
        ans = (ctypes.c_uint64 * 2)()
        info = RequestInfo()
        check(_native.load().mf_server_wait(self._h, rid, timeout_s, ans, ctypes.byref(info)))
        return _u128(ans), info

    def close(self):
        if getattr(self, "_h", None):
            _native.load().mf_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def submit(server: Server, req: Request, expanded_n: int = 36) -> int:
    if req.kind == "chunk":
        return server.submit_sym(8, expanded_n, req.start_case, req.max_cases)
    return server.submit_lunnon(req.dims)


def run_stream(server: Server, requests: Sequence[Request], expanded_n: int = 36,
               timeout_s: float = 3600.0) -> dict:
    """Submit each request at its arrival time, wait for all, summarise."""
    t0 = time.perf_counter()
    ids = []
    for req in requests:
        delay = req.arrival_s - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        ids.append(submit(server, req, expanded_n))
    results = []
    for req, rid in zip(requests, ids):
        ans, info = server.wait(rid, timeout_s)
        results.append({"rid": req.rid, "kind": req.kind, "answer": ans,
                        "latency_s": info.done_s - info.submit_s,
                        "queue_s": info.admit_s - info.submit_s,
                        "units": int(info.units), "nodes": int(info.nodes),
                        "start_case": req.start_case, "max_cases": req.max_cases,
                        "dims": list(req.dims)})
    wall = time.perf_counter() - t0
    chunk_lat = sorted(r["latency_s"] for r in results if r["kind"] == "chunk")
    all_lat = sorted(r["latency_s"] for r in results)

    def pct(v, q):
        if not v:
            return None
        k = min(len(v) - 1, max(0, int(round(q * (len(v) - 1)))))
        return v[k]

    cases = sum(r["units"] for r in results if r["kind"] == "chunk")
    nodes = sum(r["nodes"] for r in results)
    return {
        "requests": len(results),
        "wall_s": wall,
        "chunk_p50_s": pct(chunk_lat, 0.50),
        "chunk_p99_s": pct(chunk_lat, 0.99),
        "all_p50_s": pct(all_lat, 0.50),
        "all_p99_s": pct(all_lat, 0.99),
        "mean_latency_s": statistics.fmean(all_lat) if all_lat else None,
        "cases_per_s": cases / wall if wall else None,
        "nodes_per_s": nodes / wall if wall else None,
        "results": results,
    }
