"""Host side of the serving benchmark without a GPU: the seeded request
stream (8x8 chunks at MF_EXPANDED_N=36 and whole maps up to 5x6, Poisson
arrivals) and run_stream's latency and throughput bookkeeping, driven
through a stand-in server."""
from types import SimpleNamespace

from map_folding_gb300.serving import run_stream
from map_folding_gb300.workloads import TOTAL_8X8_D36, serving_stream


def test_stream_is_seeded_and_in_range():
    a = serving_stream(seed=5, requests=200, rate_per_s=50.0, chunk_cases=50_000)
    b = serving_stream(seed=5, requests=200, rate_per_s=50.0, chunk_cases=50_000)
    assert [(r.kind, r.arrival_s, r.start_case, r.dims) for r in a] == \
           [(r.kind, r.arrival_s, r.start_case, r.dims) for r in b]
    times = [r.arrival_s for r in a]
    assert times == sorted(times) and times[0] > 0
    chunks = [r for r in a if r.kind == "chunk"]
    maps = [r for r in a if r.kind == "map"]
    assert chunks and maps
    for r in chunks:
        assert r.max_cases == 50_000 and 0 <= r.start_case <= TOTAL_8X8_D36 - 50_000
    for r in maps:
        p, q = r.dims
        assert 2 <= p <= 5 and 2 <= q <= 6


class FakeServer:
    """Answers every request at once; request k takes k+1 seconds."""

    def __init__(self):
        self.calls = []

    def submit_sym(self, n, expanded_n, start_case, max_cases):
        self.calls.append(("sym", n, expanded_n, start_case, max_cases))
        return len(self.calls) - 1

    def submit_lunnon(self, dims, depth=-1):
        self.calls.append(("lunnon", tuple(dims)))
        return len(self.calls) - 1

    def wait(self, rid, timeout_s=0.0):
        kind = self.calls[rid][0]
        units = self.calls[rid][4] if kind == "sym" else 10
        info = SimpleNamespace(submit_s=100.0, admit_s=100.5, done_s=101.0 + rid, units=units,
                               nodes=1000 * (rid + 1))
        return 7 * (rid + 1), info


def test_run_stream_bookkeeping():
    reqs = serving_stream(seed=3, requests=10, rate_per_s=1e6, chunk_cases=1000)
    srv = FakeServer()
    out = run_stream(srv, reqs)
    assert out["requests"] == 10 and len(srv.calls) == 10
    for r, call in zip(reqs, srv.calls):
        if r.kind == "chunk":
            assert call == ("sym", 8, 36, r.start_case, 1000)
        else:
            assert call == ("lunnon", r.dims)
    lat = [1.0 + k for k in range(10)]
    chunk_lat = sorted(1.0 + k for k, r in enumerate(reqs) if r.kind == "chunk")
    assert [res["latency_s"] for res in out["results"]] == lat
    assert all(res["queue_s"] == 0.5 for res in out["results"])
    assert out["all_p99_s"] == max(lat) and out["chunk_p99_s"] == chunk_lat[-1]
    assert out["chunk_p50_s"] == chunk_lat[round(0.5 * (len(chunk_lat) - 1))]
    n_chunks = len(chunk_lat)
    assert out["cases_per_s"] == n_chunks * 1000 / out["wall_s"]
    assert [res["answer"] for res in out["results"]] == [7 * (k + 1) for k in range(10)]
