"""The request server: mixed 8x8 / 7x7 sym chunks and whole Lunnon maps,
submitted while others run; every result must equal the reference's count
(golden) and the same request served alone."""
import time

import pytest

pytestmark = pytest.mark.gpu

SYM = [
    # (golden key, n, expanded_n, max_cases, start_case)
    ("8x8_d36_first200", 8, 36, 200, 0),
    ("8x8_d36_120000000+200", 8, 36, 200, 120000000),
    ("8x8_d36_240192700+500", 8, 36, 500, 240192700),
    ("7x7_d24_first2000", 7, 24, 2000, 0),
    ("7x7_d24_300000+500", 7, 24, 500, 300000),
]
MAPS = ["4x5", "3x6", "2x2x4", "5x5", "1x16"]


def test_mixed_requests_match_alone_and_reference(engine, cuda, golden):
    from map_folding_gb300.serving import Server

    with Server() as srv:
        # alone: one request at a time
        alone = {}
        for key, n, e, m, s in SYM:
            alone[key] = srv.wait(srv.submit_sym(n, e, s, m))[0]
        for key in MAPS:
            dims = tuple(int(x) for x in key.split("x"))
            alone[key] = srv.wait(srv.submit_lunnon(dims))[0]
        # mixed: everything in flight at once, interleaved, twice over
        ids = []
        for rep in range(2):
            for (key, n, e, m, s), mkey in zip(SYM, MAPS):
                ids.append((key, srv.submit_sym(n, e, s, m)))
                dims = tuple(int(x) for x in mkey.split("x"))
                ids.append((mkey, srv.submit_lunnon(dims)))
        mixed = [(key, srv.wait(rid)[0]) for key, rid in ids]
    for key, n, e, m, s in SYM:
        assert alone[key] == golden["sym"][key], key
    for key in MAPS:
        assert alone[key] == golden["lunnon"][key], key
    for key, ans in mixed:
        assert ans == alone[key], key


def test_requests_admitted_while_others_run(engine, cuda, golden):
    from map_folding_gb300.serving import Server

    with Server(unit_capacity=1 << 12, max_requests=8) as srv:
        # the arena holds 4096 units: later chunks wait for memory, then run
        # while earlier ones are still on the GPU
        rids = [srv.submit_sym(7, 24, 300000, 500) for _ in range(12)]
        time.sleep(0.01)
        late = srv.submit_lunnon((4, 5), depth=10)  # 480 prefix states
        answers = [srv.wait(r)[0] for r in rids]
        ans_late, info = srv.wait(late)
    assert answers == [golden["sym"]["7x7_d24_300000+500"]] * 12
    assert ans_late == golden["lunnon"]["4x5"]
    assert info.done_s >= info.admit_s >= info.submit_s


def test_request_larger_than_arena_is_refused(engine, cuda):
    from map_folding_gb300._native import MF_ERR_CAPACITY, EngineError
    from map_folding_gb300.serving import Server

    with Server(unit_capacity=1 << 12, max_requests=8) as srv:
        with pytest.raises(EngineError) as e:
            srv.submit_lunnon((4, 5), depth=13)  # 5904 prefix states > 4096
        assert e.value.status == MF_ERR_CAPACITY


def test_poisson_stream_driver(engine, cuda):
    from map_folding_gb300.serving import Server, run_stream
    from map_folding_gb300.workloads import serving_stream

    reqs = serving_stream(seed=11, requests=6, rate_per_s=20.0, chunk_cases=300)
    with Server() as srv:
        out = run_stream(srv, reqs)
        # the same requests alone give the same answers
        for r in out["results"]:
            if r["kind"] == "chunk":
                rid = srv.submit_sym(8, 36, r["start_case"], r["max_cases"])
            else:
                rid = srv.submit_lunnon(tuple(r["dims"]))
            assert srv.wait(rid)[0] == r["answer"]
    assert out["requests"] == 6 and out["chunk_p99_s"] is not None
