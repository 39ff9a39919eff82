"""The allocation-free batched sym entry point.

mf_sym_count_cases_batched_static serves callers that cannot allocate device
memory and so cannot hand the engine a workspace: its split-item ring lives in
a fixed device array inside the library.  This test calls it through the C ABI
(ctypes on libmapfold_gb300.so) twice in a row and checks every per-case count
and the node total against the existing workspace entry point on the same
cases -- bit for bit, since the counts are exact integers.  Its run header
(error word and work accounting), which stays inside the library's array,
is read back with mf_sym_static_status, also allocation-free; a malformed
case must show up there and as UINT64_MAX in its count slot.  It lives in
its own file, collected last, and works both alone in a fresh process and
after the other tests.
"""
import ctypes

import numpy as np
import pytest

UINT64_MAX = np.uint64(2**64 - 1)

pytestmark = pytest.mark.gpu


def _lib():
    from map_folding_gb300 import _native

    return _native.load()


def _workspace_counts(lib, torch, n, start_i, stop_i, d_cyc, num):
    counts = torch.zeros(num, dtype=torch.int64, device="cuda")
    nodes = torch.zeros(1, dtype=torch.int64, device="cuda")
    ws_bytes = lib.mf_sym_workspace_bytes(None)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    rc = lib.mf_sym_count_cases_batched(n, start_i, stop_i, ctypes.c_void_p(d_cyc.data_ptr()),
                                        num, ctypes.c_void_p(counts.data_ptr()),
                                        ctypes.c_void_p(nodes.data_ptr()),
                                        ctypes.c_void_p(ws.data_ptr()), ws_bytes, None, None)
    assert rc == 0, lib.mf_last_error()
    torch.cuda.synchronize()
    return counts.cpu().numpy().view(np.uint64).copy(), int(nodes.item())


def _static_counts(lib, torch, n, start_i, stop_i, d_cyc, num, counts, nodes):
    rc = lib.mf_sym_count_cases_batched_static(n, start_i, stop_i,
                                               ctypes.c_void_p(d_cyc.data_ptr()), num,
                                               ctypes.c_void_p(counts.data_ptr()),
                                               ctypes.c_void_p(nodes.data_ptr()), None, None)
    assert rc == 0, lib.mf_last_error()
    torch.cuda.synchronize()
    return counts.cpu().numpy().view(np.uint64).copy(), int(nodes.item())


def test_static_entry_matches_workspace_entry_twice(engine, cuda):
    torch = cuda
    lib = _lib()
    plan = engine.SymPlan(7, 24)
    cycles, _ = plan.cases(150000, 20000)
    d_cyc = torch.from_numpy(np.ascontiguousarray(cycles)).cuda()
    num = len(cycles)
    want, want_nodes = _workspace_counts(lib, torch, 7, 24, 49, d_cyc, num)
    assert want_nodes > 0 and (want != np.uint64(2**64 - 1)).all()
    # Outputs start non-zero on purpose: the entry point clears what it owns.
    counts = torch.full((num,), 7, dtype=torch.int64, device="cuda")
    nodes = torch.zeros(1, dtype=torch.int64, device="cuda")
    for call in range(2):
        nodes.zero_()
        got, got_nodes = _static_counts(lib, torch, 7, 24, 49, d_cyc, num, counts, nodes)
        assert (got == want).all(), f"call {call}"
        assert got_nodes == want_nodes, f"call {call}"


def test_static_entry_rejects_oversized_ring(engine, cuda):
    torch = cuda
    lib = _lib()
    from map_folding_gb300 import BatchConfig

    cfg = BatchConfig()
    cfg.queue_capacity = 1 << 20
    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = lib.mf_sym_count_cases_batched_static(7, 24, 49, ctypes.c_void_p(buf.data_ptr()), 1,
                                               ctypes.c_void_p(out.data_ptr()), None,
                                               ctypes.byref(cfg), None)
    assert rc == 5  # MF_ERR_CAPACITY
    assert b"4096" in lib.mf_last_error()


def _static_header(lib, torch):
    from map_folding_gb300._native import RunHeader

    hdr = RunHeader()
    rc = lib.mf_sym_static_status(None, ctypes.byref(hdr))
    assert rc == 0, lib.mf_last_error()
    torch.cuda.synchronize()
    return hdr


def test_static_entry_reports_malformed_case(engine, cuda):
    torch = cuda
    lib = _lib()
    from map_folding_gb300._native import MF_RUN_MALFORMED

    plan = engine.SymPlan(7, 24)
    cycles, _ = plan.cases(150000, 256)
    cycles = np.ascontiguousarray(cycles).copy()
    num = len(cycles)
    good = torch.from_numpy(cycles.copy()).cuda()
    want, want_nodes = _workspace_counts(lib, torch, 7, 24, 49, good, num)
    # Row 5: two cells claim the same successor, so the cycle is not a
    # permutation of the 24 placed cells.
    bad_rows = cycles.copy()
    bad_rows[5, 1] = bad_rows[5, 0]
    d_bad = torch.from_numpy(bad_rows).cuda()
    counts = torch.zeros(num, dtype=torch.int64, device="cuda")
    nodes = torch.zeros(1, dtype=torch.int64, device="cuda")
    got, _ = _static_counts(lib, torch, 7, 24, 49, d_bad, num, counts, nodes)
    hdr = _static_header(lib, torch)
    assert hdr.error == MF_RUN_MALFORMED
    assert got[5] == UINT64_MAX
    # A clean call right after it: error word cleared, accounting closed,
    # counts exact.
    nodes.zero_()
    got, got_nodes = _static_counts(lib, torch, 7, 24, 49, good, num, counts, nodes)
    hdr = _static_header(lib, torch)
    assert hdr.error == 0
    assert hdr.completed == num + hdr.split_items
    assert (got == want).all() and got_nodes == want_nodes


def test_static_entry_rejects_wide_kernel(engine, cuda):
    torch = cuda
    lib = _lib()
    from map_folding_gb300 import BatchConfig

    cfg = BatchConfig()
    cfg.stack_mode = 2
    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = lib.mf_sym_count_cases_batched_static(7, 24, 49, ctypes.c_void_p(buf.data_ptr()), 1,
                                               ctypes.c_void_p(out.data_ptr()), None,
                                               ctypes.byref(cfg), None)
    assert rc == 1  # MF_ERR_ARG
