"""The allocation-free batched sym entry point.

mf_sym_count_cases_batched_static serves callers that cannot allocate device
memory and so cannot hand the engine a workspace: its split-item ring lives in
a fixed device array inside the library.  This test calls it through the C ABI
(ctypes on libmapfold_gb300.so) twice in a row and checks every per-case count
and the node total against the existing workspace entry point on the same
cases -- bit for bit, since the counts are exact integers.  It lives in its
own file, collected last, and works both alone in a fresh process and after
the other tests.
"""
import ctypes

import numpy as np
import pytest

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
