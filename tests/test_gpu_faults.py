"""Bounded device-side waits end with an error status, never a hang.

Every wait in the persistent kernels is bounded by cfg.wait_limit idle rounds.
These tests make a wait run out without faulting anything: the host-side
fault hook (mf_test_inject_fault, MF_FAULT_LOST_SPLIT) reserves one split-ring
ticket that no lane ever publishes -- a donor's message lost on the way -- so
the items queued behind it are never taken and the work accounting cannot
close.  The idle warps leave after wait_limit rounds, the last one out raises
error word MF_RUN_WAIT_LIMIT, and the host-buffer entry points return
MF_ERR_TIMEOUT within a fraction of a second.  The next, clean, call on the
same context -- with the same small wait_limit, where warps that run out of
work leave early as a matter of course -- must give the exact count again.
(The reference has no device-side waits; its analogue is CUDA_CHECK,
gpu_folding_v2.cu:101-109.)
"""
import time

import pytest

pytestmark = pytest.mark.gpu


def _inject(engine):
    from map_folding_gb300 import _native

    _native.load().mf_test_inject_fault(_native.MF_FAULT_LOST_SPLIT)


def test_lost_split_item_times_out_sym(engine, cuda, golden):
    from map_folding_gb300._native import MF_ERR_TIMEOUT, EngineError

    plan = engine.SymPlan(7, 24)
    try:
        cfg = {"wait_limit": 64}
        _inject(engine)
        t0 = time.perf_counter()
        with pytest.raises(EngineError) as err:
            plan.solve(2000, 0, "batched", cfg)
        elapsed = time.perf_counter() - t0
        assert err.value.status == MF_ERR_TIMEOUT, err.value
        assert elapsed < 30.0
        # The context is still usable and the next call is exact.
        ans, _ = plan.solve(2000, 0, "batched", cfg)
        assert ans == golden["sym"]["7x7_d24_first2000"]
    finally:
        plan.close()


def test_lost_split_item_times_out_lunnon(engine, cuda, golden):
    from map_folding_gb300._native import MF_ERR_TIMEOUT, EngineError

    plan = engine.LunnonPlan((5, 6))
    try:
        cfg = {"wait_limit": 64}
        _inject(engine)
        with pytest.raises(EngineError) as err:
            plan.count(12, "batched", cfg)
        assert err.value.status == MF_ERR_TIMEOUT, err.value
        count, _, _ = plan.count(12, "batched", cfg)
        assert count == golden["lunnon"]["5x6"]
    finally:
        plan.close()


def test_fault_hook_is_one_shot(engine, cuda, golden):
    from map_folding_gb300 import _native

    lib = _native.load()
    lib.mf_test_inject_fault(_native.MF_FAULT_LOST_SPLIT)
    lib.mf_test_inject_fault(0)  # cleared before any launch
    plan = engine.LunnonPlan((4, 5))
    try:
        count, _, _ = plan.count(8, "batched", {"wait_limit": 64})
        assert count == golden["lunnon"]["4x5"]
    finally:
        plan.close()
