"""ctypes binding of libmapfold_gb300.so (the C ABI in include/mapfold.h).

The library is the only compute path: if it has not been built this module
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libmapfold_gb300.so"

_i32 = ctypes.c_int32
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64
_p = ctypes.c_void_p
_pu64 = ctypes.POINTER(ctypes.c_uint64)

MF_OK = 0
MF_ERR_ARG = 1
MF_ERR_RANGE = 2
MF_ERR_CUDA = 3
MF_ERR_NO_DEVICE = 4
MF_ERR_CAPACITY = 5
MF_ERR_TIMEOUT = 6


class RunStats(ctypes.Structure):
    _fields_ = [
        ("setup_s", ctypes.c_double),
        ("h2d_s", ctypes.c_double),
        ("kernel_s", ctypes.c_double),
        ("d2h_s", ctypes.c_double),
        ("total_s", ctypes.c_double),
        ("units", ctypes.c_uint64),
        ("nodes", ctypes.c_uint64),
        ("tasks", ctypes.c_uint64),
        ("splits", ctypes.c_uint64),
        ("h2d_bytes", ctypes.c_uint64),
        ("d2h_bytes", ctypes.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class BatchConfig(ctypes.Structure):
    _fields_ = [
        ("block_threads", ctypes.c_uint32),
        ("blocks_per_sm", ctypes.c_uint32),
        ("node_budget", ctypes.c_uint32),
        ("hungry_factor", ctypes.c_uint32),
        ("queue_capacity", ctypes.c_uint64),
        ("wait_limit", ctypes.c_uint32),
        ("stack_mode", ctypes.c_uint32),
    ]


class SymPlanOptions(ctypes.Structure):
    _fields_ = [
        ("expanded_n", ctypes.c_int32),
        ("center_n", ctypes.c_int32),
        ("seed_start", ctypes.c_uint64),
        ("seed_count", ctypes.c_uint64),
    ]


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("unit_capacity", ctypes.c_uint64),
        ("max_requests", ctypes.c_uint32),
        ("block_threads", ctypes.c_uint32),
        ("table_bytes", ctypes.c_uint64),
        ("node_budget", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("queue_capacity", ctypes.c_uint64),
    ]


class RequestInfo(ctypes.Structure):
    _fields_ = [
        ("submit_s", ctypes.c_double),
        ("admit_s", ctypes.c_double),
        ("done_s", ctypes.c_double),
        ("units", ctypes.c_uint64),
        ("nodes", ctypes.c_uint64),
    ]


class RunHeader(ctypes.Structure):
    """mf_run_header: the 64-byte header of a persistent launch."""
    _fields_ = [
        ("units_handed_out", ctypes.c_uint64),
        ("split_head", ctypes.c_uint64),
        ("split_items", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("work_items_run", ctypes.c_uint64),
        ("error", ctypes.c_uint32),
        ("pad", ctypes.c_uint32),
        ("idle_lanes", ctypes.c_int64),
        ("warps_out", ctypes.c_uint64),
    ]


MF_RUN_MALFORMED = 1
MF_RUN_WAIT_LIMIT = 2
MF_FAULT_LOST_SPLIT = 1


class EngineError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"mapfold status {status}: {message}")
        self.status = status


# Every symbol include/mapfold.h declares, with its ctypes signature.
SIGNATURES = {
    "mf_last_error": ([], ctypes.c_char_p),
    "mf_abi_version": ([], _i32),
    "mf_lunnon_plan_create": ([_p, _i32, ctypes.POINTER(_p)], _i32),
    "mf_lunnon_plan_destroy": ([_p], None),
    "mf_lunnon_leaves": ([_p], _i32),
    "mf_lunnon_state_stride": ([_p], _u32),
    "mf_lunnon_collect": ([_p, _i32, _p, _u64, _pu64], _i32),
    "mf_lunnon_count_states": ([_p, _i32, _p, _u64, _p, _p, _p, _p], _i32),
    "mf_lunnon_count": ([_p, _i32, _i32, _p, _pu64, _pu64, _p], _i32),
    "mf_lunnon_count_range": ([_p, _i32, _u64, _u64, _i32, _p, _pu64, _pu64, _p], _i32),
    "mf_lunnon_batch_count": ([_p, _i32, _p, _p, _p, _p], _i32),
    "mf_sym_edges": ([_i32, _p], _i32),
    "mf_sym_plan_create": ([_i32, _i32, ctypes.POINTER(_p)], _i32),
    "mf_sym_plan_create_ex": ([_i32, _p, ctypes.POINTER(_p)], _i32),
    "mf_sym_plan_destroy": ([_p], None),
    "mf_sym_plan_info": ([_p, _p, _p, _p, _p, _p], _i32),
    "mf_sym_cases": ([_p, _u64, _u64, _p, _p, _u64, _pu64], _i32),
    "mf_sym_plan_case_bytes": ([_p], _u32),
    "mf_sym_count_cases": ([_i32, _i32, _i32, _p, _u64, _p, _p, _p], _i32),
    "mf_sym_workspace_bytes": ([_p], _u64),
    "mf_sym_count_cases_batched": ([_i32, _i32, _i32, _p, _u64, _p, _p, _p, _u64, _p, _p], _i32),
    "mf_sym_plan_solve": ([_p, _u64, _u64, _i32, _p, _p, _p], _i32),
    "mf_sym_plan_score": ([_p, _i32, _i32, _i32, _p, _pu64, _pu64, _p, _p], _i32),
    "mf_sym_sort_order": ([_p, _p, _u64, _i32, _p], _i32),
    "mf_sym_plan_block_costs": ([_p, _u64, _u64, _i32, _u64, _i32, _p, _p], _i32),
    "mf_sym_count_cases_batched_static": ([_i32, _i32, _i32, _p, _u64, _p, _p, _p, _p], _i32),
    "mf_sym_static_status": ([_p, _p], _i32),
    "mf_test_inject_fault": ([_u32], None),
    "mf_sym_graph_create": ([_i32, _i32, _i32, _p, _u64, _p, _p, _p, _u64, _p,
                             ctypes.POINTER(_p)], _i32),
    "mf_graph_launch": ([_p, _p], _i32),
    "mf_graph_destroy": ([_p], None),
    "mf_lunnon_batch_create": ([_p, _i32, _p, _p, ctypes.POINTER(_p)], _i32),
    "mf_lunnon_batch_run": ([_p, _p, _p], _i32),
    "mf_lunnon_batch_destroy": ([_p], None),
    "mf_server_create": ([_p, ctypes.POINTER(_p)], _i32),
    "mf_server_submit_sym": ([_p, _i32, _i32, _u64, _u64, _pu64], _i32),
    "mf_server_submit_lunnon": ([_p, _p, _i32, _i32, _pu64], _i32),
    "mf_server_poll": ([_p, _u64, ctypes.POINTER(_i32), _p, _p], _i32),
    "mf_server_wait": ([_p, _u64, ctypes.c_double, _p, _p], _i32),
    "mf_server_destroy": ([_p], None),
    "mf_sym_solve": ([_i32, _u64, _u64, _i32, _i32, _p, _p, _p], _i32),
    "mf_solve_cases": ([_u32, _u32, _u32, _p, _u32, _p], _u32),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load the engine library, failing loudly if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH.name} is not built: run `python -m map_folding_gb300.build` "
                "(the engine has no non-CUDA path)")
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def check(status: int) -> None:
    if status != MF_OK:
        msg = load().mf_last_error()
        raise EngineError(status, msg.decode() if msg else "")
