"""ctypes binding of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The product package never
imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"

_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_p = ctypes.c_void_p


class Work(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_uint64), ("steps", ctypes.c_uint64)]


def build(force: bool = False) -> Path:
    """Compile oracle.c into liboracle.so (gcc, no -march flags)."""
    src = HERE / "oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.orc_lunnon_count.argtypes = [_p, _i32, _i32, _i32, ctypes.POINTER(Work)]
        L.orc_lunnon_count.restype = _i64
        L.orc_lunnon_collect.argtypes = [_p, _i32, _i32, _p, _p, _p, _i64]
        L.orc_lunnon_collect.restype = _i64
        L.orc_lunnon_resume.argtypes = [_p, _i32, _i32, _p, _p, ctypes.POINTER(Work)]
        L.orc_lunnon_resume.restype = _u64
        L.orc_lunnon_resume_many.argtypes = [_p, _i32, _i32, _p, _p, _i64, _i32, _p,
                                             ctypes.POINTER(Work)]
        L.orc_lunnon_resume_many.restype = _u64
        L.orc_sym_edges.argtypes = [_i32, _p]
        L.orc_sym_edges.restype = None
        L.orc_sym_good.argtypes = [_p, _i32, _p, ctypes.POINTER(Work)]
        L.orc_sym_good.restype = _u64
        L.orc_sym_count.argtypes = [_p, _i32, _i32, _p, ctypes.POINTER(Work)]
        L.orc_sym_count.restype = _u64
        L.orc_sym_count_to.argtypes = [_p, _i32, _i32, _p, ctypes.POINTER(Work)]
        L.orc_sym_count_to.restype = _u64
        L.orc_sym_reps.argtypes = [_i32, _p, _p, _i64, ctypes.POINTER(_i64)]
        L.orc_sym_reps.restype = _i64
        L.orc_sym_estimate_cases.argtypes = [_i32, _i32, _i32, _p, _i64, _i32, _p]
        L.orc_sym_estimate_cases.restype = None
        L.orc_sym_expand.argtypes = [_i32, _i32, _u64, _u64, _p, _p, _i64]
        L.orc_sym_expand.restype = _i64
        L.orc_sym_count_cases.argtypes = [_i32, _i32, _p, _p, _i64, _i32, _p, _p,
                                          ctypes.POINTER(Work)]
        L.orc_sym_count_cases.restype = None
        L.orc_sym_solve.argtypes = [_i32, _i32, _u64, _u64, _i32, _p, ctypes.POINTER(Work)]
        L.orc_sym_solve.restype = _i32
        _lib = L
    return _lib


def _dims(dims):
    arr = np.ascontiguousarray(np.asarray(dims, dtype=np.int32))
    return arr, arr.ctypes.data, len(arr)


def lunnon_count(dims, res: int = 0, mod: int = 0):
    """(count, Work) for a whole map, mf.c semantics."""
    arr, ptr, nd = _dims(dims)
    w = Work()
    c = lib().orc_lunnon_count(ptr, nd, res, mod, ctypes.byref(w))
    if c < 0:
        raise ValueError(f"bad dims {dims}")
    return int(c), w


def lunnon_collect(dims, depth: int):
    """Prefix states (a, b, gapter) as uint8/uint8/uint16 arrays [S, n+1]."""
    arr, ptr, nd = _dims(dims)
    n = int(np.prod(arr))
    total = lib().orc_lunnon_collect(ptr, nd, depth, None, None, None, 0)
    if total < 0:
        raise ValueError("bad input")
    a = np.zeros((max(total, 1), n + 1), np.uint8)
    b = np.zeros((max(total, 1), n + 1), np.uint8)
    g = np.zeros((max(total, 1), n + 1), np.uint16)
    lib().orc_lunnon_collect(ptr, nd, depth, a.ctypes.data, b.ctypes.data, g.ctypes.data, total)
    return a[:total], b[:total], g[:total]


def lunnon_resume_many(dims, start_leaf: int, a, b, threads: int = 1):
    arr, ptr, nd = _dims(dims)
    a = np.ascontiguousarray(a, dtype=np.uint8)
    b = np.ascontiguousarray(b, dtype=np.uint8)
    per = np.zeros(len(a), np.uint64)
    w = Work()
    total = lib().orc_lunnon_resume_many(ptr, nd, start_leaf, a.ctypes.data, b.ctypes.data,
                                         len(a), threads, per.ctypes.data, ctypes.byref(w))
    return int(total), per, w


def sym_edges(n: int) -> np.ndarray:
    out = np.zeros((4, 64), np.uint8)
    lib().orc_sym_edges(n, out.ctypes.data)
    return out


def sym_count_to(n: int, cycle, start_i: int, stop: int):
    """(count, Work) of cycles reaching `stop` cells, sym_kernel.c semantics."""
    cy = np.zeros(64, np.uint8)
    src = np.asarray(cycle, np.uint8)
    cy[:len(src)] = src
    e = sym_edges(n)
    w = Work()
    c = lib().orc_sym_count_to(cy.ctypes.data, start_i, stop, e.ctypes.data, ctypes.byref(w))
    return int(c), w


def sym_raw_prefixes(n: int, depth: int):
    """Cycles at `depth` cells grown from the 3-cell cycle, in DFS order
    (mfah/folding.py:148-176 generate_prefixes, as byte arrays)."""
    e = sym_edges(n)
    out = []
    cy = np.zeros(64, np.uint8)
    cy[0], cy[1], cy[2] = 1, 2, 0

    def visit(i):
        if i == depth:
            out.append(cy.copy())
            return
        good = int(lib().orc_sym_good(cy.ctypes.data, i, e.ctypes.data, None))
        while good:
            j = (good & -good).bit_length() - 1
            good &= good - 1
            nxt = int(cy[j])
            cy[i] = nxt
            cy[j] = i
            visit(i + 1)
            cy[j] = nxt

    visit(3)
    return np.array(out, np.uint8).reshape(-1, 64)


def sym_reps(n: int):
    cc = _i64(0)
    k = lib().orc_sym_reps(n, None, None, 0, ctypes.byref(cc))
    cyc = np.zeros((k, 64), np.uint8)
    mult = np.zeros(k, np.uint64)
    lib().orc_sym_reps(n, cyc.ctypes.data, mult.ctypes.data, k, None)
    return cyc, mult, int(cc.value)


def sym_expand(n: int, expanded_n: int, start_case: int = 0, max_cases: int = 0):
    k = lib().orc_sym_expand(n, expanded_n, start_case, max_cases, None, None, 0)
    if k < 0:
        raise ValueError("bad input")
    cyc = np.zeros((max(k, 1), 64), np.uint8)
    mult = np.zeros(max(k, 1), np.uint64)
    lib().orc_sym_expand(n, expanded_n, start_case, max_cases, cyc.ctypes.data,
                         mult.ctypes.data, k)
    return cyc[:k], mult[:k]


def sym_estimate_cases(n: int, start_i: int, depth: int, cycles, threads: int = 1) -> np.ndarray:
    """Per-case estimate_work scores (sym_fold.cpp:235-250, :274-283)."""
    cycles = np.ascontiguousarray(cycles, dtype=np.uint8)
    scores = np.zeros(max(len(cycles), 1), np.uint64)
    lib().orc_sym_estimate_cases(n, start_i, depth, cycles.ctypes.data, len(cycles), threads,
                                 scores.ctypes.data)
    return scores[:len(cycles)]


def sym_count_cases(n: int, start_i: int, cycles, mults=None, threads: int = 1):
    cycles = np.ascontiguousarray(cycles, dtype=np.uint8)
    count = len(cycles)
    per = np.zeros(max(count, 1), np.uint64)
    s = np.zeros(2, np.uint64)
    w = Work()
    mptr = None
    if mults is not None:
        mults = np.ascontiguousarray(mults, dtype=np.uint64)
        mptr = mults.ctypes.data
    lib().orc_sym_count_cases(n, start_i, cycles.ctypes.data, mptr, count, threads,
                              per.ctypes.data, s.ctypes.data, ctypes.byref(w))
    return (int(s[1]) << 64) | int(s[0]), per[:count], w


def sym_solve(n: int, threads: int = 1, max_cases: int = 0, start_case: int = 0,
              expanded_n: int = 0):
    out = np.zeros(2, np.uint64)
    w = Work()
    rc = lib().orc_sym_solve(n, threads, max_cases, start_case, expanded_n, out.ctypes.data,
                             ctypes.byref(w))
    if rc != 0:
        raise ValueError(f"sym_solve rc={rc}")
    return (int(out[1]) << 64) | int(out[0]), w


def ref_binary(name: str):
    """Path of a reference binary built by `make -C oracle ref`, or None."""
    p = REF_DIR / name
    return p if p.exists() and os.access(p, os.X_OK) else None
