"""Build the engine's shared library and drop-in CLIs with nvcc (sm_103a).

    python -m map_folding_gb300.build          # library + CLIs, in place

Outputs (git-ignored, rebuilt on each machine):
    map_folding_gb300/libmapfold_gb300.so      the C ABI of include/mapfold.h
    map_folding_gb300/bin/gpu_folding          `gpu_folding <n> <depth>` drop-in
    map_folding_gb300/bin/sym_fold             `sym_fold n [threads] [max start]`
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libmapfold_gb300.so"
BIN = PKG / "bin"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include")]
LIB_SOURCES = ["host.cpp", "capi.cpp", "dfs_kernels.cu", "wide_kernels.cu", "serve.cu"]
# name -> (source, extra compiler flags); sym_fold9 is sym_fold's source with
# experiments/9x9/sym_fold9.cpp's options switched on.
CLI_SOURCES = {"gpu_folding": ("cli_gpu_folding.cpp", []),
               "gpu_folding_v2": ("cli_gpu_folding_v2.cpp", []),
               "sym_fold": ("cli_sym_fold.cpp", []),
               "sym_fold9": ("cli_sym_fold.cpp", ["-DMF_SYM_FOLD9"])}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the engine is built for sm_103a with nvcc")
    return cand


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    headers = (sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.inl")) + sorted(CSRC.glob("*.cuh"))
               + [ROOT / "include" / "mapfold.h"])
    cc = nvcc()
    jobs = []
    objs = []
    for src in LIB_SOURCES:
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc, *COMMON, *ARCH, "-c", str(s), "-o", str(o)])
    for name, (src, flags) in CLI_SOURCES.items():
        s = CSRC / src
        o = OBJ / f"cli_{name}.o"
        if force or _stale(o, [s] + headers):
            jobs.append([cc, *COMMON, *flags, "-c", str(s), "-o", str(o)])
    workers = min(len(jobs), os.cpu_count() or 4) or 1
    with ThreadPoolExecutor(max_workers=workers) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, jobs))
    if force or _stale(LIB, objs):
        # Link to a temporary name and rename: the linker rewrites an existing
        # output in place, which would corrupt processes that have it mapped.
        tmp = LIB.with_suffix(".so.tmp")
        _run([cc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart",
              "-Xcompiler", "-pthread"])
        os.replace(tmp, LIB)
    for name, (src, _) in CLI_SOURCES.items():
        o = OBJ / f"cli_{name}.o"
        exe = BIN / name
        if force or _stale(exe, [o, LIB]):
            _run([cc, "-o", str(exe), str(o), f"-L{PKG}", "-lmapfold_gb300",
                  f"-Xlinker=-rpath,{PKG}", "-Xcompiler", "-pthread"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
