"""The drop-in CLIs against the reference's own binaries (built from source
into oracle/_ref by `make -C oracle ref`), on every path that needs no GPU:
argument errors, trivial sizes, setup-only runs.  Exit code, stdout and
stderr must agree, apart from timing fields and the executable's path.
Skipped where the reference binaries have not been built."""
import os
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = ROOT / "oracle" / "_ref"


def _run(exe, args, env):
    e = dict(os.environ)
    for k in list(e):
        if k.startswith("MF_"):
            del e[k]
    e.update(env)
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, env=e,
                       timeout=300)
    norm = lambda s: re.sub(r"(total_s|score_s|elapsed_s)=[0-9.e+-]+", r"\1=T",
                            s.replace(str(exe), "EXE"))
    return r.returncode, norm(r.stdout), norm(r.stderr)


SYM_CASES = [
    ([], {}), (["x7"], {}), ([9], {}), ([7, 0], {}), ([7, 4, "abc"], {}),
    ([7, 4, 10, "zz"], {}), ([1], {}), ([2], {}), ([7, 4], {"MF_EXPANDED_N": "5"}),
    ([7, 4], {"MF_SETUP_ONLY": "1"}), ([7, 4], {"MF_SETUP_ONLY": "1", "MF_STREAM_CASES": "1"}),
    ([6, 4], {"MF_SETUP_ONLY": "1"}), ([8, 4], {"MF_SETUP_ONLY": "1", "MF_EXPANDED_N": "20"}),
    ([7, 1, 10, 0], {"MF_STREAM_CASES": "1", "MF_QUEUE_SIZE": "abc"}),
]


@pytest.mark.parametrize("args,env", SYM_CASES)
def test_sym_fold_matches_reference_binary(engine, args, env):
    from map_folding_gb300 import build as mfbuild

    ref = REF / "sym_fold"
    if not ref.exists():
        pytest.skip("reference sym_fold not built here")
    assert _run(mfbuild.BIN / "sym_fold", args, env) == _run(ref, args, env)


SYM9_CASES = [
    ([10], {}), ([9, 1], {"MF_CENTER_N": "4"}), ([9, 1], {"MF_CENTER_N": "7"}),
    ([9, 1], {"MF_CENTER_N": "5", "MF_SETUP_ONLY": "1"}),
    ([9, 1], {"MF_CENTER_N": "5", "MF_SETUP_ONLY": "1", "MF_CENTER_STREAM_DEDUP": "1",
              "MF_STREAM_CASES": "1", "MF_SEED_START": "1000", "MF_SEED_COUNT": "10"}),
    ([7, 1], {"MF_CENTER_N": "5", "MF_SETUP_ONLY": "1", "MF_EXPANDED_N": "25"}),
    ([9, 1], {"MF_CENTER_N": "3", "MF_SETUP_ONLY": "1"}),
    ([9, 1], {"MF_CENTER_N": "3", "MF_SETUP_ONLY": "1", "MF_EXPANDED_N": "20"}),
    ([9, 1], {"MF_CENTER_N": "5", "MF_SETUP_ONLY": "1", "MF_EXPANDED_N": "24"}),
    ([9, 1], {"MF_CENTER_N": "5", "MF_SETUP_ONLY": "1", "MF_STREAM_CASES": "1",
              "MF_SEED_START": "99999999"}),
    ([7, 1], {"MF_CENTER_N": "3", "MF_SETUP_ONLY": "1"}),
    ([8, 1], {"MF_CENTER_N": "4", "MF_SETUP_ONLY": "1", "MF_EXPANDED_N": "20"}),
    ([6, 1], {"MF_SETUP_ONLY": "1"}),
    # bad slice text: reported after the centre lines, rc 2
    ([9, 1], {"MF_CENTER_N": "5", "MF_SEED_START": "x"}),
    ([9, 1], {"MF_CENTER_N": "5", "MF_SEED_START": "3", "MF_SEED_COUNT": "y"}),
]


@pytest.mark.parametrize("args,env", SYM9_CASES)
def test_sym_fold9_matches_reference_binary(engine, args, env):
    from map_folding_gb300 import build as mfbuild

    ref = REF / "sym_fold9"
    if not ref.exists():
        pytest.skip("reference sym_fold9 not built here")
    assert _run(mfbuild.BIN / "sym_fold9", args, env) == _run(ref, args, env)


# Paths of the reference's CUDA drivers that end before any CUDA call.
GPU_FOLDING_CASES = [[], [5], [9, 5], [10, 3]]
GPU_FOLDING_V2_CASES = [[], [6], ["x", 18], [6, "y"], [10, 18], [0, 5], [6, 0], [6, 37],
                        [6, 18, 0], [6, 18, 5000, 0], [6, 18, 5000, 128, 8, 4, 0],
                        [6, 18, 5000, 128, 8, 4, 8, "q"], [6, 18, 1, 2, 3, 4, 5, 6, 7]]


@pytest.mark.parametrize("args", GPU_FOLDING_CASES)
def test_gpu_folding_errors_match_reference_binary(engine, args):
    from map_folding_gb300 import build as mfbuild

    ref = REF / "gpu_folding"
    if not ref.exists():
        pytest.skip("reference gpu_folding not built here")
    ours = _run(mfbuild.BIN / "gpu_folding", args, {})
    theirs = _run(ref, args, {})
    # usage text names "./gpu_folding" literally in both
    assert ours == theirs


@pytest.mark.parametrize("args", GPU_FOLDING_V2_CASES)
def test_gpu_folding_v2_errors_match_reference_binary(engine, args):
    from map_folding_gb300 import build as mfbuild

    ref = REF / "gpu_folding_v2"
    if not ref.exists():
        pytest.skip("reference gpu_folding_v2 not built here")
    assert _run(mfbuild.BIN / "gpu_folding_v2", args, {}) == _run(ref, args, {})
