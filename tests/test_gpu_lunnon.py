"""GPU parity of the Lunnon kernels against the reference's counts (golden,
from the reference's own mf / mf_fast binaries) and the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def shape_of(key):
    return tuple(int(x) for x in key.split("x"))


SMALL_SHAPES = ["2x2", "2x3", "2x4", "2x5", "2x6", "3x3", "3x4", "3x5", "3x6", "4x4", "4x5",
                "4x6", "5x5", "5x6", "1x8", "1x9", "1x10", "1x11", "1x12", "1x13", "1x14",
                "1x15", "1x16", "1x17", "1x18", "1x19", "1x20", "2x2x1", "2x2x2", "2x2x3",
                "2x2x4", "2x2x5", "1x1", "2x3x4", "2x2x6", "3x3x3", "2x2x2x2", "2x2x2x3",
                "2x2x2x2x2"]


@pytest.mark.parametrize("key", SMALL_SHAPES)
@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_whole_map_counts(engine, cuda, golden, key, mode):
    dims = shape_of(key)
    want = golden["lunnon"][key]
    plan = engine.LunnonPlan(dims)
    got, states, st = plan.count(-1, mode)
    assert got == want, (key, mode, got, want)


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_6x6_depth18(engine, cuda, golden, mode):
    # the reference's headline Lunnon GPU config: gpu_folding 6 18
    plan = engine.LunnonPlan((6, 6))
    got, states, st = plan.count(18, mode)
    assert states == golden["prefix_states"]["6x6@18"]
    assert got == golden["published"]["squares"]["6"]


@pytest.mark.parametrize("depth", [0, 1, 2, 5, 10, 15, 19, 20])
def test_every_split_depth_4x5(engine, cuda, golden, depth):
    plan = engine.LunnonPlan((4, 5))
    for mode in ("plain", "batched"):
        got, _, _ = plan.count(depth, mode)
        assert got == golden["lunnon"]["4x5"], (depth, mode)


def test_per_state_counts_and_nodes_match_oracle(engine, cuda, orc):
    torch = cuda
    dims, depth = (5, 5), 15
    plan = engine.LunnonPlan(dims)
    states = plan.collect(depth)
    d_states = torch.from_numpy(states).cuda()
    per = torch.zeros(len(states), dtype=torch.int64, device="cuda")
    acc = torch.zeros(2, dtype=torch.int64, device="cuda")
    plan.count_states_device(depth + 1, d_states.data_ptr(), len(states), per.data_ptr(),
                             acc.data_ptr(), acc[1:].data_ptr())
    torch.cuda.synchronize()
    a, b, g = orc.lunnon_collect(dims, depth)
    total, want_per, w = orc.lunnon_resume_many(dims, depth + 1, a, b, threads=8)
    got_per = per.cpu().numpy().view(np.uint64)
    assert (got_per == want_per).all()
    assert int(acc[0]) == total
    assert int(acc[1]) == w.nodes  # reference leaf insertions, mf.c:136-142


def test_malformed_state_is_reported(engine, cuda):
    torch = cuda
    plan = engine.LunnonPlan((4, 4))
    states = plan.collect(6)[:4].copy()
    states[1, 0] = 200  # b[0] points outside the placed leaves
    states[2, 3] = 9
    d = torch.from_numpy(states).cuda()
    per = torch.zeros(4, dtype=torch.int64, device="cuda")
    plan.count_states_device(7, d.data_ptr(), 4, per.data_ptr())
    torch.cuda.synchronize()
    got = per.cpu().numpy().view(np.uint64)
    assert got[1] == np.uint64(2**64 - 1)
    assert got[0] != np.uint64(2**64 - 1) and got[3] != np.uint64(2**64 - 1)


def test_count_states_rejects_bad_arguments(engine, cuda):
    torch = cuda
    plan = engine.LunnonPlan((3, 3))
    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(engine.EngineError):
        plan.count_states_device(11, buf.data_ptr(), 1)
    with pytest.raises(engine.EngineError):
        plan.count_states_device(3, buf.data_ptr() + 1, 1)


def test_gpu_folding_function(engine, cuda, golden):
    states, total = engine.gpu_folding(5, 15)
    assert states == 13416
    assert total == golden["lunnon"]["5x5"]
    states, total = engine.gpu_folding(4, 5, mode="plain", dims=(3, 5))
    assert total == golden["lunnon"]["3x5"]


def test_gpu_folding_v2_cli(engine, cuda, golden, orc):
    """bin/gpu_folding_v2 on its counting path (gpu_folding_v2.cu:610-699):
    the decimal count alone on stdout, the key=value lines on stderr, and
    max_states stopping after the first states of the emission order."""
    import subprocess

    from map_folding_gb300 import build

    def run(*args):
        return subprocess.run([str(build.BIN / "gpu_folding_v2"), *map(str, args)],
                              capture_output=True, text=True, timeout=300)

    r = run(5, 15)
    assert r.returncode == 0, r.stderr
    assert r.stdout == f"{golden['lunnon']['5x5']}\n"
    err = r.stderr.splitlines()
    assert err[0] == ("gpus=1 batch_size=100000 threads_per_block=128 blocks_per_sm=8 "
                      "max_queued_batches=8 max_states=0")
    assert err[1].startswith("grid=5 depth=15 states=13416 collect_s=")
    assert err[2].startswith("solve_s=") and " total_s=" in err[2]

    # the README's example invocation
    r = run(6, 18, 5000, 128, 8, 4, 8, 0)
    assert r.returncode == 0, r.stderr
    assert r.stdout == f"{golden['published']['squares']['6']}\n"
    assert "grid=6 depth=18 states=112024 collect_s=" in r.stderr

    # max_states: the subtrees of the first 1000 prefix states only
    a, b, _ = orc.lunnon_collect((5, 5), 15)
    want, _, _ = orc.lunnon_resume_many((5, 5), 16, a[:1000], b[:1000], threads=8)
    r = run(5, 15, 5000, 128, 8, 1, 8, 1000)
    assert r.returncode == 0, r.stderr
    assert r.stdout == f"{want}\n"
    assert "grid=5 depth=15 states=1000 collect_s=" in r.stderr
