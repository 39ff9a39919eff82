"""Batched uneven launch: 64 seeded map instances in one persistent
work-stealing kernel, each count bit-exact against the plain kernel and the
reference's counts."""
import pytest

pytestmark = pytest.mark.gpu


def expected_count(golden, dims):
    dims = tuple(sorted(dims)) if len(dims) == 2 else tuple(dims)
    if dims == (6, 6):
        return golden["published"]["squares"]["6"]
    key = "x".join(map(str, dims))
    if key in golden["lunnon"]:
        return golden["lunnon"][key]
    return None


def test_uneven_batch_matches_plain_and_reference(engine, cuda, golden):
    from map_folding_gb300.workloads import uneven_instances

    shapes = uneven_instances(seed=2026, count=64)
    counts, st = engine.lunnon_batch_count(shapes)
    assert st.units > 0 and st.tasks >= st.units
    for dims, got in zip(shapes, counts):
        want = expected_count(golden, dims)
        if want is not None:
            assert got == want, (dims, got, want)
        plain, _, _ = engine.LunnonPlan(dims).count(-1, "plain")
        assert got == plain, dims


@pytest.mark.parametrize("cfg", [
    {"block_threads": 64, "blocks_per_sm": 4, "node_budget": 8},
    {"block_threads": 256, "blocks_per_sm": 2, "node_budget": 1024, "hungry_factor": 16},
    {"block_threads": 128, "node_budget": 1, "queue_capacity": 64},
])
def test_batch_knobs_do_not_change_counts(engine, cuda, golden, cfg):
    shapes = [(4, 5), (1, 16), (2, 2, 4), (3, 6), (5, 5), (2, 2)]
    counts, st = engine.lunnon_batch_count(shapes, cfg=cfg)
    for dims, got in zip(shapes, counts):
        assert got == expected_count(golden, dims), (dims, cfg)


def test_depths_per_instance(engine, cuda, golden):
    shapes = [(5, 5), (5, 5), (5, 5), (4, 4)]
    counts, _ = engine.lunnon_batch_count(shapes, depths=[0, 7, 20, 16])
    assert counts == [golden["lunnon"]["5x5"]] * 3 + [golden["lunnon"]["4x4"]]
