"""CUDA-graph replay of the batched kernels and the autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sym_graph_replays_match_direct_launch(engine, cuda):
    torch = cuda
    plan = engine.SymPlan(6)
    cycles, _ = plan.cases()
    d_cyc = torch.from_numpy(np.ascontiguousarray(cycles)).cuda()
    num = len(cycles)
    direct = torch.zeros(num, dtype=torch.int64, device="cuda")
    ws = torch.empty(engine.sym_workspace_bytes(), dtype=torch.uint8, device="cuda")
    engine.count_cases_batched_device(6, 16, 36, d_cyc.data_ptr(), num, direct.data_ptr(),
                                      ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    want = direct.cpu().numpy().view(np.uint64).copy()
    counts = torch.zeros(num, dtype=torch.int64, device="cuda")
    nodes = torch.zeros(1, dtype=torch.int64, device="cuda")
    g = engine.SymGraph(6, 16, 36, d_cyc.data_ptr(), num, counts.data_ptr(), ws.data_ptr(),
                        ws.numel(), d_nodes=nodes.data_ptr())
    seen_nodes = []
    for _ in range(3):
        counts.fill_(5)
        g.launch(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert (counts.cpu().numpy().view(np.uint64) == want).all()
        seen_nodes.append(int(nodes.item()))
    g.close()
    assert len(set(seen_nodes)) == 1 and seen_nodes[0] > 0


def test_lunnon_batch_object_replays(engine, cuda, golden):
    shapes = [(4, 5), (1, 16), (2, 2, 4), (3, 6), (5, 5), (2, 2)]
    batch = engine.LunnonBatch(shapes)
    for _ in range(2):
        counts, st = batch.run()
        for dims, got in zip(shapes, counts):
            key = "x".join(map(str, dims))
            assert got == golden["lunnon"][key], dims
        assert st.units > 0 and st.kernel_s > 0
    batch.close()


def test_autotuner_keeps_counts_exact(engine, cuda, golden, tmp_path, monkeypatch):
    from map_folding_gb300 import autotune

    monkeypatch.setenv("MF_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    shapes = [(4, 5), (1, 14), (2, 2, 3), (3, 4)]
    best = autotune.tune_lunnon_batch(shapes, depth_offsets=(0, 2), block_threads=(128,),
                                      periods=(32, 64), repeats=1, use_cache=False)
    for dims, got in zip(shapes, best["counts"]):
        assert got == golden["lunnon"]["x".join(map(str, dims))]
    again = autotune.tune_lunnon_batch(shapes)  # served from the cache file
    assert again["depths"] == best["depths"]
    cfg = autotune.as_config(best)
    counts, _ = engine.lunnon_batch_count(shapes, best["depths"], cfg=cfg)
    assert counts == best["counts"]
