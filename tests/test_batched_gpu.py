"""Uneven tile batches: concurrent per-shape launches and CUDA-graph replay."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import nodal  # noqa: E402

GW = 1 / 2.93


def groups_for(shapes, B, seed):
    rng = np.random.default_rng(seed)
    out = []
    for T, n, m in shapes:
        G = (1.0 / np.array([2e6, 1.6e6, 1.3e6, 1e6])[rng.integers(0, 4, (T, n, m))]).astype(np.float32)
        v = (rng.integers(0, 2, (B, T, n)) * 0.2).astype(np.float32)
        out.append((G, v))
    return out


@pytest.mark.gpu
def test_uneven_batch_matches_oracle_and_graph_replays():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300.batched import TileBatch, TileGroup
    data = groups_for([(3, 64, 64), (2, 128, 128), (2, 256, 256), (1, 100, 40)], B=4, seed=8)
    groups = [TileGroup(torch.from_numpy(G).cuda(), torch.from_numpy(v).cuda()) for G, v in data]
    batch = TileBatch(groups, tuned=False)
    stats = batch.run(stats=True)
    torch.cuda.synchronize()
    assert all(s["status_or"] == 1 for s in stats)
    first = [o.clone() for o in batch.outputs()]
    for (G, v), o in zip(data, first):
        T, n, m = G.shape
        ref = nodal.solve_layer(v.astype(np.float64), G.astype(np.float64), n, m, T, 1, GW)
        assert np.abs(o.double().cpu().numpy() - ref).max() <= 2e-6 * np.abs(ref).max()
    batch.capture()
    for g in batch.groups:
        g.out.zero_()
    batch.replay()
    torch.cuda.synchronize()
    for a, b in zip(first, batch.outputs()):
        assert torch.equal(a, b)
    # new inputs in place, replay again: results follow the inputs
    batch.groups[0].vin.mul_(0.5)
    batch.replay()
    torch.cuda.synchronize()
    assert torch.allclose(batch.outputs()[0], first[0] * 0.5, rtol=1e-5, atol=0)


def test_autotune_cache_roundtrip(tmp_path, monkeypatch):
    from fadesim_gb300 import autotune
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_mem", None)
    assert autotune.lookup(128, 128) == {}
    autotune._store(128, 128, "line", {"vectors_per_cta": 8}, 1.5)
    monkeypatch.setattr(autotune, "_mem", None)
    assert autotune.lookup(128, 128) == {"vectors_per_cta": 8}
    assert autotune.candidates("rbsor")[0]["omega"] > 1.9


@pytest.mark.gpu
@pytest.mark.parametrize("method,n,m,ld", [("line", 40, 64, 64), ("line", 64, 64, 128), ("line", 128, 128, 256),
                                           ("line", 100, 77, 256), ("line", 256, 256, 512),
                                           ("rbsor", 96, 128, 256)])
def test_forced_layouts_match_oracle(method, n, m, ld):
    """The autotuner's shape axis: a tile solved on a larger layout than its own
    (a 64 x 64 tile on the 128 single-CTA kernel, a 128 x 128 tile on a 4-CTA
    cluster of 64-row bands, a 256 x 256 tile on a 16-CTA cluster) lands on the
    same nodal solution, the work items claimed from the device queue."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import cpp_ir_drop_accelerate as acc
    B, X = 3, 2
    (G, v), = groups_for([(X, n, m)], B=B, seed=n + m + ld)
    out, st, _ = acc.ir_drop_gs_ex(torch.from_numpy(v).cuda(), torch.from_numpy(G).cuda(), B, n, m, X, 1,
                                   g_wire=GW, method=method, kernel_ld=ld, tol_v=1e-8)
    assert st["status_or"] == 1 and st["solves"] == B * X, st
    ref = nodal.solve_layer(v.astype(np.float64), G.astype(np.float64), n, m, X, 1, GW)
    assert np.abs(out.double().cpu().numpy() - ref).max() <= 2e-6 * np.abs(ref).max()
    with pytest.raises(RuntimeError, match="kernel_ld"):
        acc.ir_drop_gs_ex(torch.from_numpy(v).cuda(), torch.from_numpy(G).cuda(), B, n, m, X, 1, g_wire=GW,
                          method=method, kernel_ld=32)


def test_autotune_candidates_cover_the_kernel_shapes():
    from fadesim_gb300 import autotune
    assert autotune.layouts(64, 64) == [64, 128]
    assert autotune.layouts(128, 100) == [128, 256]
    assert autotune.layouts(256, 256) == [256, 512]
    assert autotune.layouts(512, 300) == [512]
    lds = {c["kernel_ld"] for c in autotune.candidates("line", 128, 128)}
    assert lds == {128, 256}
