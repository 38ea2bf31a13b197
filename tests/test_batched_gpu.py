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
