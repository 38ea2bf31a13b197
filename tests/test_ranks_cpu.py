"""The multi-rank host logic on CPU: tile split, seeds, and the job-wide timing
reduction over world_size 2 gloo ranks (the benchmark's N > 1 path without its
GPU work)."""
import os
import socket

import pytest

from fadesim_gb300 import ranks

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("total, world", [(4096, 2), (4096, 3), (7, 4), (3, 8), (0, 2)])
def test_split_tiles_covers_every_tile_once(total, world):
    spans = [ranks.split_tiles(total, r, world) for r in range(world)]
    assert spans[0][0] == 0 and spans[-1][1] == total
    assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    sizes = [hi - lo for lo, hi in spans]
    assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        ranks.split_tiles(total, world, world)


def test_rank_env(monkeypatch):
    monkeypatch.setenv("RANK", "3")
    monkeypatch.setenv("WORLD_SIZE", "8")
    monkeypatch.setenv("LOCAL_RANK", "3")
    assert ranks.rank_env() == (3, 8, 3)
    assert ranks.workload_seed(1000, 3) != ranks.workload_seed(1000, 2)
    assert ranks.max_over_ranks(2.5) == 2.5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    # each rank "solves" its own units in a rank-dependent time; the job rate
    # counts every rank's units over the slowest rank's time
    ms = ranks.max_over_ranks(10.0 * (rank + 1), dist)
    rate = ranks.job_rate(262144, world, ms)
    lo, hi = ranks.split_tiles(4096, rank, world)
    with open(os.path.join(out_dir, "r%d.txt" % rank), "w") as f:
        f.write("%r %r %d %d %d\n" % (ms, rate, lo, hi, ranks.workload_seed(1000, rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_job_time(tmp_path):
    world, port = 2, _free_port()
    torch.multiprocessing.spawn(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    got = [open(tmp_path / ("r%d.txt" % r)).read().split() for r in range(world)]
    for r, (ms, rate, lo, hi, seed) in enumerate(got):
        assert float(ms) == 20.0                          # the slower rank's time on both
        assert float(rate) == 262144 * 2 / 0.020          # both ranks' units
        assert (int(lo), int(hi)) == (2048 * r, 2048 * (r + 1))
    assert got[0][4] != got[1][4]                          # weak scaling: each rank its own tiles


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        warmup, steps, gpus = 3, 1, 2
    bench.run_reference(Args())
    assert capsys.readouterr().out == ""
