"""The autotuner's search logic on the CPU, with the solver call and the clock
replaced by fakes: it keeps the fastest converged setting, drops settings
whose solves did not all converge, skips the timed repetitions of a setting
whose first call already took twice the best time, and stops timing a whole
kernel layout once its first setting lost that way to another layout."""
import pytest

torch = pytest.importorskip("torch")

from fadesim_gb300 import autotune  # noqa: E402


class FakeSolver:
    """ir_drop_gs_ex stand-in: each call advances a fake clock by the time the
    setting 'takes' and reports convergence as configured."""

    def __init__(self, cost, converged=lambda kw: True):
        self.cost, self.converged, self.now, self.calls = cost, converged, 0.0, []

    def clock(self):
        return self.now

    def __call__(self, vin, G, B, n, m, T, Y, g_wire=None, method=None, return_stats=True, **kw):
        kw = dict(kw, method=method)
        self.calls.append(kw)
        self.now += self.cost(kw) / 1e3
        return None, {"status_or": 1 if self.converged(kw) else 2}, None


@pytest.fixture
def fake(monkeypatch, tmp_path):
    def install(cost, converged=lambda kw: True):
        f = FakeSolver(cost, converged)
        monkeypatch.setattr(autotune._acc, "ir_drop_gs_ex", f)
        monkeypatch.setattr(autotune.time, "perf_counter", f.clock)
        monkeypatch.setattr(autotune.torch.cuda, "synchronize", lambda *a, **k: None)
        monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tune.json"))
        monkeypatch.setattr(autotune, "_mem", None)
        return f
    return install


def test_method_axis_on_strongly_coupled_128_tiles(fake):
    """Full 128 x 128 tiles whose cells couple the planes strongly (sum of
    g / g_wire >= 3 per tile) also time the two-level method; lookup then hands
    it back as the method to run.  Weakly coupled tiles never try it."""
    vin = torch.zeros(2, 4, 128)
    cost = lambda kw: (1.0 if kw["method"] == "line_coarse" else 2.0) + (5.0 if kw["kernel_ld"] == 256 else 0.0)
    f = fake(cost)
    strong = torch.full((4, 128, 128), 1e-3)          # sum of g / g_wire ~ 48 per tile
    kw, ms = autotune.tune(strong, vin, reps=2)
    assert kw["method"] == "line_coarse" and kw["kernel_ld"] == 128 and ms == pytest.approx(1.0)
    assert autotune.lookup(128, 128)["method"] == "line_coarse"
    assert len([c for c in f.calls if c["method"] == "line_coarse"]) == 3 * (1 + 2)
    f.calls.clear()
    weak = torch.full((4, 128, 128), 1e-6)            # ~0.05 per tile
    kw, _ = autotune.tune(weak, vin, reps=2)
    assert "method" not in kw and all(c["method"] == "line" for c in f.calls)


def test_keeps_fastest_converged_setting(fake):
    G, vin = torch.zeros(4, 128, 128), torch.zeros(2, 4, 128)
    # 128 layout: 2 ms, 8 vectors per item fastest (1.5 ms) but it does not converge
    cost = lambda kw: {0: 2.0, 8: 1.5, 32: 1.8}[kw["vectors_per_cta"]] + (10.0 if kw["kernel_ld"] == 256 else 0.0)
    f = fake(cost, converged=lambda kw: kw["vectors_per_cta"] != 8)
    kw, ms = autotune.tune(G, vin, reps=3)
    assert kw["kernel_ld"] == 128 and kw["vectors_per_cta"] == 32
    assert ms == pytest.approx(1.8)
    assert autotune.lookup(128, 128) == kw


def test_losing_layout_is_dropped_after_one_call(fake):
    G, vin = torch.zeros(4, 256, 256), torch.zeros(2, 4, 256)
    # the 512 layout takes 4x the 256 layout's time: after its first setting's
    # first call it is not timed again
    f = fake(lambda kw: 4.0 if kw["kernel_ld"] == 512 else 1.0)
    kw, _ = autotune.tune(G, vin, reps=3)
    assert kw["kernel_ld"] == 256
    calls_512 = [c for c in f.calls if c["kernel_ld"] == 512]
    assert len(calls_512) == 1
    # every 256 setting: one first call and its timed repetitions
    n256 = len([c for c in autotune.candidates("line", 256, 256) if c["kernel_ld"] == 256])
    assert len([c for c in f.calls if c["kernel_ld"] == 256]) == n256 * (1 + 3)


def test_slow_setting_on_the_winning_layout_skips_its_repetitions(fake):
    G, vin = torch.zeros(4, 64, 64), torch.zeros(2, 4, 64)
    # on the 64 layout the residual-period-1 settings are 3x slower: one call each
    cost = lambda kw: (3.0 if kw["residual_period"] == 1 else 1.0) + (0.5 if kw["kernel_ld"] == 128 else 0.0)
    f = fake(cost)
    kw, _ = autotune.tune(G, vin, reps=3)
    assert kw["kernel_ld"] == 64 and kw["residual_period"] == 0
    slow64 = [c for c in f.calls if c["kernel_ld"] == 64 and c["residual_period"] == 1]
    assert len(slow64) == 3  # vectors_per_cta 0, 8, 32: first call only


def test_no_converged_setting_raises(fake):
    G, vin = torch.zeros(2, 32, 32), torch.zeros(1, 2, 32)
    fake(lambda kw: 1.0, converged=lambda kw: False)
    with pytest.raises(RuntimeError, match="no candidate setting converged"):
        autotune.tune(G, vin)
