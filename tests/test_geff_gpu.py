"""Effective conductance matrices (the reference's FCM export and SCN labels)
from batched unit-voltage line solves."""
import io
import pickle

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import nodal  # noqa: E402


@pytest.fixture(scope="module")
def geff():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import geff as m
    return m


def test_effective_conductance_matches_reference_fcm(geff, gold):
    z = gold("sim_v1_fcm_12x10.npz")
    G = 1.0 / z["Rset"][z["states"]]
    ge = geff.effective_conductance(torch.tensor(G[None], dtype=torch.float64).cuda(), 1 / float(z["r_wire"]))
    ge = ge[0].cpu().numpy()
    assert np.abs(ge - z["g_non_ideal"]).max() <= 1e-5 * np.abs(z["g_non_ideal"]).max()


def test_fcm_currents_equal_direct_solves(geff):
    rng = np.random.default_rng(3)
    T, n, m = 3, 40, 56
    G = 1.0 / np.array([1e6, 1e5, 2e4, 5e3])[rng.integers(0, 4, (T, n, m))]
    v = rng.random((5, T, n)) * 0.3
    ge = geff.effective_conductance(torch.tensor(G).cuda(), 1 / 2.93).cpu().numpy()
    for t in range(T):
        u, d = nodal.solve(G[t], 1 / 2.93, v[:, t])
        ref = nodal.currents(G[t], u, d)
        got = geff.fcm_currents(ge[t], v[:, t])
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_scn_dataset_stream(geff, tmp_path):
    """Header and instances in the reference's pickle layout; cell states drawn
    with the reference's seed sequence; labels from the converged solve."""
    p = tmp_path / "scn.binlog"
    geff.scn_dataset(str(p), data_num=3, cbsize=(16, 16), seed=959595, batch=2)
    with open(p, "rb") as f:
        header = pickle.load(f)
        items = [(pickle.load(f), pickle.load(f)) for _ in range(3)]
    assert header == [16, 16, 1.0, 1, 74867.0, 16.9e3, 1, 2.93, 0.0]
    torch.manual_seed(959595)
    dG = 1 / 16.9e3 - 1 / 74867.0
    for wq_list, labels in items:
        wq = torch.randint(0, 2, (1, 16, 16))
        assert wq.view(-1).tolist() == wq_list
        G = (wq[0].double() * dG + 1 / 74867.0).numpy()
        u, d = nodal.solve(G, 1 / 2.93, np.eye(16))
        Y = nodal.currents(G, u, d)                        # 1 V unit responses
        ref = (Y - 1 / 74867.0) / dG
        assert np.abs(np.array(labels).reshape(16, 16) - ref).max() <= 1e-4 * np.abs(ref).max()
