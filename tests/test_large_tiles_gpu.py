"""Tiles above 128 x 128: the cluster-resident line solver against the FP64 oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import nodal  # noqa: E402

GW = 1 / 2.93
CFG1 = [2e6, 1.6e6, 1.3e6, 1e6]
STRONG = [1e6, 1 / (1e-6 + (1e-3 - 1e-6) / 3), 1 / (1e-6 + 2 * (1e-3 - 1e-6) / 3), 1e3]


@pytest.fixture(scope="module")
def acc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import cpp_ir_drop_accelerate as m
    return m


def case(seed, B, X, Y, n, m, Rset, vmax):
    rng = np.random.default_rng(seed)
    G = 1.0 / np.asarray(Rset)[rng.integers(0, len(Rset), (X, n, Y * m))]
    inp = rng.integers(0, 2, (B, X, n)) * vmax
    return inp.astype(np.float64), G


@pytest.mark.parametrize("shape,cells", [((2, 1, 2, 256, 256), "cfg1"), ((2, 2, 1, 256, 256), "strong"),
                                         ((2, 1, 1, 200, 150), "cfg1"), ((1, 1, 1, 130, 256), "strong"),
                                         ((1, 1, 1, 512, 512), "cfg1"), ((1, 1, 1, 300, 420), "cfg1")])
def test_cluster_line_solver_matches_oracle(acc, shape, cells):
    B, X, Y, n, m = shape
    Rset, vmax = (CFG1, 1.0) if cells == "cfg1" else (STRONG, 0.2)
    inp, G = case(n + m + (cells == "strong"), B, X, Y, n, m, Rset, vmax)
    cur, U, D = nodal.solve_layer(inp, G, n, m, X, Y, GW, return_planes=True)
    ti = torch.tensor(inp, dtype=torch.float32, device="cuda")
    tg = torch.tensor(G, dtype=torch.float32, device="cuda")
    planes, stats, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, g_wire=GW, ret_V=2, method="line")
    assert stats["status_or"] == 1, stats
    planes = planes.double().cpu().numpy()
    err = max(np.abs(planes[:, :, :, 0] - U).max(), np.abs(planes[:, :, :, 1] - D).max())
    assert err < (2e-7 if cells == "cfg1" else 1e-6), (err, stats)
    got, _, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, g_wire=GW, method="line")
    rel = np.abs(got.double().cpu().numpy() - cur).max() / np.abs(cur).max()
    assert rel < (2e-6 if cells == "cfg1" else 1e-4), rel


def test_cluster_line_solver_f64_and_ret_v(acc):
    B, X, Y, n, m = 2, 1, 1, 256, 200
    inp, G = case(3, B, X, Y, n, m, CFG1, 0.2)
    cur, U, D = nodal.solve_layer(inp, G, n, m, X, Y, GW, return_planes=True)
    ti = torch.tensor(inp, device="cuda")
    tg = torch.tensor(G, device="cuda")
    got = acc.ir_drop_gs(ti, tg, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    assert got.dtype == torch.float64
    assert np.abs(got.cpu().numpy() - cur).max() <= 1e-6 * np.abs(cur).max()
    v = acc.ir_drop_gs(ti, tg, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], True)
    assert np.abs(v.cpu().numpy() - (U - D)).max() < 1e-8
