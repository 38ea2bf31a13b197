"""Non-idealities: sinh-cell nonlinearity (the reference's nonlinear_cell_enable
path), lognormal conductance variation and read noise."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import nodal  # noqa: E402

GW = 1 / 2.93
R4 = np.array([2e6, 1.6e6, 1.3e6, 1e6])


def k2_params(V, R, K2):
    """get_nonlinear_params_from_K2 (conductance_variation.py:29-33)."""
    x = (K2 + math.sqrt(K2 * K2 - 4)) / 2
    a = 2 * math.log(x) / V
    return a, V / R / math.sinh(a * V)


@pytest.fixture(scope="module")
def acc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import cpp_ir_drop_accelerate as m
    return m


CASES = [
    ("sinh-cfg5", (2, 1, 2, 64, 64), R4, nodal.sinh_params(1e6, 2e6), 0.2),
    ("sinh-cfg5-128", (2, 2, 1, 128, 96), R4, nodal.sinh_params(1e6, 2e6), 0.2),
    ("k2-strong", (2, 1, 1, 48, 40), np.array([1e3, 2e4, 3e5, 1e6]),
     [1e3, 1e6, *k2_params(1, 1e3, 10.00001), *k2_params(1, 1e6, 20.00001)], 0.2),
    ("sinh-cluster-256", (1, 1, 1, 256, 256), R4, nodal.sinh_params(1e6, 2e6), 0.2),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,shape,Rset,params,vmax", CASES, ids=[c[0] for c in CASES])
def test_nonlinear_cells_match_oracle(acc, name, shape, Rset, params, vmax):
    B, X, Y, n, m = shape
    rng = np.random.default_rng(n + m)
    G = 1.0 / Rset[rng.integers(0, len(Rset), (X, n, Y * m))]
    inp = rng.random((B, X, n)) * vmax
    ti = torch.tensor(inp, dtype=torch.float32, device="cuda")
    tg = torch.tensor(G, dtype=torch.float32, device="cuda")
    planes, stats, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, g_wire=GW, nonlinear_cell_enable=True,
                                         nonlinear_params=params, ret_V=2, method="line")
    assert stats["status_or"] == 1, stats
    cur, _, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, g_wire=GW, nonlinear_cell_enable=True,
                                  nonlinear_params=params, method="line")
    planes = planes.double().cpu().numpy()
    cur = cur.double().cpu().numpy()
    Gr = G.reshape(X, n, Y, m)
    for b in range(B):
        for x in range(X):
            for y in range(Y):
                u, d, _ = nodal.solve_nonlinear(Gr[x, :, y, :], GW, inp[b, x], params)
                assert np.abs(planes[b, x, y, 0] - u).max() < 1e-6
                assert np.abs(planes[b, x, y, 1] - d).max() < 1e-6
                ref = nodal.nonlinear_currents(Gr[x, :, y, :], u, d, params)
                got = cur[b, x, y * m:(y + 1) * m]
                assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


@pytest.mark.gpu
def test_read_noise_statistics_and_determinism(acc):
    B, X, Y, n, m = 8, 4, 1, 128, 128
    rng = np.random.default_rng(1)
    G = torch.tensor(1.0 / R4[rng.integers(0, 4, (X, n, m))], dtype=torch.float32, device="cuda")
    inp = torch.tensor(rng.random((B, X, n)) * 0.2, dtype=torch.float32, device="cuda")
    clean, _, _ = acc.ir_drop_gs_ex(inp, G, B, n, m, X, Y, g_wire=GW, method="line")
    noisy, _, _ = acc.ir_drop_gs_ex(inp, G, B, n, m, X, Y, g_wire=GW, method="line", read_noise_sigma=0.01,
                                    noise_seed=42)
    again, _, _ = acc.ir_drop_gs_ex(inp, G, B, n, m, X, Y, g_wire=GW, method="line", read_noise_sigma=0.01,
                                    noise_seed=42)
    other, _, _ = acc.ir_drop_gs_ex(inp, G, B, n, m, X, Y, g_wire=GW, method="line", read_noise_sigma=0.01,
                                    noise_seed=43)
    assert torch.equal(noisy, again) and not torch.equal(noisy, other)
    rel = ((noisy - clean) / clean).double().cpu().numpy().ravel()
    # each bitline sums 128 cells with 1% independent noise: relative spread ~ 0.01 * ||I_cell|| / sum I_cell
    assert abs(rel.mean()) < 2e-4
    assert 3e-4 < rel.std() < 2e-3


def test_add_variation_matches_reference_formula():
    from fadesim_gb300.variation import add_variation
    g0 = torch.Generator()
    g0.manual_seed(557)
    G = torch.full((4, 8, 16), 1e-6)
    out = add_variation(G, sigma=0.1, rand_gen=g0)
    g1 = torch.Generator()
    g1.manual_seed(557)
    ref = G / torch.exp(torch.randn(G.shape, generator=g1) * 0.1)
    assert torch.equal(out, ref)
    assert torch.equal(add_variation(G, sigma=0, rand_gen=g1), G)


@pytest.mark.gpu
def test_add_variation_device_lognormal():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300.variation import add_variation_device
    G = torch.full((1024, 1024), 1e-6, device="cuda")
    out = add_variation_device(G, 0.1, seed=5)
    lr = torch.log(G / out).double()
    assert abs(lr.mean().item()) < 1e-3 and abs(lr.std().item() - 0.1) < 1e-3
    assert torch.equal(out, add_variation_device(G, 0.1, seed=5))
