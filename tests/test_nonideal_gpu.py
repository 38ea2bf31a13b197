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


def counter_normal(seed, a, b):
    """numpy restatement of the kernels' counter-based normal draw (splitmix64
    finaliser of seed + golden * (a * FNV prime + b + 1), then Box-Muller on its
    top and bottom 24 bits), in FP64."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        a = np.asarray(a, np.uint64)
        zz = np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15) * (a * np.uint64(0x100000001B3) + np.uint64(b) +
                                                               np.uint64(1))
        zz = (zz ^ (zz >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        zz = (zz ^ (zz >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        zz = (zz ^ (zz >> np.uint64(31))) & M
    u1 = ((zz >> np.uint64(40)).astype(np.float64) + 0.5) / 16777216.0
    u2 = (zz & np.uint64(0xFFFFFF)).astype(np.float64) / 16777216.0
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


VARIATION_STREAM = 0x7661726961


@pytest.mark.gpu
def test_add_variation_device_lognormal():
    """The device variation kernel: G / exp(sigma z) with z from the counter hash
    of (seed, offset + cell), against an FP64 numpy restatement of the draw
    (FP32 log/cos/exp: a few ulps); deterministic; the offset shifts the
    stream; log(G / out) / sigma is standard normal."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300.variation import add_variation_device
    G = torch.full((1024, 1024), 1e-6, device="cuda")
    out = add_variation_device(G, 0.1, seed=5)
    lr = torch.log(G / out).double()
    assert abs(lr.mean().item()) < 1e-3 and abs(lr.std().item() - 0.1) < 1e-3
    assert torch.equal(out, add_variation_device(G, 0.1, seed=5))
    k = np.arange(4096)
    ref = 1e-6 / np.exp(0.1 * counter_normal(5, k, VARIATION_STREAM))
    got = out.double().cpu().numpy().ravel()[:4096]
    assert np.abs(got / ref - 1).max() < 2e-6
    shifted = add_variation_device(G[:1, :8].contiguous(), 0.1, seed=5, offset=1000)
    assert torch.equal(shifted.ravel(), out.ravel()[1000:1008])


@pytest.mark.gpu
def test_variation_layer_path_bit_exact(gold):
    """Cycle-to-cycle variation (sigma 0.1) in the GPU layer path, PN and
    Ref-column: one draw per (input bit, slice, array) solve from the
    reference's generator, in its order, divided on the device; bit-exact with
    the oracle fed the same draws (same host, same generator) and the same
    droop solve -- the oracle itself reproduces the reference's own
    splitArr_matmul_nn on these fixtures (test_oracle.py)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import platform
    from fadesim_gb300 import splitarr
    from oracle import intstages

    def droop_on_host(v, G, B, rows, cols, numX, numY, out):
        cur = intstages.droop_solver(v.cpu().numpy(), G.cpu().numpy(), B, rows, cols, numX, numY)
        return out.copy_(torch.from_numpy(cur).reshape(out.shape))

    for name in ("var_pn", "var_ref"):
        z = gold("pimtorch_layer_%s.npz" % name)
        cfg = splitarr.ArrayConfig(Ron=float(z["Ron"]), Roff=float(z["Roff"]), cellBits=int(z["cellBits"]),
                                   arrRowSize=int(z["rows"]), arrColSize=int(z["cols"]),
                                   inputMaxVoltage=float(z["inputMaxVoltage"]), sigma=float(z["sigma"]))
        seed = int(z["seed"]) + 2
        y = splitarr.splitArr_matmul_nn(torch.from_numpy(z["x"]), torch.from_numpy(z["w"]), 8, 1, int(z["adc_bits"]),
                                        10, 8, str(z["arr_mode"]), torch.float32, cfg=cfg, solver=droop_on_host,
                                        rand_gen=torch.Generator().manual_seed(seed)).cpu().numpy()
        gen = torch.Generator().manual_seed(seed)
        vary = lambda shape: torch.exp(torch.randn(tuple(shape), generator=gen) * cfg.sigma).numpy()
        p = intstages.ArrayParams(Ron=float(z["Ron"]), Roff=float(z["Roff"]), cellBits=int(z["cellBits"]),
                                  rows=int(z["rows"]), cols=int(z["cols"]),
                                  inputMaxVoltage=float(z["inputMaxVoltage"]), adc_bits=int(z["adc_bits"]))
        ref = intstages.split_matmul_ex(z["x"], z["w"], p, arr=str(z["arr_mode"]), solver=intstages.droop_solver,
                                        vary=vary)
        assert np.array_equal(y, ref), name
        if platform.machine() == "x86_64":  # the fixture's own platform: same CPU draws bit for bit
            assert np.array_equal(y, z["y"]), name


@pytest.mark.gpu
def test_sinh_cluster_512_with_variation_matches_oracle(acc):
    """The large-tile non-ideal kernel as benchmarked (512 x 512 on 16-CTA
    clusters, sinh cells I = (V/R) sinh(2V)/(2V), lognormal variation sigma 0.1
    from the device kernel, inputs U[0, 0.2] V), no read noise: both planes
    within 1e-6 V and the bitline currents within 1e-4 relative of the FP64
    nonlinear nodal fixed point."""
    from fadesim_gb300.variation import add_variation_device
    B, X, n = 2, 1, 512
    rng = np.random.default_rng(512)
    G0 = torch.tensor(1.0 / R4[rng.integers(0, 4, (X, n, n))], dtype=torch.float32, device="cuda")
    tg = add_variation_device(G0, 0.1, seed=9)
    inp = rng.random((B, X, n)) * 0.2
    ti = torch.tensor(inp, dtype=torch.float32, device="cuda")
    params = nodal.sinh_params(1e6, 2e6)
    kw = dict(g_wire=GW, nonlinear_cell_enable=True, nonlinear_params=params, method="line")
    planes, stats, _ = acc.ir_drop_gs_ex(ti, tg, B, n, n, X, 1, ret_V=2, **kw)
    assert stats["status_or"] == 1, stats
    cur, st2, _ = acc.ir_drop_gs_ex(ti, tg, B, n, n, X, 1, **kw)
    assert st2["status_or"] == 1, st2
    planes = planes.double().cpu().numpy()
    cur = cur.double().cpu().numpy()
    G = tg.double().cpu().numpy()[0]
    for b in range(B):
        u, d, _ = nodal.solve_nonlinear(G, GW, inp[b, 0], params, reuse_factor=True)
        assert np.abs(planes[b, 0, 0, 0] - u).max() < 1e-6
        assert np.abs(planes[b, 0, 0, 1] - d).max() < 1e-6
        ref = nodal.nonlinear_currents(G, u, d, params)
        assert np.abs(cur[b, 0] - ref).max() <= 1e-4 * np.abs(ref).max()


@pytest.mark.gpu
def test_sinh_cluster_512_read_noise(acc):
    """The same kernel with 1% read noise: deterministic per seed, a new seed
    gives new noise, and the relative spread of the bitline currents matches
    independent 1% noise on 512 cells per column."""
    from fadesim_gb300.variation import add_variation_device
    B, X, n = 4, 1, 512
    rng = np.random.default_rng(77)
    G0 = torch.tensor(1.0 / R4[rng.integers(0, 4, (X, n, n))], dtype=torch.float32, device="cuda")
    tg = add_variation_device(G0, 0.1, seed=3)
    ti = torch.tensor(rng.random((B, X, n)) * 0.2, dtype=torch.float32, device="cuda")
    kw = dict(g_wire=GW, nonlinear_cell_enable=True, nonlinear_params=nodal.sinh_params(1e6, 2e6), method="line")
    clean, _, _ = acc.ir_drop_gs_ex(ti, tg, B, n, n, X, 1, **kw)
    noisy, st, _ = acc.ir_drop_gs_ex(ti, tg, B, n, n, X, 1, read_noise_sigma=0.01, noise_seed=42, **kw)
    again, _, _ = acc.ir_drop_gs_ex(ti, tg, B, n, n, X, 1, read_noise_sigma=0.01, noise_seed=42, **kw)
    other, _, _ = acc.ir_drop_gs_ex(ti, tg, B, n, n, X, 1, read_noise_sigma=0.01, noise_seed=43, **kw)
    assert st["status_or"] == 1, st
    assert torch.equal(noisy, again) and not torch.equal(noisy, other)
    rel = ((noisy - clean) / clean).double().cpu().numpy().ravel()
    # 512 cells of similar current per column with 1% independent noise: ~0.01 / sqrt(512) = 4.4e-4
    assert abs(rel.mean()) < 1e-4
    assert 2e-4 < rel.std() < 1e-3
