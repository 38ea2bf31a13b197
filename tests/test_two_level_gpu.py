"""Parity of the two-level line relaxation (method "line_coarse": the 128 x 128
kernel with a coarse-grid correction after every iteration) with the oracle.

On full 128 x 128 tiles of strongly coupled linear cells (the 1 kOhm - 1 MOhm
weight-slice maps of the MLP layers, uniform 1 kOhm cells) it must land within
the tolerance of the FP64 direct solve (plus the FP32 floor of the planes) in
at most half the line method's iterations; on weakly coupled tiles and on
partial tiles it runs the plain line iteration and must agree with the line
method; the currents meet the contract (1e-4 of the largest current).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import nodal  # noqa: E402

GW = 1 / 2.93
CFG1 = [2e6, 1.6e6, 1.3e6, 1e6]


@pytest.fixture(scope="module")
def acc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import cpp_ir_drop_accelerate as m
    return m


def mlp_maps(seed, X, n):
    """X weight-slice maps (2-bit cells, PN, 8-bit weights ~ N(0, 0.05^2): the three
    low slices, whose cells couple the planes strongly), [X, n, n]."""
    rng = np.random.default_rng(seed)
    out = []
    for x in range(X):
        w = rng.normal(0, 0.05, (n, n))
        wi = np.round(w / 2 ** np.ceil(np.log2(np.abs(w).max() / 255))).astype(np.int64)
        out.append(((np.where(wi > 0, wi, 0) >> (2 * (x % 3))) & 3) * ((1e-3 - 1e-6) / 3) + 1e-6)
    return np.stack(out)


def run(acc, inp, G, B, X, n, m, dtype=torch.float64, ret_V=2, **kw):
    ti = torch.tensor(inp, dtype=dtype, device="cuda").contiguous()
    tg = torch.tensor(G, dtype=dtype, device="cuda").contiguous()
    out, stats, iters = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, 1, ret_V=ret_V, return_iters=True, **kw)
    torch.cuda.synchronize()
    return out.double().cpu().numpy(), stats, iters.cpu().numpy()


@pytest.mark.parametrize("cells", ["mlp", "1k"])
@pytest.mark.parametrize("tol", [5e-7, 1e-8])
def test_two_level_matches_oracle_in_fewer_iterations(acc, cells, tol):
    B, X, n = 6, 4, 128
    rng = np.random.default_rng(7 + (cells == "1k"))
    G = mlp_maps(5, X, n) if cells == "mlp" else 1.0 / (1e3 * np.exp(0.3 * rng.standard_normal((X, n, n))))
    assert ((G / GW).sum(axis=(1, 2)) >= 3.0).all()  # every tile takes the coarse correction
    inp = rng.integers(0, 2, (B, X, n)) * 0.2
    cur, U, D = nodal.solve_layer(inp, G, n, n, X, 1, GW, return_planes=True)
    got, st, it2 = run(acc, inp, G, B, X, n, n, method="line_coarse", tol_v=tol, vectors_per_cta=B)
    assert st["status_or"] == 1, st
    dev = max(np.abs(U - inp.reshape(B, X, 1, n, 1)).max(), np.abs(D).max())
    floor = max(2e-9, 8 * 2.0 ** -23 * dev)
    err = max(np.abs(got[:, :, :, 0] - U).max(), np.abs(got[:, :, :, 1] - D).max())
    assert err <= tol + floor, (err, st)
    _, st1, it1 = run(acc, inp, G, B, X, n, n, method="line", tol_v=tol, vectors_per_cta=B)
    assert st1["status_or"] == 1
    assert it2.mean() <= 0.5 * it1.mean(), (it2.mean(), it1.mean())
    # currents (FP32 I/O, the layer path's call)
    got_i, st_i, _ = run(acc, inp, G, B, X, n, n, dtype=torch.float32, ret_V=False, method="line_coarse", tol_v=tol)
    assert st_i["status_or"] == 1
    assert np.abs(got_i[:, :, :] - cur).max() <= 1e-4 * np.abs(cur).max()


@pytest.mark.parametrize("shape", [(128, 128), (100, 128), (128, 77), (64, 64)])
def test_two_level_elsewhere_runs_the_line_iteration(acc, shape):
    """Weakly coupled full tiles (four-state 1-2 MOhm cells) and every partial or
    smaller tile: the plain line iteration, the line method's answer."""
    n, m = shape
    B, X = 4, 3
    rng = np.random.default_rng(n * 3 + m)
    G = 1.0 / np.asarray(CFG1)[rng.integers(0, 4, (X, n, m))]
    inp = rng.integers(0, 2, (B, X, n)) * 1.0
    _, U, D = nodal.solve_layer(inp, G, n, m, X, 1, GW, return_planes=True)
    got, st, it2 = run(acc, inp, G, B, X, n, m, method="line_coarse")
    ref, st1, it1 = run(acc, inp, G, B, X, n, m, method="line")
    assert st["status_or"] == 1 and st1["status_or"] == 1
    err = max(np.abs(got[:, :, :, 0] - U).max(), np.abs(got[:, :, :, 1] - D).max())
    assert err < 1e-7, err
    assert np.abs(got - ref).max() < 1e-7
    assert abs(it2.mean() - it1.mean()) <= 0.25


def test_two_level_warm_start_and_rejection(acc):
    """From the exact planes, from far-off planes (rejected, restarted from the
    ideal state): the same answer either way."""
    B, X, n = 3, 2, 128
    G = mlp_maps(9, X, n)
    inp = np.random.default_rng(3).integers(0, 2, (B, X, n)) * 0.2
    cur, U, D = nodal.solve_layer(inp, G, n, n, X, 1, GW, return_planes=True)
    ti = torch.tensor(inp, dtype=torch.float32, device="cuda")
    tg = torch.tensor(G, dtype=torch.float32, device="cuda")
    exact = np.stack([U - inp.reshape(B, X, 1, n, 1), D], axis=3)  # [B, X, 1, 2, n, n]
    for init, rejected in ((exact, False), (exact + 5.0, True)):
        tin = torch.tensor(init, dtype=torch.float32, device="cuda").contiguous()
        out, st, _ = acc.ir_drop_gs_warm(ti, tg, B, n, n, X, 1, tin, g_wire=GW, method="line_coarse")
        torch.cuda.synchronize()
        assert st["status_or"] & 1
        assert bool(st["warm_rejected"]) == rejected
        assert np.abs(out.double().cpu().numpy() - cur).max() <= 1e-4 * np.abs(cur).max()


def test_superposition_unit_responses_to_the_fp32_limit(acc):
    """The layer path's superposition on full 128 x 128 tiles solves its unit
    responses with the two-level method to the FP32 limit: every input
    vector's currents, a sum of up to 128 unit responses, then meet the
    oracle's to a few 1e-6 of the largest current (the plain stop test left
    ~1e-4)."""
    from fadesim_gb300 import splitarr
    B, X, n = 200, 3, 128
    G = mlp_maps(13, X, n)
    inp = np.random.default_rng(14).integers(0, 2, (B, X, n)) * 0.2
    cur = nodal.solve_layer(inp, G, n, n, X, 1, GW)
    cfg = splitarr.ArrayConfig(Ron=1e3, Roff=1e6, cellBits=2, arrRowSize=n, arrColSize=n, inputMaxVoltage=0.2,
                               r_wire=2.93)
    v = torch.tensor(inp, dtype=torch.float32, device="cuda").contiguous()
    tg = torch.tensor(G, dtype=torch.float32, device="cuda").contiguous()
    got = splitarr.superposition_solver(cfg)(v, tg, B, n, n, X, 1, None)
    torch.cuda.synchronize()
    got = got.double().cpu().numpy().reshape(cur.shape)
    assert np.abs(got - cur).max() <= 5e-6 * np.abs(cur).max()
