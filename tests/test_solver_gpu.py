"""Parity of the CUDA solver with the oracle, through the drop-in module.

Every converging method must land within 1e-6 V of the FP64 direct solve on
every node of both planes and within 1e-4 relative on bitline currents (the
contract); the line solver is held to a tighter 1e-7 V (FP32 output rounding
of ~1 V nodes) / 1e-6 where the cells are weak.  The reference-order method must reproduce the reference's own
iterates (FP64 to 1e-12 relative).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import nodal, sweeps  # noqa: E402

GW = 1 / 2.93
V_TOL = 1e-6       # max node error vs the FP64 oracle (V)
I_RTOL = 1e-4      # bitline current, relative to the largest current


@pytest.fixture(scope="module")
def acc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import cpp_ir_drop_accelerate as m
    return m


def make_case(seed, B, X, Y, n, m, Rset, vmax, bern=True):
    rng = np.random.default_rng(seed)
    G = 1.0 / np.asarray(Rset)[rng.integers(0, len(Rset), (X, n, Y * m))]
    if bern:
        inp = rng.integers(0, 2, (B, X, n)) * vmax
    else:
        inp = rng.random((B, X, n)) * vmax
    return inp.astype(np.float64), G


def oracle_planes(inp, G, B, X, Y, n, m):
    out, U, D = nodal.solve_layer(inp, G, n, m, X, Y, GW, return_planes=True)
    return out, U, D


def run(acc, inp, G, B, X, Y, n, m, dtype=torch.float32, ret_V=2, **kw):
    ti = torch.tensor(inp, dtype=dtype, device="cuda").contiguous()
    tg = torch.tensor(G, dtype=dtype, device="cuda").contiguous()
    out, stats, iters = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, ret_V=ret_V, return_iters=True, **kw)
    torch.cuda.synchronize()
    return out.double().cpu().numpy(), stats, iters.cpu().numpy()


CFG1 = [2e6, 1.6e6, 1.3e6, 1e6]
STRONG = [1e6, 1 / (1e-6 + (1e-3 - 1e-6) / 3), 1 / (1e-6 + 2 * (1e-3 - 1e-6) / 3), 1e3]

SHAPES = [(1, 1, 1, 5, 7), (2, 2, 3, 16, 24), (3, 1, 2, 32, 32), (2, 2, 1, 64, 64), (2, 1, 1, 100, 77),
          (2, 1, 2, 128, 128), (1, 1, 1, 128, 3), (1, 1, 1, 2, 128)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("cells", ["cfg1", "strong"])
def test_line_solver_matches_oracle(acc, shape, cells):
    B, X, Y, n, m = shape
    Rset, vmax = (CFG1, 1.0) if cells == "cfg1" else (STRONG, 0.2)
    inp, G = make_case(sum(shape) * 7 + (cells == "strong"), B, X, Y, n, m, Rset, vmax)
    cur, U, D = oracle_planes(inp, G, B, X, Y, n, m)
    planes, stats, iters = run(acc, inp, G, B, X, Y, n, m, method="line")
    assert stats["status_or"] == 1, stats
    err_u = np.abs(planes[:, :, :, 0] - U).max()
    err_d = np.abs(planes[:, :, :, 1] - D).max()
    # weak cells converge to ~1e-9 V; the returned FP32 planes then round a
    # 1 V wordline node to 6e-8 V
    tol = 1e-7 if cells == "cfg1" else V_TOL
    assert max(err_u, err_d) < tol, (err_u, err_d, stats)
    got, _, _ = run(acc, inp, G, B, X, Y, n, m, method="line", ret_V=False)
    assert np.abs(got - cur).max() <= (1e-6 if cells == "cfg1" else I_RTOL) * np.abs(cur).max()


def test_line_solver_config1_tile(acc, gold):
    """The 128x128 four-state tile of the reference's own config (seed 1, 1 V on every row)."""
    z = gold("sim_v1_128_tol1e-11.npz")
    g = 1.0 / z["Rset"][z["states"]]
    inp = np.ones((1, 1, 128))
    planes, stats, _ = run(acc, inp, g.reshape(1, 128, 128), 1, 1, 1, 128, 128, method="line")
    u, d = nodal.solve(g, GW, z["vin"])
    assert np.abs(planes[0, 0, 0, 0] - u).max() < 1e-7
    assert np.abs(planes[0, 0, 0, 1] - d).max() < 1e-8
    assert stats["iters_max"] <= 6
    # and the reference's converged sim output on the stored rows
    r = z["sample_rows"]
    assert np.abs(planes[0, 0, 0, 0][r] - z["vup_rows"]).max() < 1e-7
    cur, _, _ = run(acc, inp, g.reshape(1, 128, 128), 1, 1, 1, 128, 128, method="line", ret_V=False)
    np.testing.assert_allclose(cur[0, 0], z["iout"], rtol=1e-6)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_line_solver_dtypes(acc, dtype):
    B, X, Y, n, m = 3, 2, 2, 64, 48
    inp, G = make_case(9, B, X, Y, n, m, CFG1, 0.2, bern=False)
    cur = nodal.solve_layer(inp, G, n, m, X, Y, GW)
    got, _, _ = run(acc, inp, G, B, X, Y, n, m, dtype=dtype, ret_V=False, method="line")
    assert np.abs(got - cur).max() <= 1e-6 * np.abs(cur).max()


@pytest.mark.parametrize("shape", [(2, 1, 1, 16, 24), (1, 2, 1, 64, 64), (1, 1, 1, 128, 128),
                                   (2, 1, 2, 256, 256), (1, 1, 1, 130, 256), (1, 1, 1, 200, 150),
                                   (1, 1, 1, 512, 512), (1, 1, 1, 300, 420)])
def test_rbsor_matches_oracle(acc, shape):
    """The plain red-black SOR, single-CTA up to 128 and cluster-resident above
    (4-CTA bands up to 256, 16-CTA bands up to 512, halo rows through
    distributed shared memory, partial and empty bands included)."""
    B, X, Y, n, m = shape
    inp, G = make_case(21, B, X, Y, n, m, CFG1, 0.2)
    cur, U, D = oracle_planes(inp, G, B, X, Y, n, m)
    planes, stats, iters = run(acc, inp, G, B, X, Y, n, m, method="rbsor")
    assert stats["status_or"] == 1, stats
    err = max(np.abs(planes[:, :, :, 0] - U).max(), np.abs(planes[:, :, :, 1] - D).max())
    assert err < V_TOL, (err, stats)
    got, st2, _ = run(acc, inp, G, B, X, Y, n, m, method="rbsor", ret_V=False)
    assert st2["status_or"] == 1, st2
    assert np.abs(got - cur).max() <= I_RTOL * np.abs(cur).max()


@pytest.mark.parametrize("dt,rtol", [(np.float64, 1e-12), (np.float32, 2e-5)])
def test_sweep_order_matches_reference_iterates(acc, gold, dt, rtol):
    """Reference order: same iterates as the reference's PimTorch GS (golden) and
    as the oracle restatement, fixed sweeps and with the delta break."""
    z = gold("pimtorch_gs_8x6.npz")
    B, X, Y, n, m = [int(z[k]) for k in ["B", "numX", "numY", "rows", "cols"]]
    tdt = torch.float64 if dt == np.float64 else torch.float32
    tag = "f64" if dt == np.float64 else "f32"
    ti = torch.tensor(z["input"], dtype=tdt, device="cuda")
    tg = torch.tensor(z["G"], dtype=tdt, device="cuda")
    out, stats, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, iter_times=int(z["fixed_iters"]), g_wire=GW,
                                      beta=float(z["omega"]), method="sweeps")
    ref = z["fixed_" + tag]
    assert np.abs(out.cpu().numpy() - ref).max() <= rtol * np.abs(ref).max()
    thr = float(z["break_thr_" + tag])
    out, stats, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, iter_times=5000, g_wire=GW, beta=float(z["omega"]),
                                      enable_break=True, break_threshould=thr, method="sweeps")
    ref = z["break_" + tag]
    _, it = sweeps.ir_drop_gs(z["input"].astype(dt), z["G"].astype(dt), B, n, m, X, Y, 5000, GW,
                              float(z["omega"]), True, thr, return_iters=True)
    assert abs(stats["iters_max"] - it) <= (0 if dt == np.float64 else 2)
    assert np.abs(out.cpu().numpy() - ref).max() <= 4 * rtol * np.abs(ref).max()


def test_sweep_order_ret_v_and_larger(acc):
    B, X, Y, n, m = 2, 2, 1, 24, 40
    inp, G = make_case(5, B, X, Y, n, m, STRONG, 0.2)
    ti = torch.tensor(inp, device="cuda")
    tg = torch.tensor(G, device="cuda")
    out, _, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, X, Y, iter_times=37, beta=1.9, ret_V=True, method="sweeps")
    ref = sweeps.ir_drop_gs(inp, G, B, n, m, X, Y, 37, GW, 1.9, ret_V=True)
    assert np.abs(out.cpu().numpy() - ref).max() < 1e-12


def test_dropin_signature_and_errors(acc):
    B, X, Y, n, m = 2, 1, 1, 8, 8
    inp, G = make_case(1, B, X, Y, n, m, CFG1, 1.0)
    ti = torch.tensor(inp, dtype=torch.float32, device="cuda")
    tg = torch.tensor(G, dtype=torch.float32, device="cuda")
    out = acc.ir_drop_gs(ti, tg, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    assert out.shape == (B, X, Y * m) and out.dtype == torch.float32 and out.is_cuda
    v = acc.ir_drop_gs(ti, tg, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], True)
    assert v.shape == (B, X, Y, n, m)
    with pytest.raises(RuntimeError):
        acc.ir_drop_gs(ti.cpu(), tg, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    with pytest.raises(RuntimeError):
        acc.ir_drop_gs(ti, tg.t(), B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    with pytest.raises(RuntimeError):
        acc.ir_drop_gs(ti, tg, B, 1, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    with pytest.raises(RuntimeError):
        acc.ir_drop_gs(ti, tg.double(), B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    with pytest.raises(RuntimeError, match="nonlinear_params"):  # sinh cells need all six parameters
        acc.ir2s(ti, tg, B, n, m, X, Y, 10, 2.93, False, 1e-7, True, [1.0])
    empty = acc.ir_drop_gs(ti[:0], tg, 0, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    assert empty.shape == (0, X, Y * m)


def test_line_solver_deterministic_and_stream(acc):
    B, X, Y, n, m = 4, 2, 2, 128, 128
    inp, G = make_case(77, B, X, Y, n, m, CFG1, 0.2)
    ti = torch.tensor(inp, dtype=torch.float32, device="cuda")
    tg = torch.tensor(G, dtype=torch.float32, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        a = acc.ir_drop_gs(ti, tg, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    s.synchronize()
    b = acc.ir_drop_gs(ti, tg, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    assert torch.equal(a, b)


@pytest.mark.parametrize("n", [16, 256])  # single-CTA and cluster kernels
def test_nonfinite_input_reports_status(acc, n):
    B, X, Y, m = 2, 1, 1, n
    inp, G = make_case(3, B, X, Y, n, m, CFG1, 1.0)
    G[0, 3, 4] = np.nan
    _, stats, iters = run(acc, inp, G, B, X, Y, n, m, method="line")
    assert stats["status_or"] & 4
    # the NaN stays in its lines (fmaxf skips it in the maxima): the rest converges as usual
    # and the status flags the result, well before the iteration cap
    assert iters.max() < 10
    cur, stats, _ = run(acc, inp, G, B, X, Y, n, m, method="line", ret_V=False)
    assert stats["status_or"] & 4


def test_dropin_reports_solve_status(acc, monkeypatch):
    """ir_drop_gs reads every call's status back: a clean call matches the
    oracle and stays silent; a NaN conductance or an iteration cap far below
    what the tolerance needs warns (check_status "warn", the default), raises
    under "raise", and passes silently under "off"."""
    import warnings
    B, X, Y, n, m = 3, 2, 1, 64, 64
    inp, G = make_case(8, B, X, Y, n, m, STRONG, 1.0)
    ti = torch.tensor(inp, dtype=torch.float32, device="cuda")
    tg = torch.tensor(G, dtype=torch.float32, device="cuda")
    call = lambda g: acc.ir_drop_gs(ti, g, B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False)
    with warnings.catch_warnings():
        warnings.simplefilter("error", acc.SolveStatusWarning)
        out = call(tg)
    ref = nodal.solve_layer(inp, G, n, m, X, Y, GW)
    assert np.abs(out.double().cpu().numpy() - ref).max() <= I_RTOL * np.abs(ref).max()
    bad = tg.clone()
    bad[1, 9, 10] = float("nan")
    with pytest.warns(acc.SolveStatusWarning, match="non-finite"):
        call(bad)
    monkeypatch.setattr(acc.options, "check_status", "raise")
    with pytest.raises(acc.SolveStatusError, match="non-finite"):
        call(bad)
    monkeypatch.setattr(acc.options, "max_iters", 1)
    monkeypatch.setattr(acc.options, "tol_v", 1e-8)
    with pytest.raises(acc.SolveStatusError, match="iteration cap"):
        call(tg)
    monkeypatch.setattr(acc.options, "check_status", "off")
    with warnings.catch_warnings():
        warnings.simplefilter("error", acc.SolveStatusWarning)
        call(bad)


@pytest.mark.parametrize("method,n,cap", [("line", 64, 1), ("line", 256, 2), ("rbsor", 64, 5), ("rbsor", 256, 12)])
def test_iteration_cap_reports_status(acc, method, n, cap):
    """Forced non-convergence: a cap far below what the tolerance needs ends
    every solve with the cap status, never the converged one, at the cap."""
    B, X, Y = 3, 2, 1
    inp, G = make_case(4, B, X, Y, n, n, STRONG, 1.0)
    _, stats, iters = run(acc, inp, G, B, X, Y, n, n, method=method, max_iters=cap, tol_v=1e-8, ret_V=False)
    assert stats["status_or"] & 2 and not stats["status_or"] & 1, stats
    assert iters.min() == cap and iters.max() == cap


@pytest.mark.parametrize("tol", [5e-7, 1e-8])
@pytest.mark.parametrize("cells,n", [("cfg1", 128), ("cfg1", 64), ("strong", 64), ("cfg1", 256), ("strong", 256),
                                     ("cfg1", 512)])
def test_precision_schedule_meets_tolerance(acc, tol, cells, n):
    """The adaptive schedule (FP32 residuals, a precise one on the last
    iteration, per-tile choice of the cheaper precise form, rate carried between
    the vectors of a tile) against the FP64 oracle, with many vectors per work
    item as in a throughput run; float64 I/O so the planes come back unrounded.
    256 and 512 run on the cluster kernels."""
    B, X, Y = (24, 2, 1) if n <= 128 else (6, 1, 1)
    inp, G = make_case(21 + n, B, X, Y, n, n, CFG1 if cells == "cfg1" else STRONG, 0.2 if cells == "cfg1" else 1.0)
    _, U, D = oracle_planes(inp, G, B, X, Y, n, n)
    got, st, _ = run(acc, inp, G, B, X, Y, n, n, dtype=torch.float64, method="line", tol_v=tol, vectors_per_cta=B)
    assert st["status_or"] == 1
    # the stop test floors at 4 ulps of the largest deviation (FP32 planes); the
    # error there is within ~8 ulps:
    # ~1e-9 V for weak cells (1e-2 V drops), ~8e-7 V for strong ones (0.9 V)
    dev = max(np.abs(U - inp.reshape(B, X, 1, n, 1)).max(), np.abs(D).max())
    floor = max(2e-9, 8 * 2.0 ** -23 * dev)
    err = max(np.abs(got[:, :, :, 0] - U).max(), np.abs(got[:, :, :, 1] - D).max())
    assert err <= tol + floor, (err, st)
    # the every-iteration float-float schedule agrees with it to the same tolerance
    ref, _, _ = run(acc, inp, G, B, X, Y, n, n, dtype=torch.float64, method="line", tol_v=tol, residual_period=1)
    assert np.abs(got - ref).max() <= 2 * (tol + floor)


@pytest.fixture(scope="module")
def full_size():
    """The throughput workload's full size: 4096 tiles of 128 x 128, 64 input
    vectors each (262,144 solves), four-state 1-2 Mohm cells; two input sets."""
    B, X, n = 64, 4096, 128
    g = torch.Generator().manual_seed(11)
    states = torch.randint(0, 4, (X, n, n), generator=g)
    G = (1.0 / torch.tensor(CFG1, dtype=torch.float64))[states].float().cuda()
    va = (torch.randint(0, 2, (B, X, n), generator=g) * 0.2).float().cuda()
    vb = (torch.rand((B, X, n), generator=g) * 0.1).float().cuda()
    return B, X, n, G, va, vb


def test_full_size_linearity_and_tile_order(acc, full_size):
    """At the full size, where the oracle cannot follow: every solve converges;
    with linear cells the currents are linear in the inputs, I(a) + I(b) =
    I(a + b) to the solver's tolerance; tiles are independent, so solving them
    in another order returns the same currents in that order."""
    B, X, n, G, va, vb = full_size

    def solve(v, g):
        out, st, _ = acc.ir_drop_gs_ex(v.contiguous(), g.contiguous(), B, n, n, X, 1, method="line", tol_v=1e-8)
        assert st["solves"] == B * X and st["status_or"] == 1, st
        return out.double()

    Ia, Ib, Iab = solve(va, G), solve(vb, G), solve(va + vb, G)
    scale = Iab.abs().max().item()
    assert (Ia + Ib - Iab).abs().max().item() <= 1e-5 * scale
    perm = torch.randperm(X, generator=torch.Generator().manual_seed(5)).cuda()
    Ip = solve(va[:, perm], G[perm])
    assert (Ip - Ia[:, perm]).abs().max().item() <= 1e-5 * Ia.abs().max().item()
