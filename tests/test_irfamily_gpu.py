"""The reference extension's other exports (ir2s, ir2s_ou_local, ir2s_ou,
ir_gs_ou_local, ir_gs_ou) through the drop-in module: their iterates against the
numpy restatement (FP64 to rounding, FP32 within its precision), with and
without the delta break, and the IR2S restatement pinned to the reference's own
Python IR2S."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import sweeps  # noqa: E402

GW = 1 / 2.93


@pytest.fixture(scope="module")
def acc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import cpp_ir_drop_accelerate as m
    return m


def case(seed, B, X, Y, n, m):
    rng = np.random.default_rng(seed)
    inp = rng.integers(0, 2, (B, X, n)) * 0.2
    G = 1.0 / rng.choice([1e3, 2e4, 3e5, 1e6], size=(X, n, Y * m))
    return inp, G


def tt(a, dt):
    return torch.tensor(a, dtype=dt, device="cuda").contiguous()


TOL = {torch.float64: 1e-11, torch.float32: 3e-5}


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
@pytest.mark.parametrize("iters,brk", [(7, False), (400, True)])
def test_ir2s_family(acc, dt, iters, brk):
    B, X, Y, n, m = 3, 2, 2, 16, 12
    inp, G = case(5, B, X, Y, n, m)
    thr = 1e-9 if dt == torch.float64 else 1e-6
    np_dt = np.float64 if dt == torch.float64 else np.float32
    i64, g64 = inp.astype(np_dt), G.astype(np_dt)
    runs = [
        (acc.ir2s(tt(inp, dt), tt(G, dt), B, n, m, X, Y, iters, 2.93, brk, thr),
         sweeps.ir_family(i64, g64, B, n, m, X, Y, iters, 2.93, "ir2s", enable_break=brk, break_threshold=thr)),
        (acc.ir2s(tt(inp, dt), tt(G, dt), B, n, m, X, Y, iters, 2.93, brk, thr, False, [], True),
         sweeps.ir_family(i64, g64, B, n, m, X, Y, iters, 2.93, "ir2s", enable_break=brk, break_threshold=thr,
                          ret_V=True)),
        (acc.ir2s_ou_local(tt(inp, dt), tt(G, dt), B, n, m, X, Y, iters, 2.93, 5.0, 7.5, brk, thr),
         sweeps.ir_family(i64, g64, B, n, m, X, Y, iters, 2.93, "ir2s", loads=(5.0, 7.5), enable_break=brk,
                          break_threshold=thr)),
        (acc.ir2s_ou(tt(inp, dt), tt(G, dt), B, n, m, 4, 3, X, Y, iters, 2.93, brk, thr),
         sweeps.ir_family(i64, g64, B, n, m, X, Y, iters, 2.93, "ir2s", ou=(4, 3), enable_break=brk,
                          break_threshold=thr)),
    ]
    for got, ref in runs:
        got = got.double().cpu().numpy().reshape(ref.shape)
        assert np.abs(got - ref).max() <= TOL[dt] * np.abs(ref).max()


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
@pytest.mark.parametrize("iters,brk", [(9, False), (3000, True)])
def test_gs_ou_family(acc, dt, iters, brk):
    B, X, Y, n, m = 2, 2, 3, 16, 12
    inp, G = case(6, B, X, Y, n, m)
    thr = 1e-10 if dt == torch.float64 else 1e-6
    np_dt = np.float64 if dt == torch.float64 else np.float32
    i64, g64 = inp.astype(np_dt), G.astype(np_dt)
    runs = [
        (acc.ir_gs_ou_local(tt(inp, dt), tt(G, dt), B, n, m, X, Y, iters, GW, 0.2, 0.15, 1.7, brk, thr),
         sweeps.ir_family(i64, g64, B, n, m, X, Y, iters, GW, "gs", loads=(0.2, 0.15), beta=1.7, enable_break=brk,
                          break_threshold=thr)),
        (acc.ir_gs_ou(tt(inp, dt), tt(G, dt), B, n, m, 8, 4, X, Y, iters, GW, 1.7, brk, thr),
         sweeps.ir_family(i64, g64, B, n, m, X, Y, iters, GW, "gs", ou=(8, 4), beta=1.7, enable_break=brk,
                          break_threshold=thr)),
    ]
    for got, ref in runs:
        got = got.double().cpu().numpy().reshape(ref.shape)
        assert np.abs(got - ref).max() <= TOL[dt] * np.abs(ref).max()


def test_ir2s_matches_reference_python(acc, gold):
    z = gold("pimtorch_ir2s_8x6.npz")
    B, X, Y, n, m = (int(z[k]) for k in ("B", "numX", "numY", "rows", "cols"))
    for iters in (6, 300):
        got = acc.ir2s(tt(z["input"], torch.float64), tt(z["G"], torch.float64), B, n, m, X, Y, iters,
                       float(z["r_wire"]), False, 0.0).cpu().numpy()
        ref = z["iters_%d" % iters]
        assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def test_family_argument_errors(acc):
    inp, G = case(1, 1, 1, 1, 8, 8)
    with pytest.raises(RuntimeError):
        acc.ir_gs_ou(tt(inp, torch.float32), tt(G, torch.float32), 1, 8, 8, 3, 4, 1, 1, 5, GW, 1.9, False, 0.0)
    with pytest.raises(RuntimeError, match="nonlinear_params"):
        acc.ir2s(tt(inp, torch.float32), tt(G, torch.float32), 1, 8, 8, 1, 1, 5, 2.93, False, 0.0, True, [1e3])
    with pytest.raises(RuntimeError, match="nonlinear_params"):  # R_off below R_on
        acc.ir_gs_ou_local(tt(inp, torch.float32), tt(G, torch.float32), 1, 8, 8, 1, 1, 5, GW, 0.2, 0.2, 1.5, False,
                           0.0, True, [1e6, 1e3, 2, 1e-3, 2, 1e-6])


def nl_case(seed, B=2, X=2, Y=2, n=8, m=6):
    """Sinh cells I = b sinh(a V), a = 2, b = 1 / (a R), between 100 kohm and
    1 Mohm; inputs U[0, 0.2] V with one row at 0 V (cells under the reference's
    |V| < 1e-5 clamp)."""
    rng = np.random.default_rng(seed)
    inp = rng.uniform(0, 0.2, (B, X, n))
    inp[0, 0, 1] = 0.0
    G = 1 / rng.choice([1e5, 2e5, 5e5, 1e6], size=(X, n, Y * m))
    params = [1e5, 1e6, 2.0, 1.0 / (2.0 * 1e5), 2.0, 1.0 / (2.0 * 1e6)]
    return inp, G, params


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
@pytest.mark.parametrize("iters,brk", [(1, False), (6, False), (300, True)])
def test_nonlinear_family(acc, dt, iters, brk):
    """All five exports with the reference's sinh cells (conductances re-evaluated
    before every iteration from the iterate before the newest, deal_v clamp)
    against the numpy restatement: FP64 to rounding, FP32 within its precision."""
    B, X, Y, n, m = 2, 2, 2, 8, 6
    inp, G, params = nl_case(31 + iters)
    thr = 1e-9 if dt == torch.float64 else 1e-6
    np_dt = np.float64 if dt == torch.float64 else np.float32
    i_, g_ = inp.astype(np_dt), G.astype(np_dt)
    a, g = tt(inp, dt), tt(G, dt)
    nl = dict(nonlinear=params, enable_break=brk, break_threshold=thr)
    runs = [
        (acc.ir2s(a, g, B, n, m, X, Y, iters, 2.93, brk, thr, True, params),
         sweeps.ir_family(i_, g_, B, n, m, X, Y, iters, 2.93, "ir2s", **nl)),
        (acc.ir2s(a, g, B, n, m, X, Y, iters, 2.93, brk, thr, True, params, True),
         sweeps.ir_family(i_, g_, B, n, m, X, Y, iters, 2.93, "ir2s", ret_V=True, **nl)),
        (acc.ir2s_ou_local(a, g, B, n, m, X, Y, iters, 2.93, 5.0, 7.5, brk, thr, True, params),
         sweeps.ir_family(i_, g_, B, n, m, X, Y, iters, 2.93, "ir2s", loads=(5.0, 7.5), **nl)),
        (acc.ir2s_ou(a, g, B, n, m, 4, 3, X, Y, iters, 2.93, brk, thr, True, params),
         sweeps.ir_family(i_, g_, B, n, m, X, Y, iters, 2.93, "ir2s", ou=(4, 3), **nl)),
        (acc.ir_gs_ou_local(a, g, B, n, m, X, Y, iters, GW, 0.2, 0.15, 1.5, brk, thr, True, params),
         sweeps.ir_family(i_, g_, B, n, m, X, Y, iters, GW, "gs", loads=(0.2, 0.15), beta=1.5, **nl)),
        (acc.ir_gs_ou(a, g, B, n, m, 4, 3, X, Y, iters, GW, 1.5, brk, thr, True, params),
         sweeps.ir_family(i_, g_, B, n, m, X, Y, iters, GW, "gs", ou=(4, 3), beta=1.5, **nl)),
    ]
    for k, (got, ref) in enumerate(runs):
        got = got.double().cpu().numpy().reshape(ref.shape)
        assert np.abs(got - ref).max() <= TOL[dt] * np.abs(ref).max(), k


@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_nonlinear_sweep_order_ir_drop_gs(acc, dt):
    """ir_drop_gs with sinh cells under the reference's own sweep order: the
    restatement of its ping-pong nonlinear sweeps, fixed count and delta break,
    currents and cell voltages."""
    B, X, Y, n, m = 2, 2, 2, 8, 6
    inp, G, params = nl_case(5)
    np_dt = np.float64 if dt == torch.float64 else np.float32
    for iters, brk, thr in ((1, False, 0.0), (7, False, 0.0), (2000, True, 1e-9 if dt == torch.float64 else 1e-6)):
        got, st, _ = acc.ir_drop_gs_ex(tt(inp, dt), tt(G, dt), B, n, m, X, Y, iter_times=iters, g_wire=GW, beta=1.5,
                                       enable_break=brk, break_threshould=thr, nonlinear_cell_enable=True,
                                       nonlinear_params=params, method="sweeps")
        ref = sweeps.ir_family(inp.astype(np_dt), G.astype(np_dt), B, n, m, X, Y, iters, GW, "gs", loads=(GW, GW),
                               beta=1.5, nonlinear=params, enable_break=brk, break_threshold=thr)
        got = got.double().cpu().numpy()
        assert np.abs(got - ref).max() <= TOL[dt] * np.abs(ref).max(), iters
        assert st["solves"] == B * X * Y and 1 <= st["iters_max"] <= iters
        v, _, _ = acc.ir_drop_gs_ex(tt(inp, dt), tt(G, dt), B, n, m, X, Y, iter_times=iters, g_wire=GW, beta=1.5,
                                    enable_break=brk, break_threshould=thr, nonlinear_cell_enable=True,
                                    nonlinear_params=params, method="sweeps", ret_V=True)
        vref = sweeps.ir_family(inp.astype(np_dt), G.astype(np_dt), B, n, m, X, Y, iters, GW, "gs", loads=(GW, GW),
                                beta=1.5, nonlinear=params, enable_break=brk, break_threshold=thr, ret_V=True)
        assert np.abs(v.double().cpu().numpy() - vref).max() <= TOL[dt] * np.abs(vref).max(), iters
