"""The host-buffer entry (fadesim_ir_drop_gs_host): pipelined copies around
the same solve, checked against the FP64 oracle and the device-buffer call."""
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


def case(seed, B, X, Y, n, m):
    rng = np.random.default_rng(seed)
    G = 1.0 / np.asarray(CFG1)[rng.integers(0, 4, (X, n, Y * m))]
    inp = rng.integers(0, 2, (B, X, n)) * 0.2
    return inp, G


@pytest.mark.parametrize("group_x, pinned", [(0, True), (3, True), (2, False), (1, True)])
def test_host_currents_match_oracle(acc, group_x, pinned):
    B, X, Y, n, m = 3, 7, 2, 32, 24
    inp, G = case(5, B, X, Y, n, m)
    ti, tg = torch.tensor(inp, dtype=torch.float32), torch.tensor(G, dtype=torch.float32)
    if pinned:
        ti, tg = ti.pin_memory(), tg.pin_memory()
    out, st = acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW, group_x=group_x, return_stats=True)
    assert not out.is_cuda and out.shape == (B, X, Y * m)
    ref = nodal.solve_layer(inp, G, n, m, X, Y, GW)
    assert np.abs(out.double().numpy() - ref).max() <= 1e-6 * np.abs(ref).max()
    assert st["solves"] == B * X * Y and st["status_or"] & 1 and not st["status_or"] & 2


def test_host_status_from_device_counters(acc):
    """The groups' counters stay on the device and come back once: the stats
    cover every solve of every group, and an iteration cap far below what the
    tolerance needs is reported (warning by default, error under "raise") as
    for the device-buffer call."""
    B, X, Y, n, m = 4, 9, 1, 64, 64
    inp, G = case(11, B, X, Y, n, m)
    ti, tg = torch.tensor(inp, dtype=torch.float32).pin_memory(), torch.tensor(G, dtype=torch.float32).pin_memory()
    _, st = acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW, group_x=2, return_stats=True)
    assert st["solves"] == B * X * Y and st["status_or"] == 1 and st["iters_max"] >= 2
    with pytest.warns(acc.SolveStatusWarning):
        acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW, group_x=2, max_iters=1)
    with pytest.raises(acc.SolveStatusError):
        acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW, group_x=2, max_iters=1, check_status="raise")
    _, st = acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW, group_x=2, max_iters=1, check_status="off",
                                return_stats=True)
    assert st["solves"] == B * X * Y and st["status_or"] & 2


@pytest.mark.parametrize("ret_V", [1, 2])
def test_host_planes_layout_f64(acc, ret_V):
    B, X, Y, n, m = 2, 5, 3, 16, 12
    inp, G = case(8, B, X, Y, n, m)
    ti, tg = torch.tensor(inp).pin_memory(), torch.tensor(G).pin_memory()
    got = acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW, ret_V=ret_V, group_x=2)
    dev, _, _ = acc.ir_drop_gs_ex(ti.cuda(), tg.cuda(), B, n, m, X, Y, g_wire=GW, ret_V=ret_V)
    assert got.shape == dev.shape and got.dtype == torch.float64
    assert torch.abs(got - dev.cpu()).max().item() < 1e-8


def test_host_large_pipelined_matches_device_call(acc):
    """Many groups over the copy engines: the same currents as the device call
    on the same tensors (both converge to the tolerance; the group split can
    change which vectors share a CTA, so agreement is to the tolerance)."""
    B, X, Y, n, m = 16, 600, 1, 128, 128
    rng = np.random.default_rng(2)
    G = torch.tensor(1.0 / np.asarray(CFG1)[rng.integers(0, 4, (X, n, m))], dtype=torch.float32).pin_memory()
    inp = torch.tensor(rng.integers(0, 2, (B, X, n)) * 0.2, dtype=torch.float32).pin_memory()
    got = acc.ir_drop_gs_host(inp, G, B, n, m, X, Y, g_wire=GW)
    dev = acc.ir_drop_gs(inp.cuda(), G.cuda(), B, n, m, X, Y, 600, GW, 1.9, False, 1e-7, False, [], False).cpu()
    assert torch.abs(got - dev).max().item() <= 1e-5 * torch.abs(dev).max().item()


def test_host_argument_errors(acc):
    ti = torch.zeros((1, 1, 8))
    tg = torch.zeros((1, 8, 8))
    with pytest.raises(RuntimeError):
        acc.ir_drop_gs_host(ti.cuda(), tg, 1, 8, 8, 1, 1)
    with pytest.raises(RuntimeError):
        acc.ir_drop_gs_host(ti, tg.double(), 1, 8, 8, 1, 1)
    with pytest.raises(RuntimeError):
        acc.ir_drop_gs_host(ti, tg, 1, 8, 8, 2, 1)
    with pytest.raises(TypeError):
        acc.ir_drop_gs_host(ti, tg, 1, 8, 8, 1, 1, tol=1e-8)
    empty = acc.ir_drop_gs_host(ti[:0], tg, 0, 8, 8, 1, 1)
    assert empty.shape == (0, 1, 8)


def test_release_memory_between_calls(acc):
    """The library's pool gives its memory back on request; later calls allocate again."""
    from fadesim_gb300 import _lib
    B, X, Y, n, m = 2, 3, 1, 64, 64
    inp, G = case(11, B, X, Y, n, m)
    ti, tg = torch.tensor(inp, dtype=torch.float32).pin_memory(), torch.tensor(G, dtype=torch.float32).pin_memory()
    first = acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW)
    assert _lib.load().fadesim_release_memory() == 0
    again = acc.ir_drop_gs_host(ti, tg, B, n, m, X, Y, g_wire=GW)
    assert torch.equal(first, again)
