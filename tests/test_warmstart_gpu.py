"""The learned warm start: its CUDA kernels and gradients against a torch-CPU
FP32 reference of the same network (same bf16-rounded weights and inputs),
the solver's use of a warm start (exact, garbage -> rejected), and what a
briefly trained network gains in line iterations."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import torch.nn.functional as F  # noqa: E402

from oracle import nodal  # noqa: E402

GW = 1 / 2.93


@pytest.fixture(scope="module")
def ws():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import warmstart
    from fadesim_gb300.build import build
    build()
    return warmstart


def bf(t):
    return t.to(torch.bfloat16)


def nchw(t):
    return t.float().cpu().permute(0, 3, 1, 2)


def rel(a, b):
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


@pytest.mark.parametrize("cin,cout,H,W", [(16, 32, 16, 24), (32, 64, 8, 8), (64, 16, 12, 20), (96, 128, 8, 8)])
def test_conv_kernels_match_torch(ws, cin, cout, H, W):
    g = torch.Generator().manual_seed(cin + cout)
    N = 2
    x = bf(torch.randn((N, H, W, cin), generator=g)).cuda()
    conv = ws.Conv(cin, cout, g, "cuda")
    conv.b.copy_(torch.randn(cout, generator=g))
    y = conv.fwd(x, relu=False, f32=True)
    wr = conv.wb.float().cpu().permute(0, 3, 1, 2)
    ref = F.conv2d(nchw(x), wr, conv.b.cpu(), padding=1)
    assert rel(nchw(y), ref) < 2e-3
    # input and weight gradients for a random output gradient
    dy = bf(torch.randn((N, H, W, cout), generator=g)).cuda()
    conv.zero_grad()
    dx = conv.bwd(dy, x)
    dx_ref = torch.nn.grad.conv2d_input((N, cin, H, W), wr, nchw(dy), padding=1)
    assert rel(nchw(dx), dx_ref) < 1e-2
    dw_ref = torch.nn.grad.conv2d_weight(nchw(x), wr.shape, nchw(dy), padding=1)
    assert rel(conv.gw.cpu().permute(0, 3, 1, 2), dw_ref) < 1e-4
    assert rel(conv.gb.cpu(), nchw(dy).sum(dim=(0, 2, 3))) < 1e-4


@pytest.mark.parametrize("cin,cout,N,H,W", [(32, 32, 1, 128, 128), (32, 64, 2, 32, 32), (96, 128, 2, 16, 16),
                                             (128, 96, 1, 64, 64), (64, 32, 3, 16, 16), (128, 16, 2, 32, 32),
                                             (32, 32, 1, 24, 16)])
def test_tensor_core_conv_matches_torch(ws, cin, cout, N, H, W):
    """The tcgen05 / TMA convolution (the network's shapes: Cin a multiple of
    32, 16 x 8-pixel tiles whose input box serves all three row shifts, "same"
    padding from the TMA zero fill) against torch's FP32 convolution of the
    same bf16 operands and against the mma.sync kernel; ReLU, skip connection
    and bf16 output in the epilogue; the input gradient through the same
    kernel; the weight gradient on the tensor-core kernel (MN-major operands)
    where Cout is a multiple of 32; no bounded wait expired."""
    tc = ws._k().fadesim_conv_tc_shape(H, W, cin, cout)
    assert tc & 1 and bool(tc & 2) == (cout % 32 == 0)  # forward / weight gradient on the tensor cores
    g = torch.Generator().manual_seed(cin * 7 + cout + H)
    x = bf(torch.randn((N, H, W, cin), generator=g)).cuda()
    conv = ws.Conv(cin, cout, g, "cuda")
    conv.b.copy_(torch.randn(cout, generator=g))
    stream = torch.cuda.current_stream().cuda_stream
    y = conv.fwd(x, relu=False, f32=True)
    assert ws._k().fadesim_conv_tc_status(stream) == 0
    wr = conv.wb.float().cpu().permute(0, 3, 1, 2)
    ref = F.conv2d(nchw(x), wr, conv.b.cpu(), padding=1)
    assert rel(nchw(y), ref) < 1e-5
    legacy = conv.fwd(x, relu=False, f32=True, legacy=True)
    assert rel(y.cpu(), legacy.cpu()) < 1e-5
    skip = bf(torch.randn((N, H, W, cout), generator=g)).cuda()
    yr = conv.fwd(x, relu=True, skip=skip)
    ref2 = F.relu(ref) + nchw(skip)
    assert yr.dtype == torch.bfloat16 and rel(nchw(yr), ref2) < 1e-2
    dy = bf(torch.randn((N, H, W, cout), generator=g)).cuda()
    conv.zero_grad()
    dx = conv.bwd(dy, x)
    dx_ref = torch.nn.grad.conv2d_input((N, cin, H, W), wr, nchw(dy), padding=1)
    assert rel(nchw(dx), dx_ref) < 1e-2
    dw_ref = torch.nn.grad.conv2d_weight(nchw(x), wr.shape, nchw(dy), padding=1)
    assert rel(conv.gw.cpu().permute(0, 3, 1, 2), dw_ref) < 1e-4
    assert ws._k().fadesim_conv_tc_status(stream) == 0


def test_pool_upsample_kernels(ws):
    g = torch.Generator().manual_seed(3)
    x = bf(torch.randn((2, 8, 12, 16), generator=g)).cuda()
    p = ws._pool(x)
    assert rel(nchw(p), F.avg_pool2d(nchw(x), 2)) < 1e-2
    u = ws._pool(p, up=True)
    assert torch.equal(nchw(u), F.interpolate(nchw(p), scale_factor=2, mode="nearest"))
    d = bf(torch.randn(p.shape, generator=g)).cuda()
    pb = ws._pool(d, backward=True)             # avgpool backward: spread 1/4
    assert rel(nchw(pb), F.interpolate(nchw(d), scale_factor=2, mode="nearest") * 0.25) < 1e-2
    ub = ws._pool(bf(torch.randn(u.shape, generator=g)).cuda(), backward=True, up=True)
    assert ub.shape == p.shape


def torch_reference(net, x, target):
    """The same network in torch autograd, FP32 on the CPU, from the bf16 weights."""
    L = net.layers
    params = {}
    for k, l in L.items():
        params[k] = (l.wb.float().cpu().permute(0, 3, 1, 2).clone().requires_grad_(True),
                     l.b.cpu().clone().requires_grad_(True))
    conv = lambda k, t: F.conv2d(t, params[k][0], params[k][1], padding=1)
    xi = nchw(x)
    e1 = F.relu(conv("e1", xi))
    e2 = F.relu(conv("e2", F.avg_pool2d(e1, 2)))
    e3 = F.relu(conv("e3", F.avg_pool2d(e2, 2)))
    e4 = F.relu(conv("e4", F.avg_pool2d(e3, 2)))
    d3 = F.relu(conv("d3", F.interpolate(e4, scale_factor=2))) + e3
    d2 = F.relu(conv("d2", F.interpolate(d3, scale_factor=2))) + e2
    d1 = F.relu(conv("d1", F.interpolate(d2, scale_factor=2))) + e1
    y = conv("out", d1)
    loss = ((y[:, :2] - target.cpu().permute(0, 3, 1, 2)) ** 2).mean()
    loss.backward()
    return loss.item(), {k: (p[0].grad.permute(0, 2, 3, 1), p[1].grad) for k, p in params.items()}


def test_network_gradients_match_cpu_autograd(ws):
    net = ws.WarmStartNet(seed=1)
    g = torch.Generator().manual_seed(5)
    G = 1.0 / torch.tensor([2e6, 1.6e6, 1.3e6, 1e6])[torch.randint(0, 4, (2, 32, 32), generator=g)]
    vin = torch.randint(0, 2, (2, 32), generator=g).float() * 0.2
    x, _ = net.make_inputs(G.cuda(), vin.cuda())
    target = torch.randn((2, 32, 32, 2), generator=g).cuda() * 0.3
    for l in net.layers.values():
        l.zero_grad()
    y = net.forward(x, keep=True)
    loss, dy = net.loss_and_grad(y, target)
    net.backward(dy)
    ref_loss, ref_grads = torch_reference(net, x, target)
    assert abs(loss.item() - ref_loss) < 2e-2 * ref_loss
    for k, l in net.layers.items():
        gw, gb = ref_grads[k]
        assert rel(l.gw.cpu(), gw) < 6e-2, k
        assert rel(l.gb.cpu(), gb) < 6e-2, k


def test_solver_warm_start_exact_and_garbage(ws):
    from fadesim_gb300 import cpp_ir_drop_accelerate as acc
    rng = np.random.default_rng(2)
    n = m = 64
    B = 4
    G = 1.0 / np.array([1e6, 3.3e5, 2e4, 1e3])[rng.integers(0, 4, (1, n, m))]
    vin = rng.integers(0, 2, (B, 1, n)) * 0.2
    u, d = nodal.solve(G[0], GW, vin[:, 0])
    exact = np.stack([u - vin[:, 0, :, None], d], axis=1)[:, None, None]  # [B, 1, 1, 2, n, m]
    ti = torch.tensor(vin, dtype=torch.float32, device="cuda")
    tg = torch.tensor(G, dtype=torch.float32, device="cuda")
    cold, st0, _ = acc.ir_drop_gs_ex(ti, tg, B, n, m, 1, 1, g_wire=GW, method="line")
    warm, st1, _ = acc.ir_drop_gs_warm(ti, tg, B, n, m, 1, 1, torch.tensor(exact, dtype=torch.float32).cuda())
    assert st1["status_or"] == 1 and st1["iters_max"] <= 3 < st0["iters_max"]
    ref = nodal.currents(G[0], u, d)
    assert np.abs(warm.double().cpu().numpy()[:, 0] - ref).max() <= 1e-4 * np.abs(ref).max()
    junk = torch.full(exact.shape, 0.7, dtype=torch.float32, device="cuda")
    out, st2, _ = acc.ir_drop_gs_warm(ti, tg, B, n, m, 1, 1, junk)
    assert st2["status_or"] & 8 and st2["status_or"] & 1
    assert np.abs(out.double().cpu().numpy()[:, 0] - ref).max() <= 1e-4 * np.abs(ref).max()


@pytest.mark.parametrize("n,sinh", [(256, False), (512, False), (256, True), (512, True)])
def test_cluster_warm_start_exact_and_garbage(ws, n, sinh):
    """Warm starts on the cluster layouts (256 x 256 on 4-CTA clusters, 512 x
    512 on 16-CTA clusters; linear and sinh cells with lognormal variation):
    started from the converged planes the solve takes fewer iterations and
    returns the same currents; started from planes that are far off it discards them
    (FADESIM_ST_WARM_REJECTED), restarts from the ideal state and lands on the
    same currents again."""
    from fadesim_gb300 import cpp_ir_drop_accelerate as acc
    from fadesim_gb300.variation import add_variation_device
    B, X = 2, 1
    rng = np.random.default_rng(n + sinh)
    R4 = np.array([2e6, 1.6e6, 1.3e6, 1e6])
    G0 = torch.tensor(1.0 / R4[rng.integers(0, 4, (X, n, n))], dtype=torch.float32, device="cuda")
    tg = add_variation_device(G0, 0.1, seed=5) if sinh else G0
    vin = torch.tensor(rng.random((B, X, n)) * 0.2, dtype=torch.float32, device="cuda")
    nl = dict(nonlinear_cell_enable=True, nonlinear_params=nodal.sinh_params(1e6, 2e6)) if sinh else {}
    planes, st0, _ = acc.ir_drop_gs_ex(vin, tg, B, n, n, X, 1, g_wire=GW, ret_V=2, method="line", **nl)
    cold, st1, _ = acc.ir_drop_gs_ex(vin, tg, B, n, n, X, 1, g_wire=GW, method="line", **nl)
    assert st0["status_or"] == 1 and st1["status_or"] == 1
    init = planes.float().clone()
    init[:, :, :, 0] -= vin[:, :, None, :, None]
    wkw = dict(g_wire=GW, nonlinear_params=nodal.sinh_params(1e6, 2e6) if sinh else None)
    warm, st2, _ = acc.ir_drop_gs_warm(vin, tg, B, n, n, X, 1, init.contiguous(), **wkw)
    assert st2["status_or"] == 1 and st2["warm_rejected"] == 0
    assert st2["iters_max"] <= 3 and st2["iters_sum"] < st1["iters_sum"], (st2, st1)
    scale = cold.abs().max().item()
    assert (warm - cold).abs().max().item() <= 1e-5 * scale
    junk = torch.full(init.shape, 0.7, dtype=torch.float32, device="cuda")
    out, st3, _ = acc.ir_drop_gs_warm(vin, tg, B, n, n, X, 1, junk, **wkw)
    assert st3["status_or"] & 8 and st3["status_or"] & 1 and st3["warm_rejected"] == B * X
    assert (out - cold).abs().max().item() <= 1e-5 * scale


def test_trained_network_prediction_and_warm_solve(ws, tmp_path):
    """Train briefly on solver-generated data with the strong 2-bit cells of the
    MLP layers (1 kohm - 1 Mohm, linear in conductance, 64x64 tiles, Bernoulli
    0.2 V inputs).  What the network gains over the method without it: its
    prediction starts the solve at under half the error of the ideal state (the
    method's own start), no prediction is discarded, and the solve from it
    still lands on the oracle (the solver, not the network, decides the error).
    Whether that start saves iterations depends on the setting and is not
    asserted: on the GPU, at 128x128 after 65k training instances it saved 11%
    of the line iterations (25.1 -> 22.3), here at 64x64 after 32k it cost 25%
    (12.1 -> 15.2); the bench reports both, and what the warm start is worth
    once the network's inference is counted (a net loss)."""
    from fadesim_gb300 import cpp_ir_drop_accelerate as acc
    n = 64
    gvals = torch.tensor([1e-6 + k * (1e-3 - 1e-6) / 3 for k in range(4)])
    gen = torch.Generator().manual_seed(11)

    def batch(N):
        G = gvals[torch.randint(0, 4, (N, n, n), generator=gen)].float().cuda()
        vin = (torch.randint(0, 2, (N, n), generator=gen).float() * 0.2).cuda()
        return G, vin

    def solve_planes(G, vin):
        # one tile per instance: numX = N tiles, one input vector each
        N = G.shape[0]
        planes, _, _ = acc.ir_drop_gs_ex(vin[None].contiguous(), G.contiguous(), 1, n, n, N, 1, g_wire=GW, ret_V=2,
                                         method="line")
        p = planes[0, :, 0].clone()  # [N, 2, n, n]
        p[:, 0] -= vin[:, :, None]
        return p

    net = ws.WarmStartNet(seed=0)
    losses = []
    for step in range(1000):
        G, vin = batch(32)
        x, _ = net.make_inputs(G, vin)
        tgt = ws.solver_targets(G, vin, solve_planes)
        losses.append(net.train_step(x, tgt, lr=1e-3).item())
    assert np.mean(losses[-20:]) < 0.5 * np.mean(losses[:20])
    net.save(str(tmp_path / "net.pt"))
    net2 = ws.WarmStartNet(seed=99)
    net2.load(str(tmp_path / "net.pt"))
    N = 64
    G, vin = batch(N)
    pred = net2.predict_planes(G, vin)
    true = solve_planes(G, vin)
    assert float((pred - true).norm() / true.norm()) < 0.5  # the ideal state is 1.0 away
    init = pred[None, :, None].contiguous()
    ti = vin[None].contiguous()
    _, st_cold, _ = acc.ir_drop_gs_ex(ti, G, 1, n, n, N, 1, g_wire=GW, method="line")
    cur, st_warm, _ = acc.ir_drop_gs_warm(ti, G, 1, n, n, N, 1, init)
    assert st_warm["status_or"] == 1 and st_cold["status_or"] == 1, (st_warm, st_cold)
    assert st_warm["warm_rejected"] == 0
    print("line iterations per solve: cold %.2f, warm %.2f" % (st_cold["iters_sum"] / N, st_warm["iters_sum"] / N))
    Gn = G.double().cpu().numpy()
    vn = vin.double().cpu().numpy()
    for k in range(4):
        u, d = nodal.solve(Gn[k], GW, vn[k])
        ref = nodal.currents(Gn[k], u, d)
        assert np.abs(cur[0, k].double().cpu().numpy() - ref).max() <= 1e-4 * np.abs(ref).max()
