"""Train the warm-start network on solver-generated tiles and measure what it buys.

``train_and_evaluate`` generates random tiles (four-state cells, Bernoulli
wordline inputs), solves them with the line solver for the targets, trains with
Adam, then on a fresh inference batch reports the prediction error, the network's
own throughput, and for both solvers the iterations (line) or sweeps (red-black
SOR) from the ideal state and from the prediction, the fallback (rejection) rate
and the end-to-end solves/s including inference.

  python -m fadesim_gb300.warmstart_eval [--size 128] [--train 200000] [--infer 8192] [--cells weak|strong|sinh]
  python -m fadesim_gb300.warmstart_eval --conv [--conv-shape N,H,W,Cin,Cout]   (one convolution, both kernels)
"""
import argparse
import json
import time

import torch

from . import cpp_ir_drop_accelerate as acc
from . import warmstart as ws

R_STATES = (2e6, 1.6e6, 1.3e6, 1e6)
# 2-bit cells between 1 kohm and 1 Mohm, linear in conductance (the MLP layers' arrays)
G_STRONG = tuple(1e-6 + k * (1e-3 - 1e-6) / 3 for k in range(4))
# sinh cells I = (V / R) sinh(2V) / (2V) between 1 and 2 Mohm: [R_on, R_off, a_on, b_on, a_off, b_off]
SINH_PARAMS = (1e6, 2e6, 2.0, 1.0 / (2.0 * 1e6), 2.0, 1.0 / (2.0 * 2e6))


def _timed(fn):
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    r = fn()
    e1.record()
    torch.cuda.synchronize()
    return r, e0.elapsed_time(e1) / 1e3


def train_and_evaluate(size=128, train_instances=200000, batch=64, infer=8192, lr=1e-3, g_wire=1 / 2.93, seed=0,
                       cells="weak", sor_omegas=(1.96, 1.98), sor_sample=304):
    """Train on ``train_instances`` solver-generated tiles of the given cells
    ("weak": four states 1-2 Mohm; "strong": 2-bit 1 kohm - 1 Mohm; both with
    Bernoulli 0.2 V inputs; "sinh": the large non-ideal setting -- four states
    1-2 Mohm with lognormal variation sigma 0.1, sinh cells, inputs uniform in
    [0, 0.2] V), then on a fresh batch of ``infer`` tiles report the
    prediction error, the network's throughput, and for the line solver and the
    plain red-black SOR the iterations / sweeps from the ideal state and from
    the prediction, the fallback rate (predictions the line solver discarded)
    and solves/s with and without the warm start, inference included."""
    n = size
    gvals = torch.tensor(G_STRONG if cells == "strong" else [1.0 / r for r in R_STATES])
    gen = torch.Generator().manual_seed(seed)
    sinh = cells == "sinh"
    nl = dict(nonlinear_cell_enable=True, nonlinear_params=SINH_PARAMS) if sinh else {}
    draws = [0]

    def draw(N):
        G = gvals[torch.randint(0, len(gvals), (N, n, n), generator=gen)].float().cuda()
        if sinh:
            # the large non-ideal setting: lognormal variation, inputs uniform in [0, 0.2] V
            from .variation import add_variation_device
            draws[0] += 1
            G = add_variation_device(G, 0.1, seed=seed * 1000 + draws[0])
            vin = (torch.rand((N, n), generator=gen) * 0.2).cuda()
        else:
            vin = (torch.randint(0, 2, (N, n), generator=gen).float() * 0.2).cuda()
        return G, vin

    def solve_planes(G, vin):
        N = G.shape[0]
        planes, _, _ = acc.ir_drop_gs_ex(vin[None].contiguous(), G.contiguous(), 1, n, n, N, 1, g_wire=g_wire,
                                         ret_V=2, method="line", **nl)
        p = planes[0, :, 0].clone()
        p[:, 0] -= vin[:, :, None]
        return p

    net = ws.WarmStartNet(seed=seed)
    steps = max(1, train_instances // batch)
    t0 = time.perf_counter()
    losses = []
    for _ in range(steps):
        G, vin = draw(batch)
        x, _ = net.make_inputs(G, vin)
        losses.append(net.train_step(x, ws.solver_targets(G, vin, solve_planes), lr=lr))
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    G, vin = draw(infer)
    net.predict_planes(G[:batch], vin[:batch])  # warm-up
    pred, t_inf = _timed(lambda: net.predict_planes(G, vin))
    true = solve_planes(G, vin)
    rel = float((pred - true).norm() / true.norm())
    ti = vin[None].contiguous()
    init = pred[None, :, None].contiguous()
    (_, cold, _), t_cold = _timed(lambda: acc.ir_drop_gs_ex(ti, G, 1, n, n, infer, 1, g_wire=g_wire, method="line",
                                                            **nl))
    (_, warm, _), t_warm = _timed(lambda: acc.ir_drop_gs_warm(ti, G, 1, n, n, infer, 1, init, g_wire=g_wire,
                                                              nonlinear_params=SINH_PARAMS if sinh else None))
    line = {"iters_mean_cold": cold["iters_sum"] / cold["solves"], "iters_mean_warm": warm["iters_sum"] / warm["solves"],
            "iters_saved_frac": 1 - warm["iters_sum"] / cold["iters_sum"],
            "fallback_rate": warm["warm_rejected"] / warm["solves"],
            "solves_per_s_cold": infer / t_cold, "solves_per_s_warm_excl_inference": infer / t_warm,
            "solves_per_s_warm_incl_inference": infer / (t_warm + t_inf)}
    line["net_gain_incl_inference"] = line["solves_per_s_warm_incl_inference"] / line["solves_per_s_cold"]
    out = {
        "tile": "%dx%d" % (n, n), "cells": cells, "train_instances": steps * batch, "train_s": train_s,
        "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
        "infer_batch": infer, "infer_instances_per_s": infer / t_inf, "prediction_rel_err": rel,
        "line": line, "rbsor": {},
    }
    k = min(sor_sample, infer)
    tis = vin[None, :k].contiguous()
    Gs = G[:k].contiguous()
    inits = pred[None, :k, None].contiguous()
    for w in sor_omegas:
        (_, c, _), tc = _timed(lambda: acc.ir_drop_gs_ex(tis, Gs, 1, n, n, k, 1, g_wire=g_wire, method="rbsor",
                                                         omega=w))
        (_, wm, _), tw = _timed(lambda: acc.ir_drop_gs_warm(tis, Gs, 1, n, n, k, 1, inits, g_wire=g_wire,
                                                            method="rbsor", omega=w))
        r = {"sweeps_mean_cold": c["iters_sum"] / c["solves"], "sweeps_mean_warm": wm["iters_sum"] / wm["solves"],
             "sweeps_saved_frac": 1 - wm["iters_sum"] / c["iters_sum"], "solves_per_s_cold": k / tc,
             "solves_per_s_warm_incl_inference": k / (tw + t_inf * k / infer)}
        r["net_gain_incl_inference"] = r["solves_per_s_warm_incl_inference"] / r["solves_per_s_cold"]
        out["rbsor"]["omega_%.2f" % w] = r
    return out


def conv_throughput(N=64, H=128, W=128, cin=64, cout=32, reps=10, legacy=False):
    """Time one 3x3 convolution of the network (default: the d1 layer, 64 -> 32
    channels at 128 x 128, batch 64) on the tensor-core kernel (tcgen05 / TMA)
    or, with ``legacy``, the mma.sync kernel.  Returns ms per launch and
    TFLOP/s (2 * 9 * Cin * Cout flops per output pixel)."""
    g = torch.Generator().manual_seed(1)
    x = torch.randn((N, H, W, cin), generator=g).to(torch.bfloat16).cuda()
    conv = ws.Conv(cin, cout, g, "cuda")
    for _ in range(2):
        conv.fwd(x, relu=True, legacy=legacy)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        conv.fwd(x, relu=True, legacy=legacy)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    flops = 2.0 * 9 * cin * cout * N * H * W
    out = {"kernel": "mma.sync" if legacy else "tcgen05+TMA", "shape": "N%d %dx%d %d->%d" % (N, H, W, cin, cout),
           "ms": ms, "tflops": flops / (ms / 1e3) / 1e12}
    if not legacy:
        # the weight gradient of the same layer (tensor cores where Cin and Cout are multiples of 32)
        dy = torch.randn((N, H, W, cout), generator=g).to(torch.bfloat16).cuda()
        for _ in range(2):
            conv.bwd(dy, x, need_dx=False)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            conv.bwd(dy, x, need_dx=False)
        e1.record()
        torch.cuda.synchronize()
        wms = e0.elapsed_time(e1) / reps
        out.update({"wgrad_tc": bool(ws._k().fadesim_conv_tc_shape(H, W, cin, cout) & 2), "wgrad_ms": wms,
                    "wgrad_tflops": flops / (wms / 1e3) / 1e12})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--train", type=int, default=200000, help="training instances")
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--infer", type=int, default=8192)
    ap.add_argument("--cells", default="weak", choices=["weak", "strong", "sinh"])
    ap.add_argument("--conv", action="store_true",
                    help="only time one network convolution on both kernels (for profiling)")
    ap.add_argument("--conv-shape", default="64,128,128,64,32", help="N,H,W,Cin,Cout of --conv")
    a = ap.parse_args()
    if a.conv:
        from .build import build
        build()
        N, H, W, cin, cout = (int(v) for v in a.conv_shape.split(","))
        print(json.dumps([conv_throughput(N, H, W, cin, cout), conv_throughput(N, H, W, cin, cout, legacy=True)]))
        return
    print(json.dumps(train_and_evaluate(a.size, a.train, a.batch, a.infer, cells=a.cells,
                                        sor_omegas=() if a.cells == "sinh" or a.size > 128 else (1.96, 1.98))))


if __name__ == "__main__":
    main()
