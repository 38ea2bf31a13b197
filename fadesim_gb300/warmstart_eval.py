"""Train the warm-start network on solver-generated tiles and measure what it buys.

``train_and_evaluate`` generates random tiles (four-state cells, Bernoulli
wordline inputs), solves them with the line solver for the targets, trains with
Adam, then on a fresh inference batch reports the prediction error, the network's
own throughput, and for both solvers the iterations (line) or sweeps (red-black
SOR) from the ideal state and from the prediction, the fallback (rejection) rate
and the end-to-end solves/s including inference.

  python -m fadesim_gb300.warmstart_eval [--size 128] [--steps 600] [--infer 8192]
"""
import argparse
import json
import time

import torch

from . import cpp_ir_drop_accelerate as acc
from . import warmstart as ws

R_STATES = (2e6, 1.6e6, 1.3e6, 1e6)


def _timed(fn):
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    r = fn()
    e1.record()
    torch.cuda.synchronize()
    return r, e0.elapsed_time(e1) / 1e3


def train_and_evaluate(size=128, steps=600, batch=32, infer=8192, lr=1e-3, g_wire=1 / 2.93, seed=0,
                       sor_omegas=(1.90, 1.96), sor_sample=256):
    n = size
    Rs = torch.tensor(R_STATES)
    gen = torch.Generator().manual_seed(seed)

    def draw(N):
        G = (1.0 / Rs[torch.randint(0, len(R_STATES), (N, n, n), generator=gen)]).float().cuda()
        vin = (torch.randint(0, 2, (N, n), generator=gen).float() * 0.2).cuda()
        return G, vin

    def solve_planes(G, vin):
        N = G.shape[0]
        planes, _, _ = acc.ir_drop_gs_ex(vin[None].contiguous(), G.contiguous(), 1, n, n, N, 1, g_wire=g_wire,
                                         ret_V=2, method="line")
        p = planes[0, :, 0].clone()
        p[:, 0] -= vin[:, :, None]
        return p

    net = ws.WarmStartNet(seed=seed)
    t0 = time.perf_counter()
    losses = []
    for _ in range(steps):
        G, vin = draw(batch)
        x, _ = net.make_inputs(G, vin)
        losses.append(net.train_step(x, ws.solver_targets(G, vin, solve_planes), lr=lr))
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    G, vin = draw(infer)
    pred, t_inf = _timed(lambda: net.predict_planes(G, vin))
    true = solve_planes(G, vin)
    rel = float((pred - true).norm() / true.norm())
    ti = vin[None].contiguous()
    init = pred[None, :, None].contiguous()
    (_, cold, _), t_cold = _timed(lambda: acc.ir_drop_gs_ex(ti, G, 1, n, n, infer, 1, g_wire=g_wire, method="line"))
    (_, warm, _), t_warm = _timed(lambda: acc.ir_drop_gs_warm(ti, G, 1, n, n, infer, 1, init, g_wire=g_wire))
    rejected = int(warm["status_or"] & 8)
    out = {
        "tile": "%dx%d" % (n, n), "train_instances": steps * batch, "train_s": train_s,
        "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
        "infer_batch": infer, "infer_instances_per_s": infer / t_inf, "prediction_rel_err": rel,
        "line": {"iters_mean_cold": cold["iters_sum"] / cold["solves"], "iters_mean_warm": warm["iters_sum"] / warm["solves"],
                 "solves_per_s_cold": infer / t_cold, "solves_per_s_warm_incl_inference": infer / (t_warm + t_inf),
                 "any_rejected": bool(rejected)},
        "rbsor": {},
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
        out["rbsor"]["omega_%.2f" % w] = {
            "sweeps_mean_cold": c["iters_sum"] / c["solves"], "sweeps_mean_warm": wm["iters_sum"] / wm["solves"],
            "sweeps_saved_frac": 1 - wm["iters_sum"] / c["iters_sum"], "solves_per_s_cold": k / tc,
            "solves_per_s_warm_incl_inference": k / (tw + t_inf * k / infer)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--infer", type=int, default=8192)
    a = ap.parse_args()
    print(json.dumps(train_and_evaluate(a.size, a.steps, a.batch, a.infer)))


if __name__ == "__main__":
    main()
