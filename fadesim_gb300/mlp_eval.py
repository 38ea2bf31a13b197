"""Layer-level PimTorch inference on the GPU: an MLP 784-512-512-10 of Linear_sp
layers evaluated on crossbars.

Weights ~ N(0, 0.05^2) (torch seed 3), quantised to signed 8-bit and mapped as
differential (PN) pairs onto 2-bit cells (4 slices per weight) in 128 x 128
crossbars with 1 kohm / 1 Mohm cells and 2.93 ohm wires; inputs are a batch of
256 synthetic 28 x 28 images uniform in [0, 255], fed bit-serially (8 cycles,
1-bit DAC, 0.2 V read); every slice x cycle goes through the IR-drop solve, then
an 8-bit ADC and shift-add (fixedPoint/nn/modules/linear_split.py,
splitArrayArithmetic.py:1161-1260).  ReLU between layers, no bias.

``run`` times one batch through the three layers with a given solver strategy:
"direct" solves every (tile, input vector) pair; "direct_coarse" does the same
with the two-level line relaxation (method "line_coarse": a coarse-grid
correction after every iteration on the strongly coupled tiles);
"superposition" solves each tile's unit responses (to the FP32 limit) and forms
the currents by linearity (linear cells, no read noise); "superposition_fast"
stops its unit responses at the plain stop test's FP32 floor.

  python -m fadesim_gb300.mlp_eval [--batch 256]
"""
import argparse
import json

import torch

from . import splitarr

SIZES = (784, 512, 512, 10)


def config():
    return splitarr.ArrayConfig(Ron=1e3, Roff=1e6, cellBits=2, arrRowSize=128, arrColSize=128, inputMaxVoltage=0.2,
                                r_wire=2.93)


def build(seed=3):
    g = torch.Generator().manual_seed(seed)
    return [(torch.randn((o, i), generator=g) * 0.05).cuda() for i, o in zip(SIZES[:-1], SIZES[1:])]


def solves_per_batch(batch, cfg, input_bits=8, weight_bits=8):
    rows, cols = cfg.arrRowSize, cfg.arrColSize
    total = []
    for i, o in zip(SIZES[:-1], SIZES[1:]):
        numX, numY = -(-i // rows), -(-o // cols)
        total.append(input_bits * batch * numX * numY * (weight_bits // cfg.cellBits) * 2)
    return total


def forward(x, weights, cfg, solver):
    for k, w in enumerate(weights):
        x = splitarr.splitArr_matmul_nn(x, w.t().contiguous(), 8, 1, 8, 10, 8, "PN", torch.float32, cfg=cfg,
                                        solver=solver)
        if k + 1 < len(weights):
            x = torch.relu(x)
    return x


def run(batch=256, strategy="direct", seed=3, reps=1):
    from . import cpp_ir_drop_accelerate as acc
    cfg = config()
    weights = build(seed)
    g = torch.Generator().manual_seed(seed + 1)
    x = torch.randint(0, 256, (batch, SIZES[0]), generator=g).float().cuda()
    if strategy.startswith("superposition"):
        solver = splitarr.superposition_solver(cfg, fp32_limit=strategy == "superposition")
    else:
        solver = splitarr.default_solver(cfg)
    method = acc.options.method
    if strategy == "direct_coarse":
        acc.options.method = "line_coarse"
    try:
        y = forward(x, weights, cfg, solver)  # warm-up (builds, tunes nothing)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            y = forward(x, weights, cfg, solver)
        e1.record()
        torch.cuda.synchronize()
    finally:
        acc.options.method = method
    ms = e0.elapsed_time(e1) / reps
    per_layer = solves_per_batch(batch, cfg)
    return y, {"ms_per_batch": ms, "solves_per_batch": sum(per_layer), "solves_per_layer": per_layer,
               "solves_per_s": sum(per_layer) / (ms / 1e3), "images_per_s": batch / (ms / 1e3)}


def current_agreement(batch=256, seed=3, fp32_limit=True):
    """Largest difference, relative to the largest current, between the two
    strategies' bitline currents on the solver call of layer 1 (all four weight
    slices of both arrays, all 8 input cycles of the batch)."""
    cfg = config()
    w = build(seed)[0]
    g = torch.Generator().manual_seed(seed + 1)
    x = torch.randint(0, 256, (batch, SIZES[0]), generator=g).float().cuda()
    seen = {}
    direct = splitarr.default_solver(cfg)

    def first_call(v, G, B, rows, cols, numX, numY, out):
        if not seen:
            seen["args"] = (v.clone(), G.clone(), B, rows, cols, numX, numY)
        return direct(v, G, B, rows, cols, numX, numY, out)

    splitarr.splitArr_matmul_nn(x, w.t().contiguous(), 8, 1, 8, 10, 8, "PN", torch.float32, cfg=cfg, solver=first_call)
    v, G, B, rows, cols, numX, numY = seen["args"]
    a = direct(v, G, B, rows, cols, numX, numY, None)
    b = splitarr.superposition_solver(cfg, fp32_limit)(v, G, B, rows, cols, numX, numY, None).reshape(a.shape)
    return float(((a - b).abs().max() / a.abs().max()).item())


def evaluate(batch=256):
    """The strategies on the same batch (direct solves, the same with the
    two-level method, superposition with unit responses to the FP32 limit and
    stopped at the floor), with their agreement.  The 8-bit ADC
    makes the network's outputs jump with any change of the currents near a code
    boundary (one code of the top input bit and weight slice moves a layer-1
    output by ~10%), so output-level agreement is shown next to the same
    comparison between two tolerances of the direct solve."""
    from . import cpp_ir_drop_accelerate as acc
    yd, direct = run(batch, "direct")
    yc, coarse = run(batch, "direct_coarse")
    coarse["equal_outputs_frac_vs_direct"] = float(((yd - yc).abs() == 0).float().mean().item())
    ys, sup = run(batch, "superposition")
    sup["max_rel_current_diff_vs_direct"] = current_agreement(batch)
    sup["equal_outputs_frac_vs_direct"] = float(((yd - ys).abs() == 0).float().mean().item())
    yf, fast = run(batch, "superposition_fast")
    fast["max_rel_current_diff_vs_direct"] = current_agreement(batch, fp32_limit=False)
    fast["equal_outputs_frac_vs_direct"] = float(((yd - yf).abs() == 0).float().mean().item())
    tol = acc.options.tol_v
    acc.options.tol_v = tol * 0.02
    try:
        yt, _ = run(batch, "direct")
    finally:
        acc.options.tol_v = tol
    direct["equal_outputs_frac_vs_tol_x0.02"] = float(((yd - yt).abs() == 0).float().mean().item())
    direct["tol_v"] = tol
    return {"workload": "MLP 784-512-512-10, batch %d, 128x128 PN crossbars, 2-bit cells (1k/1M ohm), 8 input "
                        "cycles at 0.2 V, 8-bit ADC" % batch, "direct": direct, "direct_coarse": coarse,
            "superposition": sup, "superposition_fast": fast}


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--batch", type=int, default=256)
    print(json.dumps(evaluate(ap.parse_args().batch)))
