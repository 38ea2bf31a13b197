"""Throughput of the crossbar IR-drop solve on GB300.

Workload (one step): 4096 independent 128x128 crossbar tiles, 64 input vectors
each (262,144 tile x vector solves), four-state cells R in {2e6, 1.6e6, 1.3e6,
1e6} ohm drawn uniformly, 2.93 ohm wire segments, wordline inputs
Bernoulli(0.5) in {0, 0.2} V, bitlines grounded, FP32.  Every solve is driven
to an estimated 5e-7 V of the nodal solution (the metric's 1e-6 V bound with a
2x margin on the estimate; --tol changes it); a seeded sample of 512 solves,
run exactly as the timed ones, is checked against the FP64 oracle before
timing.  Data are synthetic (seeded numpy generators).

Metric: 128x128 crossbar solves per second, whole job.  ``value`` is measured
with inputs resident in HBM; ``e2e`` through the public host-buffer call
(``ir_drop_gs_host``) with pinned host buffers and the host<->device copies,
which the library pipelines with the solve, inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank solves its own 4096 tiles (weak scaling, no
collective on the data path); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TILES = 4096
N_VEC = 64
ROWS = COLS = 128
R_STATES = np.array([2e6, 1.6e6, 1.3e6, 1e6])
R_WIRE = 2.93
V_READ = 0.2
METRIC = "128x128 crossbar solves/s (<=1e-6 V node error)"
TOL_V = 5e-7  # stop when the estimated max node error is below this (volts)
UNIT = "solves/s"
# algorithmic HBM bytes per solve: G amortised over the tile's vectors, the
# input vector and the output currents, FP32
BYTES_PER_SOLVE = (ROWS * COLS * 4) / N_VEC + ROWS * 4 + COLS * 4
# algorithmic shared-memory bytes per node update of a line pass: the node's own
# value read for the residual and again for the update, one write, the other
# plane's node, the cell conductance, and the input voltage on bitline passes
SMEM_BYTES_PER_NODE_UPDATE = 4 * (2 + 1 + 1 + 1 + 0.5)
SMEM_BYTES_PER_CLK_SM = 128  # shared-memory bandwidth per SM per clock (32 banks x 4 B), nominal
N_SMS = 152
# algorithmic FP32 flops per node update of a line pass, an FMA counted as two
# flops like the peak below: the residual (cell voltage and its difference from
# the node: 2 adds; the two neighbour differences and their sum: 3 adds; the
# cell term, an FMA: 2), the Thomas forward step c r + c y (a multiply and an
# FMA: 3), the backward step y + c x (an FMA: 2) and the relaxed update
# omega x + own (an FMA: 2)
FP32_FLOPS_PER_NODE_UPDATE = 14
FP32_FLOPS_PER_CLK_SM = 256  # 128 FP32 lanes x 2 flops (FMA)


def fp32_roofline(node_updates, kern_ms, sm_mhz):
    """The line kernel against the FP32 pipe: algorithmic FP32 flops of its node
    updates per second over the nominal FMA rate at the sampled clock, both
    counting an FMA as two flops."""
    achieved = FP32_FLOPS_PER_NODE_UPDATE * node_updates / (kern_ms / 1e3) / 1e12
    peak = FP32_FLOPS_PER_CLK_SM * N_SMS * sm_mhz * 1e6 / 1e12
    return {"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_kind": "nominal: 128 FP32 FMA lanes/clk/SM x 2 flops at the sampled clock",
            "flops_per_node_update": FP32_FLOPS_PER_NODE_UPDATE, "fma_counts_as": 2}


def measured_smem_peak(torch, lib, reps=5):
    """Shared-memory read bandwidth of this GPU (GB/s), measured with the
    library's probe kernel (fadesim_smem_read_probe): 16 CTAs of 1024 threads
    per SM, 4096 conflict-free 16-byte reads per thread, best of ``reps`` CUDA-
    event timings, no clock changes."""
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    blocks, iters = 16 * sms, 4096
    sink = torch.zeros(blocks, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    if lib.fadesim_smem_read_probe(sink.data_ptr(), blocks, 512, st.cuda_stream) != 0:
        raise RuntimeError("shared-memory probe launch failed")
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        lib.fadesim_smem_read_probe(sink.data_ptr(), blocks, iters, st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return blocks * 1024 * iters * 16 / (best / 1e3) / 1e9, sms


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """Per-solve DRAM bytes of the line kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "line_relax_f32_128x128.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_solve"):
            return float(line.split("=")[1].split()[0])
    return None


class Clocks:
    """nvidia-smi sampler over the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_workload(seed, n_tiles=N_TILES, n_vec=N_VEC):
    rng = np.random.default_rng(seed)
    states = rng.integers(0, 4, (n_tiles, ROWS, COLS), dtype=np.int8)
    G = (1.0 / R_STATES)[states].astype(np.float32)                  # [numX=tiles, rows, cols]
    vin = (rng.integers(0, 2, (n_vec, n_tiles, ROWS)) * V_READ).astype(np.float32)  # [B, numX, rows]
    return G, vin


def cpu_baseline(seconds=12.0, max_solves=4096):
    """The reference's Au solve (C restatement of V1 nodeBasedGS) on all host
    cores over a bounded sample of the same workload."""
    from oracle import augs
    augs.build()
    threads = augs.max_threads()
    G, vin = make_workload(12345, n_tiles=64, n_vec=1)
    w = float(np.float32(1.95))
    done, t0 = 0, time.perf_counter()
    batch = threads
    while True:
        k0 = done % 64
        idx = [(k0 + q) % 64 for q in range(batch)]
        augs.solve_many(G[idx].astype(np.float64), vin[0, idx].astype(np.float64), R_WIRE, 100000, w, True, 1e-9)
        done += batch
        el = time.perf_counter() - t0
        if el >= seconds or done >= max_solves:
            break
    return {"value": done / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d solves of 128x128 (Au lexicographic GS, omega 1.95, delta tol 1e-9 which meets "
                      "1e-6 V) over %d threads in %.1f s" % (done, threads, el)}


def cpu_mixed_baseline(seconds_per_size=4.0, sizes=(64, 128, 256), tiles_by_size=None):
    """The reference's Au solve on all host cores for the mixed-size batch,
    extrapolated from a stratified sample: each tile size timed on its own
    bounded sample (same cells, Bernoulli 0.2 V inputs, omega 1.95, delta tol
    1e-9), the batch's rate then the harmonic combination by the batch's
    share of each size."""
    from oracle import augs
    augs.build()
    threads = augs.max_threads()
    w = float(np.float32(1.95))
    rates, notes = {}, []
    for n in sizes:
        rng = np.random.default_rng(100 + n)
        G = (1.0 / R_STATES)[rng.integers(0, 4, (threads, n, n))].astype(np.float64)
        v = (rng.integers(0, 2, (threads, n)) * V_READ).astype(np.float64)
        done, t0 = 0, time.perf_counter()
        while True:
            augs.solve_many(G, v, R_WIRE, 200000, w, True, 1e-9)
            done += threads
            el = time.perf_counter() - t0
            if el >= seconds_per_size:
                break
        rates[n] = done / el
        notes.append("%d of %dx%d in %.1f s" % (done, n, n, el))
    share = tiles_by_size or {n: 1 for n in sizes}
    tot = float(sum(share[n] for n in sizes))
    mix = tot / sum(share[n] / rates[n] for n in sizes)
    return {"value": mix, "unit": UNIT, "cores": threads, "kind": "port",
            "by_size": {str(n): rates[n] for n in sizes},
            "sample": "stratified: " + ", ".join(notes) + " (Au lexicographic GS, omega 1.95, delta tol 1e-9, "
                      "%d threads); the batch rate combines them by its tile shares" % threads}


def side_figure(fn):
    """One of the figures reported beside the headline: an error in it is
    reported in its place instead of taking the JSON line with it (a CUDA error
    that leaves the context unusable still ends the run at the next launch)."""
    try:
        return fn()
    except (ArithmeticError, AttributeError, LookupError, RuntimeError, TypeError, ValueError) as e:
        return {"error": "%s: %s" % (type(e).__name__, e)}


def workload_name(tiles):
    """The benchmarked workload, named the same way on both arms."""
    return ("%d tiles x %d vectors of 128x128 per rank (ir_drop_gs layout B=%d, numX=%d, numY=1), 4-state cells, "
            "2.93 ohm wires, Bernoulli 0.2 V inputs" % (tiles, N_VEC, N_VEC, tiles))


def run_reference(args):
    from fadesim_gb300.ranks import rank_env
    if rank_env()[0] != 0:
        return  # the host-core reference runs once, on rank 0
    steps = []
    for _ in range(args.warmup):
        cpu_baseline(seconds=2.0)
    for _ in range(args.steps):
        steps.append(cpu_baseline(seconds=6.0))
    v = statistics.median(s["value"] for s in steps)
    cb = dict(steps[-1])
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(args.tiles),
                       "solver": "reference Au GS (V1 nodeBasedGS, C restatement) on host cores, each step a "
                                 "bounded sample of the workload (see cpu_baseline.sample)"},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def mixed_batch(torch, tol, n_tiles=4096, n_vec=64, seed=2, steps=3):
    """4096 tiles with sizes drawn uniformly from {64, 128, 256}^2 (square), 64
    Bernoulli 0.2 V vectors each, one CUDA-graph replay per step."""
    from fadesim_gb300 import cpp_ir_drop_accelerate as _acc
    from fadesim_gb300.batched import TileBatch, TileGroup
    rng = np.random.default_rng(seed)
    sizes = rng.choice([64, 128, 256], size=n_tiles)
    groups = []
    for n in (64, 128, 256):
        T = int((sizes == n).sum())
        states = rng.integers(0, 4, (T, n, n), dtype=np.int8)
        G = torch.from_numpy((1.0 / R_STATES)[states].astype(np.float32)).cuda()
        v = torch.from_numpy((rng.integers(0, 2, (n_vec, T, n)) * V_READ).astype(np.float32)).cuda()
        groups.append(TileGroup(G, v))
    batch = TileBatch(groups, g_wire=1 / R_WIRE, tol_v=tol, tuned=True)
    t0 = time.perf_counter()
    tuned = batch.tune()  # the autotuner on a sample of every group (outside the timed region)
    tune_s = time.perf_counter() - t0
    st = batch.run(stats=True)
    batch.capture()
    batch.replay()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        batch.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # the plain red-black SOR on a sample of the same mix (the comparator at every size)
    rb = {}
    for g in groups:
        k, nv = min(g.T, 152), 4  # enough work items to fill the GPU
        vs, Gs = g.vin[:nv, :k].contiguous(), g.G[:k].contiguous()
        _acc.ir_drop_gs_ex(vs, Gs, nv, g.n, g.n, k, 1, g_wire=1 / R_WIRE, method="rbsor", tol_v=tol)
        torch.cuda.synchronize()
        p0 = time.perf_counter()
        _, rst, _ = _acc.ir_drop_gs_ex(vs, Gs, nv, g.n, g.n, k, 1, g_wire=1 / R_WIRE, method="rbsor", tol_v=tol)
        torch.cuda.synchronize()
        rb[str(g.n)] = {"solves_per_s": k * nv / (time.perf_counter() - p0),
                        "sweeps_mean": rst["iters_sum"] / max(1, rst["solves"]), "status_or": rst["status_or"]}
    # the mix at the red-black rates: total time = sum over sizes of solves / rate
    rb_mix = batch.solves / sum(g.solves / rb[str(g.n)]["solves_per_s"] for g in groups)
    return {"workload": "4096 tiles, sizes uniform in {64,128,256}^2, 64 vectors each, one CUDA graph",
            "tol_v": tol,
            "tuned": {k: v[0] for k, v in tuned.items()}, "tune_s": tune_s,
            "plain_rbsor_by_size": rb, "plain_rbsor_mix_solves_per_s": rb_mix,
            "tiles_by_size": {str(g.n): g.T for g in groups}, "solves_per_step": batch.solves,
            "ms_per_step": ms, "solves_per_s": batch.solves / (ms / 1e3),
            "nodes_per_s": sum(g.solves * 2 * g.n * g.n for g in groups) / (ms / 1e3),
            "iters_max_by_size": {str(g.n): s["iters_max"] for g, s in zip(groups, st)},
            "status_or": int(np.bitwise_or.reduce([s["status_or"] for s in st])),
            "speedup_vs_plain_rbsor_mix": batch.solves / (ms / 1e3) / rb_mix}


def large_nonideal(torch, acc, n_tiles=1024, n_vec=32, seed=5):
    """1024 tiles of 512x512 on 16-CTA clusters with sinh cells I = (V/R)
    sinh(2V)/(2V), lognormal R variation (sigma 0.1), 1% Gaussian read noise, 32
    inputs per tile uniform in [0, 0.2] V."""
    from fadesim_gb300.variation import add_variation_device
    rng = np.random.default_rng(seed)
    n = 512
    states = rng.integers(0, 4, (n_tiles, n, n), dtype=np.int8)
    G = torch.from_numpy((1.0 / R_STATES)[states].astype(np.float32)).cuda()
    G = add_variation_device(G, 0.1, seed=seed)
    v = torch.from_numpy((rng.random((n_vec, n_tiles, n)) * V_READ).astype(np.float32)).cuda()
    params = [1e6, 2e6, 2.0, 1.0 / (2.0 * 1e6), 2.0, 1.0 / (2.0 * 2e6)]
    kw = dict(g_wire=1 / R_WIRE, nonlinear_cell_enable=True, nonlinear_params=params, method="line",
              read_noise_sigma=0.01, noise_seed=seed)
    _, st, _ = acc.ir_drop_gs_ex(v, G, n_vec, n, n, n_tiles, 1, **kw)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    acc.ir_drop_gs_ex(v, G, n_vec, n, n, n_tiles, 1, return_stats=False, **kw)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"workload": "%d tiles 512x512 (16-CTA clusters) x %d vectors U[0,0.2] V, sinh cells a=2, "
                        "lognormal sigma 0.1, 1%% read noise" % (n_tiles, n_vec),
            "solves": n_tiles * n_vec, "ms": ms, "solves_per_s": n_tiles * n_vec / (ms / 1e3),
            "node_updates_per_s": n_tiles * n_vec * 2 * n * n * st["iters_sum"] / st["solves"] / (ms / 1e3),
            "line_iters_mean": st["iters_sum"] / st["solves"], "status_or": st["status_or"]}


def reference_sweep_order(torch, acc, G, vin, k=2, sweeps=600, omega=1.90):
    """The reference extension's algorithm on this GPU at the reference's
    settings: ``iter_times`` point-SOR sweeps of the two planes in its order
    (one launch per sweep, a thread per line), no early break, FP32; k tiles x
    all their vectors.  Returns solves/s and the sample's max node error against
    the FP64 oracle (the sweep count is the reference's, not a tolerance)."""
    from oracle import nodal
    nv = vin.shape[0]
    tg = torch.from_numpy(np.ascontiguousarray(G[:k])).cuda()
    ti = torch.from_numpy(np.ascontiguousarray(vin[:, :k])).cuda()
    kw = dict(iter_times=sweeps, beta=omega, g_wire=1 / R_WIRE, method="sweeps")
    acc.ir_drop_gs_ex(ti[:1, :1].contiguous(), tg[:1].contiguous(), 1, ROWS, COLS, 1, 1, **kw)  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    acc.ir_drop_gs_ex(ti, tg, nv, ROWS, COLS, k, 1, return_stats=False, **kw)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    planes, _, _ = acc.ir_drop_gs_ex(ti[:4, :1].contiguous(), tg[:1].contiguous(), 4, ROWS, COLS, 1, 1, ret_V=2,
                                     **kw)
    planes = planes.double().cpu().numpy()
    u, d = nodal.solve(G[0].astype(np.float64), 1 / R_WIRE, vin[:4, 0].astype(np.float64))
    err = float(max(np.abs(planes[:, 0, 0, 0] - u).max(), np.abs(planes[:, 0, 0, 1] - d).max()))
    return {"solves_per_s": nv * k / (ms / 1e3), "sweeps": sweeps, "omega": omega, "sample": "%d tiles x %d "
            "vectors, FP32" % (k, nv), "max_node_err_v_sample": err,
            "note": "the reference's ir_drop_gs algorithm (split_arr_matmul.cu:27-119,204-333) restated in "
                    "csrc/sweeps.cu at its default 600 sweeps, omega 1.90"}


def check_accuracy(acc, G, vin, torch, k=None):
    """Max node error over both planes of k tiles x all their vectors, solved as
    the timed run solves them (same options, one work item per tile), against
    the FP64 oracle.  Float64 inputs give float64 planes, so the comparison is
    not limited by FP32 rounding of the output (the solve itself is FP32)."""
    from oracle import nodal
    k = k or (8 if ROWS <= 128 else 2)
    nv = vin.shape[0]
    tg = torch.from_numpy(G[:k].astype(np.float64)).cuda()
    ti = torch.from_numpy(np.ascontiguousarray(vin[:, :k]).astype(np.float64)).cuda()
    planes, _, _ = acc.ir_drop_gs_ex(ti, tg, nv, ROWS, COLS, k, 1, g_wire=1 / R_WIRE, ret_V=2, method="line",
                                     vectors_per_cta=nv)
    planes = planes.cpu().numpy()
    # the currents as the timed run returns them (FP32 in and out)
    cur, _, _ = acc.ir_drop_gs_ex(ti.float(), tg.float(), nv, ROWS, COLS, k, 1, g_wire=1 / R_WIRE, method="line",
                                  vectors_per_cta=nv)
    cur = cur.double().cpu().numpy()
    err = cerr = 0.0
    for x in range(k):
        u, d = nodal.solve(G[x].astype(np.float64), 1 / R_WIRE, vin[:, x].astype(np.float64))
        err = max(err, np.abs(planes[:, x, 0, 0] - u).max(), np.abs(planes[:, x, 0, 1] - d).max())
        ref = nodal.currents(G[x].astype(np.float64), u, d)
        cerr = max(cerr, np.abs(cur[:, x] - ref).max() / np.abs(ref).max())
    return err, cerr


def run_ours(args):
    import torch
    from fadesim_gb300 import ranks
    rank, world, local = ranks.rank_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from fadesim_gb300 import cpp_ir_drop_accelerate as acc
    from fadesim_gb300.build import build
    build()
    acc.options.tol_v = args.tol  # every call below, the drop-in included

    G, vin = make_workload(ranks.workload_seed(1000, rank), n_tiles=args.tiles)
    tg = torch.from_numpy(G).cuda()
    ti = torch.from_numpy(vin).cuda()
    B, X, Y = N_VEC, args.tiles, 1
    gw = 1 / R_WIRE
    err, cerr = check_accuracy(acc, G, vin, torch)
    stream = torch.cuda.current_stream()

    def step():
        if args.quick_method != "line":  # profiling the plain comparator
            return acc.ir_drop_gs_ex(ti, tg, B, ROWS, COLS, X, Y, g_wire=gw, method=args.quick_method,
                                     return_stats=False)[0]
        return acc.ir_drop_gs(ti, tg, B, ROWS, COLS, X, Y, 600, gw, 1.9, False, 1e-7, False, [], False)

    for _ in range(max(3, args.warmup)):
        out = step()
    torch.cuda.synchronize()
    _, stats, _ = acc.ir_drop_gs_ex(ti, tg, B, ROWS, COLS, X, Y, g_wire=gw, method=args.quick_method)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for s in range(args.steps):
            ev[s][0].record(stream)
            out = step()
            ev[s][1].record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    kern_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    ms = ranks.max_over_ranks(t0.elapsed_time(t1), dist, "cuda")
    solves_per_step = B * X * Y
    value = ranks.job_rate(solves_per_step * args.steps, world, ms)
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "quick": True, "tiles": X,
                              "tile_size": ROWS,
                              "kernel_ms": kern_ms, "line_iters_mean": stats["iters_sum"] / max(1, stats["solves"]),
                              "max_node_err_v_sample": err, "max_rel_current_err_sample": cerr,
                              "clocks": clk.summary()}))
        if dist:
            dist.destroy_process_group()
        return

    # end to end through the public host-buffer call (fadesim_ir_drop_gs_host):
    # pinned host inputs in, currents out, the library's copies pipelined with
    # the solve over tile groups; host-synchronous, timed on the host clock
    hG = torch.from_numpy(G).pin_memory()
    hv = torch.from_numpy(vin).pin_memory()
    hout = torch.empty((B, X, Y * COLS), dtype=torch.float32).pin_memory()
    del out
    for _ in range(max(3, args.warmup)):
        acc.ir_drop_gs_host(hv, hG, B, ROWS, COLS, X, Y, 600, gw, out=hout)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    h0 = time.perf_counter()
    for _ in range(args.steps):
        acc.ir_drop_gs_host(hv, hG, B, ROWS, COLS, X, Y, 600, gw, out=hout)
    torch.cuda.synchronize()
    e2e_ms = ranks.max_over_ranks((time.perf_counter() - h0) * 1e3, dist, "cuda")
    e2e_value = ranks.job_rate(solves_per_step * args.steps, world, e2e_ms)
    # the same through the device-buffer drop-in with the caller's own copies
    # (copy in, solve, copy out in sequence on one stream), for comparison
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        o = acc.ir_drop_gs(hv.cuda(non_blocking=True), hG.cuda(non_blocking=True), B, ROWS, COLS, X, Y, 600, gw,
                           1.9, False, 1e-7, False, [], False)
        hout.copy_(o, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_serial_value = ranks.job_rate(solves_per_step * args.steps, world,
                                      ranks.max_over_ranks(e0.elapsed_time(e1), dist, "cuda"))

    # the same step under the other residual precisions (one timed step each)
    variants = {}
    for vname, kw in [("fp32_residual_only", dict(residual_period=-1)), ("native_fp64_residual", dict(residual="fp64")),
                      ("float_float_every_iteration", dict(residual_period=1)), ("tol_1e-8", dict(tol_v=1e-8))]:
        acc.ir_drop_gs_ex(ti, tg, B, ROWS, COLS, X, Y, g_wire=gw, method="line", return_stats=False, **kw)
        v0 = torch.cuda.Event(enable_timing=True)
        v1 = torch.cuda.Event(enable_timing=True)
        v0.record(stream)
        acc.ir_drop_gs_ex(ti, tg, B, ROWS, COLS, X, Y, g_wire=gw, method="line", return_stats=False, **kw)
        v1.record(stream)
        torch.cuda.synchronize()
        variants[vname + "_solves_per_s"] = solves_per_step / (v0.elapsed_time(v1) / 1e3)

    # the mixed-size batch (tiles of 64, 128 and 256)
    def mixed_section():
        m = mixed_batch(torch, args.tol)
        if rank == 0 and world == 1:
            # the reference's CPU algorithm on the same mix (stratified sample, host cores)
            shares = {int(k): v for k, v in m["tiles_by_size"].items()}
            m["cpu_baseline"] = cpu_mixed_baseline(tiles_by_size=shares)
            m["speedup_vs_cpu_reference"] = m["solves_per_s"] / m["cpu_baseline"]["value"]
        return m

    def mlp_section():
        # the layer-level MLP inference (PimTorch Linear_sp path on crossbars)
        from fadesim_gb300 import mlp_eval
        return mlp_eval.evaluate(256)

    mixed = side_figure(mixed_section) if not args.no_mixed else None
    large = side_figure(lambda: large_nonideal(torch, acc)) if not args.no_mixed else None
    mlp = side_figure(mlp_section) if not args.no_mixed else None
    def warm_section():
        from fadesim_gb300.warmstart_eval import train_and_evaluate
        # config 4 as specified (200k solver-generated instances of the four-state
        # 1-2 Mohm cells) and the strong 1 kohm - 1 Mohm cells of the MLP layers,
        # where the line solver needs ~20 iterations instead of 2
        from fadesim_gb300.warmstart_eval import conv_throughput
        conv_tc, conv_legacy = conv_throughput(), conv_throughput(legacy=True)
        bf16_peak = 1929.8
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                bf16_peak = float(json.load(f)["bf16_tflops"])
        except (OSError, ValueError, KeyError):
            pass
        return {"conv_roofline": {"bound": "tensor", "achieved": conv_tc["tflops"], "peak": bf16_peak,
                                  "unit": "TFLOP/s", "frac": conv_tc["tflops"] / bf16_peak,
                                  "peak_kind": "measured cuBLAS bf16 burst", "tensor_core": conv_tc,
                                  "mma_sync_kernel": conv_legacy},
                "weak_cells": train_and_evaluate(size=ROWS, train_instances=200000, batch=64, infer=8192,
                                                 cells="weak"),
                "strong_cells": train_and_evaluate(size=ROWS, train_instances=65536, batch=64, infer=8192,
                                                   cells="strong"),
                # the large non-ideal setting: 512 x 512 sinh cells with variation, on the
                # cluster kernels (the network is fully convolutional: any tile size)
                "sinh_cells_512": train_and_evaluate(size=512, train_instances=4096, batch=8, infer=512,
                                                     cells="sinh", sor_omegas=())}

    warm = side_figure(warm_section) if not args.no_warm else None

    # the plain red-black SOR kernel on a bounded sample of the same workload
    nps = 256
    tgs = tg[:nps // 16].contiguous()
    tis = ti[:16, :nps // 16].contiguous()
    acc.ir_drop_gs_ex(tis[:, :2].contiguous(), tgs[:2].contiguous(), 16, ROWS, COLS, 2, 1, g_wire=gw, method="rbsor")
    torch.cuda.synchronize()
    p0 = time.perf_counter()
    _, rb_stats, _ = acc.ir_drop_gs_ex(tis, tgs, 16, ROWS, COLS, nps // 16, 1, g_wire=gw, method="rbsor")
    torch.cuda.synchronize()
    rb_value = nps / (time.perf_counter() - p0)

    # the reference's own GPU algorithm at its defaults (ir_drop_gs: 600 point
    # sweeps at omega 1.90, no break; NN/commonConst.py:251-253), restated in
    # csrc/sweeps.cu, on 2 tiles x 64 vectors, with its error against the oracle
    ref_sweeps = reference_sweep_order(torch, acc, G, vin)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    hbm_peak, peak_kind = peaks()
    achieved = BYTES_PER_SOLVE * solves_per_step / (kern_ms / 1e3) / 1e9
    traffic = profiled_traffic()
    clk = clk_summary = clk.summary()
    node_updates = stats["iters_sum"] / max(1, stats["solves"]) * 2 * ROWS * COLS * solves_per_step
    smem_achieved = SMEM_BYTES_PER_NODE_UPDATE * node_updates / (kern_ms / 1e3) / 1e9
    smem_nominal = SMEM_BYTES_PER_CLK_SM * N_SMS * (clk_summary.get("sm_mhz") or 2070.0) * 1e6 / 1e9
    with Clocks(local) as pclk:
        smem_peak, sms = measured_smem_peak(torch, acc._lib.load())
    probe_clk = pclk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_name(X),
                   "solver": "block line relaxation: FP32 tridiagonal line solves; residual in FP32, and in "
                             "float-float (FP64-class) arithmetic on the iteration expected to be the last, which "
                             "must pass the stop test; tol %.0e V (estimated max node error)" % args.tol,
                   "method_note": "the headline solves every (tile, vector) from the ideal state, without the "
                                  "learned warm start: its speed-up over the plain red-black SOR comes from "
                                  "replacing point SOR by exact line solves; the learned warm start is reported "
                                  "separately (learned_warm_start)",
                   "accuracy_sample": "%d tiles x %d vectors solved as timed, FP64 oracle, both planes and "
                                      "the FP32 currents" % (8, N_VEC),
                   "l2": "inputs %.0f MB vs 129 MB L2, no flush" % ((G.nbytes + vin.nbytes) / 1e6),
                   "max_node_err_v_sample": err, "max_rel_current_err_sample": cerr,
                   "line_iters_mean": stats["iters_sum"] / max(1, stats["solves"]),
                   "line_iters_max": stats["iters_max"],
                   "plain_rbsor_solves_per_s": rb_value,
                   "plain_rbsor_sweeps_mean": rb_stats["iters_sum"] / max(1, rb_stats["solves"]),
                   "speedup_vs_plain_rbsor": value / world / rb_value,
                   "reference_sweep_order": ref_sweeps,
                   "speedup_vs_reference_sweep_order": value / world / ref_sweeps["solves_per_s"], **variants,
                   "e2e_path": "ir_drop_gs_host: pinned host buffers, copies pipelined over 8 tile groups on "
                               "3 streams, host clock",
                   "e2e_serial_copies_solves_per_s": e2e_serial_value,
                   "mixed_sizes": mixed, "large_nonideal": large, "mlp_layers": mlp, "learned_warm_start": warm},
        "roofline": {"bound": "smem", "achieved": smem_achieved, "peak": smem_peak, "unit": "GB/s",
                     "frac": smem_achieved / smem_peak,
                     "peak_kind": "measured: shared-memory read probe (fadesim_smem_read_probe, %d CTAs x 1024 "
                                  "threads, conflict-free 16-byte reads, best of 5) at %s MHz"
                                  % (16 * sms, probe_clk.get("sm_mhz")),
                     "bytes_per_node_update": SMEM_BYTES_PER_NODE_UPDATE, "node_updates_per_launch": node_updates,
                     "traffic": traffic * solves_per_step if traffic else None,
                     "traffic_note": "DRAM bytes per launch (ncu dram__bytes_read + write, profiles/"
                                     "line_relax_f32_128x128.txt, per solve x solves); shared-memory traffic is "
                                     "the achieved figure itself",
                     "kernel": "line_relax_kernel<128,NL=0,FULL=1>", "kernel_ms": kern_ms,
                     "smem_nominal": {"peak": smem_nominal, "frac": smem_achieved / smem_nominal,
                                      "peak_kind": "nominal 128 B/clk/SM x %d SMs at the sampled clock" % N_SMS},
                     "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                             "peak_kind": peak_kind, "algorithmic_bytes_per_launch": BYTES_PER_SOLVE * solves_per_step,
                             "traffic": traffic * solves_per_step if traffic else None},
                     "fp32": fp32_roofline(node_updates, kern_ms, clk_summary.get("sm_mhz") or 2070.0),
                     "note": "the line passes run on shared-memory-resident planes: shared memory is the bounding "
                             "resource the fraction is quoted against (the kernel is issue-bound below it, see "
                             "profiles/); HBM carries only G, inputs and currents"},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(G.nbytes + vin.nbytes), "d2h_bytes_per_step": int(hout.numel() * 4)},
        "gpu_launches": args.steps,
        "clocks": clk_summary,
    }
    if world == 1:  # the host-core baseline is timed at N = 1 only (rank 0 is the only rank left here)
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tiles", type=int, default=N_TILES, help="128x128 tiles per rank (64 vectors each)")
    ap.add_argument("--tol", type=float, default=TOL_V, help="stop tolerance, estimated max node error (V)")
    ap.add_argument("--no-mixed", action="store_true",
                    help="skip the mixed-size (64/128/256), large non-ideal (512) and MLP-layer figures")
    ap.add_argument("--no-warm", action="store_true", help="skip training/evaluating the learned warm start")
    ap.add_argument("--quick", action="store_true",
                    help="time the device-resident solve only (no e2e, comparator or CPU baseline); for profiling")
    ap.add_argument("--quick-method", default="line", choices=["line", "rbsor"],
                    help="with --quick: the solver timed (rbsor: the plain red-black SOR, for profiling)")
    ap.add_argument("--size", type=int, default=128,
                    help="with --quick: tile size N (N x N tiles; 256 and 512 run on the cluster kernels)")
    ap.add_argument("--only-large", type=int, default=0, metavar="TILES",
                    help="run only the 512x512 sinh-cell figure on TILES tiles and print it (for profiling)")
    args = ap.parse_args()
    if args.only_large:
        import torch
        from fadesim_gb300 import cpp_ir_drop_accelerate as acc
        from fadesim_gb300.build import build
        build()
        acc.options.tol_v = args.tol
        print(json.dumps(large_nonideal(torch, acc, n_tiles=args.only_large)))
        return
    if args.size != 128:
        if not args.quick:
            ap.error("--size is a --quick (profiling) option; the metric is quoted on 128x128 tiles")
        global ROWS, COLS
        ROWS = COLS = args.size
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
