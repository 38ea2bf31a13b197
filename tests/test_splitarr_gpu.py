"""GPU integer stages of the bit-sliced matmul, bit-exact with the reference.

The fixtures were produced by the reference's own ``splitArr_matmul_nn`` with a
deterministic stand-in for the IR-drop solve (oracle.intstages.droop_solver).
Here the same stand-in replaces the solve, fed with the input voltages and
conductance maps the CUDA kernels build, so the comparison covers quantisation,
bit slicing, conductance mapping, ADC and shift-add end to end.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import intstages  # noqa: E402


@pytest.fixture(scope="module")
def sa():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import splitarr
    return splitarr


def droop_on_host(v, G, B, rows, cols, numX, numY, out):
    cur = intstages.droop_solver(v.cpu().numpy(), G.cpu().numpy(), B, rows, cols, numX, numY)
    out.copy_(torch.from_numpy(cur).reshape(out.shape))
    return out


def per_map(recorded, nmaps):
    """The layer driver solves all (slice, array) maps of a layer in one call,
    stacked along the tile axis; split that recorded call into one
    (vectors, conductances, currents) triple per map, in slice-major order."""
    (v_all, G_all, cur), = recorded
    numX = G_all.shape[0] // nmaps
    return [(v_all[:, k * numX:(k + 1) * numX].copy(), G_all[k * numX:(k + 1) * numX].copy(),
             cur[:, k * numX:(k + 1) * numX].copy()) for k in range(nmaps)]


@pytest.mark.parametrize("name", ["c3like", "signed"])
def test_split_matmul_bit_exact_vs_reference(sa, gold, name):
    z = gold("pimtorch_split_%s.npz" % name)
    cfg = sa.ArrayConfig(Ron=float(z["Ron"]), Roff=float(z["Roff"]), cellBits=int(z["cellBits"]),
                         arrRowSize=int(z["rows"]), arrColSize=int(z["cols"]),
                         inputMaxVoltage=float(z["inputMaxVoltage"]))
    y = sa.splitArr_matmul_nn(torch.from_numpy(z["x"]), torch.from_numpy(z["w"]), 8, 1, int(z["adc_bits"]), 10, 8,
                              "PN", torch.float32, cfg=cfg, solver=droop_on_host)
    assert np.array_equal(y.cpu().numpy(), z["y"])


def test_split_matmul_matches_oracle_with_gpu_solver_currents(sa):
    """With the real CUDA solve, the integer stages agree with the oracle's
    restatement fed the same (GPU-solved) currents."""
    rng = np.random.default_rng(4)
    x = rng.integers(0, 256, (3, 70)).astype(np.float32)
    w = (rng.standard_normal((70, 40)) * 0.05).astype(np.float32)
    cfg = sa.ArrayConfig(cellBits=2, arrRowSize=32, arrColSize=32, inputMaxVoltage=0.2)
    recorded = []

    def record(v, G, B, rows, cols, numX, numY, out):
        r = sa.default_solver(cfg)(v, G, B, rows, cols, numX, numY, out)
        recorded.append((v.cpu().numpy(), G.cpu().numpy(), r.cpu().numpy().copy()))
        return r

    y = sa.splitArr_matmul_nn(torch.from_numpy(x), torch.from_numpy(w), 8, 1, 8, 10, 8, "PN", torch.float32, cfg=cfg,
                              solver=record)
    recorded = per_map(recorded, 8)   # 4 slices x (positive, negative)
    p = intstages.ArrayParams(Ron=1e3, Roff=1e6, cellBits=2, rows=32, cols=32, inputMaxVoltage=0.2, adc_bits=8)
    # replay: the oracle calls its solver per (input bit, slice, array) with one bit's
    # vectors; pick those rows out of the recorded all-bit solves
    calls = iter(range(10 ** 6))
    state = {"k": 0}

    def replay(in_v, G, B, rows, cols, numX, numY):
        k = state["k"]
        state["k"] += 1
        i, rem = divmod(k, 8)           # oracle order: bit i, slice j, pos then neg
        j, pn = divmod(rem, 2)
        v_all, G_rec, cur = recorded[j * 2 + pn]
        assert np.array_equal(G_rec, G)
        assert np.array_equal(v_all[i * B:(i + 1) * B], in_v)
        return cur[i * B:(i + 1) * B]

    ref = intstages.split_matmul(x, w, p, replay)
    assert np.array_equal(y.cpu().numpy(), ref)


def test_map_grouping_gives_the_same_bits(sa, gold, monkeypatch):
    """The layer driver's batching of weight-slice maps into one solver call
    (bounded by MAP_GROUP_BYTES) changes nothing: one map per call, a few per
    call and all in one give the same output bits."""
    z = gold("pimtorch_split_c3like.npz")
    cfg = sa.ArrayConfig(Ron=float(z["Ron"]), Roff=float(z["Roff"]), cellBits=int(z["cellBits"]),
                         arrRowSize=int(z["rows"]), arrColSize=int(z["cols"]),
                         inputMaxVoltage=float(z["inputMaxVoltage"]))
    run = lambda: sa.splitArr_matmul_nn(torch.from_numpy(z["x"]), torch.from_numpy(z["w"]), 8, 1, int(z["adc_bits"]),
                                        10, 8, "PN", torch.float32, cfg=cfg, solver=droop_on_host).cpu().numpy()
    whole = run()
    v_bytes = z["x"].shape[0] * 8 * 4   # bytes of one map's input vectors per row of tiles
    for budget in (1, 2 * v_bytes * 64):
        monkeypatch.setattr(sa, "MAP_GROUP_BYTES", budget)
        assert np.array_equal(run(), whole)
    assert np.array_equal(whole, z["y"])


def layer_cfg(sa, z):
    return sa.ArrayConfig(Ron=float(z["Ron"]), Roff=float(z["Roff"]), cellBits=int(z["cellBits"]),
                          arrRowSize=int(z["rows"]), arrColSize=int(z["cols"]),
                          inputMaxVoltage=float(z["inputMaxVoltage"]),
                          inputVmode=str(z["input_mode"]) if "input_mode" in z else "complement_code")


@pytest.mark.parametrize("name", ["ref_c2", "ref_signed", "negpulse_pn_dac2", "negpulse_ref"])
def test_ref_and_negpulse_bit_exact_vs_reference(sa, gold, name):
    """Ref-column arrays (two reference columns per block, offset weights) and
    negative-pulse inputs, against the reference's splitArr_matmul_nn."""
    z = gold("pimtorch_layer_%s.npz" % name)
    dac = int(z["dac_bits"]) if "dac_bits" in z else 1
    y = sa.splitArr_matmul_nn(torch.from_numpy(z["x"]), torch.from_numpy(z["w"]), 8, dac, int(z["adc_bits"]), 10, 8,
                              str(z["arr_mode"]), torch.float32, cfg=layer_cfg(sa, z), solver=droop_on_host)
    assert np.array_equal(y.cpu().numpy(), z["y"])


@pytest.mark.parametrize("name", ["conv_pn", "conv_ref_stride"])
def test_conv2d_sp_bit_exact_vs_reference(sa, gold, name):
    """Conv2d_sp evaluation: unfold by addressing in the slicing kernel, bias in
    float32 or mapped to a ones row, NCHW output from the shift-add kernel; the
    second case has an input row the unfold never reads holding the largest
    value (it must not set the quantisation scale)."""
    z = gold("pimtorch_layer_%s.npz" % name)
    get = lambda k, d: tuple(int(t) for t in np.broadcast_to(z[k], 2)) if k in z else d
    layer = sa.Conv2d_sp(int(z["conv_in_channels"]), int(z["conv_out_channels"]), get("conv_kernel_size", None),
                         stride=get("conv_stride", (1, 1)), padding=get("conv_padding", (0, 0)),
                         dilation=get("conv_dilation", (1, 1)), adc_bit_width=int(z["adc_bits"]),
                         phy_arr_mode=str(z["arr_mode"]), use_fp_bias=bool(z["use_fp_bias"]),
                         cfg=layer_cfg(sa, z), solver=droop_on_host)
    with torch.no_grad():
        layer.fp_weight.copy_(torch.from_numpy(z["weight"]))
        layer.fp_bias.copy_(torch.from_numpy(z["bias"]))
    layer.eval()
    y = layer(torch.from_numpy(z["x"]).cuda())
    assert tuple(y.shape) == z["y"].shape
    assert np.array_equal(y.cpu().numpy(), z["y"])


def test_conv2d_sp_with_gpu_solver_matches_oracle(sa):
    """Real CUDA solves under a Ref-column convolution: the oracle's
    restatement, replaying the recorded currents, gives the same bits."""
    rng = np.random.default_rng(9)
    x = rng.standard_normal((2, 3, 6, 6)).astype(np.float32)
    wgt = (rng.standard_normal((8, 3, 3, 3)) * 0.2).astype(np.float32)
    bias = rng.standard_normal(8).astype(np.float32)
    cfg = sa.ArrayConfig(cellBits=1, arrRowSize=16, arrColSize=8, inputMaxVoltage=0.5)
    recorded = []

    def record(v, G, B, rows, cols, numX, numY, out):
        r = sa.default_solver(cfg)(v, G, B, rows, cols, numX, numY, out)
        recorded.append((v.cpu().numpy(), G.cpu().numpy(), r.cpu().numpy().copy()))
        return r

    y = sa.conv2d_split(torch.from_numpy(x), torch.from_numpy(wgt), torch.from_numpy(bias), 1, 1, 1, adcBits=10,
                        arrType="Ref", cfg=cfg, solver=record)
    recorded = per_map(recorded, 8)   # 8 one-bit slices, one Ref array
    p = intstages.ArrayParams(Ron=1e3, Roff=1e6, cellBits=1, rows=16, cols=8, inputMaxVoltage=0.5, adc_bits=10)
    state = {"k": 0}

    def replay(in_v, G, B, rows, cols, numX, numY):
        k = state["k"]
        state["k"] += 1
        i, j = divmod(k, 8)           # oracle order: bit i, slice j (one Ref array)
        v_all, G_rec, cur = recorded[j]
        assert np.array_equal(G_rec, G)
        assert np.array_equal(v_all[i * B:(i + 1) * B], in_v)
        return cur[i * B:(i + 1) * B]

    ref = intstages.conv2d_sp(x, wgt, bias, p, padding=(1, 1), arr="Ref", solver=replay)
    assert np.array_equal(y.cpu().numpy(), ref)


def test_superposition_solver_matches_direct(sa):
    """Currents by linearity (unit responses of each tile, then one FP32 matrix
    product) equal the direct per-vector solves to the solver tolerance."""
    rng = np.random.default_rng(12)
    cfg = sa.ArrayConfig(Ron=1e3, Roff=1e6, cellBits=2, arrRowSize=64, arrColSize=64, inputMaxVoltage=0.2)
    B, numX, numY, n = 300, 2, 2, 64
    states = rng.integers(0, 4, (numX, n, numY * n))
    G = torch.tensor(states * cfg.cellDeltaConduct + cfg.cellMinConduct, dtype=torch.float32).cuda()
    v = torch.tensor(rng.integers(0, 2, (B, numX, n)) * 0.2, dtype=torch.float32).cuda()
    direct = sa.default_solver(cfg)(v, G, B, n, n, numX, numY, None)
    sup = sa.superposition_solver(cfg)(v, G, B, n, n, numX, numY, torch.empty_like(direct))
    assert (sup - direct).abs().max().item() <= 1e-5 * direct.abs().max().item()


def test_mlp_layer_path_runs_both_strategies(sa):
    """The layer-level MLP (784-512-512-10, 2-bit cells on 128x128 PN crossbars)
    on a small batch: both solver strategies give nearly the same outputs."""
    from fadesim_gb300 import mlp_eval
    r = mlp_eval.evaluate(batch=20)   # 160 vectors per call: more than a tile's 128 rows
    assert r["direct"]["solves_per_batch"] == sum(mlp_eval.solves_per_batch(20, mlp_eval.config()))
    # over all eight maps of layer 1 the two strategies' currents agree to about
    # 1e-4 of the largest current: the superposition sums up to 128 unit
    # responses, each with the FP32 floor of its planes
    assert r["superposition"]["max_rel_current_diff_vs_direct"] < 2e-4


def test_mlp_first_layer_end_to_end_against_oracle(sa):
    """The MLP configuration itself, end to end: the first layer (784 -> 512,
    weights N(0, 0.05^2), 2-bit cells of 1 kohm - 1 Mohm on 128x128 PN
    crossbars, 0.2 V reads, 8-bit ADC) on two synthetic images through the GPU
    path with the real CUDA solves.  The oracle's restatement of the integer
    stages, fed the recorded currents, gives the same output bits, and the
    recorded currents of one (slice, array) map match the FP64 nodal solve of
    the same voltages and conductances within the 1e-4 current contract."""
    from fadesim_gb300 import mlp_eval
    from oracle import nodal
    cfg = mlp_eval.config()
    w = mlp_eval.build(3)[0]                                   # [512, 784]
    g = torch.Generator().manual_seed(4)
    x = torch.randint(0, 256, (2, 784), generator=g).float()
    recorded = []

    def record(v, G, B, rows, cols, numX, numY, out):
        r = sa.default_solver(cfg)(v, G, B, rows, cols, numX, numY, out)
        recorded.append((v.cpu().numpy(), G.cpu().numpy(), r.cpu().numpy().copy()))
        return r

    y = sa.splitArr_matmul_nn(x, w.t().contiguous(), 8, 1, 8, 10, 8, "PN", torch.float32, cfg=cfg, solver=record)
    recorded = per_map(recorded, 8)   # 4 slices x (positive, negative)
    p = intstages.ArrayParams(Ron=1e3, Roff=1e6, cellBits=2, rows=128, cols=128, inputMaxVoltage=0.2, adc_bits=8)
    state = {"k": 0}

    def replay(in_v, G, B, rows, cols, numX, numY):
        k = state["k"]
        state["k"] += 1
        i, rem = divmod(k, 8)           # oracle order: bit i, slice j, pos then neg
        j, pn = divmod(rem, 2)
        v_all, G_rec, cur = recorded[j * 2 + pn]
        assert np.array_equal(G_rec, G)
        assert np.array_equal(v_all[i * B:(i + 1) * B], in_v)
        return cur[i * B:(i + 1) * B]

    ref = intstages.split_matmul(x.numpy(), w.t().contiguous().cpu().numpy(), p, replay)
    assert np.array_equal(y.cpu().numpy(), ref)
    # the currents of the most significant slice's positive array on two tiles, against FP64
    v_all, G_rec, cur = recorded[3 * 2]
    numX, rows, cols = 7, 128, 128
    for x_t, y_t in ((0, 0), (6, 3)):
        Gt = G_rec[x_t, :, y_t * cols:(y_t + 1) * cols].astype(np.float64)
        vin = v_all[:, x_t].astype(np.float64)
        u, d = nodal.solve(Gt, 1 / cfg.r_wire, vin)
        ref_i = nodal.currents(Gt, u, d)
        got = cur[:, x_t, y_t * cols:(y_t + 1) * cols].astype(np.float64)
        assert np.abs(got - ref_i).max() <= 1e-4 * np.abs(ref_i).max()
