"""The CPU oracle against fixtures produced by the reference itself."""
import numpy as np
import pytest

from oracle import augs, intstages, nodal, sweeps

GW = 1 / 2.93


def test_port_reproduces_reference_sim(gold):
    z = gold("sim_v1_16x24.npz")
    g = 1.0 / z["Rset"][z["states"]]
    up, dn, io, sw = augs.solve(g, z["vin"], float(z["r_wire"]), 100000, float(z["omega"]), True, float(z["tol"]))
    # the reference prints 13 significant digits
    np.testing.assert_allclose(up, z["vup"], rtol=2e-12, atol=1e-15)
    np.testing.assert_allclose(dn, z["vdown"], rtol=2e-12, atol=1e-17)
    np.testing.assert_allclose(io, z["iout"], rtol=2e-11)
    assert sw == int(z["sweeps"])


def test_port_readme_config_sweeps(gold):
    z = gold("sim_v1_128_readme.npz")
    g = 1.0 / z["Rset"][z["states"]]
    _, _, io, sw = augs.solve(g, z["vin"], 2.93, 100000, float(z["omega"]), True, 1e-8)
    assert sw == int(z["sweeps"]) == 1513
    np.testing.assert_allclose(io, z["iout"], rtol=2e-11)


def test_direct_solve_matches_converged_reference(gold):
    z = gold("sim_v1_16x24.npz")
    g = 1.0 / z["Rset"][z["states"]]
    u, d = nodal.solve(g, GW, z["vin"])
    assert np.abs(u - z["vup"]).max() < 1e-9
    assert np.abs(d - z["vdown"]).max() < 1e-9
    z = gold("sim_v1_128_tol1e-11.npz")
    g = 1.0 / z["Rset"][z["states"]]
    u, d = nodal.solve(g, GW, z["vin"])
    r = z["sample_rows"]
    assert np.abs(u[r] - z["vup_rows"]).max() < 3e-9
    assert np.abs(d[r] - z["vdown_rows"]).max() < 3e-9
    np.testing.assert_allclose(nodal.currents(g, u, d), z["iout"], rtol=5e-8)


def test_reference_delta_stop_is_loose(gold):
    """At its own settings (tol 1e-8 on the sweep delta) the reference stops ~1e-6 V short."""
    z = gold("sim_v1_128_tol1e-8.npz")
    g = 1.0 / z["Rset"][z["states"]]
    u, d = nodal.solve(g, GW, z["vin"])
    r = z["sample_rows"]
    err = max(np.abs(u[r] - z["vup_rows"]).max(), np.abs(d[r] - z["vdown_rows"]).max())
    assert 5e-7 < err < 5e-6
    assert int(z["sweeps"]) == 1509


def test_dense_and_sparse_direct_agree():
    rng = np.random.default_rng(3)
    g = 1.0 / rng.choice([1e3, 1e4, 1e6], size=(12, 9))
    vin = rng.random(12)
    u1, d1 = nodal.solve(g, GW, vin)
    u2, d2 = nodal.solve(g, GW, vin, dense=True)
    assert np.abs(u1 - u2).max() < 1e-13 and np.abs(d1 - d2).max() < 1e-13
    # several vectors at once give the same answer
    V = rng.random((3, 12))
    U, D = nodal.solve(g, GW, V)
    u3, d3 = nodal.solve(g, GW, V[2])
    assert np.abs(U[2] - u3).max() < 1e-14


def test_direct_solve_kcl_residual():
    rng = np.random.default_rng(4)
    g = 1.0 / rng.choice([1e3, 1e6], size=(7, 5))
    vin = rng.random(7)
    A, b = nodal.assemble(g, GW, vin)
    u, d = nodal.solve(g, GW, vin)
    x = np.empty(2 * 35)
    x[0::2] = u.ravel()
    x[1::2] = d.ravel()
    assert np.abs(A @ x - b).max() < 1e-14
    # current into the array equals current out through the bitline terminals
    i_in = (GW * (vin - u[:, 0])).sum()
    i_out = (GW * d[-1, :]).sum()
    assert abs(i_in - i_out) < 1e-12 * abs(i_in) + 1e-18


@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-13), (np.float32, 5e-6)])
def test_sweep_order_matches_pimtorch(gold, dt, tol):
    z = gold("pimtorch_gs_8x6.npz")
    B, X, Y, n, m = [int(z[k]) for k in ["B", "numX", "numY", "rows", "cols"]]
    tag = "f64" if dt == np.float64 else "f32"
    r = sweeps.ir_drop_gs(z["input"].astype(dt), z["G"].astype(dt), B, n, m, X, Y, int(z["fixed_iters"]), GW,
                          float(z["omega"]))
    ref = z["fixed_" + tag]
    assert np.abs(r - ref).max() <= tol * np.abs(ref).max()
    r = sweeps.ir_drop_gs(z["input"].astype(dt), z["G"].astype(dt), B, n, m, X, Y, 5000, GW, float(z["omega"]),
                          True, float(z["break_thr_" + tag]))
    ref = z["break_" + tag]
    assert np.abs(r - ref).max() <= 4 * tol * np.abs(ref).max()


@pytest.mark.parametrize("name", ["c3like", "signed"])
def test_integer_stages_bit_exact(gold, name):
    z = gold("pimtorch_split_%s.npz" % name)
    kw = {k: z[k].item() for k in ["Ron", "Roff", "cellBits", "rows", "cols", "inputMaxVoltage", "adc_bits"]}
    p = intstages.ArrayParams(**kw)
    y = intstages.split_matmul(z["x"], z["w"], p, intstages.droop_solver)
    assert y.dtype == np.float32
    assert np.array_equal(y, z["y"])


LAYER_LINEAR = ["ref_c2", "ref_signed", "negpulse_pn_dac2", "negpulse_ref"]
LAYER_CONV = ["conv_pn", "conv_ref_stride"]


def layer_params(z):
    kw = {k: z[k].item() for k in ["Ron", "Roff", "cellBits", "rows", "cols", "inputMaxVoltage", "adc_bits"]}
    if "dac_bits" in z:
        kw["dac_bits"] = int(z["dac_bits"])
    return intstages.ArrayParams(**kw)


@pytest.mark.parametrize("name", LAYER_LINEAR)
def test_ref_and_negpulse_stages_bit_exact(gold, name):
    """Ref-column arrays and negative-pulse inputs against the reference's own
    splitArr_matmul_nn (same droop solve)."""
    z = gold("pimtorch_layer_%s.npz" % name)
    y = intstages.split_matmul_ex(z["x"], z["w"], layer_params(z), arr=str(z["arr_mode"]),
                                  neg_pulse=str(z["input_mode"]) == "neg_pulse", solver=intstages.droop_solver)
    assert y.dtype == np.float32
    assert np.array_equal(y, z["y"])


def torch_variation_draws(sigma, seed):
    """The reference's variation draws, exp(sigma N(0,1)) from a torch CPU
    generator seeded like its network generator (seed + 2), in call order."""
    import torch
    gen = torch.Generator()
    gen.manual_seed(int(seed) + 2)
    return lambda shape: torch.exp(torch.randn(tuple(shape), generator=gen) * sigma).numpy()


@pytest.mark.parametrize("name", ["var_pn", "var_ref"])
def test_variation_stages_bit_exact(gold, name):
    """Cycle-to-cycle variation (sigma 0.1) in the layer path: the restatement's
    draw order -- input bit outer, slice inner, positive before negative -- and
    its G / exp(sigma N) reproduce the reference's splitArr_matmul_nn bit for bit
    (same droop solve); without the draws the result differs."""
    pytest.importorskip("torch")
    z = gold("pimtorch_layer_%s.npz" % name)
    p = layer_params(z)
    vary = torch_variation_draws(float(z["sigma"]), int(z["seed"]))
    y = intstages.split_matmul_ex(z["x"], z["w"], p, arr=str(z["arr_mode"]), solver=intstages.droop_solver,
                                  vary=vary)
    assert y.dtype == np.float32
    assert np.array_equal(y, z["y"])
    y0 = intstages.split_matmul_ex(z["x"], z["w"], p, arr=str(z["arr_mode"]), solver=intstages.droop_solver)
    assert not np.array_equal(y0, z["y"])


@pytest.mark.parametrize("name", LAYER_CONV)
def test_conv2d_sp_bit_exact(gold, name):
    """Conv2d_sp evaluation (unfold, split matmul, bias, fold) against the reference module."""
    z = gold("pimtorch_layer_%s.npz" % name)
    pair = lambda k, d: tuple(np.broadcast_to(z[k], 2)) if k in z else d
    y = intstages.conv2d_sp(z["x"], z["weight"], z["bias"], layer_params(z), stride=pair("conv_stride", (1, 1)),
                            padding=pair("conv_padding", (0, 0)), dilation=pair("conv_dilation", (1, 1)),
                            arr=str(z["arr_mode"]), use_fp_bias=bool(z["use_fp_bias"]), solver=intstages.droop_solver)
    assert y.shape == z["y"].shape
    assert np.array_equal(y, z["y"])


def test_converged_sweeps_reach_direct_solution():
    """The sweep-order restatement converges to the direct solve (same system)."""
    rng = np.random.default_rng(5)
    n, m = 6, 5
    g = 1.0 / rng.choice([1e3, 3e3, 1e4], size=(n, m))
    vin = rng.random(n)
    r = sweeps.ir_drop_gs(vin.reshape(1, 1, n), g.reshape(1, n, m), 1, n, m, 1, 1, 4000, GW, 1.5, ret_V=False)
    u, d = nodal.solve(g, GW, vin)
    np.testing.assert_allclose(r.reshape(m), nodal.currents(g, u, d), rtol=1e-10)


def test_fcm_file_format_and_oracle(gold):
    """The FCM export of the reference's sim (unit-voltage solve per wordline):
    our writer reproduces its file text byte for byte from the same numbers, and
    the FP64 oracle's unit responses give the same non-ideal conductances."""
    from fadesim_gb300 import geff
    z = gold("sim_v1_fcm_12x10.npz")
    st, Rset, g_ref = z["states"], z["Rset"], z["g_non_ideal"]
    assert geff.fcm_text(st, Rset, g_ref) == str(z["text"])
    G = 1.0 / Rset[st]
    n = G.shape[0]
    u, d = nodal.solve(G, 1 / float(z["r_wire"]), np.eye(n))
    g_or = nodal.currents(G, u, d)
    assert np.abs(g_or - g_ref).max() <= 1e-9 * np.abs(g_ref).max()


@pytest.mark.parametrize("iters", [6, 300])
def test_ir2s_restatement_matches_reference(gold, iters):
    """The IR2S iteration restated from the CUDA extension (persistent line
    sums) against the reference's Python IR2S (sums recomputed each iteration):
    the same iterates up to FP64 rounding."""
    z = gold("pimtorch_ir2s_8x6.npz")
    B, X, Y, n, m = (int(z[k]) for k in ("B", "numX", "numY", "rows", "cols"))
    r = sweeps.ir_family(z["input"], z["G"], B, n, m, X, Y, iters, float(z["r_wire"]), "ir2s")
    ref = z["iters_%d" % iters]
    assert np.abs(r - ref).max() <= 1e-12 * np.abs(ref).max()


def test_ir_family_consistency():
    """Structural identities of the OU and load variants: a whole-tile OU and
    wire-valued loads reduce each to its plain solver; IR2S converges to the
    nodal solution."""
    rng = np.random.default_rng(1)
    B, X, Y, n, m = 2, 2, 2, 8, 6
    inp = rng.integers(0, 2, (B, X, n)) * 0.2
    G = 1 / rng.choice([1e3, 2e4, 3e5, 1e6], size=(X, n, Y * m))
    gs = sweeps.ir_drop_gs(inp, G, B, n, m, X, Y, 40, GW, 1.9)
    for kw in (dict(), dict(ou=(n, m)), dict(loads=(GW, GW))):
        r = sweeps.ir_family(inp, G, B, n, m, X, Y, 40, GW, "gs", beta=1.9, **kw)
        assert np.abs(r - gs).max() <= 1e-13 * np.abs(gs).max()
    conv = sweeps.ir_family(inp, G, B, n, m, X, Y, 400, 2.93, "ir2s")
    assert np.abs(conv - nodal.solve_layer(inp, G, n, m, X, Y, GW)).max() <= 1e-12 * np.abs(conv).max()
    for kw in (dict(ou=(n, m)), dict(loads=(2.93, 2.93))):
        r = sweeps.ir_family(inp, G, B, n, m, X, Y, 400, 2.93, "ir2s", **kw)
        assert np.abs(r - conv).max() <= 1e-13 * np.abs(conv).max()


def _nl_case(seed, B=2, X=2, Y=2, n=8, m=6):
    rng = np.random.default_rng(seed)
    inp = rng.uniform(0, 0.2, (B, X, n))
    inp[0, 0, 1] = 0.0                                   # a row at 0 V: cells under the deal_v clamp
    G = 1 / rng.choice([1e5, 2e5, 5e5, 1e6], size=(X, n, Y * m))
    return inp, G, nodal.sinh_params(1e5, 1e6, a=2.0)


def test_nonlinear_sweeps_converge_to_nodal_fixed_point():
    """The nonlinear sweep restatement (conductances from the iterate before the
    newest) converges to the FP64 fixed point of the nonlinear nodal system."""
    inp, G, params = _nl_case(3)
    B, X, Y, n, m = 2, 2, 2, 8, 6
    r = sweeps.ir_drop_gs_nonlinear(inp, G, B, n, m, X, Y, 400, GW, 1.5, params)
    Gr = G.reshape(X, n, Y, m)
    for b in range(B):
        for x in range(X):
            for y in range(Y):
                u, d, _ = nodal.solve_nonlinear(Gr[x, :, y, :], GW, inp[b, x], params)
                ref = nodal.nonlinear_currents(Gr[x, :, y, :], u, d, params)
                got = r[b, x, y * m:(y + 1) * m]
                assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("iters", [1, 2, 5, 40])
def test_nonlinear_family_matches_sweep_restatement(iters):
    """The family's nonlinear bookkeeping (a lagged copy of the planes) against
    the literal ping-pong restatement of ir_drop_gs: identical iterates for the
    plain sweep, its whole-tile OU and its wire-valued loads."""
    inp, G, params = _nl_case(4)
    B, X, Y, n, m = 2, 2, 2, 8, 6
    ref = sweeps.ir_drop_gs_nonlinear(inp, G, B, n, m, X, Y, iters, GW, 1.3, params)
    for kw in (dict(), dict(ou=(n, m)), dict(loads=(GW, GW))):
        r = sweeps.ir_family(inp, G, B, n, m, X, Y, iters, GW, "gs", beta=1.3, nonlinear=params, **kw)
        assert np.abs(r - ref).max() <= 1e-13 * np.abs(ref).max(), kw


def test_nonlinear_ir2s_family_fixed_point_and_linear_limit():
    """Nonlinear IR2S converges to the nonlinear nodal solution (its loads equal
    to the wire resistance make it the plain tile), the OU/load variants reduce
    to it, and as a -> 0 (b = 1/(a R)) the cells turn linear."""
    inp, G, params = _nl_case(5)
    B, X, Y, n, m = 2, 2, 2, 8, 6
    conv = sweeps.ir_family(inp, G, B, n, m, X, Y, 600, 2.93, "ir2s", nonlinear=params)
    Gr = G.reshape(X, n, Y, m)
    for b in range(B):
        for x in range(X):
            for y in range(Y):
                u, d, _ = nodal.solve_nonlinear(Gr[x, :, y, :], GW, inp[b, x], params)
                ref = nodal.nonlinear_currents(Gr[x, :, y, :], u, d, params)
                assert np.abs(conv[b, x, y * m:(y + 1) * m] - ref).max() <= 1e-9 * np.abs(ref).max()
    for kw in (dict(ou=(n, m)), dict(loads=(2.93, 2.93))):
        r = sweeps.ir_family(inp, G, B, n, m, X, Y, 600, 2.93, "ir2s", nonlinear=params, **kw)
        assert np.abs(r - conv).max() <= 1e-13 * np.abs(conv).max(), kw
    lin = sweeps.ir_family(inp, G, B, n, m, X, Y, 30, 2.93, "ir2s")
    a = 1e-4
    weak = [1e5, 1e6, a, 1 / (a * 1e5), a, 1 / (a * 1e6)]
    r = sweeps.ir_family(inp, G, B, n, m, X, Y, 30, 2.93, "ir2s", nonlinear=weak)
    assert np.abs(r - lin).max() <= 1e-7 * np.abs(lin).max()


def test_nonlinear_family_float32_tracks_float64():
    """The FP32 form of the nonlinear family (arithmetic in the dtype of G, as
    the reference's tensor ops) stays within FP32 rounding of the FP64 one."""
    inp, G, params = _nl_case(6)
    B, X, Y, n, m = 2, 2, 2, 8, 6
    for mode, wire, kw in (("gs", GW, dict(ou=(4, 3), beta=1.2)), ("ir2s", 2.93, dict(loads=(5.0, 7.5)))):
        r64 = sweeps.ir_family(inp, G, B, n, m, X, Y, 12, wire, mode, nonlinear=params, **kw)
        r32 = sweeps.ir_family(inp.astype(np.float32), G.astype(np.float32), B, n, m, X, Y, 12, wire, mode,
                               nonlinear=params, **kw)
        assert r32.dtype == np.float32
        assert np.abs(r32 - r64).max() <= 1e-5 * np.abs(r64).max(), mode


def test_nonlinear_reused_factor_matches_picard():
    """The factor-reusing nonlinear oracle (one factorisation, x += A0^-1 (b -
    A(x) x)) lands on the Picard fixed point."""
    rng = np.random.default_rng(4)
    n, m = 48, 40
    G = 1.0 / np.array([2e6, 1.6e6, 1.3e6, 1e6])[rng.integers(0, 4, (n, m))]
    G = G / np.exp(0.1 * rng.standard_normal((n, m)))
    vin = rng.random(n) * 0.2
    p = nodal.sinh_params(1e6, 2e6)
    u, d, _ = nodal.solve_nonlinear(G, 1 / 2.93, vin, p)
    u2, d2, _ = nodal.solve_nonlinear(G, 1 / 2.93, vin, p, reuse_factor=True)
    assert max(np.abs(u - u2).max(), np.abs(d - d2).max()) < 1e-12
