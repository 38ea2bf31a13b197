"""Generate the golden fixtures in this directory from the reference itself.

Runs only where the reference tree is present (it reads it from the
directory in $FADESIM_REFERENCE, by default /root/reference).  Three sources:

1. The reference's crossbarHspice V1 ``sim``, compiled from its own sources by
   ``make -C oracle ref`` into ``oracle/_ref/sim``, run on seeded configs written
   as explicit per-cell ``setCellR`` lines (its ``randSetR`` is unseeded).
2. The reference's PimTorch modules, imported through a throw-away package in a
   temporary directory: the six ``fixedPoint/nn`` files and
   ``fixedPoint/nn/modules/conv_split.py`` are copied there unchanged except
   that the import-time JIT build and ``chdir`` in ``commonConst.py`` are
   removed (the CUDA source does not compile against this
   torch and there is no GPU here).  Nothing from that copy is kept.
3. Their outputs, saved as small .npz files next to this script.

Usage: python tests/golden/make_golden.py [sim] [pimtorch] [layers] [variation] [fcm] [ir2s] [simtext] [sim2text]
"""
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
REF = os.environ.get("FADESIM_REFERENCE", "/root/reference")
NN = os.path.join(REF, "pimtorch", "pimfixedpoint", "fixedPoint", "nn")
SIM = os.path.join(REPO, "oracle", "_ref", "sim")

from oracle import intstages  # noqa: E402


def sim_run(states, Rset, vin, r_wire, iters, w, tol):
    n, m = states.shape
    lines = ["useRtypeReRAMCell yes",
             "cellRstates %d %s" % (len(Rset), " ".join("%.17g" % r for r in Rset)),
             "arraySize %d %d" % (n, m), "selector no", "line_resistance %.17g" % r_wire]
    for i in range(n):
        for j in range(m):
            lines.append("setCellR %d %d %d" % (i, j, states[i, j]))
    lines += ["setUseLine left -1", "setUseLine down -1"]
    for i in range(n):
        lines.append("setLineV left %d %.17g" % (i, vin[i]))
    lines += ["setLineV down -1 0", "senseBitlineI down -1",
              "nodebasedGSMethod %d %.17g 0 yes %.17g" % (iters, w, tol)]
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "cfg"), "w") as f:
            f.write("\n".join(lines) + "\n")
        out = subprocess.run([SIM, "cfg"], cwd=td, capture_output=True, text=True, check=True).stdout
        with open(os.path.join(td, "fastmode_nodebasedGS.out")) as f:
            txt = f.read()
    vup_s, rest = txt.split("vup = ")[1].split("vdown = ")
    vdn_s, iout_s = rest.split("iout = ")
    arr = lambda s: np.array([float(x) for x in s.split()])
    rec = re.findall(r"iter times =\s+(\d+)", out)
    sweeps = int(rec[-1]) + 1 if rec else iters
    return arr(vup_s).reshape(n, m), arr(vdn_s).reshape(n, m), arr(iout_s), sweeps


def sim_fixtures():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref"], check=True)
    Rset = np.array([2e6, 1.6e6, 1.3e6, 1e6])
    w = float(np.float32(1.95))  # the reference parses omega with stof
    # small non-square tile, mixed wordline voltages, converged hard
    rng = np.random.default_rng(7)
    st = rng.integers(0, 4, (16, 24))
    vin = rng.integers(0, 2, 16) * 0.2 + 0.05
    u, d, io, sw = sim_run(st, Rset, vin, 2.93, 100000, w, 1e-11)
    np.savez_compressed(os.path.join(HERE, "sim_v1_16x24.npz"), states=st, Rset=Rset, vin=vin, r_wire=2.93,
                        omega=w, tol=1e-11, vup=u, vdown=d, iout=io, sweeps=sw)
    # 128x128, four states drawn uniformly from seed 1, 1 V on every row
    st = np.random.default_rng(1).integers(0, 4, (128, 128))
    vin = np.ones(128)
    for tol, tag in [(1e-8, "tol1e-8"), (1e-11, "tol1e-11")]:
        u, d, io, sw = sim_run(st, Rset, vin, 2.93, 100000, w, tol)
        rows = np.arange(0, 128, 8)
        np.savez_compressed(os.path.join(HERE, "sim_v1_128_%s.npz" % tag), states=st, Rset=Rset, vin=vin,
                            r_wire=2.93, omega=w, tol=tol, sample_rows=rows, vup_rows=u[rows], vdown_rows=d[rows],
                            iout=io, sweeps=sw)
    # the README's example: every cell in state 2
    st = np.full((128, 128), 2)
    u, d, io, sw = sim_run(st, Rset, vin, 2.93, 100000, w, 1e-8)
    np.savez_compressed(os.path.join(HERE, "sim_v1_128_readme.npz"), states=st, Rset=Rset, vin=vin, r_wire=2.93,
                        omega=w, tol=1e-8, iout=io, sweeps=sw)


def import_pimtorch():
    td = tempfile.mkdtemp(prefix="pimtorch_shim_")
    pkg = os.path.join(td, "fixedPoint")
    os.makedirs(os.path.join(pkg, "nn"))
    open(os.path.join(pkg, "__init__.py"), "w").close()
    open(os.path.join(pkg, "nn", "__init__.py"), "w").close()
    for f in ["conductance_variation.py", "fixedPointArithmetic.py", "ir_drop_solve.py",
              "splitArrayArithmetic.py", "ir_drop_compensate.py"]:
        shutil.copy(os.path.join(NN, f), os.path.join(pkg, "nn", f))
    os.makedirs(os.path.join(pkg, "nn", "modules"))
    open(os.path.join(pkg, "nn", "modules", "__init__.py"), "w").close()
    shutil.copy(os.path.join(NN, "modules", "conv_split.py"), os.path.join(pkg, "nn", "modules", "conv_split.py"))
    with open(os.path.join(NN, "commonConst.py")) as f:
        src = f.read()
    # drop the import-time chdir and JIT build of the CUDA extension
    src = re.sub(r"\n    print\(\"now the working dir is \{\}\.\"\.format\(os\.getcwd\(\)\)\)\n"
                 r"    if os\.getcwd\(\)\[-5:\]!=\"point\":\n        os\.chdir\(\"\.\./\"\)\n"
                 r"    cpp_ir_drop_accelerate = load\(.*?verbose = True\)\n",
                 "\n    cpp_ir_drop_accelerate = None\n", src, flags=re.S)
    assert "cpp_ir_drop_accelerate = None" in src, "commonConst.py layout changed"
    with open(os.path.join(pkg, "nn", "commonConst.py"), "w") as f:
        f.write(src)
    sys.path.insert(0, td)
    import fixedPoint.nn.commonConst as cc
    import fixedPoint.nn.ir_drop_solve as ids
    import fixedPoint.nn.splitArrayArithmetic as sa
    return td, cc, ids, sa


def set_params(cc, p):
    P = cc.phyArrParams
    for k in ["Ron", "Roff", "cellMaxConduct", "cellMinConduct", "cellBits", "arrRowSize", "arrColSize",
              "inputMaxVoltage", "r_wire", "cellDeltaConduct", "adcUseI"]:
        setattr(P, k, getattr(p, k))
    P.crx_size = p.arrRowSize * p.arrColSize


class _DroopSolve:
    """Stand-in for the extension module: returns oracle.intstages.droop_solver."""

    def ir_drop_gs(self, in_b, G, bsize, rows, cols, numX, numY, *rest):
        import torch
        return torch.from_numpy(intstages.droop_solver(in_b.numpy(), G.numpy(), bsize, rows, cols, numX, numY))


def pimtorch_fixtures():
    import torch
    td, cc, ids, sa = import_pimtorch()
    try:
        # (a) the PimTorch GS sweep order, batchBybatch, fixed sweeps (and with break)
        P = cc.phyArrParams
        out = {}
        rng = np.random.default_rng(11)
        B, X, Y, n, m = 3, 2, 2, 8, 6
        inp = (rng.integers(0, 2, (B, X, n)) * 0.2).astype(np.float64)
        G = 1.0 / rng.choice([1e3, 2e4, 3e5, 1e6], size=(X, n, Y * m))
        P.arrRowSize = n
        P.ir_drop_GS_method_beta_scale = 1.9
        P.ir_drop_GS_method_mode = cc.GS_method.batchBybatch
        P.r_wire = 2.93
        for dt, tag in [(torch.float64, "f64"), (torch.float32, "f32")]:
            P.ir_drop_iter_time = 40
            P.ir_drop_less_than_thresholdBreak_enable = False
            r = ids.ir_drop_accurate_GSMethod(torch.tensor(inp, dtype=dt), torch.tensor(G, dtype=dt), B, X, Y, m)
            out["fixed_" + tag] = r.numpy()
            P.ir_drop_iter_time = 5000
            P.ir_drop_less_than_thresholdBreak_enable = True
            P.ir_drop_less_than_threshold = 1e-9 if tag == "f64" else 1e-6
            r = ids.ir_drop_accurate_GSMethod(torch.tensor(inp, dtype=dt), torch.tensor(G, dtype=dt), B, X, Y, m)
            out["break_" + tag] = r.numpy()
        np.savez_compressed(os.path.join(HERE, "pimtorch_gs_8x6.npz"), input=inp, G=G, B=B, numX=X, numY=Y, rows=n,
                            cols=m, omega=1.9, r_wire=2.93, fixed_iters=40, break_thr_f64=1e-9, break_thr_f32=1e-6,
                            **out)
        # (b) integer stages through splitArr_matmul_nn with a deterministic solve
        P.cpp_ir_drop_accelerate_flag = True
        P.cpp_ir_drop_accelerate = _DroopSolve()
        P.IRdropMode = cc.ir_drop_mode.accurate_GS_math
        P.useOUSize = False
        P.sigma = 0
        cases = [
            ("c3like", dict(Ron=1e3, Roff=1e6, cellBits=2, rows=32, cols=32, inputMaxVoltage=0.2, adc_bits=8),
             lambda r: r.integers(0, 256, (5, 100)).astype(np.float32),
             lambda r: (r.standard_normal((100, 70)) * 0.05).astype(np.float32)),
            ("signed", dict(Ron=1e3, Roff=1e6, cellBits=1, rows=64, cols=64, inputMaxVoltage=1.0, adc_bits=10),
             lambda r: r.standard_normal((4, 150)).astype(np.float32),
             lambda r: (r.standard_normal((150, 90)) * 0.1).astype(np.float32)),
        ]
        for name, kw, mkx, mkw in cases:
            p = intstages.ArrayParams(**kw)
            set_params(cc, p)
            r = np.random.default_rng(len(name))
            x, w = mkx(r), mkw(r)
            cc.variations.reset_all()
            y = sa.splitArr_matmul_nn(torch.from_numpy(x), torch.from_numpy(w), 8, 1, p.adc_bits, 10, 8,
                                      cc.phyArrMode.PN, torch.float32)
            np.savez_compressed(os.path.join(HERE, "pimtorch_split_%s.npz" % name), x=x, w=w, y=y.numpy(),
                                **{k: v for k, v in kw.items()})
    finally:
        shutil.rmtree(td, ignore_errors=True)


def ir2s_fixture():
    """The reference's Python IR2S iteration (ir_drop_solve.py:35-72) on a seeded
    layer, FP64, a few and many iterations."""
    import torch
    td, cc, ids, sa = import_pimtorch()
    try:
        P = cc.phyArrParams
        rng = np.random.default_rng(17)
        B, X, Y, n, m = 3, 2, 2, 8, 6
        inp = (rng.integers(0, 2, (B, X, n)) * 0.2).astype(np.float64)
        G = 1.0 / rng.choice([1e3, 2e4, 3e5, 1e6], size=(X, n, Y * m))
        P.arrRowSize = n
        P.r_wire = 2.93
        P.ir_drop_less_than_thresholdBreak_enable = False
        out = {}
        for iters in (6, 300):
            P.ir_drop_iter_time = iters
            r = ids.ir_drop_ir2s_fastsolve(torch.tensor(inp), torch.tensor(G), B, X, Y, m)
            out["iters_%d" % iters] = r.numpy()
        np.savez_compressed(os.path.join(HERE, "pimtorch_ir2s_8x6.npz"), input=inp, G=G, B=B, numX=X, numY=Y,
                            rows=n, cols=m, r_wire=2.93, **out)
    finally:
        shutil.rmtree(td, ignore_errors=True)


def fcm_fixture():
    """The reference's FCM export (``FCM gen``): the non-ideal conductance matrix
    of a seeded 12x10 array from one unit-voltage solve per wordline
    (crossbarHspice/2dArray.cc:949-1008), saved with the file text."""
    rng = np.random.default_rng(31)
    n, m = 12, 10
    Rset = [2e6, 1.6e6, 1.3e6, 1e6]
    st = rng.integers(0, 4, (n, m))
    lines = ["useRtypeReRAMCell yes",
             "cellRstates %d %s" % (len(Rset), " ".join("%.17g" % r for r in Rset)),
             "arraySize %d %d" % (n, m), "selector no", "line_resistance %.17g" % 2.93]
    for i in range(n):
        for j in range(m):
            lines.append("setCellR %d %d %d" % (i, j, st[i, j]))
    lines += ["setUseLine left -1", "setUseLine down -1", "setLineV left -1 1", "setLineV down -1 0",
              "senseBitlineI down -1", "FCM gen IR_FCM.conf"]
    with tempfile.TemporaryDirectory() as td:
        with open(os.path.join(td, "cfg"), "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run([SIM, "cfg"], cwd=td, capture_output=True, text=True, check=True)
        with open(os.path.join(td, "IR_FCM.conf")) as f:
            txt = f.read()
    tok = txt.split()
    assert int(tok[0]) == n and int(tok[1]) == m and int(tok[2]) == len(Rset)
    g = np.array([float(t) for t in tok[3 + len(Rset) + n * m:]]).reshape(n, m)
    np.savez_compressed(os.path.join(HERE, "sim_v1_fcm_12x10.npz"), states=st, Rset=np.array(Rset), r_wire=2.93,
                        g_non_ideal=g, text=np.array(txt))


SIM_TEXT_CFG = """% a 6x5 array in the reference's config language, exercising the commands
// the fast path reads (comments, whole-array setters, per-line overrides) and
// netlist-only ones that it skips
topString .title twoDArray
useRtypeReRAMCell yes
cellRstates 4 2e6 1.6e6 1.3e6 1e6
arraySize 6 5
selector no
line_resistance 2.93
setCellR -1 -1 2
setCellR 0 -1 3
setCellR -1 4 0
setCellR 2 1 1
setCellR 5 3 3
setUseLine left -1
setUseLine down -1
setLineV left -1 0.1
setLineV left 1 0.25
setLineV left 4 0
setLineV down -1 0
senseBitlineI down -1
nodebasedGSMethod 100000 1.9 0 yes 1e-13
FCM gen fcm.conf
setLineV left 2 0.3
FCM test fcm.conf
"""


def sim_text_fixture():
    """The reference's own output files for a committed config: byte-level
    layout of fastmode_nodebasedGS.out, IR_FCM.out (both modes) and the FCM
    file, and the stdout lines that its scripts parse.  Every nodeBasedGS call
    rewrites fastmode_nodebasedGS.out (FCM gen's unit solves too) and both FCM
    modes write IR_FCM.out, so each file is taken from a run of the config cut
    after the command that writes it."""
    with open(os.path.join(HERE, "sim_v1_6x5.cfg"), "w") as f:
        f.write(SIM_TEXT_CFG)

    def run(upto, td):
        cut = SIM_TEXT_CFG.index(upto) + len(upto)
        with open(os.path.join(td, "config"), "w") as f:
            f.write(SIM_TEXT_CFG[:cut] + "\n")
        return subprocess.run([SIM], cwd=td, capture_output=True, text=True, check=True).stdout

    with tempfile.TemporaryDirectory() as td:
        out = run("nodebasedGSMethod 100000 1.9 0 yes 1e-13", td)
        keep = [ln for ln in out.splitlines()
                if re.match(r"(evalutate|threshould|error I sum|set array size|setCellR)", ln)]
        with open(os.path.join(HERE, "sim_v1_6x5.stdout"), "w") as f:
            f.write("\n".join(keep) + "\n")
        shutil.copy(os.path.join(td, "fastmode_nodebasedGS.out"), os.path.join(HERE, "sim_v1_6x5.nodebasedGS.out"))
        run("FCM gen fcm.conf", td)
        shutil.copy(os.path.join(td, "IR_FCM.out"), os.path.join(HERE, "sim_v1_6x5.IR_FCM_gen.out"))
        shutil.copy(os.path.join(td, "fcm.conf"), os.path.join(HERE, "sim_v1_6x5.fcm.conf"))
        run("FCM test fcm.conf", td)
        shutil.copy(os.path.join(td, "IR_FCM.out"), os.path.join(HERE, "sim_v1_6x5.IR_FCM_test.out"))


SIM2_TEXT_CFG = """# the V2 simulator's dialect: '#' comments, cellRStates, no selector command;
% a 6x7 array (V2 reads wordline segments from the [m][n+1] bitline table, in
// range for n <= m <= n+1)
topString .title twoDArray
useRtypeReRAMCell yes
cellRStates 4 2e6 1.6e6 1.3e6 1e6
arraySize 6 7
line_resistance 2.93
setCellR -1 -1 1
setCellR 0 -1 3
setCellR -1 6 0
setCellR 2 1 2
setCellR 5 3 3
setUseLine left -1
setUseLine down -1
setLineV left -1 0.2
setLineV left 3 0.05
setLineV down -1 0
senseBitlineI down -1
nodebasedGSMethod 100000 1.9 0 yes 1e-13
"""


def sim2_text_fixture():
    """The reference's V2 ``sim`` (``make -C oracle ref2``) on a committed V2
    config: its fastmode_nodebasedGS.out and the solve lines of default.log."""
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref2"], check=True)
    with open(os.path.join(HERE, "sim_v2_6x7.cfg"), "w") as f:
        f.write(SIM2_TEXT_CFG)
    with tempfile.TemporaryDirectory() as td:
        shutil.copy(os.path.join(HERE, "sim_v2_6x7.cfg"), os.path.join(td, "config"))
        out = subprocess.run([SIM + "2"], cwd=td, capture_output=True, text=True, check=True).stdout
        assert "Run end && Succeed" in out, out
        shutil.copy(os.path.join(td, "fastmode_nodebasedGS.out"), os.path.join(HERE, "sim_v2_6x7.nodebasedGS.out"))
        with open(os.path.join(td, "default.log")) as f:
            keep = [ln for ln in f.read().splitlines() if re.match(r"(threshould|error I sum|Set array size)", ln)]
        with open(os.path.join(HERE, "sim_v2_6x7.log"), "w") as f:
            f.write("\n".join(keep) + "\n")


def pimtorch_layer_fixtures():
    """Ref-column arrays, negative-pulse inputs and Conv2d_sp evaluation, through
    the reference's own splitArr_matmul_nn and Conv2d_sp with the droop solve."""
    import torch
    td, cc, ids, sa = import_pimtorch()
    try:
        import fixedPoint.nn.modules.conv_split as cs
        P = cc.phyArrParams
        P.cpp_ir_drop_accelerate_flag = True
        P.cpp_ir_drop_accelerate = _DroopSolve()
        P.IRdropMode = cc.ir_drop_mode.accurate_GS_math
        P.useOUSize = False
        P.useBNN = False
        P.sigma = 0
        # linear layers: (name, params, input mode, array mode, dac bits, x, w)
        lin = [
            ("ref_c2", dict(Ron=1e3, Roff=1e6, cellBits=2, rows=32, cols=24, inputMaxVoltage=0.2, adc_bits=8),
             "complement_code", "Ref", 1,
             lambda r: r.integers(0, 256, (6, 90)).astype(np.float32),
             lambda r: (r.standard_normal((90, 50)) * 0.05).astype(np.float32)),
            ("ref_signed", dict(Ron=1e3, Roff=1e6, cellBits=1, rows=64, cols=64, inputMaxVoltage=1.0, adc_bits=10),
             "complement_code", "Ref", 1,
             lambda r: r.standard_normal((4, 130)).astype(np.float32),
             lambda r: (r.standard_normal((130, 70)) * 0.1).astype(np.float32)),
            ("negpulse_pn_dac2", dict(Ron=1e3, Roff=1e6, cellBits=2, rows=32, cols=32, inputMaxVoltage=0.3,
                                      adc_bits=9, dac_bits=2),
             "neg_pulse", "PN", 2,
             lambda r: r.standard_normal((5, 75)).astype(np.float32),
             lambda r: (r.standard_normal((75, 40)) * 0.08).astype(np.float32)),
            ("negpulse_ref", dict(Ron=1e3, Roff=1e6, cellBits=1, rows=32, cols=16, inputMaxVoltage=1.0, adc_bits=10),
             "neg_pulse", "Ref", 1,
             lambda r: r.standard_normal((3, 40)).astype(np.float32),
             lambda r: (r.standard_normal((40, 33)) * 0.1).astype(np.float32)),
        ]
        for name, kw, imode, amode, dac, mkx, mkw in lin:
            p = intstages.ArrayParams(**kw)
            set_params(cc, p)
            P.inputVmode = getattr(cc.input_v_mode, imode)
            r = np.random.default_rng(100 + len(name))
            x, w = mkx(r), mkw(r)
            y = sa.splitArr_matmul_nn(torch.from_numpy(x), torch.from_numpy(w), 8, dac, p.adc_bits, 10, 8,
                                      getattr(cc.phyArrMode, amode), torch.float32)
            np.savez_compressed(os.path.join(HERE, "pimtorch_layer_%s.npz" % name), x=x, w=w, y=y.numpy(),
                                input_mode=imode, arr_mode=amode, **dict(kw, dac_bits=dac))
        # Conv2d_sp: (name, params, array mode, use_fp_bias, conv args, input shape, big value at an
        # input row the unfold never reads)
        conv = [
            ("conv_pn", dict(Ron=1e3, Roff=1e6, cellBits=2, rows=32, cols=32, inputMaxVoltage=0.2, adc_bits=8),
             "PN", True, dict(in_channels=3, out_channels=10, kernel_size=(3, 3), stride=1, padding=1),
             (2, 3, 9, 9), None),
            ("conv_ref_stride", dict(Ron=1e3, Roff=1e6, cellBits=1, rows=16, cols=16, inputMaxVoltage=1.0,
                                     adc_bits=10),
             "Ref", False, dict(in_channels=4, out_channels=20, kernel_size=(2, 3), stride=(3, 1), padding=(0, 1),
                                dilation=(1, 2)),
             (2, 4, 11, 7), 5),
        ]
        for name, kw, amode, fpb, cargs, shape, hole in conv:
            p = intstages.ArrayParams(**kw)
            set_params(cc, p)
            P.inputVmode = cc.input_v_mode.complement_code
            r = np.random.default_rng(200 + len(name))
            torch.manual_seed(7)
            layer = cs.Conv2d_sp(**cargs, bias=True, input_bit_width=8, output_bit_width=10, weight_bit_width=8,
                                 dac_bit_width=1, adc_bit_width=p.adc_bits,
                                 phy_arr_mode=getattr(cc.phyArrMode, amode), use_fp_bias=fpb)
            x = r.standard_normal(shape).astype(np.float32)
            if hole is not None:
                x[:, :, hole, :] = 40.0
            layer.eval()
            with torch.no_grad():
                y = layer(torch.from_numpy(x))
            np.savez_compressed(os.path.join(HERE, "pimtorch_layer_%s.npz" % name), x=x,
                                weight=layer.fp_weight.detach().numpy(), bias=layer.fp_bias.detach().numpy(),
                                y=y.numpy(), arr_mode=amode, use_fp_bias=fpb,
                                **{"conv_" + k: np.array(v) for k, v in cargs.items()}, **kw)
    finally:
        shutil.rmtree(td, ignore_errors=True)


def variation_fixtures():
    """Cycle-to-cycle conductance variation in the layer path: the reference's
    splitArr_matmul_nn with phyArrParams.sigma = 0.1, its network generator
    reset to the default seed first (variations.reset_all), the droop solve
    standing in for the IR-drop solve; a PN and a Ref-column case."""
    import torch
    td, cc, ids, sa = import_pimtorch()
    try:
        P = cc.phyArrParams
        P.cpp_ir_drop_accelerate_flag = True
        P.cpp_ir_drop_accelerate = _DroopSolve()
        P.IRdropMode = cc.ir_drop_mode.accurate_GS_math
        P.useOUSize = False
        P.useBNN = False
        P.inputVmode = cc.input_v_mode.complement_code
        cases = [
            ("var_pn", dict(Ron=1e3, Roff=1e6, cellBits=2, rows=32, cols=32, inputMaxVoltage=0.2, adc_bits=8), "PN",
             lambda r: r.integers(0, 256, (4, 70)).astype(np.float32),
             lambda r: (r.standard_normal((70, 40)) * 0.05).astype(np.float32)),
            ("var_ref", dict(Ron=1e3, Roff=1e6, cellBits=1, rows=32, cols=16, inputMaxVoltage=1.0, adc_bits=10), "Ref",
             lambda r: r.standard_normal((3, 40)).astype(np.float32),
             lambda r: (r.standard_normal((40, 20)) * 0.1).astype(np.float32)),
        ]
        for name, kw, amode, mkx, mkw in cases:
            p = intstages.ArrayParams(**kw)
            set_params(cc, p)
            P.sigma = 0.1
            r = np.random.default_rng(300 + len(name))
            x, w = mkx(r), mkw(r)
            cc.variations.reset_all()
            y = sa.splitArr_matmul_nn(torch.from_numpy(x), torch.from_numpy(w), 8, 1, p.adc_bits, 10, 8,
                                      getattr(cc.phyArrMode, amode), torch.float32)
            np.savez_compressed(os.path.join(HERE, "pimtorch_layer_%s.npz" % name), x=x, w=w, y=y.numpy(),
                                arr_mode=amode, sigma=0.1, seed=cc.variations.var_defaultSeed, **kw)
    finally:
        shutil.rmtree(td, ignore_errors=True)


if __name__ == "__main__":
    which = sys.argv[1:] or ["sim", "pimtorch", "layers", "variation", "fcm", "ir2s", "simtext", "sim2text"]
    if "sim2text" in which:
        sim2_text_fixture()
    if "simtext" in which:
        sim_text_fixture()
    if "ir2s" in which:
        ir2s_fixture()
    if "sim" in which:
        sim_fixtures()
    if "fcm" in which:
        fcm_fixture()
    if "pimtorch" in which:
        pimtorch_fixtures()
    if "layers" in which:
        pimtorch_layer_fixtures()
    if "variation" in which:
        variation_fixtures()
    print("fixtures written to", HERE)
