"""The ``sim`` config front-end end to end on the GPU: the reference's own
configs in, its output files out, against its converged results."""
import io
import os
import re

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def sim():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fadesim_gb300 import sim as m
    return m


def text(name):
    with open(os.path.join(HERE, name)) as f:
        return f.read()


def run(sim, cfg, tmp_path):
    buf = io.StringIO()
    a = sim.Array2D(out=buf, cwd=str(tmp_path))
    a.read_config(cfg)
    return a, buf.getvalue()


def sim_config(states, Rset, vin, r_wire, w, tol):
    """The config layout of the fixtures' generator (tests/golden/make_golden.py)."""
    n, m = states.shape
    lines = ["useRtypeReRAMCell yes", "cellRstates %d %s" % (len(Rset), " ".join("%.17g" % r for r in Rset)),
             "arraySize %d %d" % (n, m), "selector no", "line_resistance %.17g" % r_wire]
    lines += ["setCellR %d %d %d" % (i, j, states[i, j]) for i in range(n) for j in range(m)]
    lines += ["setUseLine left -1", "setUseLine down -1"]
    lines += ["setLineV left %d %.17g" % (i, vin[i]) for i in range(n)]
    lines += ["setLineV down -1 0", "senseBitlineI down -1", "nodebasedGSMethod 100000 %.17g 0 yes %.17g" % (w, tol)]
    return "\n".join(lines) + "\n"


def test_nodebased_gs_file_matches_reference(sim, tmp_path):
    cfg = text("sim_v1_6x5.cfg")
    cfg = cfg[:cfg.index("\nFCM gen") + 1]
    a, out = run(sim, cfg, tmp_path)
    got = (tmp_path / "fastmode_nodebasedGS.out").read_text()
    ref = text("sim_v1_6x5.nodebasedGS.out")
    # same layout: line count and field widths
    assert [len(ln) for ln in got.splitlines()[1:]] == [len(ln) for ln in ref.splitlines()[1:]]
    _, u, d, i = sim.parse_nodebased_out(got)
    _, ur, dr, ir = sim.parse_nodebased_out(ref)
    assert np.abs(u - ur).max() < 1e-10 and np.abs(d - dr).max() < 1e-10
    np.testing.assert_allclose(i, ir, rtol=1e-6)
    # the stdout lines the reference's scripts parse, twice (the reference solves twice)
    ev = [ln for ln in out.splitlines() if ln.startswith("evalutate")]
    assert ev == [ln for ln in text("sim_v1_6x5.stdout").splitlines() if ln.startswith("evalutate")]
    assert len(re.findall(r"^threshould break, iter times =  \d+$", out, re.M)) == 2
    assert len(re.findall(r"^nodebase fast mode time = \S+ s$", out, re.M)) == 2
    err = float(re.findall(r"^error I sum = (\S+)$", out, re.M)[-1])
    assert err < 1e-11  # KCL mismatch of the converged planes (amperes, summed over all nodes)


@pytest.mark.parametrize("fixture, bound", [("sim_v1_16x24.npz", 3e-9), ("sim_v1_128_tol1e-11.npz", 2e-8)])
def test_reference_fixtures_through_config(sim, gold, tmp_path, fixture, bound):
    z = gold(fixture)
    cfg = sim_config(z["states"], z["Rset"], z["vin"], float(z["r_wire"]), float(z["omega"]), float(z["tol"]))
    run(sim, cfg, tmp_path)
    _, u, d, i = sim.parse_nodebased_out((tmp_path / "fastmode_nodebasedGS.out").read_text())
    if "vup" in z.files:
        assert np.abs(u - z["vup"]).max() < bound and np.abs(d - z["vdown"]).max() < bound
    else:
        r = z["sample_rows"]
        assert np.abs(u[r] - z["vup_rows"]).max() < bound and np.abs(d[r] - z["vdown_rows"]).max() < bound
    np.testing.assert_allclose(i, z["iout"], rtol=1e-6)


def test_fcm_gen_matches_reference(sim, tmp_path):
    cfg = text("sim_v1_6x5.cfg")
    cfg = cfg[:cfg.index("\nsetLineV left 2 0.3") + 1]
    run(sim, cfg, tmp_path)
    got = (tmp_path / "fcm.conf").read_text().splitlines()
    ref = text("sim_v1_6x5.fcm.conf").splitlines()
    n = 6
    assert got[:2 + n] == ref[:2 + n]          # header, states of R, cell states: same bytes
    g = np.array([[float(x) for x in ln.split()] for ln in got[2 + n:]])
    gr = np.array([[float(x) for x in ln.split()] for ln in ref[2 + n:]])
    assert [len(ln) for ln in got] == [len(ln) for ln in ref]
    np.testing.assert_allclose(g, gr, rtol=1e-6)
    io_got = (tmp_path / "IR_FCM.out").read_text()
    io_ref = text("sim_v1_6x5.IR_FCM_gen.out")
    assert len(io_got) == len(io_ref)
    np.testing.assert_allclose([float(x) for x in io_got.split("=")[1].split()],
                               [float(x) for x in io_ref.split("=")[1].split()], rtol=1e-6)


def test_cli_reads_config_from_cwd(sim, tmp_path, monkeypatch, capsys):
    cfg = text("sim_v1_6x5.cfg")
    (tmp_path / "config").write_text(cfg[:cfg.index("\nFCM gen") + 1])
    monkeypatch.chdir(tmp_path)
    assert sim.main([]) == 0
    out = capsys.readouterr().out
    assert "threshould break, iter times =" in out
    assert (tmp_path / "fastmode_nodebasedGS.out").exists()


def test_config_omega_runs_fixed_relaxation(sim, tmp_path, monkeypatch):
    """FADESIM_SIM_OMEGA=config: the line relaxation at the config's w, so an
    omega search over the config sees the iteration count change with w."""
    cfg = text("sim_v1_6x5.cfg")
    base = cfg[:cfg.index("\nnodebasedGSMethod") + 1]
    monkeypatch.setenv("FADESIM_SIM_OMEGA", "config")
    iters = {}
    for w in (1.0, 1.8):
        a, out = run(sim, base + "nodebasedGSMethod 100000 %g 0 yes 1e-12\n" % w, tmp_path)
        iters[w] = a.solves[-1][3]
        _, u, d, _ = sim.parse_nodebased_out((tmp_path / "fastmode_nodebasedGS.out").read_text())
        _, ur, dr, _ = sim.parse_nodebased_out(text("sim_v1_6x5.nodebasedGS.out"))
        assert np.abs(u - ur).max() < 1e-10
    assert iters[1.0] < iters[1.8]


def test_v2_config_end_to_end(sim, tmp_path, monkeypatch, capsys):
    """The V2 dialect through its CLI: fastmode_nodebasedGS.out against the
    reference V2 sim's converged file, default.log with the solve lines."""
    (tmp_path / "config").write_text(text("sim_v2_6x7.cfg"))
    monkeypatch.chdir(tmp_path)
    assert sim.main(["--v2"]) == 0
    assert capsys.readouterr().out.endswith("--------Run end && Succeed---------\n")
    got = (tmp_path / "fastmode_nodebasedGS.out").read_text()
    ref = text("sim_v2_6x7.nodebasedGS.out")
    assert [len(ln) for ln in got.splitlines()[1:]] == [len(ln) for ln in ref.splitlines()[1:]]
    _, u, d, i = sim.parse_nodebased_out(got)
    _, ur, dr, ir = sim.parse_nodebased_out(ref)
    assert np.abs(u - ur).max() < 1e-10 and np.abs(d - dr).max() < 1e-10
    np.testing.assert_allclose(i, ir, rtol=1e-6)
    log = (tmp_path / "default.log").read_text()
    assert "Set array size to ( 6, 7 )" in log
    assert re.search(r"^threshould break, iter times =  \d+$", log, re.M)
