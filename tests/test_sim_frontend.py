"""The ``sim`` config front-end on the CPU: config reading, the output file
layouts against the reference's own files, the KCL check, FCM test mode, and
the configs it refuses.  The fixtures under tests/golden/sim_v1_6x5.* are the
reference V1 ``sim`` run on the committed sim_v1_6x5.cfg."""
import io
import os

import numpy as np
import pytest

from fadesim_gb300 import sim
from oracle import augs

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def text(name):
    with open(os.path.join(HERE, name)) as f:
        return f.read()


def config_upto(cmd):
    """The committed config cut before the first line starting with ``cmd``."""
    cfg = text("sim_v1_6x5.cfg")
    return cfg[:cfg.index("\n" + cmd) + 1]


def read(cfg):
    buf = io.StringIO()
    a = sim.Array2D(out=buf)
    a.read_config(cfg)
    return a, buf.getvalue()


def test_config_state_matches_reference():
    a, out = read(config_upto("nodebasedGSMethod"))
    ref = text("sim_v1_6x5.stdout").splitlines()
    # the stdout lines of the setters, as the reference prints them
    for ln in out.splitlines():
        if ln.startswith(("set array size", "setCellR")):
            assert ln in ref
    # cell states as the reference's FCM file lists them
    tok = text("sim_v1_6x5.fcm.conf").split()
    n, m, k = int(tok[0]), int(tok[1]), int(tok[2])
    assert (a.n, a.m, len(a.cellR_states)) == (n, m, k)
    np.testing.assert_array_equal(a.arr, np.array([int(x) for x in tok[3 + k:3 + k + n * m]]).reshape(n, m))
    np.testing.assert_array_equal(a.v[1], [0.1, 0.25, 0.1, 0.1, 0.0, 0.1])
    assert a.wire_conductance() == 1 / 2.93
    assert a.vmm_boundary()


def test_nodebased_out_layout_is_byte_exact():
    txt = text("sim_v1_6x5.nodebasedGS.out")
    err, u, d, i = sim.parse_nodebased_out(txt)
    assert sim.format_nodebased_out(err, u, d, i) == txt


def test_err_i_sum_is_the_reference_kcl_check():
    """On the C restatement's planes (the reference's GS iterate, reproduced
    sweep for sweep) the KCL sum prints as the reference printed it."""
    a, _ = read(config_upto("nodebasedGSMethod"))
    g = a.conductances()
    up, dn, _, sweeps = augs.solve(g, a.v[1], 2.93, 100000, float(np.float32(1.9)), True, 1e-13)
    ref = [ln for ln in text("sim_v1_6x5.stdout").splitlines() if ln.startswith("error I sum")][0]
    assert "error I sum = " + sim._fmt_g(a.err_i_sum(up, dn, g)) == ref
    assert "threshould break, iter times =  %d" % (sweeps - 1) in text("sim_v1_6x5.stdout")


def test_fcm_test_mode_reproduces_reference_file(tmp_path):
    """FCM test reads G_eff from the FCM file and writes I = v G_eff: the same
    sums in the same order as the reference, so the same bytes."""
    (tmp_path / "fcm.conf").write_text(text("sim_v1_6x5.fcm.conf"))
    cfg = config_upto("nodebasedGSMethod") + "setLineV left 2 0.3\nFCM test fcm.conf\n"
    a = sim.Array2D(out=io.StringIO(), cwd=str(tmp_path))
    a.read_config(cfg)
    assert (tmp_path / "IR_FCM.out").read_text() == text("sim_v1_6x5.IR_FCM_test.out")


def test_fcm_test_mode_rejects_other_arrays(tmp_path):
    (tmp_path / "fcm.conf").write_text(text("sim_v1_6x5.fcm.conf"))
    buf = io.StringIO()
    a = sim.Array2D(out=buf, cwd=str(tmp_path))
    a.read_config(config_upto("nodebasedGSMethod") + "setCellR 0 0 1\nFCM test fcm.conf\n")
    assert "fcm config file wrong, has wrong cell states" in buf.getvalue()
    assert not (tmp_path / "IR_FCM.out").exists()


def test_fcm_gen_iout_layout():
    txt = text("sim_v1_6x5.IR_FCM_gen.out")
    vals = [float(x) for x in txt.split("iout = ")[1].split()]
    assert sim.format_fcm_iout(vals, trailing_space=True) == txt


@pytest.mark.parametrize("extra, msg", [
    ("setLineR up 2 3 5.0\n", "one wire resistance"),
    ("rload all 100\n", "one wire resistance"),
    ("setLineV down 1 0.1\n", "bitline end"),
    ("setCellR 1 1 7\n", "outside the 4 resistance states"),
])
def test_refused_configs(extra, msg):
    a, _ = read(config_upto("nodebasedGSMethod") + extra)
    with pytest.raises(sim.SimError, match=msg):
        a.set_paras("nodebasedGSMethod", "100000 1.9 0 yes 1e-13")


def test_rload_on_unused_segments_is_accepted():
    """RULine[i][m] (the open right end) and RDLine[j][0] (the open top) are not
    read by the nodal system."""
    a, _ = read(config_upto("nodebasedGSMethod") + "rload right 50\nrload up 70\n")
    assert a.wire_conductance() == 1 / 2.93


def test_general_boundary_and_other_commands():
    a, out = read(config_upto("nodebasedGSMethod") + "setUseLine up 2\nbuild out\nfastsolve 10 0\nfooBar 1\n")
    assert not a.vmm_boundary()
    assert "build: not provided" in out and "fastsolve: not provided" in out
    assert "wrong commnd" in out


def test_index_out_of_range_raises():
    with pytest.raises(sim.SimError):
        read("arraySize 4 4\nsetCellR 4 0 1\n")


def test_rand_pick_keeps_reference_cumulative_sum():
    """randSetR accumulates p from its third entry on (``if (i>1)``), so with
    p = (0.2, 0.3, 0.5) the thresholds are 0.2, 0.3, 0.8."""
    class Seq:
        def __init__(self, vals):
            self.vals = iter(vals)

        def integers(self, lo, hi):
            return next(self.vals)
    a = sim.Array2D(out=io.StringIO())
    got = a._rand_pick([0.2, 0.3, 0.5], 6, Seq([1999, 2000, 2999, 3000, 7999, 8000]))
    np.testing.assert_array_equal(got, [0, 1, 1, 2, 2, 2])
    with pytest.raises(sim.SimError):
        a._rand_pick([0.2, 0.3], 1, Seq([0]))


# -- the V2 dialect (tests/golden/sim_v2_6x7.*: the reference's V2 sim) ------------

def read_v2(cfg):
    a = sim.Array2DV2(out=io.StringIO())
    a.read_config(cfg)
    return a


def v2_config_upto(cmd):
    cfg = text("sim_v2_6x7.cfg")
    return cfg[:cfg.index("\n" + cmd) + 1]


def test_v2_config_and_kcl_check():
    a = read_v2(v2_config_upto("nodebasedGSMethod"))
    assert a.logbuf[0] == text("sim_v2_6x7.log").splitlines()[0]      # "Set array size to ( 6, 7 )"
    assert (a.n, a.m) == (6, 7) and a.cellR_states == [2e6, 1.6e6, 1.3e6, 1e6]
    np.testing.assert_array_equal(a.v[1], [0.2, 0.2, 0.2, 0.05, 0.2, 0.2])
    g = a.conductances()
    # V2 reads w with stod (V1: stof)
    up, dn, _, sweeps = augs.solve(g, a.v[1], 2.93, 100000, 1.9, True, 1e-13)
    log = text("sim_v2_6x7.log").splitlines()
    assert "threshould break, iter times =  %d" % (sweeps - 1) in log
    assert "error I sum = " + sim._fmt_g(a.err_i_sum(up, dn, g)) in log
    ref = sim.parse_nodebased_out(text("sim_v2_6x7.nodebasedGS.out"))
    assert np.abs(up - ref[1]).max() < 1e-12 and np.abs(dn - ref[2]).max() < 1e-12
    assert sim.format_nodebased_out(*ref) == text("sim_v2_6x7.nodebasedGS.out")


@pytest.mark.parametrize("line, msg", [
    ("selector no", "Unknown command: selector"),          # registered in V1 only
    ("cellRstates 2 1e6 2e6", "Unknown command: cellRstates"),
    ("setLineV middle 0 1", "Direction should be"),
    ("setLineR left 0 0 1", "setLineR up\\|down"),
    ("nodebasedGSMethod 100 1.9", "args number not matched \\(<3\\)"),
    ("nodebasedGSMethod 100 1.9 0 yes", "args number not matched \\(!=5\\)"),
    ("nodebasedGSMethod 100 1.9 1 yes 1e-9", "mode bit 0 is not supported now"),
    ("nodebasedGSMethod 100 1.9 4 yes 1e-9", "mode bit 2 is not supported now"),
])
def test_v2_errors_name_the_line(line, msg):
    cfg = v2_config_upto("nodebasedGSMethod")
    with pytest.raises(sim.SimError, match="line %d: .*%s" % (cfg.count("\n") + 1, msg)):
        read_v2(cfg + line + "\n")


def test_v2_segment_table_shapes():
    """V2 reads wordline segments from the bitline table: in range for
    n <= m <= n+1, otherwise the whole table must be uniform."""
    cfg = "arraySize 4 4\nline_resistance 2\nsetLineR down 3 0 9\n"
    assert read(cfg)[0].wire_conductance() == 0.5     # V1: RDLine[3][0] is the open top of bitline 3
    with pytest.raises(sim.SimError, match="one wire resistance"):
        read_v2(cfg).wire_conductance()               # V2: also the driver segment of wordline 3
    a = read_v2("arraySize 4 8\nline_resistance 2\nsetLineR down 7 0 9\n")
    with pytest.raises(sim.SimError, match="one wire resistance"):
        a.wire_conductance()


def test_v2_main_reports_errors(tmp_path, monkeypatch, capsys):
    (tmp_path / "config").write_text("arraySize 4 4\nselector no\n")
    monkeypatch.chdir(tmp_path)
    assert sim.main(["--v2"]) == 1
    out = capsys.readouterr().out
    assert out.startswith("Error(s) occured in line 2: Unknown command: selector")
    assert "Set array size to ( 4, 4 )" in out
