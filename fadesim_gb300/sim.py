"""Drop-in for the reference's V1 crossbar simulator, ``sim <config>``, on its
fast read (VMM) path, with the nodal solve on the GPU.

    python -m fadesim_gb300.sim [config] [-debug]
    python -m fadesim_gb300.sim --v2 [config]      (the V2 simulator's dialect)

The config is the reference's own command file (crossbarHspice/GenArray.cc:72-83:
one command per line, ``%`` and ``//`` lines skipped), read into the same array
state that ``array2D::setParas`` builds (crossbarHspice/2dArray.cc:24-873):
array size, cell resistance states and the state of every cell, the per-segment
line resistances, the line voltages and which lines are driven.  The commands
that evaluate the array are

  nodebasedGSMethod iters w mode [yes tol]   2dArray.cc:51-112 -> fastmode_nodebasedGS.out
  FCM gen|test [file]                        2dArray.cc:841-1011 -> IR_FCM.out (+ the FCM file)

and the output files keep the reference's layout byte for byte (2dArray.cc:1648-1679,
986-1008), so scripts that parse them (crossbarHspice/tests/print_best_omega.py,
check_iout.py) run unchanged; so do the stdout lines those scripts parse.

What differs is the solver.  The reference runs point Gauss-Seidel sweeps
(2dArray.cc:1551-1610) until the largest change of a sweep is below ``tol`` and
writes that iterate; here the same nodal system is solved by the GPU block line
relaxation to an estimated maximum node error of ``tol`` volts (floored at the
solver's working precision), so the files hold the converged voltages: the
reference's own iterate at ``tol`` 1e-8 is ~1.6e-6 V away from them, at 1e-11
within ~2e-9 V.  The iteration count printed on the "threshould break" line is
the line solver's (0-based index of its last iteration, as the reference
prints the index of its last sweep); ``w`` is the point-GS relaxation factor
and is ignored unless ``FADESIM_SIM_OMEGA=config`` is set, which runs the line
relaxation at that fixed factor instead of its adaptive one.

The GPU solver takes one wire conductance for every segment and grounded
bitline ends.  A config whose used segments differ (``setLineR``, ``rload``) or
whose bitline ends are driven (``setLineV down``) is refused with an error, as
are the netlist-only commands' outputs (``build``: SPICE netlist generation)
and the other solvers (``fastsolve``, ``ir_*``, the general-boundary GS), which
print a notice and are skipped.
"""
import os
import sys
import time

import numpy as np

_DIRS = {"up": 0, "left": 1, "down": 2, "right": 3}

# Commands that only shape the SPICE netlist or the transient stimulus; the
# fast path does not read what they set.
_NETLIST_ONLY = {"topString", "bottomString", "mode", "dc", "ac", "capacitance", "capacity", "setLineV++",
                 "senseCellV", "senseBitlineI", "senseWordlineI", "simpleWriteOne", "simpleWriteZero",
                 "simpleReadOut", "useRtypeReRAMCell", "selector"}
# Commands that run a solver this front-end does not provide.
_OTHER_SOLVERS = {"build", "fastsolve", "iras_table", "ir_aihwkit", "ir_scichina", "ir_neurosim", "ir_free",
                  "ir_pbia"}


class SimError(RuntimeError):
    """A config the fast path cannot evaluate (the reference throws or
    misbehaves on most of these)."""


def check_yes(s):
    """checkYes (2dArray.cc:16-22)."""
    return s.lower() in ("yes", "1", "true", "y", "t")


def _stof(s):
    """std::stof: the value rounded to float32, then widened back."""
    return float(np.float32(float(s)))


def _fmt_g(x):
    """operator<< on a double with the stream's default format (%g, 6 digits)."""
    return "%g" % x


def _fmt_e20(x):
    """std::scientific, setprecision(12), setw(20)."""
    return "%20.12e" % x


class Array2D:
    """The state ``array2D::setParas`` keeps for a single crossbar (2dArray.h:25-80):
    cell states ``arr`` [n, m], cell resistance states, per-segment wordline
    resistances RULine [n, m+1] (segment j feeds node (i, j) from its left) and
    bitline resistances RDLine [m, n+1] (segment i+1 joins node (i, j) to the
    one below it, RDLine[j][n] to the bitline end), line voltages v[d] and
    driven flags bv[d] per side d (up, left, down, right)."""

    def __init__(self, out=None, cwd="."):
        self.out = out if out is not None else sys.stdout
        self.cwd = cwd
        self.debug = False
        self.n = self.m = 0
        self.cellR_states = []
        self.inputV_states = []
        self.fast_mode = False
        self.r_load = [-1.0] * 4
        self.set_array_size(0, 0)
        self.solves = []  # (u, d, iout, iters) of every solve, for callers

    def log(self, *a):
        print(*a, file=self.out)

    def path(self, name):
        return os.path.join(self.cwd, name)

    def set_array_size(self, n, m):
        """setArraySize (2dArray.h:31-48)."""
        self.n, self.m = n, m
        self.arr = np.zeros((n, m), dtype=np.int64)
        self.RULine = np.zeros((n, m + 1))
        self.RDLine = np.zeros((m, n + 1))
        self.v = [np.zeros(m), np.zeros(n), np.zeros(m), np.zeros(n)]
        self.bv = [np.zeros(m, np.int64), np.zeros(n, np.int64), np.zeros(m, np.int64), np.zeros(n, np.int64)]
        self.r_load = [-1.0] * 4

    # -- config reading -------------------------------------------------------

    def read_config(self, text):
        """phyArray::readConfig (GenArray.cc:72-83): the first word of a line is
        the command, the rest of that line its arguments."""
        for line in text.splitlines():
            words = line.split(None, 1)
            if not words:
                continue
            cmd = words[0]
            if cmd.startswith("%") or cmd.startswith("//"):
                continue
            self.set_paras(cmd, words[1] if len(words) > 1 else "")

    def set_paras(self, s, t):
        """array2D::setParas (2dArray.cc:24-873), the commands the fast path reads."""
        a = t.split()
        if self.debug:
            self.log(s, t)
        if s == "arraySize":
            self.set_array_size(int(a[0]), int(a[1]))
            self.log("set array size to wordline = %d bitline = %d" % (self.n, self.m))
        elif s == "nodebasedGSMethod":
            self._cmd_nodebased_gs(a)
        elif s == "inputVstates":
            k = int(a[0])
            self.inputV_states = [float(x) for x in a[1:1 + k]]
        elif s == "randSetInputV":
            self._cmd_rand_set_input_v(a)
        elif s == "randSetR":
            self._cmd_rand_set_r(a)
        elif s == "cellRstates":
            k = int(a[0])
            self.cellR_states = [float(x) for x in a[1:1 + k]]
        elif s == "fastmode":
            if a and check_yes(a[0]):
                self.fast_mode = True
                k = int(a[1])
                self.cellR_states = [float(x) for x in a[2:2 + k]]
            else:
                self.fast_mode = False
            self.log("fast mode " + ("on" if self.fast_mode else "off"))
        elif s == "line_resistance":
            r = float(a[0])
            self.RULine[:] = r
            self.RDLine[:] = r
            self.log("set line_resistance to " + _fmt_g(r))
        elif s == "rload":
            self._cmd_rload(a[0], float(a[1]))
        elif s == "setLineR":
            x, y, z = int(a[1]), int(a[2]), float(a[3])
            tgt = self.RULine if a[0] == "up" else self.RDLine
            tgt[self._at(tgt.shape[0], x), self._at(tgt.shape[1], y)] = z
        elif s in ("setUseLine", "setNotUseLine", "setUseLine++"):
            d = _DIRS.get(a[0], 0)
            val = {"setUseLine": 1, "setNotUseLine": 0, "setUseLine++": 2}[s]
            xs = [int(x) for x in a[1:]] if s != "setUseLine++" else [int(a[1])]
            for x in xs:
                if x == -1:
                    self.bv[d][:] = val
                else:
                    self.bv[d][self._at(len(self.bv[d]), x)] = val
        elif s == "setLineV":
            d, x, y = _DIRS.get(a[0], 0), int(a[1]), float(a[2])
            if x == -1:
                self.v[d][:] = y
            else:
                self.v[d][self._at(len(self.v[d]), x)] = y
        elif s == "setCellR":
            x, y, z = int(a[0]), int(a[1]), int(a[2])
            self.log("setCellR %d %d %d" % (x, y, z))
            rows = slice(None) if x == -1 else self._at(self.n, x)
            cols = slice(None) if y == -1 else self._at(self.m, y)
            self.arr[rows, cols] = z
        elif s == "FCM":
            self._cmd_fcm(a)
        elif s in _NETLIST_ONLY:
            pass
        elif s in _OTHER_SOLVERS:
            self.log("%s: not provided by this front-end (nodebasedGSMethod and FCM are), skipped" % s)
        else:
            self.log("wrong commnd")
        return True

    @staticmethod
    def _at(size, i):
        """vector::at: an index outside [0, size) throws."""
        if not 0 <= i < size:
            raise SimError("index %d out of range [0, %d)" % (i, size))
        return i

    def _cmd_rload(self, side, r):
        """rload (2dArray.cc:282-310)."""
        if side == "all":
            self.RULine[:, 0] = self.RULine[:, -1] = r
            self.RDLine[:, 0] = self.RDLine[:, -1] = r
            self.r_load = [r] * 4
            self.log("set all line resistance load to r_load %s omega" % _fmt_g(r))
        elif side in ("left", "right"):
            self.RULine[:, 0 if side == "left" else -1] = r
            self.r_load[1 if side == "left" else 3] = r
        elif side in ("down", "up"):
            self.RDLine[:, 0 if side == "up" else -1] = r
            self.r_load[0 if side == "up" else 2] = r
        self.log("set " + side + " line resistance load to r_load " + _fmt_g(r) + " omega")

    def _rand_pick(self, p, count, rng):
        """The cumulative draw of randSetR / randSetInputV (2dArray.cc:121-219),
        including its running sum that starts at the third entry (``if (i>1)``)."""
        p = list(p)
        if abs(sum(p) - 1) > 1e-6:
            raise SimError("Error: p sum is not 1")
        for i in range(2, len(p)):
            p[i] += p[i - 1]
        out = np.empty(count, dtype=np.int64)
        for c in range(count):
            rd = int(rng.integers(0, 10000))
            out[c] = next((k for k in range(len(p)) if p[k] * 10000 > rd), len(p) - 1)
        return out

    def _cmd_rand_set_r(self, a):
        rng = np.random.default_rng(int(time.time()))
        k = len(self.cellR_states)
        self.arr[:] = self._rand_pick([float(x) for x in a[:k]], self.n * self.m, rng).reshape(self.n, self.m)
        self.log("randSetR finish")

    def _cmd_rand_set_input_v(self, a):
        d = _DIRS.get(a[0], 0)
        k = len(self.inputV_states)
        rng = np.random.default_rng(int(time.time()))
        idx = self._rand_pick([float(x) for x in a[1:1 + k]], len(self.v[d]), rng)
        self.v[d][:] = np.asarray(self.inputV_states)[idx]
        self.log("randSetInputV " + a[0] + " finish")

    # -- the fast VMM path ------------------------------------------------------

    def conductances(self):
        if not len(self.cellR_states):
            raise SimError("no cell resistance states (cellRstates / fastmode yes)")
        if self.arr.size and (self.arr.min() < 0 or self.arr.max() >= len(self.cellR_states)):
            raise SimError("cell state outside the %d resistance states" % len(self.cellR_states))
        return 1.0 / np.asarray(self.cellR_states, dtype=np.float64)[self.arr]

    def wire_conductance(self):
        """The one wire conductance the GPU solve takes.  nodeBasedGS reads the
        wordline segments RULine[i][0..m-1] and the bitline segments
        RDLine[j][1..n] (2dArray.cc:1561-1587); they must all be equal."""
        used = self._used_segments()
        if not used.size or np.any(used <= 0):
            raise SimError("line resistance not set (line_resistance)")
        if np.any(used != used[0]):
            raise SimError("the GPU solver takes one wire resistance; this config sets %d different line "
                           "segment values (setLineR / rload)" % len(np.unique(used)))
        return 1.0 / used[0]

    def _used_segments(self):
        return np.concatenate([self.RULine[:, :self.m].ravel(), self.RDLine[:, 1:].ravel()])

    def vmm_boundary(self):
        """check_status (2dArray.cc:85-101): wordlines driven from the left only,
        bitlines sensed at the bottom only."""
        return not (np.any(self.bv[0] == 1) or np.any(self.bv[1] == 0) or np.any(self.bv[2] == 0)
                    or np.any(self.bv[3] == 1))

    def solve(self, tol, omega=0.0, max_iters=0):
        """The converged voltages of the system nodeBasedGS iterates on
        (vin = v[left], bitline ends at v[down]): (vup, vdown, iters, status)."""
        if np.any(self.v[2] != 0):
            raise SimError("the GPU solver grounds every bitline end; setLineV down must be 0")
        g = self.conductances()
        gw = self.wire_conductance()
        import torch
        from . import cpp_ir_drop_accelerate as acc
        n, m = self.n, self.m
        inp = torch.tensor(self.v[1], dtype=torch.float64).reshape(1, 1, n).cuda()
        G = torch.tensor(g, dtype=torch.float64).reshape(1, n, m).cuda()
        planes, st, it = acc.ir_drop_gs_ex(inp, G, 1, n, m, 1, 1, g_wire=gw, ret_V=2, tol_v=tol,
                                           omega=omega if omega > 0 else None,
                                           max_iters=max_iters if max_iters > 0 else None, return_iters=True)
        p = planes.reshape(2, n, m).cpu().numpy()
        return p[0], p[1], int(it.reshape(-1)[0]), int(st["status_or"])

    def err_i_sum(self, vup, vdown, g):
        """nodeBasedGS's KCL check (2dArray.cc:1619-1645): the absolute current
        mismatch summed over the wordline nodes of columns 1..m-1 and the bitline
        nodes of rows 0..n-2, with the wire conductance 1/RDLine[0][0]."""
        gw = 1.0 / self.RDLine[0, 0]
        n, m = self.n, self.m
        s = 0.0
        if m > 2:
            s += np.abs((vup[:, :-2] - vup[:, 1:-1] + vup[:, 2:] - vup[:, 1:-1]) * gw
                        + (vdown[:, 1:-1] - vup[:, 1:-1]) * g[:, 1:-1]).sum()
        if m > 1:
            s += np.abs((vup[:, m - 2] - vup[:, m - 1]) * gw + (vdown[:, m - 1] - vup[:, m - 1]) * g[:, m - 1]).sum()
        s += np.abs((vup[0] - vdown[0]) * g[0] + ((vdown[1] - vdown[0]) if n > 1 else 0.0) * gw).sum()
        if n > 2:
            s += np.abs((vup[1:-1] - vdown[1:-1]) * g[1:-1]
                        + (vdown[:-2] - vdown[1:-1] + vdown[2:] - vdown[1:-1]) * gw).sum()
        return float(s)

    def _cmd_nodebased_gs(self, a):
        """nodebasedGSMethod iter_time w mode [yes threshold] (2dArray.cc:51-112)."""
        iter_time, w, mode, enable_break, thr = -1, 1.0, 0, False, 0.0
        for cnt, tok in enumerate(a):
            if cnt == 0:
                iter_time = int(tok)
            elif cnt == 1:
                w = _stof(tok)
            elif cnt == 2:
                mode = int(tok)
            else:
                if check_yes(tok):
                    enable_break = True
                    thr = float(a[cnt + 1]) if cnt + 1 < len(a) else 0.0
                break
        self.log("evalutate ir drop using GS-method, w = %s , print to file fastmode_nodebasedGS.out" % _fmt_g(w))
        if mode & 2:
            raise SimError("nodebasedGSMethod mode bit 2 (write the initial estimate without iterating) is not "
                           "provided by this front-end")
        if not (self.n >= 2 and self.m >= 2):
            self.log("nodebase fast mode m and n should greater than 2")
            return
        res = self._nodebased_gs(iter_time, w, enable_break, thr)
        if self.vmm_boundary():
            self.log("evalutate ir drop using GS-method (special version for vmm only), w = %s , print to file "
                     "fastmode_nodebasedGS.out" % _fmt_g(w))
            # the reference solves the same system a second time; its result is this one
            self._report(*res)
        else:
            self.log("general GS-method (a boundary other than left-driven wordlines and grounded bitlines) is "
                     "not provided by this front-end, skipped")
        self.log("\n")

    def _nodebased_gs(self, iter_time, w, enable_break, thr):
        from . import cpp_ir_drop_accelerate as acc
        tol = thr if enable_break and thr > 0 else acc.options.tol_v
        omega = float(w) if os.environ.get("FADESIM_SIM_OMEGA", "") == "config" else 0.0
        t0 = time.perf_counter()
        vup, vdown, iters, status = self.solve(tol, omega, iter_time if omega > 0 else 0)
        elapsed = time.perf_counter() - t0
        res = (vup, vdown, iters, status, enable_break, elapsed)
        self._report(*res)
        return res

    def _report(self, vup, vdown, iters, status, enable_break, elapsed):
        g = self.conductances()
        self.log("nodebase fast mode time = %s s" % _fmt_g(elapsed))
        from ._lib import ST_MAXITER, ST_NONFINITE
        if status & (ST_MAXITER | ST_NONFINITE):
            self.log("warning: the line solve stopped without meeting its tolerance (status %d)" % status)
        elif enable_break:
            self.log("threshould break, iter times =  %d" % (iters - 1))
        iout = ((vup - vdown) * g).sum(axis=0)
        err = self.err_i_sum(vup, vdown, g)
        with open(self.path("fastmode_nodebasedGS.out"), "w") as f:
            f.write(format_nodebased_out(err, vup, vdown, iout))
        self.log("error I sum = " + _fmt_g(err))
        self.solves.append((vup, vdown, iout, iters))

    # -- FCM ------------------------------------------------------------------------

    def _cmd_fcm(self, a):
        """FCM [test|gen] [file] (2dArray.cc:841-867, IR_FCM :869-1011)."""
        mode = a[0] if a else "test"
        test = mode == "test"
        file = a[1] if len(a) > 1 else ("IR_FCM.out" if test else "IR_FCM.conf")
        if test:
            self.log("Test according to IR_FCM.conf, and test output to file IR_FCM.out")
            self._fcm_test(file)
        else:
            self.log("Generate G', i.e., G_non_ideal corresponding to origin G with line resistance effect, to file "
                     + file)
            self._fcm_gen(file)

    def _fcm_test(self, file):
        """Mode 0 (2dArray.cc:873-939): read the FCM file, check it against this
        array, write I_j = sum_i G_eff[i][j] v_i."""
        with open(self.path(file)) as f:
            tok = f.read().split()
        n, m, k = int(tok[0]), int(tok[1]), int(tok[2])
        if not (n == self.n and m == self.m and k == len(self.cellR_states)):
            self.log("fcm config file has wrong parameters!")
            return
        pos = 3
        for i in range(k):
            if abs(float(tok[pos + i]) - self.cellR_states[i]) > 1e-5:
                self.log("fcm config file wrong, has wrong r states")
                return
        pos += k
        states = np.array([int(x) for x in tok[pos:pos + n * m]]).reshape(n, m)
        if np.any(states != self.arr):
            self.log("fcm config file wrong, has wrong cell states")
            return
        pos += n * m
        g_eff = np.array([float(x) for x in tok[pos:pos + n * m]]).reshape(n, m)
        iout = np.zeros(m)
        for i in range(n):
            iout += g_eff[i] * self.v[1][i]
        with open(self.path("IR_FCM.out"), "w") as f:
            f.write(format_fcm_iout(iout, trailing_space=False))

    def _fcm_gen(self, file):
        """Mode 1 (2dArray.cc:940-1008): one unit-voltage solve per wordline gives
        G_eff; write I = v G_eff to IR_FCM.out and the FCM file."""
        g = self.conductances()
        gw = self.wire_conductance()
        import torch
        from . import geff
        G = torch.tensor(g, dtype=torch.float64).reshape(1, self.n, self.m).cuda()
        g_eff = geff.effective_conductance(G, gw, 1.0, tol_v=1e-13)[0].cpu().numpy()
        iout = np.zeros(self.m)
        for i in range(self.n):
            iout += g_eff[i] * self.v[1][i]
        with open(self.path("IR_FCM.out"), "w") as f:
            f.write(format_fcm_iout(iout, trailing_space=True))
        with open(self.path(file), "w") as f:
            f.write(geff.fcm_text(self.arr, self.cellR_states, g_eff))
        self.g_eff = g_eff


# Commands the V2 simulator registers (crossbarHspice/V2/main.cpp:84-115); any
# other name is an error there.
_V2_COMMANDS = {"empty", "arraySize", "line_resistance", "setLineR", "rload", "setUseLine", "setNotUseLine",
                "setUseLine++", "setLineV", "setLineV++", "setCellR", "cellRStates", "inputVStates", "topString",
                "bottomString", "build", "capacity", "capacitance", "senseCellV", "senseBitlineI",
                "senseWordlineI", "simpleWriteOne", "simpleWriteZero", "randSetInputV", "useRtypeReRAMCell",
                "randSetR", "dc", "ac", "simpleReadOut", "nodebasedGSMethod"}


class Array2DV2(Array2D):
    """The V2 simulator's dialect (crossbarHspice/V2): the same array state and
    fast path, with its command names (``cellRStates``, ``inputVStates``), ``#``
    comments, an error for any unregistered command or malformed argument list
    (V2/command.h:63-118, caught in V2/main.cpp:27-31 with the line number), a
    single ``nodebasedGSMethod`` solve with ``w`` read by stod and mode bits 0
    and 2 refused (V2/concrete_command.h:1097-1135, 1186-1210), messages
    collected into default.log, and wordline segments read from RDLine
    (V2/concrete_command.h:1214 aliases RULine to it)."""

    def __init__(self, out=None, cwd="."):
        self.logbuf = []
        super().__init__(out, cwd)

    def log(self, *a):
        self.logbuf.append(" ".join(str(x) for x in a))

    def read_config(self, text):
        """read_file_and_execute (V2/main.cpp:48-59); an error names its line."""
        for no, line in enumerate(text.splitlines(), 1):
            words = line.split(None, 1)
            if not words or words[0] in ("%", "//", "#"):
                continue
            try:
                self.set_paras(words[0], words[1] if len(words) > 1 else "")
            except (SimError, ValueError, IndexError) as e:
                raise SimError("line %d: %s" % (no, e)) from None

    def set_paras(self, s, t):
        if s not in _V2_COMMANDS:
            raise SimError("Unknown command: " + s)
        a = t.split()
        if s in ("setUseLine", "setNotUseLine", "setUseLine++", "setLineV", "setLineV++") and a[0] not in _DIRS:
            raise SimError("Arg str not matched Direction should be up|left|down|right.")
        if s == "cellRStates":
            return super().set_paras("cellRstates", t)
        if s == "inputVStates":
            return super().set_paras("inputVstates", t)
        if s == "setLineR" and a[0] not in ("up", "down"):
            raise SimError("Arg Direction not matched:setLineR up|down x:int y:int r:double")
        if s == "arraySize":
            self.set_array_size(int(a[0]), int(a[1]))
            self.log("Set array size to ( %d, %d )" % (self.n, self.m))
            return True
        if s == "empty":
            return True
        return super().set_paras(s, t)

    def _used_segments(self):
        """Wordline segment (i, j) is RDLine[i][j] here, which exists in the
        [m][n+1] RDLine only when n <= m <= n+1; any other shape reads past it
        in the reference, so it needs one uniform resistance everywhere."""
        if self.n <= self.m <= self.n + 1:
            return np.concatenate([self.RDLine[:self.n, :self.m].ravel(), self.RDLine[:, 1:].ravel()])
        return self.RDLine.ravel()

    def _cmd_nodebased_gs(self, a):
        if len(a) < 3:
            raise SimError("args number not matched (<3)")
        if len(a) > 3 and len(a) != 5:
            raise SimError("args number not matched (!=5)")
        iter_time, w, mode = int(a[0]), float(a[1]), int(a[2])
        enable_break = len(a) > 3 and check_yes(a[3])
        thr = float(a[4]) if enable_break else 0.0
        if mode & 1:
            raise SimError("mode bit 0 is not supported now")
        if not (self.n >= 2 and self.m >= 2):
            raise SimError("m and n should greater than 2")
        if mode & 4:
            raise SimError("mode bit 2 is not supported now")
        if mode & 2:
            raise SimError("nodebasedGSMethod mode bit 1 (write the initial estimate without iterating) is not "
                           "provided by this front-end")
        self._nodebased_gs(iter_time, w, enable_break, thr)

    def _report(self, vup, vdown, iters, status, enable_break, elapsed):
        self.log("time = %s s" % _fmt_g(elapsed))
        from ._lib import ST_MAXITER, ST_NONFINITE
        g = self.conductances()
        if status & (ST_MAXITER | ST_NONFINITE):
            self.log("warning: the line solve stopped without meeting its tolerance (status %d)" % status)
        elif enable_break:
            self.log("threshould break, iter times =  %d" % (iters - 1))
        else:
            self.log("iter times = %d" % iters)
        iout = ((vup - vdown) * g).sum(axis=0)
        err = self.err_i_sum(vup, vdown, g)
        with open(self.path("fastmode_nodebasedGS.out"), "w") as f:
            f.write(format_nodebased_out(err, vup, vdown, iout))
        self.log("error I sum = " + _fmt_g(err))
        self.solves.append((vup, vdown, iout, iters))

    def write_log(self):
        """print_log_to_default_file (V2/main.cpp:61-66)."""
        with open(self.path("default.log"), "w") as f:
            f.write("\n--------Operation Log---------\n\n")
            f.write("".join(ln + "\n" for ln in self.logbuf))
            f.write("--------Log end--------\n")


def format_nodebased_out(err, vup, vdown, iout):
    """fastmode_nodebasedGS.out (2dArray.cc:1648-1679)."""
    lines = ["error I sum = " + _fmt_g(err), "vup = "]
    lines += ["".join(_fmt_e20(x) for x in row) for row in vup]
    lines += ["", "vdown = "]
    lines += ["".join(_fmt_e20(x) for x in row) for row in vdown]
    lines += ["", "iout = ", "".join(_fmt_e20(x) for x in iout)]
    return "\n".join(lines) + "\n"


def format_fcm_iout(iout, trailing_space):
    """IR_FCM.out: an empty line, "iout = ", the currents (2dArray.cc:931-938 in
    test mode; 976-985 in gen mode, where each value is followed by a space)."""
    sep = " " if trailing_space else ""
    return "\niout = \n" + "".join(_fmt_e20(x) + sep for x in iout) + "\n"


def parse_nodebased_out(text):
    """(err, vup, vdown, iout) from a fastmode_nodebasedGS.out text."""
    head, rest = text.split("vup = ", 1)
    up_s, rest = rest.split("vdown = ", 1)
    dn_s, io_s = rest.split("iout = ", 1)
    err = float(head.split("=")[1])
    rows = lambda s: np.array([[float(x) for x in ln.split()] for ln in s.strip().splitlines()])
    return err, rows(up_s), rows(dn_s), np.array([float(x) for x in io_s.split()])


def main_v2(argv):
    """V2/main.cpp:17-46: the config file (default ``config``), the log in
    default.log, errors reported with their line."""
    path = argv[0] if argv else "config"
    arr = Array2DV2()
    try:
        with open(path) as f:
            arr.read_config(f.read())
    except SimError as e:
        print("Error(s) occured in %s" % e)
        print("\n--------Operation Log---------\n")
        for ln in arr.logbuf:
            print(ln)
        print("--------Log end--------")
        return 1
    print("Log print to default.log")
    arr.write_log()
    print("--------Run end && Succeed---------")
    return 0


def main(argv=None):
    """main.cc:9-44: no argument reads ``config``; ``config -debug`` echoes every
    command; ``-3DH`` (the 3-D netlist generator) is not provided.  ``--v2``
    first reads the config in the V2 simulator's dialect instead."""
    argv = sys.argv[1:] if argv is None else argv
    if argv and argv[0] == "--v2":
        return main_v2(argv[1:])
    if len(argv) > 2:
        print("argc number wrong")
        return 0
    path = argv[0] if argv else "config"
    arr = Array2D()
    if len(argv) == 2:
        if argv[1] == "-debug":
            arr.debug = True
            print("in debug mode")
        elif argv[1] in ("-3DH", "-3dh"):
            print("3-D arrays (-3DH) are not provided by this front-end")
            return 1
    try:
        with open(path) as f:
            arr.read_config(f.read())
    except SimError as e:
        print("error: %s" % e)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
