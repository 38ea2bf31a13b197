"""Drop-in for PimTorch's ``cpp_ir_drop_accelerate`` extension module.

PimTorch builds that module from ``fixedPoint/SplitArrCuda/split_arr_matmul.cu``
at import (``fixedPoint/nn/commonConst.py:278-280``) and calls
``phyArrParams.cpp_ir_drop_accelerate.ir_drop_gs(...)`` for every input bit,
weight slice and PN array (``fixedPoint/nn/splitArrayArithmetic.py:488-511``).
This module exposes the same function with the same arguments, checks, output
shapes and dtype handling; the solve runs in ``libfadesim_gb300.so``.

What differs is the answer's definition under the default method: the
reference runs ``iter_times`` node sweeps with relaxation ``beta`` (or stops on
its delta break), which at PimTorch's defaults (600 sweeps, beta 1.9) leaves a
128x128 array millivolts from the nodal solution.  Here every (tile, vector)
pair is solved to ``options.tol_v`` (1e-8 V) of the nodal solution, so results
match the reference's converged solver.  ``options.method = "sweeps"`` (or
``FADESIM_METHOD=sweeps`` in the environment) reproduces the reference's own
sweep order for exactly ``iter_times`` sweeps instead.

Solve status.  The reference returns whatever its sweeps reached.  Here every
solve also reports whether it met the tolerance, hit the iteration cap, or met
non-finite values; ``ir_drop_gs`` reads that status back after each call and,
with ``options.check_status`` "warn" (the default, or ``FADESIM_CHECK_STATUS``),
issues a ``SolveStatusWarning`` for a capped or non-finite solve, with "raise"
raises ``SolveStatusError``, with "off" skips the read (no host synchronisation).
"""
import ctypes
import math
import os
import warnings
from dataclasses import dataclass

import torch

from . import _lib

_METHODS = {"auto": _lib.METHOD_AUTO, "line": _lib.METHOD_LINE, "rbsor": _lib.METHOD_RBSOR,
            "sweeps": _lib.METHOD_SWEEPS, "line_coarse": _lib.METHOD_LINE_COARSE}


@dataclass
class SolverOptions:
    """Knobs the reference does not have; set them here, never in commonConst.py."""
    method: str = os.environ.get("FADESIM_METHOD", "auto")
    tol_v: float = 1e-8
    max_iters: int = 0           # 0: method default
    residual_period: int = 0     # 0: adaptive; k > 0: precise residual every k line iterations; -1: FP32 only
    omega: float = 0.0           # 0: adaptive (line) / size formula (rbsor)
    vectors_per_cta: int = 0     # 0: automatic
    residual: str = "ff"         # precise residual: "ff" (float-float on the FP32 pipe) or "fp64"
    read_noise_sigma: float = 0.0  # > 0: Gaussian read noise, sigma relative to each cell current
    noise_seed: int = 0
    check_status: str = os.environ.get("FADESIM_CHECK_STATUS", "warn")  # "warn", "raise" or "off"
    kernel_ld: int = 0           # 0: layout by tile size; 32/64/128 tile per CTA, 256/512 tile per cluster
    fp32_limit: bool = False     # line_coarse, full 128x128 tiles: iterate past the FP32 floor until the corrections stall

    def to_c(self, method=None):
        m = method if method is not None else self.method
        if m not in _METHODS:
            raise ValueError("unknown method %r (one of %s)" % (m, sorted(_METHODS)))
        if self.residual not in ("fp64", "ff"):
            raise ValueError("residual must be 'fp64' or 'ff'")
        return _lib.SolveOpts(_METHODS[m], float(self.tol_v), int(self.max_iters), int(self.residual_period),
                              float(self.omega), int(self.vectors_per_cta), 1 if self.residual == "fp64" else 0,
                              float(self.read_noise_sigma), int(self.noise_seed) & (2 ** 64 - 1),
                              int(self.kernel_ld), 1 if self.fp32_limit else 0)


options = SolverOptions()


class SolveStatusWarning(RuntimeWarning):
    """A solve stopped at its iteration cap or met non-finite values."""


class SolveStatusError(RuntimeError):
    """Raised instead of SolveStatusWarning under check_status = "raise"."""


def status_message(status_or, solves, method):
    """What the OR of the per-solve status bits says went wrong, or None.  An
    iteration cap is a failure for the converging methods only: the sweep
    method runs exactly iter_times sweeps, as the reference does."""
    problems = []
    if status_or & _lib.ST_NONFINITE:
        problems.append("non-finite values (NaN or inf in the inputs or the iterate)")
    if (status_or & _lib.ST_MAXITER) and method != "sweeps":
        problems.append("the iteration cap before reaching the tolerance")
    if not problems:
        return None
    return "IR-drop solve: at least one of %d solves ended with %s" % (solves, " and ".join(problems))


def resolved_method(method, row_size, col_size):
    """The method "auto" runs: the line relaxation up to 512 x 512, else the sweep order."""
    if method == "auto":
        return "line" if max(row_size, col_size) <= 512 else "sweeps"
    return method


def check_solve_status(stats, method, policy):
    """Apply the check_status policy to a stats dict (solves, status_or, ...)."""
    if policy == "off" or stats is None:
        return
    if policy not in ("warn", "raise"):
        raise ValueError("check_status must be 'warn', 'raise' or 'off'")
    msg = status_message(int(stats["status_or"]), int(stats["solves"]), method)
    if msg is None:
        return
    if policy == "raise":
        raise SolveStatusError(msg)
    warnings.warn(msg, SolveStatusWarning, stacklevel=3)


def _check_input(t, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError("%s must be a CUDA tensor" % name)
    if not t.is_contiguous():
        raise RuntimeError("%s must be contiguous" % name)


def _solve(input, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire, beta, enable_break,
           break_threshould, nonlinear_cell_enable, nonlinear_params, ret_V, opts, want_stats, want_iters, out=None):
    _check_input(input, "input")
    _check_input(G, "G")
    if row_size < 2:
        raise RuntimeError("row_size should be >=2")
    if col_size < 2:
        raise RuntimeError("col_size should be >=2")
    if input.dtype not in (torch.float32, torch.float64) or G.dtype != input.dtype:
        raise RuntimeError("input and G must both be float32 or both float64")
    if input.device != G.device:
        raise RuntimeError("input and G must be on the same device")
    if input.numel() != batch_size * numX * row_size:
        raise RuntimeError("input must hold batch_size*numX*row_size elements")
    if G.numel() != numX * row_size * numY * col_size:
        raise RuntimeError("G must hold numX*row_size*numY*col_size elements")
    lib = _lib.load()
    dtype = _lib.F64 if input.dtype == torch.float64 else _lib.F32
    if ret_V == 2:
        shape = (batch_size, numX, numY, 2, row_size, col_size)
    elif ret_V:
        shape = (batch_size, numX, numY, row_size, col_size)
    else:
        shape = (batch_size, numX, numY * col_size)
    if out is None:
        out = torch.empty(shape, dtype=input.dtype, device=input.device)
    elif (not out.is_contiguous() or out.dtype != input.dtype or out.device != input.device
          or out.numel() != math.prod(shape)):
        raise RuntimeError("out must be a contiguous %s tensor of %d elements on %s" % (input.dtype, math.prod(shape),
                                                                                      input.device))
    iters = None
    if want_iters:
        iters = torch.empty((batch_size, numX, numY), dtype=torch.int32, device=input.device)
    params = [float(v) for v in (nonlinear_params or [])]
    cparams = (ctypes.c_double * max(1, len(params)))(*params) if params else None
    stats = _lib.SolveStats()
    with torch.cuda.device(input.device):
        stream = torch.cuda.current_stream(input.device).cuda_stream
        rc = lib.fadesim_ir_drop_gs_ex(dtype, input.data_ptr(), G.data_ptr(), int(batch_size), int(row_size),
                                       int(col_size), int(numX), int(numY), int(iter_times), float(g_wire),
                                       float(beta), int(bool(enable_break)), float(break_threshould),
                                       int(bool(nonlinear_cell_enable)), cparams, len(params), 2 if ret_V == 2 else int(bool(ret_V)),
                                       out.data_ptr(), ctypes.byref(opts),
                                       ctypes.byref(stats) if want_stats else None,
                                       iters.data_ptr() if want_iters else None, stream)
    _lib.check(rc)
    return out, (stats if want_stats else None), iters


def ir_drop_gs(input, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire, beta, enable_break,
               break_threshould, nonlinear_cell_enable, nonlinear_params, ret_V=False):
    """Same contract as the reference's ``ir_drop_gs`` (split_arr_matmul.cu:204-220).

    input [batch, numX, rows] and G [numX, rows, numY*cols], contiguous CUDA,
    float32 or float64; returns bitline currents [batch, numX, numY*cols], or
    the cell voltages [batch, numX, numY, rows, cols] when ``ret_V``.  The
    solves' status is checked per ``options.check_status``.
    """
    check = options.check_status != "off"
    out, st, _ = _solve(input, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire, beta,
                        enable_break, break_threshould, nonlinear_cell_enable, nonlinear_params, ret_V,
                        options.to_c(), check, False)
    if check:
        check_solve_status(dict(solves=int(st.solves), status_or=int(st.status_or)),
                           resolved_method(options.method, row_size, col_size), options.check_status)
    return out


def ir_drop_gs_ex(input, G, batch_size, row_size, col_size, numX, numY, iter_times=600, g_wire=1 / 2.93, beta=1.9,
                  enable_break=False, break_threshould=1e-7, nonlinear_cell_enable=False, nonlinear_params=(),
                  ret_V=False, method=None, tol_v=None, max_iters=None, residual_period=None, omega=None,
                  vectors_per_cta=None, residual=None, read_noise_sigma=None, noise_seed=None, kernel_ld=None,
                  fp32_limit=None, return_stats=True, return_iters=False, out=None):
    """``ir_drop_gs`` with explicit solver options (``ret_V=2`` returns both node
    planes, [batch, numX, numY, 2, rows, cols]).  Returns (out, stats, iters):
    stats is a dict (solves, iters_sum, iters_max, status_or) and iters an int32
    [batch, numX, numY] tensor of per-solve iterations (None unless asked).  ``out``
    may be a preallocated contiguous tensor of the output's size."""
    o = SolverOptions(**{k: v for k, v in vars(options).items()})
    for k, v in dict(tol_v=tol_v, max_iters=max_iters, residual_period=residual_period, omega=omega,
                     vectors_per_cta=vectors_per_cta, residual=residual, read_noise_sigma=read_noise_sigma,
                     noise_seed=noise_seed, kernel_ld=kernel_ld, fp32_limit=fp32_limit).items():
        if v is not None:
            setattr(o, k, v)
    out, st, it = _solve(input, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire, beta,
                         enable_break, break_threshould, nonlinear_cell_enable, nonlinear_params, ret_V,
                         o.to_c(method), return_stats, return_iters, out=out)
    stats = None
    if st is not None:
        stats = dict(solves=int(st.solves), iters_sum=int(st.iters_sum), iters_max=int(st.iters_max),
                     status_or=int(st.status_or), warm_rejected=int(st.warm_rejected))
    return out, stats, it


def ir_drop_gs_host(input, G, batch_size, row_size, col_size, numX, numY, iter_times=600, g_wire=1 / 2.93, beta=1.9,
                    enable_break=False, break_threshould=1e-7, nonlinear_cell_enable=False, nonlinear_params=(),
                    ret_V=False, out=None, group_x=0, return_stats=False, device=None, **opt):
    """``ir_drop_gs`` on host (CPU) tensors: the library copies input and G in and
    the result out itself, pipelined over groups of ``group_x`` values of numX
    (0: automatic) so one group's copies overlap another's solve.  Pinned
    (``pin_memory()``) tensors let the copies run asynchronously.  Returns the
    CPU result (and the stats dict with ``return_stats``); ``opt`` takes the
    ``SolverOptions`` fields per call, as ``ir_drop_gs_ex`` does."""
    for t, name in ((input, "input"), (G, "G")):
        if not isinstance(t, torch.Tensor) or t.is_cuda:
            raise RuntimeError("%s must be a CPU tensor" % name)
        if not t.is_contiguous():
            raise RuntimeError("%s must be contiguous" % name)
    if row_size < 2 or col_size < 2:
        raise RuntimeError("row_size and col_size should be >=2")
    if input.dtype not in (torch.float32, torch.float64) or G.dtype != input.dtype:
        raise RuntimeError("input and G must both be float32 or both float64")
    if input.numel() != batch_size * numX * row_size or G.numel() != numX * row_size * numY * col_size:
        raise RuntimeError("input / G sizes do not match batch_size, numX, numY, row_size, col_size")
    o = SolverOptions(**{k: v for k, v in vars(options).items()})
    for k, v in opt.items():
        if not hasattr(o, k):
            raise TypeError("unknown solver option %r" % k)
        setattr(o, k, v)
    if ret_V == 2:
        shape = (batch_size, numX, numY, 2, row_size, col_size)
    elif ret_V:
        shape = (batch_size, numX, numY, row_size, col_size)
    else:
        shape = (batch_size, numX, numY * col_size)
    if out is None:
        out = torch.empty(shape, dtype=input.dtype, pin_memory=input.is_pinned())
    elif out.is_cuda or not out.is_contiguous() or out.dtype != input.dtype or out.numel() != math.prod(shape):
        raise RuntimeError("out must be a contiguous CPU %s tensor of %d elements" % (input.dtype, math.prod(shape)))
    lib = _lib.load()
    params = [float(v) for v in (nonlinear_params or [])]
    cparams = (ctypes.c_double * max(1, len(params)))(*params) if params else None
    stats = _lib.SolveStats()
    want = return_stats or o.check_status != "off"
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = lib.fadesim_ir_drop_gs_host(_lib.F64 if input.dtype == torch.float64 else _lib.F32, input.data_ptr(),
                                         G.data_ptr(), int(batch_size), int(row_size), int(col_size), int(numX),
                                         int(numY), int(iter_times), float(g_wire), float(beta),
                                         int(bool(enable_break)), float(break_threshould),
                                         int(bool(nonlinear_cell_enable)), cparams, len(params),
                                         2 if ret_V == 2 else int(bool(ret_V)), out.data_ptr(),
                                         ctypes.byref(o.to_c()), ctypes.byref(stats) if want else None,
                                         int(group_x), stream)
    _lib.check(rc)
    st = dict(solves=int(stats.solves), iters_sum=int(stats.iters_sum), iters_max=int(stats.iters_max),
              status_or=int(stats.status_or), warm_rejected=int(stats.warm_rejected)) if want else None
    # the groups' counters come back once, after the call's own final synchronisation
    check_solve_status(st, resolved_method(o.method, row_size, col_size), o.check_status)
    if return_stats:
        return out, st
    return out


def _family(cname, input, G, batch_size, row_size, col_size, numX, numY, out_rows, ret_V, nonlinear_cell_enable,
            nonlinear_params, *cargs):
    """Shared checks and launch of the IR2S / OU exports (their own iterates):
    cargs are the C entry's arguments up to the break threshold; the sinh-cell
    arguments (and ret_V, for ir2s) follow them."""
    _check_input(input, "input")
    _check_input(G, "G")
    if row_size < 2:
        raise RuntimeError("row_size should be >=2")
    if col_size < 2:
        raise RuntimeError("col_size should be >=2")
    if input.dtype not in (torch.float32, torch.float64) or G.dtype != input.dtype:
        raise RuntimeError("input and G must both be float32 or both float64")
    lib = _lib.load()
    shape = (batch_size, numX, numY, row_size, col_size) if ret_V else (batch_size, out_rows, numY * col_size)
    out = torch.empty(shape, dtype=input.dtype, device=input.device)
    dtype = _lib.F64 if input.dtype == torch.float64 else _lib.F32
    params = [float(v) for v in (nonlinear_params or [])] if nonlinear_cell_enable else []
    cparams = (ctypes.c_double * len(params))(*params) if params else None
    nl = (int(bool(nonlinear_cell_enable)), cparams, len(params))
    tail = (int(bool(ret_V)),) if cname == "ir2s" else ()
    with torch.cuda.device(input.device):
        stream = torch.cuda.current_stream(input.device).cuda_stream
        rc = getattr(lib, "fadesim_" + cname)(dtype, input.data_ptr(), G.data_ptr(), *cargs, *nl, *tail,
                                              out.data_ptr(), stream)
    _lib.check(rc)
    return out


# The reference module's other exports (split_arr_matmul.cu:1429-1437): the IR2S
# iteration and the operation-unit (OU) variants, reproducing their iterates,
# with linear or sinh cells (nonlinear_params = [R_on, R_off, a_on, b_on, a_off,
# b_off], commonConst.py:207).
def ir2s(input, G, batch_size, row_size, col_size, numX, numY, iter_times, r_wire, enable_break, break_threshould,
         nonlinear_cell_enable=False, nonlinear_params=(), ret_V=False):
    """ir2s (split_arr_matmul.cu:419-545): the IR-drop-to-source iteration with
    the wire resistance r_wire (also the source and ground loads)."""
    return _family("ir2s", input, G, batch_size, row_size, col_size, numX, numY, numX, ret_V,
                   nonlinear_cell_enable, nonlinear_params, batch_size, row_size, col_size, numX, numY, iter_times,
                   float(r_wire), int(bool(enable_break)), float(break_threshould))


def ir2s_ou_local(input, G, batch_size, row_size, col_size, numX, numY, iter_times, r_wire, r_load_left,
                  r_load_down, enable_break, break_threshould, nonlinear_cell_enable=False, nonlinear_params=()):
    """ir2s_ou_local (split_arr_matmul.cu:565-680): ir2s of one OU-sized array
    with source and ground load resistances."""
    return _family("ir2s_ou_local", input, G, batch_size, row_size, col_size, numX, numY, numX, False,
                   nonlinear_cell_enable, nonlinear_params, batch_size, row_size, col_size, numX, numY, iter_times,
                   float(r_wire), float(r_load_left), float(r_load_down), int(bool(enable_break)),
                   float(break_threshould))


def ir2s_ou(input, G, batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY, iter_times, r_wire,
            enable_break, break_threshould, nonlinear_cell_enable=False, nonlinear_params=()):
    """ir2s_ou (split_arr_matmul.cu:953-1084): every OU of the array at once, each
    through the lumped wire outside it; currents per OU row group
    [batch, numX * rows/ou_row_size, numY * cols]."""
    return _family("ir2s_ou", input, G, batch_size, row_size, col_size, numX, numY,
                   numX * (row_size // max(1, ou_row_size)), False, nonlinear_cell_enable, nonlinear_params,
                   batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY, iter_times, float(r_wire),
                   int(bool(enable_break)), float(break_threshould))


def ir_gs_ou_local(input, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire, g_load_left,
                   g_load_down, beta, enable_break, break_threshould, nonlinear_cell_enable=False,
                   nonlinear_params=()):
    """ir_gs_ou_local (split_arr_matmul.cu:690-813): the ir_drop_gs sweep of one
    OU-sized array with source and ground load conductances."""
    return _family("ir_gs_ou_local", input, G, batch_size, row_size, col_size, numX, numY, numX, False,
                   nonlinear_cell_enable, nonlinear_params, batch_size, row_size, col_size, numX, numY, iter_times,
                   float(g_wire), float(g_load_left), float(g_load_down), float(beta), int(bool(enable_break)),
                   float(break_threshould))


def ir_gs_ou(input, G, batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY, iter_times, g_wire,
             beta, enable_break, break_threshould, nonlinear_cell_enable=False, nonlinear_params=()):
    """ir_gs_ou (split_arr_matmul.cu:1197-1310): the sweep on every OU of the
    array at once; currents per OU row group [batch, numX * rows/ou_row_size,
    numY * cols]."""
    return _family("ir_gs_ou", input, G, batch_size, row_size, col_size, numX, numY,
                   numX * (row_size // max(1, ou_row_size)), False, nonlinear_cell_enable, nonlinear_params,
                   batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY, iter_times, float(g_wire),
                   float(beta), int(bool(enable_break)), float(break_threshould))


def ir_drop_gs_warm(input, G, batch_size, row_size, col_size, numX, numY, init, g_wire=1 / 2.93, tol_v=None,
                    residual=None, return_iters=False, method="line", omega=None, nonlinear_params=None,
                    read_noise_sigma=None, noise_seed=None):
    """Line solve from given initial planes ``init`` [batch, numX, numY, 2, rows, cols]
    (FP32 wordline deviations u - vin and bitline voltages d, e.g. a learned
    prediction), any tile size up to 512 x 512; ``nonlinear_params`` (the six
    sinh-cell parameters) for sinh cells.  Returns (currents, stats, iters)."""
    _check_input(input, "input")
    _check_input(G, "G")
    _check_input(init, "init")
    if init.dtype != torch.float32 or init.numel() != batch_size * numX * numY * 2 * row_size * col_size:
        raise RuntimeError("init must be float32 [batch, numX, numY, 2, rows, cols]")
    o = SolverOptions(**{k: v for k, v in vars(options).items()})
    if tol_v is not None:
        o.tol_v = tol_v
    if residual is not None:
        o.residual = residual
    if omega is not None:
        o.omega = omega
    if read_noise_sigma is not None:
        o.read_noise_sigma = read_noise_sigma
    if noise_seed is not None:
        o.noise_seed = noise_seed
    if nonlinear_params is not None and len(nonlinear_params) != 6:
        raise RuntimeError("nonlinear_params: [R_on, R_off, a_on, b_on, a_off, b_off]")
    nl = (ctypes.c_double * 6)(*[float(v) for v in nonlinear_params]) if nonlinear_params is not None else None
    out = torch.empty((batch_size, numX, numY * col_size), dtype=input.dtype, device=input.device)
    iters = torch.empty((batch_size, numX, numY), dtype=torch.int32, device=input.device) if return_iters else None
    st = _lib.SolveStats()
    lib = _lib.load()
    with torch.cuda.device(input.device):
        rc = lib.fadesim_ir_drop_gs_warm(_lib.F64 if input.dtype == torch.float64 else _lib.F32, input.data_ptr(),
                                         G.data_ptr(), batch_size, row_size, col_size, numX, numY, float(g_wire),
                                         init.data_ptr(), 1 if nl is not None else 0, nl, 6 if nl is not None else 0,
                                         out.data_ptr(), ctypes.byref(o.to_c(method)), ctypes.byref(st),
                                         iters.data_ptr() if return_iters else None,
                                         torch.cuda.current_stream(input.device).cuda_stream)
    _lib.check(rc)
    return out, dict(solves=int(st.solves), iters_sum=int(st.iters_sum), iters_max=int(st.iters_max),
                     status_or=int(st.status_or), warm_rejected=int(st.warm_rejected)), iters
