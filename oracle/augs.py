"""ctypes front of ``au_gs.c`` (the C restatement of V1 nodeBasedGS).

Test infrastructure only: see ``oracle/__init__.py``.  ``build()`` compiles the
library with ``make -C oracle port``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libaugs.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build():
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        lib.au_gs_solve.restype = ctypes.c_int
        lib.au_gs_solve.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_double, _dp, _dp, _dp]
        lib.au_gs_solve_many.restype = ctypes.c_int
        lib.au_gs_solve_many.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, _dp, _ip]
        lib.au_gs_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def solve(g, vin, r_wire, iters, w, enable_break=True, tol=1e-8, vout=None):
    """One lexicographic GS/SOR solve; returns (vup, vdown, iout, sweeps)."""
    lib = _load()
    g = np.ascontiguousarray(g, np.float64)
    n, m = g.shape
    vin = np.ascontiguousarray(vin, np.float64).reshape(n)
    vout = np.zeros(m) if vout is None else np.ascontiguousarray(vout, np.float64).reshape(m)
    up = np.empty((n, m))
    dn = np.empty((n, m))
    io = np.empty(m)
    s = lib.au_gs_solve(n, m, _p(g), _p(vin), _p(vout), float(r_wire), int(iters), float(w), int(bool(enable_break)),
                        float(tol), _p(up), _p(dn), _p(io))
    if s < 0:
        raise ValueError("au_gs_solve failed (%d)" % s)
    return up, dn, io, s


def solve_many(g, vin, r_wire, iters, w, enable_break=True, tol=1e-8):
    """count independent solves on all OpenMP threads; g [K, n, m], vin [K, n]."""
    lib = _load()
    g = np.ascontiguousarray(g, np.float64)
    K, n, m = g.shape
    vin = np.ascontiguousarray(vin, np.float64).reshape(K, n)
    io = np.empty((K, m))
    sw = np.empty(K, np.int32)
    rc = lib.au_gs_solve_many(K, n, m, _p(g), _p(vin), float(r_wire), int(iters), float(w), int(bool(enable_break)),
                              float(tol), _p(io), sw.ctypes.data_as(_ip))
    if rc != 0:
        raise ValueError("au_gs_solve_many failed (%d)" % rc)
    return io, sw


def max_threads():
    return int(_load().au_gs_max_threads())
