"""ctypes binding of ``libfadesim_gb300.so`` (the C ABI in include/fadesim_gb300.h).

The library is built in-tree by ``fadesim_gb300.build``.  There is no fallback:
if the library cannot be loaded every solve raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfadesim_gb300.so")

F32 = 0
F64 = 1
METHOD_AUTO, METHOD_LINE, METHOD_RBSOR, METHOD_SWEEPS, METHOD_LINE_COARSE = 0, 1, 2, 3, 4
ST_CONVERGED, ST_MAXITER, ST_NONFINITE, ST_WARM_REJECTED = 1, 2, 4, 8


class SolveOpts(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("tol_v", ctypes.c_double), ("max_iters", ctypes.c_int),
                ("residual_period", ctypes.c_int), ("omega", ctypes.c_double), ("vectors_per_cta", ctypes.c_int),
                ("residual_kind", ctypes.c_int), ("read_noise_sigma", ctypes.c_double),
                ("noise_seed", ctypes.c_ulonglong), ("kernel_ld", ctypes.c_int), ("fp32_limit", ctypes.c_int)]


class SolveStats(ctypes.Structure):
    _fields_ = [("solves", ctypes.c_int64), ("iters_sum", ctypes.c_int64), ("iters_max", ctypes.c_int),
                ("status_or", ctypes.c_int), ("warm_rejected", ctypes.c_int64)]


_lib = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double

EXPORTS = {
    "fadesim_ir_drop_gs_f32": [_vp, _vp, _i, _i, _i, _i, _i, _i, _d, _d, _i, _d, _i, _vp, _i, _i, _vp, _vp],
    "fadesim_ir_drop_gs_f64": [_vp, _vp, _i, _i, _i, _i, _i, _i, _d, _d, _i, _d, _i, _vp, _i, _i, _vp, _vp],
    "fadesim_ir_drop_gs_ex": [_i, _vp, _vp, _i, _i, _i, _i, _i, _i, _d, _d, _i, _d, _i, _vp, _i, _i, _vp,
                              ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _vp, _vp],
    "fadesim_ir_drop_gs_host": [_i, _vp, _vp, _i, _i, _i, _i, _i, _i, _d, _d, _i, _d, _i, _vp, _i, _i, _vp,
                                ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _i, _vp],
    "fadesim_ir_drop_gs_warm": [_i, _vp, _vp, _i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i, _vp,
                                ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveStats), _vp, _vp],
    "fadesim_release_memory": [],
    "fadesim_last_error": [],
    "fadesim_version": [],
    "fadesim_ir_drop_gs_noalloc_f32": [_vp, _vp, _i, _i, _i, _i, _i, _d, _vp, _vp],
    "fadesim_quantize_f32": [_vp, ctypes.c_longlong, _i, _vp, _vp],
    "fadesim_slice_inputs_f32": [_vp, _i, _i, _i, _i, _i, _i, ctypes.c_float, _vp, _vp],
    "fadesim_map_conductance_f32": [_vp, _i, _i, _i, _i, _i, _i, _i, _i, _i, ctypes.c_float, ctypes.c_float, _vp, _vp],
    "fadesim_adc_shift_add_f32": [_vp, _i, _i, _i, _i, _i, _i, ctypes.c_float, ctypes.c_float, ctypes.c_float, _i, _i,
                                  _i, _i, _i, _vp, _vp],
    "fadesim_slice_inputs_im2col_f32": [_vp] + [_i] * 19 + [ctypes.c_float, _vp, _vp],
    "fadesim_map_conductance_ref_f32": [_vp] + [_i] * 10 + [ctypes.c_float, ctypes.c_float, _vp, _vp],
    "fadesim_adc_shift_add_ex_f32": [_vp] + [_i] * 7 + [ctypes.c_float] * 3 + [_i] * 5 + [ctypes.c_float, _vp, _i,
                                                                                         _vp, _vp],
    "fadesim_vary_conductance_f32": [_vp, _vp, ctypes.c_longlong, _d, ctypes.c_ulonglong, ctypes.c_ulonglong, _vp,
                                     _vp],
    "fadesim_ir2s": [_i, _vp, _vp] + [_i] * 6 + [_d, _i, _d, _i, _vp, _i, _i, _vp, _vp],
    "fadesim_ir2s_ou_local": [_i, _vp, _vp] + [_i] * 6 + [_d, _d, _d, _i, _d, _i, _vp, _i, _vp, _vp],
    "fadesim_ir2s_ou": [_i, _vp, _vp] + [_i] * 8 + [_d, _i, _d, _i, _vp, _i, _vp, _vp],
    "fadesim_ir_gs_ou_local": [_i, _vp, _vp] + [_i] * 6 + [_d, _d, _d, _d, _i, _d, _i, _vp, _i, _vp, _vp],
    "fadesim_ir_gs_ou": [_i, _vp, _vp] + [_i] * 8 + [_d, _d, _i, _d, _i, _vp, _i, _vp, _vp],
    "fadesim_noalloc_scratch_bytes": [],
    "fadesim_noalloc_last_error": [],
    "fadesim_noalloc_last_status": [ctypes.POINTER(SolveStats), _vp],
    "fadesim_smem_read_probe": [_vp, _i, _i, _vp],
}


def load():
    """Load the library once; raise ImportError with the reason if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libfadesim_gb300.so is not built (run fadesim_gb300.build.build()); "
                          "there is no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in EXPORTS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        if name in ("fadesim_last_error", "fadesim_version", "fadesim_noalloc_last_error"):
            fn.restype = ctypes.c_char_p
        elif name == "fadesim_noalloc_scratch_bytes":
            fn.restype = ctypes.c_size_t
        else:
            fn.restype = ctypes.c_int
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        msg = load().fadesim_last_error().decode()
        raise RuntimeError(msg or ("fadesim call failed with code %d" % rc))
