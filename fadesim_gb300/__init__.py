"""GB300-native crossbar IR-drop solver with PimTorch's ``cpp_ir_drop_accelerate``
interface.

``fadesim_gb300.cpp_ir_drop_accelerate`` is a drop-in for the module PimTorch
builds from ``fixedPoint/SplitArrCuda/split_arr_matmul.cu``; its solves run in
the hand-written CUDA kernels of ``libfadesim_gb300.so`` (sm_103a), reached
through the C ABI declared in ``include/fadesim_gb300.h``.
"""
from . import _lib  # noqa: F401

__all__ = ["cpp_ir_drop_accelerate", "build"]


def build(verbose=False):
    from .build import build as _build
    return _build(verbose)
