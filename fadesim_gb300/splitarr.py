"""PimTorch's bit-sliced crossbar matmul and ``Linear_sp`` layer on the GPU.

Mirrors ``splitArr_matmul_nn`` (pimtorch/pimfixedpoint/fixedPoint/nn/
splitArrayArithmetic.py:1161-1228) and the PN, whole-array branch of ``matmul``
(:442-1018) for the default PimTorch settings -- PN weight arrays, complement-
code inputs, 1-bit DAC, no OU, no BNN, no compensation -- and
``Linear_sp.forward`` (fixedPoint/nn/modules/linear_split.py:53-78).  The
integer stages (quantisation, PN split, bit slicing, conductance mapping, ADC,
shift-add) run in the CUDA kernels of ``libfadesim_gb300.so`` and are bit-exact
with the reference's float32 arithmetic given the same currents; the currents
come from the IR-drop solve (``cpp_ir_drop_accelerate.ir_drop_gs`` unless a
``solver`` is passed).  The solves of one (weight slice, array) pair cover all
input-bit cycles at once: the input bits are stacked on the batch.

Array and device parameters come from an object with ``phyArrParams``'s
attribute names, so the reference's own ``commonConst.phyArrParams`` can be
passed unchanged; ``ArrayConfig`` holds the same defaults.
"""
import math
from dataclasses import dataclass, field

import torch

from . import _lib
from . import cpp_ir_drop_accelerate as _acc


@dataclass
class ArrayConfig:
    """The phyArrParams fields these stages read (commonConst.py:187-269), with
    derived constants computed in the reference's order."""
    Ron: float = 1e3
    Roff: float = 1e6
    cellBits: int = 1
    arrRowSize: int = 64
    arrColSize: int = 64
    inputMaxVoltage: float = 1.0
    r_wire: float = 2.93
    sigma: float = 0.0
    ir_drop_iter_time: int = 600
    ir_drop_GS_method_beta_scale: float = 1.90
    ir_drop_less_than_thresholdBreak_enable: bool = False
    ir_drop_less_than_threshold: float = 1e-7
    nonlinear_cell_enable: bool = False
    nonlinear_params: list = field(default_factory=list)

    @property
    def cellMaxConduct(self):
        return 1 / self.Ron

    @property
    def cellMinConduct(self):
        return 1 / self.Roff

    @property
    def cellDeltaConduct(self):
        return (self.cellMaxConduct - self.cellMinConduct) / (2 ** self.cellBits - 1)

    @property
    def adcUseI(self):
        return self.arrRowSize * (self.cellMaxConduct - self.cellMinConduct) * self.inputMaxVoltage


def _fixed_point_position(max_abs, bit_width, pn):
    """fixedPointArithmetic.py:19-27."""
    if math.isclose(max_abs, 0.0):
        max_abs = 1e-12
    if pn:
        return math.ceil(math.log2(max_abs / ((1 << bit_width) - 1)))
    return math.ceil(math.log2(max_abs / ((1 << (bit_width - 1)) - 1)))


def _stream():
    return torch.cuda.current_stream().cuda_stream


def quantize(x, bit_width, pn):
    """quantization_tensor (fixedPointArithmetic.py:76-96) -> (int32 tensor, s)."""
    lib = _lib.load()
    x = x.contiguous()
    s = _fixed_point_position(float(x.abs().max().item()), bit_width, pn)
    q = torch.empty(x.shape, dtype=torch.int32, device=x.device)
    _lib.check(lib.fadesim_quantize_f32(x.data_ptr(), x.numel(), s, q.data_ptr(), _stream()))
    return q, s


def default_solver(cfg):
    def solve(v, G, B, rows, cols, numX, numY, out):
        return _acc.ir_drop_gs_ex(v, G, B, rows, cols, numX, numY, iter_times=cfg.ir_drop_iter_time,
                                  g_wire=1 / cfg.r_wire, beta=cfg.ir_drop_GS_method_beta_scale,
                                  enable_break=cfg.ir_drop_less_than_thresholdBreak_enable,
                                  break_threshould=cfg.ir_drop_less_than_threshold,
                                  nonlinear_cell_enable=cfg.nonlinear_cell_enable,
                                  nonlinear_params=cfg.nonlinear_params, return_stats=False, out=out)[0]
    return solve


def splitArr_matmul_nn(input, w, inputBits, dacBits, adcBits, outputBits, weightBits, arrType="PN",
                       float_type=torch.float32, cfg=None, solver=None):
    """Same arguments as the reference; ``arrType`` is "PN" or an enum whose name is
    "PN"; ``cfg`` is a phyArrParams-like object (default ``ArrayConfig()``);
    ``solver(v, G, B, rows, cols, numX, numY, out)`` may replace the IR-drop solve."""
    cfg = cfg if cfg is not None else ArrayConfig()
    name = getattr(arrType, "name", arrType)
    if name != "PN":
        raise NotImplementedError("only the PN array mode is implemented (Ref mode is not)")
    if float_type != torch.float32:
        raise NotImplementedError("the integer-stage kernels are float32, as Linear_sp's default fp_type")
    if dacBits != 1:
        raise Exception("[Error] Complement code input mode, but dac is not 1 bit. dacbits = {}".format(dacBits))
    if getattr(cfg, "useOUSize", False) or getattr(cfg, "useBNN", False):
        raise NotImplementedError("OU and BNN modes are not implemented")
    if getattr(cfg, "sigma", 0) != 0:
        raise NotImplementedError("conductance variation: use fadesim_gb300.variation on the maps")
    if weightBits % cfg.cellBits != 0:
        raise Exception("[Error] cellbit is not factor of weight_bit")
    lib = _lib.load()
    solver = solver or default_solver(cfg)
    with torch.no_grad():
        x = input.to(device="cuda", dtype=torch.float32).contiguous()
        w = w.to(device=x.device, dtype=torch.float32).contiguous()
        B, insize = x.shape
        outsize = w.shape[1]
        xq, s1 = quantize(x, inputBits, pn=False)
        wq, s2 = quantize(w, weightBits, pn=True)
        rows, cols = cfg.arrRowSize, cfg.arrColSize
        numX = -(-insize // rows)
        numY = -(-outsize // cols)
        nbits = len(range(0, inputBits, dacBits))
        nslices = len(range(0, weightBits, cfg.cellBits))
        inputV = cfg.inputMaxVoltage / (2 ** dacBits - 1)
        st = _stream()
        v = torch.empty((nbits * B, numX, rows), dtype=torch.float32, device=x.device)
        _lib.check(lib.fadesim_slice_inputs_f32(xq.data_ptr(), B, insize, rows, numX, nbits, dacBits, inputV,
                                                v.data_ptr(), st))
        I = torch.empty((nslices, 2, nbits * B, numX, numY * cols), dtype=torch.float32, device=x.device)
        G = torch.empty((numX, rows, numY * cols), dtype=torch.float32, device=x.device)
        for j in range(nslices):
            for pn in (0, 1):
                _lib.check(lib.fadesim_map_conductance_f32(wq.data_ptr(), insize, outsize, rows, cols, numX, numY,
                                                           j * cfg.cellBits, cfg.cellBits, pn, cfg.cellDeltaConduct,
                                                           cfg.cellMinConduct, G.data_ptr(), st))
                r = solver(v, G, nbits * B, rows, cols, numX, numY, I[j, pn])
                if r is not None and r.data_ptr() != I[j, pn].data_ptr():
                    I[j, pn].copy_(r.reshape(I[j, pn].shape))
        out = torch.empty((B, outsize), dtype=torch.float32, device=x.device)
        scale = rows * (2 ** dacBits - 1) * (2 ** cfg.cellBits - 1) / (2 ** adcBits - 1)
        _lib.check(lib.fadesim_adc_shift_add_f32(I.data_ptr(), nbits, nslices, B, numX, numY * cols, outsize,
                                                 cfg.adcUseI, float(2 ** adcBits - 1), scale, s1 + s2, dacBits,
                                                 cfg.cellBits, inputBits, 1, out.data_ptr(), st))
        return out


class Linear_sp(torch.nn.Module):
    """Linear_sp (fixedPoint/nn/modules/linear_split.py:13-79): float training,
    crossbar-simulated evaluation through ``splitArr_matmul_nn``."""

    def __init__(self, in_features, out_features, bias=True, input_bit_width=8, output_bit_width=10,
                 weight_bit_width=8, dac_bit_width=1, adc_bit_width=10, phy_arr_mode="PN",
                 fp_type=torch.float32, use_fp_bias=True, cfg=None, solver=None):
        super().__init__()
        self.inSize, self.outSize = in_features, out_features
        self.hasBias, self.useFpBias = bias, use_fp_bias
        self.inputBits, self.outputBits, self.weightBits = input_bit_width, output_bit_width, weight_bit_width
        self.adcBits, self.dacBits = adc_bit_width, dac_bit_width
        self.phyArrMode, self.fp_type = phy_arr_mode, fp_type
        self.cfg, self.solver = cfg, solver
        self.fp_weight = torch.nn.Parameter(torch.empty((out_features, in_features), dtype=fp_type))
        self.fp_bias = torch.nn.Parameter(torch.zeros(out_features, dtype=fp_type)) if bias else None
        torch.nn.init.kaiming_uniform_(self.fp_weight, a=math.sqrt(5))

    def forward(self, input):
        if self.training:
            return torch.nn.functional.linear(input, self.fp_weight, self.fp_bias)
        if self.hasBias and not self.useFpBias:
            input = torch.cat((input, input.new_ones(input.size(0), 1)), 1)
            logic = torch.cat((self.fp_weight.t(), self.fp_bias.unsqueeze(0)), 0)
        else:
            logic = self.fp_weight.t()
        out = splitArr_matmul_nn(input, logic, self.inputBits, self.dacBits, self.adcBits, self.outputBits,
                                 self.weightBits, self.phyArrMode, self.fp_type, cfg=self.cfg, solver=self.solver)
        if self.hasBias and self.useFpBias:
            out = out + self.fp_bias.to(out.device)
        return out
