"""PimTorch's bit-sliced crossbar matmul and its ``Linear_sp`` / ``Conv2d_sp``
layers on the GPU.

Mirrors ``splitArr_matmul_nn`` (pimtorch/pimfixedpoint/fixedPoint/nn/
splitArrayArithmetic.py:1161-1260) and the whole-array branch of ``matmul``
(:442-1018) -- PN or Ref-column weight arrays, complement-code or
negative-pulse inputs, no OU, no BNN, no compensation -- with
``Linear_sp.forward`` (fixedPoint/nn/modules/linear_split.py:53-78) and
``Conv2d_sp.forward`` (fixedPoint/nn/modules/conv_split.py:89-136) on top.  The
integer stages (quantisation, PN split or Ref offset, bit slicing with the
convolution's unfold done by addressing, conductance mapping, ADC,
reference-column subtraction, shift-add, bias, fold) run in the CUDA kernels
of ``libfadesim_gb300.so`` and are bit-exact with the reference's float32
arithmetic given the same currents; the currents come from the IR-drop solve
(``cpp_ir_drop_accelerate.ir_drop_gs`` unless a ``solver`` is passed).  The
solves of one (weight slice, array) pair cover all input-bit cycles at once:
the input bits are stacked on the batch -- unless the cells vary from cycle to
cycle (``sigma != 0``), when every (input bit, slice, array) solve gets its own
draw of the variation, in the reference's order and from its generator.

Array and device parameters come from an object with ``phyArrParams``'s
attribute names, so the reference's own ``commonConst.phyArrParams`` can be
passed unchanged; ``ArrayConfig`` holds the same defaults.
"""
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from . import cpp_ir_drop_accelerate as _acc
from . import variation as _variation


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
    inputVmode: str = "complement_code"   # or "neg_pulse" (commonConst.py:170-172,224)

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


def default_solver(cfg, tol_v=None, method=None, fp32_limit=None):
    """The IR-drop solve of the drop-in module with the array's parameters
    (tol_v, method, fp32_limit None: the module-wide options); the solves'
    status is checked per the module's ``options.check_status``, as
    ``ir_drop_gs`` does."""
    def solve(v, G, B, rows, cols, numX, numY, out):
        policy = _acc.options.check_status
        r, st, _ = _acc.ir_drop_gs_ex(v, G, B, rows, cols, numX, numY, iter_times=cfg.ir_drop_iter_time,
                                      g_wire=1 / cfg.r_wire, beta=cfg.ir_drop_GS_method_beta_scale,
                                      enable_break=cfg.ir_drop_less_than_thresholdBreak_enable,
                                      break_threshould=cfg.ir_drop_less_than_threshold,
                                      nonlinear_cell_enable=cfg.nonlinear_cell_enable,
                                      nonlinear_params=cfg.nonlinear_params, tol_v=tol_v, method=method,
                                      fp32_limit=fp32_limit, return_stats=policy != "off", out=out)
        _acc.check_solve_status(st, _acc.resolved_method(method or _acc.options.method, rows, cols), policy)
        return r
    return solve


def superposition_solver(cfg, fp32_limit=True):
    """IR-drop currents by linearity, for linear cells without read noise.

    The bitline currents of a tile are then a linear map of its wordline
    voltages, I = V M, M [rows, numY*cols] the tile's effective conductance
    matrix.  M comes from one solver call with ``rows`` unit vectors per tile
    (row r driven at the DAC level inputV, the others at 0 V), and every input
    vector's currents are one FP32 matrix product: rows solves per tile instead
    of one per vector, exact up to the solver tolerance.  A vector's currents
    sum up to ``rows`` unit responses, so these are solved 500x tighter than the
    module tolerance, and (``fp32_limit``, the default) on full 128 x 128 tiles
    with the two-level method to the FP32 limit: a unit response's currents
    come from the bitline ends, small nodes that keep converging after the
    largest ones reach the FP32 floor (4 ulps of the largest deviation), where
    the plain stop test leaves them up to ~3e-4 of their own size off (the
    currents then differ from direct solves by ~1e-4 of the largest instead of
    ~1e-6, at ~1/4 of the time).  Used with the same
    (v, G, B, rows, cols, numX, numY, out) interface as ``default_solver``; calls
    with no more vectors than rows solve directly."""
    direct = default_solver(cfg)
    if getattr(cfg, "nonlinear_cell_enable", False):
        raise ValueError("superposition needs linear cells: nonlinear (sinh) cells are not a linear map")

    def solve(v, G, B, rows, cols, numX, numY, out):
        if B <= rows:
            return direct(v, G, B, rows, cols, numX, numY, out)
        if _acc.options.read_noise_sigma > 0:
            raise ValueError("superposition needs noise-free cells: read noise is not a linear map")
        lv = float(v.abs().max().item()) or 1.0  # unit drive level: the largest input voltage
        unit = torch.zeros((rows, numX, rows), dtype=v.dtype, device=v.device)
        r = torch.arange(rows, device=v.device)
        unit[r, :, r] = lv
        full = fp32_limit and rows == 128 and cols == 128
        M = default_solver(cfg, tol_v=_acc.options.tol_v * 2e-3, method="line_coarse" if full else None,
                           fp32_limit=True if full else None)(unit, G, rows, rows, cols, numX, numY, None)
        M = M.reshape(rows, numX, numY * cols).permute(1, 0, 2) * (1.0 / lv)
        tf32 = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False  # full FP32 products
        try:
            res = torch.bmm(v.reshape(B, numX, rows).permute(1, 0, 2), M)  # [numX, B, numY*cols]
        finally:
            torch.backends.cuda.matmul.allow_tf32 = tf32
        out = res.permute(1, 0, 2) if out is None else out.copy_(res.permute(1, 0, 2).reshape(out.shape))
        return out

    return solve


def _mode_name(v, default):
    v = default if v is None else v
    return getattr(v, "name", v)


def _check_modes(arr, in_mode, dacBits, cfg):
    if arr not in ("PN", "Ref"):
        raise NotImplementedError("array mode %r (PN and Ref are implemented)" % (arr,))
    if in_mode not in ("complement_code", "neg_pulse"):
        raise NotImplementedError("input mode %r" % (in_mode,))
    if in_mode == "complement_code" and dacBits != 1:
        raise Exception("[Error] Complement code input mode, but dac is not 1 bit. dacbits = {}".format(dacBits))
    if getattr(cfg, "useOUSize", False) or getattr(cfg, "useBNN", False):
        raise NotImplementedError("OU and BNN modes are not implemented")


# bytes of repeated input vectors and currents that one batched solver call of
# the layer driver may hold (the maps of a layer are grouped to stay under it)
MAP_GROUP_BYTES = 1 << 30


def _split_matmul_core(xq, geom, M, insize, has_ones, ones_q, s1, w, inputBits, dacBits, adcBits, weightBits, arr,
                       neg_pulse, cfg, solver, bias=None, L=0, rand_gen=None):
    """The bit-serial, bit-sliced product of splitArr_matmul_nn from quantised
    inputs: xq is an int32 NCHW image (geom = N, C, H, W, kh, kw, sh, sw, ph,
    pw, dh, dw; a linear layer is the 1x1 case) whose unfold has M rows and
    insize columns (plus a ones column if has_ones); w [insize(+1), outsize]
    float weights.  Returns float32 [M, outsize], or [M/L, outsize, L] if L.

    With ``cfg.sigma != 0`` every solve gets its own conductance variation, as
    in the reference's ``matmul`` (splitArrayArithmetic.py:758-760 PN, :788
    Ref): one draw of exp(sigma N(0,1)) per cell of the padded map for every
    (input bit, weight slice, array) call, in the reference's loop order --
    input bit outer, slice inner, the positive array before the negative one
    (:1197-1217, :1247-1251) -- from ``rand_gen`` (default
    ``variation.variations.rand_gen_network``).  The input bits then cannot
    share one solve per map, so each bit's vectors are solved on their own."""
    lib = _lib.load()
    if weightBits % cfg.cellBits != 0:
        raise Exception("[Error] cellbit is not factor of weight_bit")
    solver = solver or default_solver(cfg)
    dev = xq.device
    K = insize + (1 if has_ones else 0)
    outsize = w.shape[1]
    rows, cols = cfg.arrRowSize, cfg.arrColSize
    numX = -(-K // rows)
    numY = -(-outsize // cols)
    nbits = len(range(0, inputBits, dacBits))
    nslices = len(range(0, weightBits, cfg.cellBits))
    inputV = cfg.inputMaxVoltage / (2 ** dacBits - 1)
    st = _stream()
    v = torch.empty((nbits * M, numX, rows), dtype=torch.float32, device=dev)
    _lib.check(lib.fadesim_slice_inputs_im2col_f32(xq.data_ptr(), *geom, int(bool(has_ones)), int(ones_q), rows, numX,
                                                   nbits, dacBits, int(bool(neg_pulse)), inputV, v.data_ptr(), st))
    ref = arr == "Ref"
    wq, s2 = quantize(w, weightBits, pn=not ref)
    cb = cols + 2 if ref else cols
    narr = 1 if ref else 2
    I = torch.empty((nslices, narr, nbits * M, numX, numY * cb), dtype=torch.float32, device=dev)
    G = torch.empty((numX, rows, numY * cb), dtype=torch.float32, device=dev)
    plus = 2 ** (weightBits - 1)

    def map_slice(j, a, G):
        if ref:
            _lib.check(lib.fadesim_map_conductance_ref_f32(wq.data_ptr(), K, outsize, rows, cols, numX, numY,
                                                           j * cfg.cellBits, cfg.cellBits, plus,
                                                           2 ** weightBits - 1, cfg.cellDeltaConduct,
                                                           cfg.cellMinConduct, G.data_ptr(), st))
        else:
            _lib.check(lib.fadesim_map_conductance_f32(wq.data_ptr(), K, outsize, rows, cols, numX, numY,
                                                       j * cfg.cellBits, cfg.cellBits, a, cfg.cellDeltaConduct,
                                                       cfg.cellMinConduct, G.data_ptr(), st))

    def solve_into(vv, GG, nb, dst):
        r = solver(vv, GG, nb, rows, cb, numX, numY, dst)
        if r is not None and r.data_ptr() != dst.data_ptr():
            dst.copy_(r.reshape(dst.shape))

    sigma = float(getattr(cfg, "sigma", 0) or 0)
    if sigma == 0:
        # the (slice, array) maps solved together: stacked along the tile axis,
        # each with all input bits' vectors (one launch per layer instead of one
        # per map; each (tile, vector) solve is the same), in groups whose
        # repeated inputs and currents stay within MAP_GROUP_BYTES
        nm = nslices * narr
        per_map = v.numel() * 4 + I[0, 0].numel() * 4
        g = max(1, min(nm, MAP_GROUP_BYTES // max(1, per_map)))
        maps = torch.empty((g * numX, rows, numY * cb), dtype=torch.float32, device=dev)
        for k0 in range(0, nm, g):
            gk = min(g, nm - k0)
            for k in range(gk):
                j, a = divmod(k0 + k, narr)
                map_slice(j, a, maps[k * numX:(k + 1) * numX])
            if gk == 1:
                j, a = divmod(k0, narr)
                solve_into(v, maps[:numX], nbits * M, I[j, a])
                continue
            vv = v.repeat(1, gk, 1)
            res = torch.empty((nbits * M, gk * numX, numY * cb), dtype=torch.float32, device=dev)
            r = solver(vv, maps[:gk * numX], nbits * M, rows, cb, gk * numX, numY, res)
            if r is not None and r.data_ptr() != res.data_ptr():
                res.copy_(r.reshape(res.shape))
            dst = I.reshape(nm, nbits * M, numX, numY * cb)[k0:k0 + gk]
            dst.copy_(res.reshape(nbits * M, gk, numX, numY * cb).permute(1, 0, 2, 3))
    else:
        gen = rand_gen if rand_gen is not None else _variation.variations.rand_gen_network
        maps = torch.empty((nslices, narr) + tuple(G.shape), dtype=torch.float32, device=dev)
        for j in range(nslices):
            for a in range(narr):
                map_slice(j, a, maps[j, a])
        div = torch.empty(G.shape, dtype=torch.float32, device=dev)
        for i in range(nbits):
            for j in range(nslices):
                for a in range(narr):
                    div.copy_(_variation.variation_divisor(tuple(G.shape), sigma, gen))
                    _lib.check(lib.fadesim_vary_conductance_f32(maps[j, a].data_ptr(), div.data_ptr(), G.numel(),
                                                                0.0, 0, 0, G.data_ptr(), st))
                    solve_into(v[i * M:(i + 1) * M], G, M, I[j, a, i * M:(i + 1) * M])
    shape = (M // L, outsize, L) if L else (M, outsize)
    out = torch.empty(shape, dtype=torch.float32, device=dev)
    scale = rows * (2 ** dacBits - 1) * (2 ** cfg.cellBits - 1) / (2 ** adcBits - 1)
    b = None
    if bias is not None:
        b = bias.detach().to(device=dev, dtype=torch.float32).contiguous()
    _lib.check(lib.fadesim_adc_shift_add_ex_f32(I.data_ptr(), cols if ref else 0, nbits, nslices, M, numX, numY * cb,
                                                outsize, cfg.adcUseI, float(2 ** adcBits - 1), scale, s1 + s2,
                                                dacBits, cfg.cellBits, inputBits, 0 if neg_pulse else 1,
                                                float(plus), b.data_ptr() if b is not None else None, int(L),
                                                out.data_ptr(), st))
    return out


def splitArr_matmul_nn(input, w, inputBits, dacBits, adcBits, outputBits, weightBits, arrType="PN",
                       float_type=torch.float32, cfg=None, solver=None, rand_gen=None):
    """Same arguments as the reference; ``arrType`` is "PN" / "Ref" or an enum
    with that name; ``cfg`` is a phyArrParams-like object (default
    ``ArrayConfig()``; its ``inputVmode`` selects complement-code or
    negative-pulse inputs, its ``sigma`` the conductance variation);
    ``solver(v, G, B, rows, cols, numX, numY, out)`` may replace the IR-drop
    solve; ``rand_gen`` is the variation's generator (default
    ``variation.variations.rand_gen_network``, the reference's)."""
    cfg = cfg if cfg is not None else ArrayConfig()
    arr = _mode_name(arrType, "PN")
    in_mode = _mode_name(getattr(cfg, "inputVmode", None), "complement_code")
    _check_modes(arr, in_mode, dacBits, cfg)
    if float_type != torch.float32:
        raise NotImplementedError("the integer-stage kernels are float32, as Linear_sp's default fp_type")
    with torch.no_grad():
        x = input.to(device="cuda", dtype=torch.float32).contiguous()
        w = w.to(device=x.device, dtype=torch.float32).contiguous()
        B, insize = x.shape
        xq, s1 = quantize(x, inputBits, pn=False)
        geom = (B, insize, 1, 1, 1, 1, 1, 1, 0, 0, 1, 1)
        return _split_matmul_core(xq, geom, B, insize, False, 0, s1, w, inputBits, dacBits, adcBits, weightBits, arr,
                                  in_mode == "neg_pulse", cfg, solver, rand_gen=rand_gen)


def _covered(n, k, s, p, d, on):
    """Which of n input positions an unfold with kernel k, stride s, padding p,
    dilation d and on outputs reads."""
    cov = np.zeros(n, dtype=bool)
    for o in range(on):
        for t in range(k):
            h = o * s - p + t * d
            if 0 <= h < n:
                cov[h] = True
    return cov


def conv2d_split(input, weight, bias, stride=1, padding=0, dilation=1, inputBits=8, dacBits=1, adcBits=10,
                 outputBits=10, weightBits=8, arrType="PN", use_fp_bias=True, cfg=None, solver=None, rand_gen=None):
    """Conv2d_sp's evaluation (fixedPoint/nn/modules/conv_split.py:89-136):
    unfold, splitArr_matmul_nn against the weights reshaped [Cout, C*kh*kw] and
    transposed, float32 bias (or a bias row in the array driven by ones when
    ``use_fp_bias`` is False), fold to [N, Cout, OH, OW].  The unfold is done by
    addressing inside the slicing kernel and the fold by the output layout of
    the shift-add kernel; results equal the reference's bit for bit given the
    same currents.  Zero padding only, groups 1."""
    cfg = cfg if cfg is not None else ArrayConfig()
    arr = _mode_name(arrType, "PN")
    in_mode = _mode_name(getattr(cfg, "inputVmode", None), "complement_code")
    _check_modes(arr, in_mode, dacBits, cfg)
    pair = lambda t: tuple(t) if isinstance(t, (tuple, list)) else (t, t)
    (sh, sw), (ph, pw), (dh, dw) = pair(stride), pair(padding), pair(dilation)
    with torch.no_grad():
        x = input.to(device="cuda", dtype=torch.float32).contiguous()
        wt = weight.to(device=x.device, dtype=torch.float32)
        N, C, H, W = x.shape
        Cout, Cw, kh, kw = wt.shape
        if Cw != C:
            raise NotImplementedError("grouped convolutions are not supported by Conv2d_sp's evaluation path")
        OH = (H + 2 * ph - dh * (kh - 1) - 1) // sh + 1
        OW = (W + 2 * pw - dw * (kw - 1) - 1) // sw + 1
        if OH < 1 or OW < 1:
            raise RuntimeError("input too small for the kernel")
        ones = bias is not None and not use_fp_bias
        rmask = torch.from_numpy(_covered(H, kh, sh, ph, dh, OH)).to(x.device)
        cmask = torch.from_numpy(_covered(W, kw, sw, pw, dw, OW)).to(x.device)
        max_abs = float(x[:, :, rmask][:, :, :, cmask].abs().max().item()) if N else 0.0
        if ones:
            max_abs = max(max_abs, 1.0)
        s1 = _fixed_point_position(max_abs, inputBits, False)
        xq = torch.empty(x.shape, dtype=torch.int32, device=x.device)
        lib = _lib.load()
        _lib.check(lib.fadesim_quantize_f32(x.data_ptr(), x.numel(), s1, xq.data_ptr(), _stream()))
        ones_q = int(np.rint(np.float32(1.0) / np.float32(2.0 ** s1))) if ones else 0
        wm = wt.reshape(Cout, -1).t()
        if ones:
            wm = torch.cat((wm, bias.detach().to(wm).reshape(1, -1)), 0)
        geom = (N, C, H, W, kh, kw, sh, sw, ph, pw, dh, dw)
        L = OH * OW
        out = _split_matmul_core(xq, geom, N * L, C * kh * kw, ones, ones_q, s1, wm.contiguous(), inputBits, dacBits,
                                 adcBits, weightBits, arr, in_mode == "neg_pulse", cfg, solver,
                                 bias=bias if (bias is not None and use_fp_bias) else None, L=L, rand_gen=rand_gen)
        return out.reshape(N, Cout, OH, OW)


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


class Conv2d_sp(torch.nn.Module):
    """Conv2d_sp (fixedPoint/nn/modules/conv_split.py:29-136): float training,
    crossbar-simulated evaluation through ``conv2d_split``.  Zero padding and
    groups = 1 in evaluation, as the reference's unfold path supports."""

    def __init__(self, in_channels, out_channels, kernel_size, stride=1, padding=0, dilation=1, groups=1, bias=True,
                 padding_mode="zeros", input_bit_width=8, output_bit_width=10, weight_bit_width=8, dac_bit_width=1,
                 adc_bit_width=10, phy_arr_mode="PN", fp_type=torch.float32, use_fp_bias=True, cfg=None, solver=None):
        super().__init__()
        if groups <= 0:
            raise ValueError("groups must be a positive integer")
        if in_channels % groups != 0:
            raise ValueError("in_channels must be divisible by groups")
        if out_channels % groups != 0:
            raise ValueError("out_channels must be divisible by groups")
        pair = lambda t: tuple(t) if isinstance(t, (tuple, list)) else (t, t)
        self.in_channels, self.out_channels = in_channels, out_channels
        self.kernel_size, self.stride = pair(kernel_size), pair(stride)
        self.padding, self.dilation = pair(padding), pair(dilation)
        self.groups, self.padding_mode = groups, padding_mode
        self.hasBias, self.useFpBias = bias, use_fp_bias
        self.inputBits, self.outputBits, self.weightBits = input_bit_width, output_bit_width, weight_bit_width
        self.adcBits, self.dacBits = adc_bit_width, dac_bit_width
        self.phyArrMode, self.fp_type = phy_arr_mode, fp_type
        self.cfg, self.solver = cfg, solver
        self.fp_weight = torch.nn.Parameter(torch.empty((out_channels, in_channels // groups, *self.kernel_size),
                                                        dtype=fp_type))
        self.fp_bias = torch.nn.Parameter(torch.empty(out_channels, dtype=fp_type)) if bias else None
        torch.nn.init.kaiming_uniform_(self.fp_weight, a=math.sqrt(5))
        if self.fp_bias is not None:
            fan_in = self.fp_weight[0].numel()
            bound = 1 / math.sqrt(fan_in) if fan_in else 0
            torch.nn.init.uniform_(self.fp_bias, -bound, bound)

    def forward(self, input):
        if self.training:
            if self.padding_mode != "zeros":
                pad = (self.padding[1], self.padding[1], self.padding[0], self.padding[0])
                return torch.nn.functional.conv2d(torch.nn.functional.pad(input, pad, mode=self.padding_mode),
                                                  self.fp_weight, self.fp_bias, self.stride, 0, self.dilation,
                                                  self.groups)
            return torch.nn.functional.conv2d(input, self.fp_weight, self.fp_bias, self.stride, self.padding,
                                              self.dilation, self.groups)
        if self.groups != 1 or self.padding_mode != "zeros":
            raise NotImplementedError("crossbar evaluation supports groups=1 and zero padding")
        return conv2d_split(input, self.fp_weight, self.fp_bias if self.hasBias else None, self.stride, self.padding,
                            self.dilation, self.inputBits, self.dacBits, self.adcBits, self.outputBits,
                            self.weightBits, self.phyArrMode, self.useFpBias, cfg=self.cfg, solver=self.solver)
