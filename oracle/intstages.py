"""numpy restatement of PimTorch's integer stages around the IR-drop solve.

Test infrastructure only: see ``oracle/__init__.py``.

Covers the whole-array (no OU) path of ``splitArr_matmul_nn`` / ``matmul`` for
PN and Ref-column arrays, complement-code and negative-pulse inputs, and the
``Conv2d_sp`` evaluation path around it:

* fixed-point quantisation, s = ceil(log2(max|x| / (2^(b-1)-1))) for Normal and
  ceil(log2(max|x| / (2^b-1))) for PN, x_int = round-half-even(x / 2^s)
  (fixedPointArithmetic.py:19-27,76-96);
* PN split into positive and negative magnitudes (splitArrayArithmetic.py:1191-1195);
* input bit i = (x_int >> i) & 1, weight slice j = (w >> j) & (2^cellBits-1)
  (splitArrayArithmetic.py:1199-1215);
* zero padding to whole tiles, G = slice*dG + Gmin, inputs * inputV
  (splitArrayArithmetic.py:705-757);
* ADC code = round(I / adcUseI * (2^adc-1)), no clamp (splitArrayArithmetic.py:835-836);
* sum over row tiles, crop, * rows*(2^dac-1)*(2^cell-1)/(2^adc-1), pos - neg
  (splitArrayArithmetic.py:961-978);
* shift-add: output +/- out * 2^(i+j+s1+s2), the top input bit subtracted
  (complement code) (splitArrayArithmetic.py:1224-1227);
* negative-pulse inputs: bit i of a negative input is -((|x| >> i) & mask),
  every bit added (splitArrayArithmetic.py:1183-1187,1202-1203);
* Ref-column arrays: weights quantised as Normal, offset by 2^(b-1) and
  clamped to 2^b-1 (:1229-1242), two reference columns per column block (state 0
  and state 1, :758-771), the state-0 column's code subtracted from every
  column and, for slice 0, 2^(b-1) times the state-1 column's (:980-996);
* Conv2d_sp: unfold, matmul, fold (fixedPoint/nn/modules/conv_split.py:106-134);
* cycle-to-cycle variation: every map divided by exp(sigma N(0,1)) per cell,
  one draw per (input bit, slice, array) call in the reference's loop order
  (conductance_variation.py:6-13, splitArrayArithmetic.py:758-760,788); the
  draws come from a caller's function (the reference's are torch's CPU
  generator, which this restatement does not re-derive).

Every float step is float32 with the reference's operation order; scalar
operands are rounded to float32 first, which is what torch does for a float32
tensor combined with a Python scalar on the CPU.
"""
import math

import numpy as np

f32 = np.float32


class ArrayParams:
    """The phyArrParams / ConstForSplitArray fields these stages read
    (commonConst.py:45-50,187-236), with derived constants computed in the
    reference's order."""

    def __init__(self, Ron=1e3, Roff=1e6, cellBits=1, rows=64, cols=64, inputMaxVoltage=1.0, r_wire=2.93,
                 input_bits=8, weight_bits=8, dac_bits=1, adc_bits=10):
        self.Ron = Ron
        self.Roff = Roff
        self.cellMaxConduct = 1 / Ron
        self.cellMinConduct = 1 / Roff
        self.cellBits = cellBits
        self.arrRowSize = rows
        self.arrColSize = cols
        self.inputMaxVoltage = inputMaxVoltage
        self.r_wire = r_wire
        self.cellDeltaConduct = (self.cellMaxConduct - self.cellMinConduct) / (2 ** cellBits - 1)
        self.adcUseI = rows * (self.cellMaxConduct - self.cellMinConduct) * inputMaxVoltage
        self.input_bits = input_bits
        self.weight_bits = weight_bits
        self.dac_bits = dac_bits
        self.adc_bits = adc_bits


def fixed_point_position(max_abs, bit_width, pn):
    if math.isclose(max_abs, 0.0):
        max_abs = 1e-12
    if pn:
        return math.ceil(math.log2(max_abs / ((1 << bit_width) - 1)))
    return math.ceil(math.log2(max_abs / ((1 << (bit_width - 1)) - 1)))


def quantize(x, bit_width, pn):
    x = np.asarray(x, f32)
    max_abs = float(np.abs(x).max())
    s = fixed_point_position(max_abs, bit_width, pn)
    return np.round(x / f32(pow(2, s))).astype(np.int32), s


def ideal_solver(in_v, G, B, rows, cols, numX, numY):
    """I = sum_i v_i G_ij, summed sequentially in float64 then rounded to float32."""
    in_v = np.asarray(in_v, np.float64).reshape(B, numX, rows, 1)
    G = np.asarray(G, np.float64).reshape(1, numX, rows, numY * cols)
    return np.cumsum(in_v * G, axis=2)[:, :, -1, :].astype(f32)


def slice_matmul(in_b, g_pos, g_neg, p, solver, vary=None):
    """One input-bit x weight-slice product through two IR-drop solves.

    in_b [B, insize] in {0,1}; g_pos/g_neg [insize, outsize] cell states.
    vary(shape), if given, returns the float32 divisors exp(sigma N(0,1)) of a
    cycle-to-cycle variation draw; it is called for the positive map, then the
    negative one (splitArrayArithmetic.py:758-760).
    Returns float32 [B, outsize] (matmul PN branch, splitArrayArithmetic.py:698-978).
    """
    B, insize = in_b.shape
    outsize = g_pos.shape[1]
    rows, cols = p.arrRowSize, p.arrColSize
    inputV = p.inputMaxVoltage / (2 ** p.dac_bits - 1)
    pad_in = (-insize) % rows
    pad_out = (-outsize) % cols
    in_b = np.pad(in_b, ((0, 0), (0, pad_in)))
    g_pos = np.pad(g_pos, ((0, pad_in), (0, pad_out)))
    g_neg = np.pad(g_neg, ((0, pad_in), (0, pad_out)))
    true_in, true_out = insize + pad_in, outsize + pad_out
    numX, numY = true_in // rows, true_out // cols
    in_f = (in_b.astype(f32) * f32(inputV)).reshape(B, numX, rows)
    Gp = (g_pos.astype(f32) * f32(p.cellDeltaConduct) + f32(p.cellMinConduct)).reshape(numX, rows, true_out)
    Gn = (g_neg.astype(f32) * f32(p.cellDeltaConduct) + f32(p.cellMinConduct)).reshape(numX, rows, true_out)
    if vary is not None:
        Gp = (Gp / np.asarray(vary(Gp.shape), f32)).astype(f32)
        Gn = (Gn / np.asarray(vary(Gn.shape), f32)).astype(f32)
    Ip = np.asarray(solver(in_f, Gp, B, rows, cols, numX, numY), f32)
    In = np.asarray(solver(in_f, Gn, B, rows, cols, numX, numY), f32)
    levels = f32(2 ** p.adc_bits - 1)
    cp = np.round((Ip / f32(p.adcUseI)) * levels)
    cn = np.round((In / f32(p.adcUseI)) * levels)
    scale = f32(rows * (2 ** p.dac_bits - 1) * (2 ** p.cellBits - 1) / (2 ** p.adc_bits - 1))
    op = cp.sum(axis=1, dtype=f32)[:, :outsize] * scale
    on = cn.sum(axis=1, dtype=f32)[:, :outsize] * scale
    return (op - on).astype(f32)


def split_matmul(x, w, p, solver=ideal_solver, return_codes=False):
    """splitArr_matmul_nn for the PN array mode (splitArrayArithmetic.py:1161-1228).

    x [B, insize] float, w [insize, outsize] float.  Returns float32 [B, outsize].
    """
    x = np.asarray(x, f32)
    w = np.asarray(w, f32)
    B = x.shape[0]
    xi, s1 = quantize(x, p.input_bits, pn=False)
    wi, s2 = quantize(w, p.weight_bits, pn=True)
    wpos = np.where(wi < 0, 0, wi).astype(np.int32)
    wneg = np.abs(np.where(wi > 0, 0, wi)).astype(np.int32)
    out = np.zeros((B, w.shape[1]), f32)
    mask_cell = (1 << p.cellBits) - 1
    mask_in = (1 << p.dac_bits) - 1
    for i in range(0, p.input_bits, p.dac_bits):
        in_b = (xi >> i) & mask_in
        for j in range(0, p.weight_bits, p.cellBits):
            gp = (wpos >> j) & mask_cell
            gn = (wneg >> j) & mask_cell
            o = slice_matmul(in_b, gp, gn, p, solver)
            k = f32(2.0 ** (i + j + s1 + s2))
            if i != p.input_bits - 1:
                out = (out + o * k).astype(f32)
            else:
                out = (out - o * k).astype(f32)
    return out


def droop_solver(in_v, G, B, rows, cols, numX, numY):
    """Deterministic stand-in for the IR-drop solve used to pin the integer stages.

    Ideal currents times a column-dependent droop, all in float64 with a
    sequential sum, rounded once to float32: the same bits on any IEEE host.
    """
    ideal = ideal_solver(in_v, G, B, rows, cols, numX, numY).astype(np.float64)
    j = np.arange(numY * cols) % cols
    return (ideal * (1.0 - 0.0031 * (j % 11) - 0.0007 * (j // 11))).astype(f32)


def slice_matmul_ref(in_v, g, j, p, solver, vary=None):
    """One input-bit x weight-slice product on a Ref-column array
    (matmul, splitArrayArithmetic.py:758-771 map, :818 solve, :835-836 ADC,
    :980-996 reference-column subtraction).

    in_v [B, insize] input levels (signed for negative pulses); g [insize,
    outsize] cell states of slice j; vary as for slice_matmul, one draw for the
    whole map with its reference columns (:788).  Returns float32 [B, outsize].
    """
    B, insize = in_v.shape
    outsize = g.shape[1]
    rows, cols = p.arrRowSize, p.arrColSize
    inputV = p.inputMaxVoltage / (2 ** p.dac_bits - 1)
    pad_in = (-insize) % rows
    pad_out = (-outsize) % cols
    in_v = np.pad(in_v, ((0, 0), (0, pad_in)))
    g = np.pad(g, ((0, pad_in), (0, pad_out)))
    true_in, true_out = insize + pad_in, outsize + pad_out
    numX, numY = true_in // rows, true_out // cols
    extra = np.zeros((true_in, numY, 2), g.dtype)
    extra[..., 1] = 1
    g = np.concatenate([g.reshape(true_in, numY, cols), extra], axis=2)
    G = (g.astype(f32) * f32(p.cellDeltaConduct) + f32(p.cellMinConduct)).reshape(numX, rows, numY * (cols + 2))
    if vary is not None:
        G = (G / np.asarray(vary(G.shape), f32)).astype(f32)
    in_f = (in_v.astype(f32) * f32(inputV)).reshape(B, numX, rows)
    I = np.asarray(solver(in_f, G, B, rows, cols + 2, numX, numY), f32)
    code = np.round((I / f32(p.adcUseI)) * f32(2 ** p.adc_bits - 1)).reshape(B, numX, numY, cols + 2)
    code = code - code[..., cols:cols + 1]
    if j == 0:
        plus = 2 ** (p.weight_bits - 1)
        code = code - np.round(code[..., cols + 1:cols + 2] * f32(plus))
    scale = f32(rows * (2 ** p.dac_bits - 1) * (2 ** p.cellBits - 1) / (2 ** p.adc_bits - 1))
    return (code[..., :cols].sum(axis=1, dtype=f32).reshape(B, -1)[:, :outsize] * scale).astype(f32)


def split_matmul_ex(x, w, p, arr="PN", neg_pulse=False, solver=ideal_solver, vary=None):
    """splitArr_matmul_nn (splitArrayArithmetic.py:1161-1260) for PN or Ref
    arrays and complement-code or negative-pulse inputs; vary(shape) draws the
    conductance variation of every map in the reference's call order (input
    bit outer, slice inner, positive before negative)."""
    x = np.asarray(x, f32)
    w = np.asarray(w, f32)
    B = x.shape[0]
    xi, s1 = quantize(x, p.input_bits, pn=False)
    if not neg_pulse and p.dac_bits != 1:
        raise ValueError("complement-code inputs need a 1-bit DAC")
    mask_cell = (1 << p.cellBits) - 1
    mask_in = (1 << p.dac_bits) - 1

    def in_bits(i):
        b = (xi >> i) & mask_in
        if neg_pulse:
            b = np.where(xi < 0, -((np.abs(xi) >> i) & mask_in), b)
        return b

    def sign(i):
        return -1 if (i == p.input_bits - 1 and not neg_pulse) else 1

    out = np.zeros((B, w.shape[1]), f32)
    if arr == "PN":
        wi, s2 = quantize(w, p.weight_bits, pn=True)
        wpos = np.where(wi < 0, 0, wi).astype(np.int32)
        wneg = np.abs(np.where(wi > 0, 0, wi)).astype(np.int32)
        for i in range(0, p.input_bits, p.dac_bits):
            ib = in_bits(i)
            for j in range(0, p.weight_bits, p.cellBits):
                o = slice_matmul(ib, (wpos >> j) & mask_cell, (wneg >> j) & mask_cell, p, solver, vary)
                t = o * f32(2.0 ** (i + j + s1 + s2))
                out = (out + t if sign(i) > 0 else out - t).astype(f32)
        return out
    wi, s2 = quantize(w, p.weight_bits, pn=False)
    plus = 2 ** (p.weight_bits - 1)
    wi = np.minimum(wi + plus, 2 ** p.weight_bits - 1).astype(np.int32)
    for i in range(0, p.input_bits, p.dac_bits):
        ib = in_bits(i)
        for j in range(0, p.weight_bits, p.cellBits):
            o = slice_matmul_ref(ib, (wi >> j) & mask_cell, j, p, solver, vary)
            t = o * f32(2.0 ** (i + j + s1 + s2))
            out = (out + t if sign(i) > 0 else out - t).astype(f32)
    return out


def unfold(x, kh, kw, stride=(1, 1), padding=(0, 0), dilation=(1, 1)):
    """torch.nn.functional.unfold as a [N*L, C*kh*kw] matrix (rows = output
    positions, columns ordered channel, kernel row, kernel column)."""
    x = np.asarray(x)
    N, C, H, W = x.shape
    sh, sw = stride
    ph, pw = padding
    dh, dw = dilation
    OH = (H + 2 * ph - dh * (kh - 1) - 1) // sh + 1
    OW = (W + 2 * pw - dw * (kw - 1) - 1) // sw + 1
    xp = np.pad(x, ((0, 0), (0, 0), (ph, ph), (pw, pw)))
    cols = np.empty((N, OH, OW, C, kh, kw), x.dtype)
    for ki in range(kh):
        for kj in range(kw):
            cols[:, :, :, :, ki, kj] = xp[:, :, ki * dh:ki * dh + sh * (OH - 1) + 1:sh,
                                          kj * dw:kj * dw + sw * (OW - 1) + 1:sw].transpose(0, 2, 3, 1)
    return cols.reshape(N * OH * OW, C * kh * kw), OH, OW


def conv2d_sp(x, weight, bias, p, stride=(1, 1), padding=(0, 0), dilation=(1, 1), arr="PN", neg_pulse=False,
              use_fp_bias=True, solver=ideal_solver, vary=None):
    """Conv2d_sp evaluation (conv_split.py:106-134): unfold, the split matmul
    against W reshaped [Cout, C*kh*kw] and transposed, bias in float32 (or
    mapped to an extra array row driven by ones), fold back to NCHW."""
    x = np.asarray(x, f32)
    weight = np.asarray(weight, f32)
    N = x.shape[0]
    Cout, _, kh, kw = weight.shape
    cols, OH, OW = unfold(x, kh, kw, stride, padding, dilation)
    wm = weight.reshape(Cout, -1).T
    if bias is not None and not use_fp_bias:
        cols = np.concatenate([cols, np.ones((cols.shape[0], 1), f32)], axis=1)
        wm = np.concatenate([wm, np.asarray(bias, f32)[None]], axis=0)
    y = split_matmul_ex(cols, wm, p, arr=arr, neg_pulse=neg_pulse, solver=solver, vary=vary)
    if bias is not None and use_fp_bias:
        y = (y + np.asarray(bias, f32)).astype(f32)
    return np.ascontiguousarray(y.reshape(N, OH * OW, Cout).transpose(0, 2, 1)).reshape(N, Cout, OH, OW)
