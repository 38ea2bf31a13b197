"""Learned warm start for the crossbar solve.

A BF16 convolutional encoder-decoder maps a tile's normalised conductance map
and its wordline voltages to predicted node-voltage deviations from the ideal
state (wordline u - vin, bitline d); the line solver starts from that
prediction and iterates to the same tolerance as from zero, and rejects the
prediction when its first correction is as large as the solution.  Every
layer runs in the project's CUDA kernels (``csrc/warmnet_tc.cu``: 3x3
convolutions and their input gradients as implicit GEMMs on the tcgen05
tensor cores, fed by TMA, accumulating in tensor memory; ``csrc/warmnet.cu``:
weight gradients, the convolutions of levels too small for the 128-pixel
tile, pooling, upsampling, ReLU, MSE, Adam); torch tensors only hold the
buffers.

Architecture (NHWC, "same" 3x3 convolutions, 4 levels):
  e1 = relu(conv(x, 32->32))            @ S      (x: 2 used input channels, 30 zero)
  e2 = relu(conv(pool(e1), 32->64))     @ S/2
  e3 = relu(conv(pool(e2), 64->96))     @ S/4
  e4 = relu(conv(pool(e3), 96->128))    @ S/8
  d3 = relu(conv(up(e4), 128->96)) + e3 @ S/4
  d2 = relu(conv(up(d3), 96->64)) + e2  @ S/2
  d1 = relu(conv(up(d2), 64->32)) + e1  @ S
  y  = conv(d1, 32->32)                 @ S      (2 output channels used, FP32)
Inputs: channel 0 = G / max(G) of the tile, channel 1 = vin_i / max(vin) on row
i.  Targets: deviations / (0.05 max(vin)).
"""
import math
import os

import torch

from . import _lib

CH = [32, 64, 96, 128]
CIN = 32   # padded input channels (2 used): every layer's Cin a multiple of 32, for the tensor-core kernel
COUT = 32  # padded output channels (2 used)
TARGET_SCALE = 0.05

_SIGS = {
    "fadesim_conv3x3_fwd_bf16": "vvpvviiiiiiv",
    "fadesim_conv3x3_wgrad_bf16": "vvpiiiiiv",
    "fadesim_weight_flip_bf16": "vviiiv",
    "fadesim_bias_grad_bf16": "vpliv",
    "fadesim_pool_bf16": "vviiiiiiv",
    "fadesim_relu_bwd_bf16": "vvvlv",
    "fadesim_add_bf16": "vvvlv",
    "fadesim_mse_f32": "pppvliiv",
    "fadesim_adam_f32": "pvppplffffiv",
    "fadesim_conv_tc_status": "v",
    "fadesim_conv_tc_shape": "iiii",
}


def _bind():
    import ctypes
    lib = _lib.load()
    m = {"v": ctypes.c_void_p, "p": ctypes.c_void_p, "i": ctypes.c_int, "l": ctypes.c_longlong, "f": ctypes.c_float}
    for name, sig in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = [m[c] for c in sig]
        fn.restype = ctypes.c_int
    return lib


_L = None


def _k():
    global _L
    if _L is None:
        _L = _bind()
    return _L


def _st():
    return torch.cuda.current_stream().cuda_stream


def _chk(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (%d)" % (what, rc))


def _p(t):
    return t.data_ptr() if t is not None else None


class Conv:
    """One 3x3 convolution: FP32 master weights, bf16 copy, Adam moments."""

    def __init__(self, cin, cout, gen, device):
        fan = 9 * cin
        w = torch.randn((cout, 3, 3, cin), generator=gen) * math.sqrt(2.0 / fan)
        self.cin, self.cout = cin, cout
        self.w = w.to(device).contiguous()
        self.b = torch.zeros(cout, device=device)
        self.wb = self.w.to(torch.bfloat16).contiguous()
        self.gw = torch.zeros_like(self.w)
        self.gb = torch.zeros_like(self.b)
        self.mw, self.vw = torch.zeros_like(self.w), torch.zeros_like(self.w)
        self.mb, self.vb = torch.zeros_like(self.b), torch.zeros_like(self.b)
        self.flip = torch.empty((cin, 3, 3, cout), dtype=torch.bfloat16, device=device)

    def fwd(self, x, relu, skip=None, f32=False, legacy=False):
        """legacy: run the mma.sync kernel even where the tensor-core kernel applies."""
        N, H, W, _ = x.shape
        y = torch.empty((N, H, W, self.cout), dtype=torch.float32 if f32 else torch.bfloat16, device=x.device)
        flags = (1 if relu else 0) | (2 if skip is not None else 0) | (4 if f32 else 0) | (8 if legacy else 0)
        _chk(_k().fadesim_conv3x3_fwd_bf16(_p(x), _p(self.wb), _p(self.b), _p(skip), _p(y), N, H, W, self.cin,
                                           self.cout, flags, _st()), "conv fwd")
        return y

    def bwd(self, dz, x, need_dx=True):
        """dz: gradient at the conv output (pre-activation); x: conv input."""
        N, H, W, _ = x.shape
        _chk(_k().fadesim_conv3x3_wgrad_bf16(_p(dz), _p(x), _p(self.gw), N, H, W, self.cin, self.cout, _st()),
             "conv wgrad")
        _chk(_k().fadesim_bias_grad_bf16(_p(dz), _p(self.gb), N * H * W, self.cout, _st()), "bias grad")
        if not need_dx:
            return None
        _chk(_k().fadesim_weight_flip_bf16(_p(self.wb), _p(self.flip), self.cin, self.cout, self.cin, _st()), "flip")
        dx = torch.empty((N, H, W, self.cin), dtype=torch.bfloat16, device=x.device)
        _chk(_k().fadesim_conv3x3_fwd_bf16(_p(dz), _p(self.flip), None, None, _p(dx), N, H, W, self.cout, self.cin, 0,
                                           _st()), "conv dgrad")
        return dx

    def zero_grad(self):
        self.gw.zero_()
        self.gb.zero_()

    def adam(self, lr, step, b1=0.9, b2=0.999, eps=1e-8):
        _chk(_k().fadesim_adam_f32(_p(self.w), _p(self.wb), _p(self.gw), _p(self.mw), _p(self.vw), self.w.numel(),
                                   lr, b1, b2, eps, step, _st()), "adam")
        _chk(_k().fadesim_adam_f32(_p(self.b), None, _p(self.gb), _p(self.mb), _p(self.vb), self.b.numel(), lr, b1,
                                   b2, eps, step, _st()), "adam")

    def state(self):
        return {k: getattr(self, k).cpu() for k in ("w", "b", "mw", "vw", "mb", "vb")}

    def load(self, st):
        for k, v in st.items():
            getattr(self, k).copy_(v)
        self.wb.copy_(self.w.to(torch.bfloat16))


def _pool(x, backward=False, up=False):
    N, H, W, C = x.shape
    if up and not backward:
        y = torch.empty((N, 2 * H, 2 * W, C), dtype=x.dtype, device=x.device)
        _chk(_k().fadesim_pool_bf16(_p(x), _p(y), N, H, W, C, 0, 1, _st()), "upsample")
    elif up:
        y = torch.empty((N, H // 2, W // 2, C), dtype=x.dtype, device=x.device)
        _chk(_k().fadesim_pool_bf16(_p(x), _p(y), N, H // 2, W // 2, C, 1, 1, _st()), "upsample bwd")
    elif not backward:
        y = torch.empty((N, H // 2, W // 2, C), dtype=x.dtype, device=x.device)
        _chk(_k().fadesim_pool_bf16(_p(x), _p(y), N, H, W, C, 0, 0, _st()), "pool")
    else:
        y = torch.empty((N, 2 * H, 2 * W, C), dtype=x.dtype, device=x.device)
        _chk(_k().fadesim_pool_bf16(_p(x), _p(y), N, 2 * H, 2 * W, C, 1, 0, _st()), "pool bwd")
    return y


def _relu_bwd(dy, act):
    dz = torch.empty_like(dy)
    _chk(_k().fadesim_relu_bwd_bf16(_p(dy), _p(act), _p(dz), dy.numel(), _st()), "relu bwd")
    return dz


def _add(a, b):
    c = torch.empty_like(a)
    _chk(_k().fadesim_add_bf16(_p(a), _p(b), _p(c), a.numel(), _st()), "add")
    return c


class WarmStartNet:
    """The encoder-decoder; ``device`` must be CUDA (no CPU path)."""

    def __init__(self, seed=0, device="cuda"):
        gen = torch.Generator()
        gen.manual_seed(seed)
        c1, c2, c3, c4 = CH
        self.layers = {
            "e1": Conv(CIN, c1, gen, device), "e2": Conv(c1, c2, gen, device), "e3": Conv(c2, c3, gen, device),
            "e4": Conv(c3, c4, gen, device), "d3": Conv(c4, c3, gen, device), "d2": Conv(c3, c2, gen, device),
            "d1": Conv(c2, c1, gen, device), "out": Conv(c1, COUT, gen, device),
        }
        self.layers["out"].w.mul_(0.1)
        self.layers["out"].wb.copy_(self.layers["out"].w.to(torch.bfloat16))
        self.step = 0
        self.cache = None

    # ---- data ----------------------------------------------------------------
    @staticmethod
    def make_inputs(G, vin):
        """G [N, n, m] (any float), vin [N, n] -> bf16 NHWC input [N, n, m, CIN] and the
        per-instance target scale [N]."""
        N, n, m = G.shape
        x = torch.zeros((N, n, m, CIN), dtype=torch.float32, device=G.device)
        gmax = G.reshape(N, -1).amax(dim=1).clamp_min(1e-30)
        vmax = vin.abs().amax(dim=1)
        x[..., 0] = G / gmax[:, None, None]
        x[..., 1] = (vin / vmax.clamp_min(1e-30)[:, None])[:, :, None]
        scale = (TARGET_SCALE * vmax).clamp_min(1e-12)
        return x.to(torch.bfloat16).contiguous(), scale

    # ---- forward / backward --------------------------------------------------
    def forward(self, x, keep=False):
        L = self.layers
        e1 = L["e1"].fwd(x, True)
        p1 = _pool(e1)
        e2 = L["e2"].fwd(p1, True)
        p2 = _pool(e2)
        e3 = L["e3"].fwd(p2, True)
        p3 = _pool(e3)
        e4 = L["e4"].fwd(p3, True)
        u3 = _pool(e4, up=True)
        a3 = L["d3"].fwd(u3, True)
        d3 = _add(a3, e3)
        u2 = _pool(d3, up=True)
        a2 = L["d2"].fwd(u2, True)
        d2 = _add(a2, e2)
        u1 = _pool(d2, up=True)
        a1 = L["d1"].fwd(u1, True)
        d1 = _add(a1, e1)
        y = L["out"].fwd(d1, False, f32=True)
        if keep:
            self.cache = dict(x=x, e1=e1, p1=p1, e2=e2, p2=p2, e3=e3, p3=p3, e4=e4, u3=u3, a3=a3, u2=u2, a2=a2,
                              u1=u1, a1=a1, d1=d1)
        return y

    def backward(self, dy):
        """dy: bf16 gradient at the output [N, S, S, COUT]; accumulates parameter gradients."""
        c, L = self.cache, self.layers
        dd1 = L["out"].bwd(dy, c["d1"])
        du1 = L["d1"].bwd(_relu_bwd(dd1, c["a1"]), c["u1"])
        dd2 = _pool(du1, backward=True, up=True)
        du2 = L["d2"].bwd(_relu_bwd(dd2, c["a2"]), c["u2"])
        dd3 = _pool(du2, backward=True, up=True)
        du3 = L["d3"].bwd(_relu_bwd(dd3, c["a3"]), c["u3"])
        de4 = _pool(du3, backward=True, up=True)
        dp3 = L["e4"].bwd(_relu_bwd(de4, c["e4"]), c["p3"])
        de3 = _add(dd3, _pool(dp3, backward=True))
        dp2 = L["e3"].bwd(_relu_bwd(de3, c["e3"]), c["p2"])
        de2 = _add(dd2, _pool(dp2, backward=True))
        dp1 = L["e2"].bwd(_relu_bwd(de2, c["e2"]), c["p1"])
        de1 = _add(dd1, _pool(dp1, backward=True))
        L["e1"].bwd(_relu_bwd(de1, c["e1"]), c["x"], need_dx=False)

    def loss_and_grad(self, y, target):
        """MSE over the 2 used channels; returns (loss tensor, bf16 dy)."""
        N, S1, S2, _ = y.shape
        loss = torch.zeros(1, device=y.device)
        dy = torch.empty(y.shape, dtype=torch.bfloat16, device=y.device)
        _chk(_k().fadesim_mse_f32(_p(y), _p(target), _p(dy), _p(loss), N * S1 * S2, COUT, 2, _st()), "mse")
        return loss, dy

    def train_step(self, x, target, lr=1e-3):
        for l in self.layers.values():
            l.zero_grad()
        y = self.forward(x, keep=True)
        loss, dy = self.loss_and_grad(y, target)
        self.backward(dy)
        self.step += 1
        for l in self.layers.values():
            l.adam(lr, self.step)
        self.cache = None
        return loss

    # ---- use as a warm start -------------------------------------------------
    def predict_planes(self, G, vin):
        """G [N, n, m], vin [N, n] -> FP32 planes [N, 2, n, m]: predicted wordline
        deviations u - vin and bitline voltages d."""
        x, scale = self.make_inputs(G, vin)
        y = self.forward(x)
        return (y[..., :2].permute(0, 3, 1, 2) * scale[:, None, None, None]).contiguous()

    def state_dict(self):
        return {"step": self.step, "layers": {k: l.state() for k, l in self.layers.items()}}

    def load_state_dict(self, sd):
        self.step = sd["step"]
        for k, st in sd["layers"].items():
            self.layers[k].load(st)

    def save(self, path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        torch.save(self.state_dict(), path)

    def load(self, path):
        self.load_state_dict(torch.load(path, map_location="cpu"))


def solver_targets(G, vin, solve_planes):
    """Training targets from the solver itself: deviations scaled like the output."""
    planes = solve_planes(G, vin)  # [N, 2, n, m]: wordline deviation, bitline voltage
    vmax = vin.abs().amax(dim=1)
    scale = (TARGET_SCALE * vmax).clamp_min(1e-12)
    return (planes / scale[:, None, None, None]).permute(0, 2, 3, 1).contiguous()
