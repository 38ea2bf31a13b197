"""Cycle-to-cycle conductance variation of the cells.

``add_variation`` draws like the reference (conductance_variation.py:6-13):
G / exp(sigma * N(0, 1)) with the normal draws taken from a torch CPU generator
(PimTorch passes ``variations.rand_gen_network``, commonConst.py:122-154), so
the same generator state gives the same numbers as the reference; the division
runs on G's device (``fadesim_vary_conductance_f32``, one correctly rounded
FP32 division per cell, as torch's).  ``variations`` mirrors the reference's
generator holder (default seed 555; the network generator is seeded 557 and
reset per test batch with ``network_gen_reset``); the layer path
(``splitarr``) draws from ``variations.rand_gen_network`` unless given another
generator.

``add_variation_device`` draws on the GPU instead, from a counter hash of
(seed, cell): different numbers from the reference's generator, same
distribution (R becomes R * exp(sigma * z), the lognormal spread of the
large-tile non-ideal configuration), the same on every run and device, with no
host round trip.
"""
import torch

from . import _lib


class variations:
    """The reference's generator holder (commonConst.py:122-154), same seeds."""
    var_defaultSeed = 555
    rand_gen_memCMOS = torch.Generator()
    rand_gen_mirrored = torch.Generator()
    rand_gen_network = torch.Generator()
    rand_gen_memCMOS.manual_seed(var_defaultSeed)
    rand_gen_mirrored.manual_seed(var_defaultSeed + 1)
    rand_gen_network.manual_seed(var_defaultSeed + 2)

    @staticmethod
    def network_gen_reset(seed=var_defaultSeed):
        variations.rand_gen_network.manual_seed(seed + 2)

    @staticmethod
    def mirrored_gen_reset(seed=var_defaultSeed):
        variations.rand_gen_mirrored.manual_seed(seed + 1)

    @staticmethod
    def memCMOS_gen_reset(seed=var_defaultSeed):
        variations.rand_gen_memCMOS.manual_seed(seed)

    @staticmethod
    def reset_all(seed=var_defaultSeed):
        variations.memCMOS_gen_reset(seed)
        variations.mirrored_gen_reset(seed)
        variations.network_gen_reset(seed)


def variation_divisor(shape, sigma, rand_gen=None):
    """exp(sigma * N(0, 1)) for every cell of ``shape``, drawn on the CPU from
    ``rand_gen`` exactly as the reference draws them (float32)."""
    return torch.exp(torch.randn(shape, generator=rand_gen) * sigma)


def _divide_on_device(G, divisor, out=None):
    """out = G / divisor on G's CUDA device in the library's kernel."""
    lib = _lib.load()
    out = torch.empty_like(G) if out is None else out
    d = divisor.to(device=G.device, dtype=torch.float32).contiguous()
    _lib.check(lib.fadesim_vary_conductance_f32(G.data_ptr(), d.data_ptr(), G.numel(), 0.0, 0, 0, out.data_ptr(),
                                                torch.cuda.current_stream(G.device).cuda_stream))
    return out


def add_variation(conductance, sigma=0, rand_gen=None):
    """G / exp(sigma * N(0, 1)) with the reference's draws (see the module text)."""
    if isinstance(conductance, torch.Tensor):
        div = variation_divisor(conductance.shape, sigma, rand_gen)
        if conductance.is_cuda and conductance.dtype == torch.float32:
            return _divide_on_device(conductance.contiguous(), div)
        return conductance / div.to(conductance.device)
    if isinstance(conductance, (float, int)):
        return conductance / variation_divisor([1], sigma, rand_gen)
    raise TypeError("add_variation takes a tensor or a number, not %s" % type(conductance).__name__)


def add_variation_device(conductance, sigma, seed, offset=0):
    """G / exp(sigma * z) with z a standard normal per cell from a counter hash
    of (seed, offset + cell index): float32 CUDA tensors, in the library's kernel."""
    if not (isinstance(conductance, torch.Tensor) and conductance.is_cuda and conductance.dtype == torch.float32):
        raise TypeError("add_variation_device takes a float32 CUDA tensor")
    if not sigma >= 0:
        raise ValueError("sigma must be >= 0")
    lib = _lib.load()
    G = conductance.contiguous()
    out = torch.empty_like(G)
    _lib.check(lib.fadesim_vary_conductance_f32(G.data_ptr(), None, G.numel(), float(sigma),
                                                int(seed) & (2 ** 64 - 1), int(offset) & (2 ** 64 - 1),
                                                out.data_ptr(), torch.cuda.current_stream(G.device).cuda_stream))
    return out
