"""Cycle-to-cycle conductance variation of the cells.

``add_variation`` follows the reference exactly (conductance_variation.py:6-13):
G / exp(sigma * N(0, 1)), the normal draws taken from a torch CPU generator
(PimTorch passes ``variations.rand_gen_network``, commonConst.py:122-154) and
moved to G's device, so the same generator state gives the same bits as the
reference.  ``add_variation_device`` draws on the GPU from a seeded device
generator for large batches (different numbers, same distribution): R becomes
R * exp(sigma * N(0, 1)), the lognormal spread of the large-tile non-ideal
configuration.
"""
import torch


def add_variation(conductance, sigma=0, rand_gen=None):
    if isinstance(conductance, torch.Tensor):
        return conductance / torch.exp(torch.randn(conductance.shape, generator=rand_gen) * sigma).to(
            conductance.device)
    if isinstance(conductance, (float, int)):
        return conductance / torch.exp(torch.randn([1], generator=rand_gen) * sigma)
    raise Exception("Conductance variation for data type {} is not implemented.".format(type(conductance)))


def add_variation_device(conductance, sigma, seed):
    g = torch.Generator(device=conductance.device)
    g.manual_seed(int(seed))
    noise = torch.randn(conductance.shape, generator=g, device=conductance.device, dtype=conductance.dtype)
    return conductance / torch.exp(noise * sigma)
