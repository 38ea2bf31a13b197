"""The line iteration's stop rule and relaxation schedule (csrc/line_common.cuh
LineStop, driven as csrc/line_impl.cuh drives it), restated in Python around an
FP64 numpy emulation of the block line relaxation, on the CPU.

What is checked is the rule's promise, separately from FP32 rounding: when it
says stop, the iterate is within the tolerance (plus its floor, 4 FP32 ulps of
the largest deviation) of the nodal solution, for weak and strong cells,
several sizes and both tolerances the benchmarks use, with the rate and
relaxation factor carried from one input vector of a tile to the next.  Also
the identity behind the fused current epilogue.  The restatement mirrors the
device code; a change there must be mirrored here.
"""
import math

import numpy as np
import pytest

from oracle import nodal

GW = 1 / 2.93
EPS32 = 1.1920929e-07


class LineStop:
    def __init__(self, omega_fixed=0.0, rate_hint=0.0, omega_prev=0.0):
        self.adapt = not (omega_fixed > 0)
        self.omega_hint = omega_prev
        self.omega = 1.0 if self.adapt else omega_fixed
        self.it = 0
        self.h0 = self.h1 = self.h2 = self.h3 = 0.0
        self.hint = self.rho = rate_hint
        self.first = 0.0

    def final_rate(self):
        return self.first if self.first > 0 else self.hint

    def update(self, delta, vm, tol):
        self.it += 1
        prev = self.h0
        self.h3, self.h2, self.h1, self.h0 = self.h2, self.h1, self.h0, delta
        if self.it == 1:
            return delta <= 0
        floor_v = 4 * EPS32 * vm
        ratio = delta / prev if prev > 0 else 0.0
        rate3 = math.pow(delta / self.h3, 1 / 3) if (self.it >= 4 and self.h3 > 0) else 0.0
        rho = max(ratio, rate3, self.omega - 1)
        if self.omega > 1:
            rho = max(rho, 0.5)
        self.rho = rho
        if self.it == 2:
            self.first = ratio
        est = delta * rho / (1 - rho) if rho < 0.999 else math.inf
        stalled = delta <= floor_v and ratio >= 0.9
        if self.adapt:
            w = self.omega
            if self.it == 3 and self.omega_hint > 1:
                self.omega = self.omega_hint
            elif self.it == 3 and 0.05 < ratio < 1:
                self.omega = min(1.95, 2 / (1 + math.sqrt(1 - ratio)))
            elif self.it == 12 and w > 1 and w - 1 + 0.02 < rate3 < 1:
                mu2 = (rate3 + w - 1) ** 2 / (rate3 * w * w)
                if mu2 < 1:
                    w2 = 2 / (1 + math.sqrt(1 - mu2))
                    if w2 > w + 0.01:
                        self.omega = min(1.95, w2)
        return est <= max(tol, floor_v) or stalled


def thomas(lower, diag, upper, rhs):
    """Tridiagonal solves along the last axis, batched over the first."""
    L = diag.shape[-1]
    c = np.zeros_like(diag)
    y = np.zeros_like(rhs)
    p = diag[:, 0]
    c[:, 0] = upper[:, 0] / p
    y[:, 0] = rhs[:, 0] / p
    for k in range(1, L):
        p = diag[:, k] - lower[:, k] * c[:, k - 1]
        c[:, k] = upper[:, k] / p
        y[:, k] = (rhs[:, k] - lower[:, k] * y[:, k - 1]) / p
    x = np.zeros_like(rhs)
    x[:, -1] = y[:, -1]
    for k in range(L - 2, -1, -1):
        x[:, k] = y[:, k] - c[:, k] * x[:, k + 1]
    return x


def line_solve(g, vin, tol, rate_hint=0.0, omega_prev=0.0, max_iters=400):
    """Block line relaxation of one tile and one input vector from the ideal
    state, stopped by LineStop; returns (u, d, iterations, stop)."""
    n, m = g.shape
    # wordline rows: source link + right link (absent at the end) + cell
    wl_diag = GW + np.where(np.arange(m) < m - 1, GW, 0.0)[None, :] + g
    wl_low = np.full((n, m), -GW)
    wl_up = np.where(np.arange(m) < m - 1, -GW, 0.0)[None, :].repeat(n, 0)
    # bitline columns: upper link (absent at the top) + lower link + cell
    bl_diag = (np.where(np.arange(n) > 0, GW, 0.0)[:, None] + GW + g).T
    bl_low = np.where(np.arange(n) > 0, -GW, 0.0)[None, :].repeat(m, 0)
    bl_up = np.full((m, n), -GW)
    u = np.repeat(vin[:, None], m, 1).astype(np.float64)
    d = np.zeros((n, m))
    stop = LineStop(0.0, rate_hint, omega_prev)
    for it in range(1, max_iters + 1):
        w = stop.omega
        rhs = g * d
        rhs[:, 0] += GW * vin
        du = thomas(wl_low, wl_diag, wl_up, rhs) - u
        u = u + w * du
        dd = thomas(bl_low, bl_diag, bl_up, (g * u).T).T - d
        d = d + w * dd
        delta = w * max(np.abs(du).max(), np.abs(dd).max())
        vm = max(np.abs(u - vin[:, None]).max(), np.abs(d).max())
        if stop.update(delta, vm, tol):
            return u, d, it, stop
    raise AssertionError("no convergence in %d iterations" % max_iters)


CFG1 = [2e6, 1.6e6, 1.3e6, 1e6]
STRONG = [1e3, 2e4, 3e5, 1e6]


@pytest.mark.parametrize("n", [16, 48, 64])
@pytest.mark.parametrize("cells,vmax", [(CFG1, 0.2), (STRONG, 1.0)])
@pytest.mark.parametrize("tol", [5e-7, 1e-8])
def test_stop_rule_keeps_its_promise(n, cells, vmax, tol):
    rng = np.random.default_rng(n + int(1e9 * tol))
    g = 1.0 / rng.choice(cells, (n, n))
    rate, omega, iters = 0.0, 0.0, []
    for v in range(4):                                    # the vectors of one tile, in order
        vin = rng.integers(0, 2, n) * vmax
        u, d, it, stop = line_solve(g, vin, tol, rate, omega)
        ue, de = nodal.solve(g, GW, vin)
        err = max(np.abs(u - ue).max(), np.abs(d - de).max())
        dev = max(np.abs(u - vin[:, None]).max(), np.abs(d).max())
        assert err <= tol + 4 * EPS32 * dev, (v, it, err, stop.omega)
        rate, omega = stop.final_rate(), stop.omega
        iters.append(it)
    # weak cells: a few block iterations, as the kernel's counts on the GPU
    if cells is CFG1:
        assert max(iters) <= 4


def test_ground_link_currents_after_an_unrelaxed_bitline_pass():
    """The current epilogue's identity (csrc/line_impl.cuh outputs): after a
    bitline pass at omega 1 every bitline equation holds, so summed down a
    column the wire terms telescope and the column current sum_i g (u - d)
    equals gw d_(n-1) -- from any wordline plane, converged or not.  Over-
    relaxed passes break it, which is why the kernel sums the cells then."""
    rng = np.random.default_rng(9)
    n, m = 40, 24
    g = 1.0 / rng.choice(STRONG, (n, m))
    u = rng.uniform(0, 1, (n, m))
    d_old = rng.uniform(0, 0.1, (n, m))
    bl_diag = (np.where(np.arange(n) > 0, GW, 0.0)[:, None] + GW + g).T
    bl_low = np.where(np.arange(n) > 0, -GW, 0.0)[None, :].repeat(m, 0)
    bl_up = np.full((m, n), -GW)
    d_star = thomas(bl_low, bl_diag, bl_up, (g * u).T).T
    for w, holds in ((1.0, True), (1.5, False)):
        d = d_old + w * (d_star - d_old)
        summed = (g * (u - d)).sum(axis=0)
        link = GW * d[-1]
        gap = np.abs(summed - link).max() / np.abs(summed).max()
        assert (gap < 1e-12) == holds, (w, gap)
