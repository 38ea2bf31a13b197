"""The two-level line relaxation (csrc/coarse_impl.cuh, the TWO variant of
csrc/line_impl.cuh's 128 x 128 kernel) restated on the CPU.

Checked here: the coarse operator it relies on (P^T A P holds no cell
conductance for P = [Phi; Phi]); the compiled factor table against its
generator and against a dense coarse solve; the kernel's restriction and
prolongation index arithmetic (segment slots, lane column weights, the warp
sums, the clamped edges) against the interpolation matrices; the coarse
solve's four products in the kernel's loop order; and the method itself --
block line Gauss-Seidel at omega 1 with the coarse correction after every
iteration, stopped by the line stop rule with its rate taken at least 0.2 --
against the FP64 nodal solution, with far fewer iterations than the plain
schedule on strongly coupled cells.  The restatement mirrors the device
code; a change there must be mirrored here.
"""
import os

import numpy as np
import pytest

from fadesim_gb300 import coarse_tables as ct
from oracle import nodal

import test_stop_rule_cpu as tsr

GW = tsr.GW


def test_coarse_operator_has_no_cell_terms():
    n = m = 32
    P = np.kron(ct.hat(n, 8), ct.hat(m, 8))       # Phi, node (i, j) -> i * m + j
    P2 = np.zeros((2 * n * m, P.shape[1]))
    P2[0::2], P2[1::2] = P, P                       # the oracle interleaves u, d per node
    g = 1.0 / np.random.default_rng(1).uniform(1e3, 1e6, (n, m))
    A = nodal.assemble(g, GW, np.zeros(n))[0] / GW
    A0 = nodal.assemble(np.zeros((n, m)), GW, np.zeros(n))[0] / GW
    Ac, Ac0 = P2.T @ A @ P2, P2.T @ A0 @ P2
    assert np.abs(Ac - Ac0).max() <= 1e-12 * np.abs(Ac0).max()
    assert np.abs(Ac0 - ct.coarse_matrix(n, m, 8)).max() <= 1e-12 * np.abs(Ac0).max()


def test_table_header_is_generated_and_solves_the_coarse_system():
    path = os.path.join(os.path.dirname(ct.__file__), "csrc", "coarse_tables.h")
    with open(path) as f:
        assert f.read() == ct.header_text()
    t = ct.table().astype(np.float64)
    Zr, Zc, lr, lc = t[:256].reshape(16, 16), t[256:512].reshape(16, 16), t[512:528], t[528:544]
    R = np.random.default_rng(2).standard_normal((16, 16))
    E = Zr @ ((Zr.T @ R @ Zc) / (lr[:, None] + lc[None, :])) @ Zc.T
    ref = np.linalg.solve(ct.coarse_matrix(), R.ravel()).reshape(16, 16)
    assert np.abs(E - ref).max() <= 1e-6 * np.abs(ref).max()


def lo_slot(k):
    return k // 8 if k % 8 < 4 else k // 8 + 1


def t_of(k):
    r = k % 8
    return (r + 4.5) / 8 if r < 4 else (r - 3.5) / 8


def clamp(I):
    return min(max(I, 0), 15)


def device_restrict(r):
    """coarse_restrict_slot over the 128 layout: thread (bitline j, segment s)."""
    R = np.zeros((16, 16))
    S = np.zeros((128, 4, 6))
    for j in range(128):
        for s in range(4):
            for k in range(32):
                i = 32 * s + k
                S[j, s, lo_slot(k)] += (1 - t_of(k)) * r[i, j]
                S[j, s, lo_slot(k) + 1] += t_of(k) * r[i, j]
    for w in range(16):                 # a warp's eight bitlines, one coarse column
        for s in range(4):
            for a in range(6):
                mid = side_lo = side_hi = 0.0
                for l in range(8):
                    t = (l + 4.5) / 8 if l < 4 else (l - 3.5) / 8
                    Sa = S[8 * w + l, s, a]
                    mid += (t if l < 4 else 1 - t) * Sa
                    if l < 4:
                        side_lo += (1 - t) * Sa
                    else:
                        side_hi += t * Sa
                I = clamp(4 * s - 1 + a)
                R[I, w] += mid
                R[I, clamp(w - 1)] += side_lo
                R[I, clamp(w + 1)] += side_hi
    return R


def device_prolong(E):
    pe = np.zeros((128, 128))
    for j in range(128):
        l, w = j & 7, j >> 3
        tj = (l + 4.5) / 8 if l < 4 else (l - 3.5) / 8
        J0, J1 = clamp(w - 1 if l < 4 else w), clamp(w if l < 4 else w + 1)
        for s in range(4):
            Ej = [(1 - tj) * E[clamp(4 * s - 1 + a), J0] + tj * E[clamp(4 * s - 1 + a), J1] for a in range(6)]
            for k in range(32):
                t = t_of(k)
                pe[32 * s + k, j] = (1 - t) * Ej[lo_slot(k)] + t * Ej[lo_slot(k) + 1]
    return pe


def test_restriction_and_prolongation_index_arithmetic():
    Pr, Pc = ct.hat(128, 8), ct.hat(128, 8)
    rng = np.random.default_rng(3)
    r = rng.standard_normal((128, 128))
    assert np.abs(device_restrict(r) - Pr.T @ r @ Pc).max() < 1e-12
    E = rng.standard_normal((16, 16))
    assert np.abs(device_prolong(E) - Pr @ E @ Pc.T).max() < 1e-12
    # a slot is complete after node 8 a + 3 (a < 4): no later node feeds it
    for a in range(4):
        later = [k for k in range(8 * a + 4, 32) if a in (lo_slot(k), lo_slot(k) + 1)]
        assert later == []


def test_coarse_solve_loop_order():
    """coarse_solve: entry p = (I, J) summed by two threads over alternate terms."""
    t = ct.table().astype(np.float64)
    Zr, Zc, lr, lc = t[:256], t[256:512], t[512:528], t[528:544]
    ZcT = Zc.reshape(16, 16).T.ravel()
    R = np.random.default_rng(4).standard_normal(256)

    def prod(fa, fb):
        out = np.zeros(256)
        for p in range(256):
            I, J = p >> 4, p & 15
            out[p] = sum(fa(I, J, 2 * q + h) * fb(I, J, 2 * q + h) for h in (0, 1) for q in range(8))
        return out

    T1 = prod(lambda I, J, K: Zr[K * 16 + I], lambda I, J, K: R[K * 16 + J])
    T2 = prod(lambda I, J, K: T1[I * 16 + K], lambda I, J, K: Zc[K * 16 + J])
    T2 = T2 / (lr[np.arange(256) >> 4] + lc[np.arange(256) & 15])
    T1 = prod(lambda I, J, K: Zr[I * 16 + K], lambda I, J, K: T2[K * 16 + J])
    E = prod(lambda I, J, K: T1[I * 16 + K], lambda I, J, K: ZcT[K * 16 + J])
    ref = np.linalg.solve(ct.coarse_matrix(), R)
    assert np.abs(E - ref).max() <= 1e-6 * np.abs(ref).max()


def two_level_solve(g, vin, tol, max_iters=200, c=8):
    """The kernel's two-level iteration in FP64 (deviation planes, gw units)."""
    n, m = g.shape
    gs = g / GW
    Pr, Pc, Zr, Zc, lr, lc = ct.factors(n, m, c)
    wl_diag = 1 + np.where(np.arange(m) < m - 1, 1.0, 0.0)[None, :] + gs
    wl_low = np.full((n, m), -1.0)
    wl_up = np.where(np.arange(m) < m - 1, -1.0, 0.0)[None, :].repeat(n, 0)
    bl_diag = (np.where(np.arange(n) > 0, 1.0, 0.0)[:, None] + 1 + gs).T
    bl_low = np.where(np.arange(n) > 0, -1.0, 0.0)[None, :].repeat(m, 0)
    bl_up = np.full((m, n), -1.0)
    U = np.zeros((n, m))
    D = np.zeros((n, m))
    stop = tsr.LineStop(1.0)
    pem = 0.0
    for it in range(1, max_iters + 1):
        Ua = U + vin[:, None]
        left = np.concatenate([np.zeros((n, 1)), U[:, :-1]], 1) - U
        right = np.concatenate([U[:, 1:] - U[:, :-1], np.zeros((n, 1))], 1)
        du = tsr.thomas(wl_low, wl_diag, wl_up, left + right + gs * (D - Ua))
        U = U + du
        Ua = U + vin[:, None]
        up = np.concatenate([np.zeros((1, m)), D[:-1, :] - D[1:, :]], 0)
        down = np.concatenate([D[1:, :], np.zeros((1, m))], 0) - D
        dd = tsr.thomas(bl_low, bl_diag, bl_up, (up + down + gs * (Ua - D)).T).T
        D = D + dd
        delta = max(np.abs(du).max(), np.abs(dd).max()) + pem
        vm = max(np.abs(U).max(), np.abs(D).max())
        if floor_update(stop, delta, vm, tol, 0.2):
            return U, D, it
        Rc = Pr.T @ (gs * dd) @ Pc                 # the wordline residual after the bitline pass
        E = Zr @ ((Zr.T @ Rc @ Zc) / (lr[:, None] + lc[None, :])) @ Zc.T
        Pe = Pr @ E @ Pc.T
        U, D = U + Pe, D + Pe
        pem = np.abs(Pe).max()
    raise AssertionError("no convergence")


def floor_update(stop, delta, vm, tol, rho_floor):
    """LineStop.update with the rate taken at least rho_floor (update<true>)."""
    import math
    stop.it += 1
    prev = stop.h0
    stop.h3, stop.h2, stop.h1, stop.h0 = stop.h2, stop.h1, stop.h0, delta
    if stop.it == 1:
        return delta <= 0
    floor_v = 4 * tsr.EPS32 * vm
    ratio = delta / prev if prev > 0 else 0.0
    rate3 = math.pow(delta / stop.h3, 1 / 3) if (stop.it >= 4 and stop.h3 > 0) else 0.0
    rho = max(ratio, rate3, stop.omega - 1, rho_floor)
    stop.rho = rho
    est = delta * rho / (1 - rho)
    return est <= max(tol, floor_v) or (delta <= floor_v and ratio >= 0.9)


def mlp_slice(rng, n, j):
    """A weight-slice map of the 1 kOhm - 1 MOhm MLP layers (2-bit cells, PN)."""
    w = rng.normal(0, 0.05, (n, n))
    wi = np.round(w / 2 ** np.ceil(np.log2(np.abs(w).max() / 255))).astype(np.int64)
    return ((np.where(wi > 0, wi, 0) >> (2 * j)) & 3) * ((1e-3 - 1e-6) / 3) + 1e-6


@pytest.mark.parametrize("n,kind", [(64, "1k"), (128, "mlp"), (128, "1k")])
@pytest.mark.parametrize("tol", [5e-7, 1e-8])
def test_two_level_keeps_the_stop_promise_in_fewer_iterations(n, kind, tol):
    rng = np.random.default_rng(n + len(kind))
    g = mlp_slice(rng, n, 0) if kind == "mlp" else 1.0 / (1e3 * np.exp(0.3 * rng.standard_normal((n, n))))
    vin = rng.integers(0, 2, n) * 0.2
    assert (g / GW).sum() >= 3.0  # the kernel takes the coarse correction on such tiles
    u_ref, d_ref = nodal.solve(g, GW, vin)
    U, D, it2 = two_level_solve(g, vin, tol)
    err = max(np.abs(U + vin[:, None] - u_ref).max(), np.abs(D - d_ref).max())
    bound = max(tol, 4 * tsr.EPS32 * max(np.abs(U).max(), np.abs(D).max()))
    assert err <= bound
    _, _, it1, _ = tsr.line_solve(g, vin, tol)
    assert it2 <= 0.5 * it1, (it2, it1)


def _thomas32(lower, diag, upper, rhs):
    """FP32 line solves (pivots from the exact recurrence, rounded, as the
    kernel's float-float pivots give them)."""
    f32 = np.float32
    L = diag.shape[-1]
    c = np.zeros(diag.shape, f32)
    y = np.zeros(rhs.shape, f32)
    p = diag[:, 0]
    c[:, 0] = f32(1.0 / p)
    y[:, 0] = rhs[:, 0].astype(f32) * c[:, 0]
    for k in range(1, L):
        p = diag[:, k] - lower[:, k] * upper[:, k - 1] / p
        c[:, k] = f32(1.0 / p)
        y[:, k] = (rhs[:, k].astype(f32) + y[:, k - 1]) * c[:, k]
    x = np.zeros(rhs.shape, f32)
    x[:, -1] = y[:, -1]
    for k in range(L - 2, -1, -1):
        x[:, k] = y[:, k] + c[:, k] * x[:, k + 1]
    return x


def fp32_limit_update(stop, delta, vm, tol, rho_floor):
    """LineStop.update<true> with fp32_limit: below the floor, run until the
    corrections make under 15% progress over three iterations."""
    import math
    stop.it += 1
    prev = stop.h0
    stop.h3, stop.h2, stop.h1, stop.h0 = stop.h2, stop.h1, stop.h0, delta
    if stop.it == 1:
        return delta <= 0
    floor_v = 4 * tsr.EPS32 * vm
    ratio = delta / prev if prev > 0 else 0.0
    rate3 = math.pow(delta / stop.h3, 1 / 3) if (stop.it >= 4 and stop.h3 > 0) else 0.0
    rho = max(ratio, rate3, stop.omega - 1, rho_floor)
    est = delta * rho / (1 - rho)
    return est <= tol or (delta <= floor_v and stop.it >= 4 and delta >= 0.85 * stop.h3)


def unit_response_fp32(g, r, vlevel=0.2, max_iters=200):
    """A unit response (row r driven) by the two-level iteration in FP32 with
    exact residuals rounded to FP32 (as the precise iterations give them) and
    the FP32-limit stop; returns (bitline currents from the ground link, its)."""
    f32 = np.float32
    n, m = g.shape
    gs = g / GW
    vin = np.zeros(n)
    vin[r] = vlevel
    Pr, Pc, Zr, Zc, lr, lc = ct.factors(n, m, 8)
    wl = (np.full((n, m), -1.0), 1 + np.where(np.arange(m) < m - 1, 1.0, 0.0)[None, :] + gs,
          np.where(np.arange(m) < m - 1, -1.0, 0.0)[None, :].repeat(n, 0))
    bl = (np.where(np.arange(n) > 0, -1.0, 0.0)[None, :].repeat(m, 0),
          (np.where(np.arange(n) > 0, 1.0, 0.0)[:, None] + 1 + gs).T, np.full((m, n), -1.0))
    U = np.zeros((n, m), f32)
    D = np.zeros((n, m), f32)
    stop = tsr.LineStop(1.0)
    pem = 0.0
    for it in range(1, max_iters + 1):
        U64, D64 = U.astype(np.float64), D.astype(np.float64)
        left = np.concatenate([np.zeros((n, 1)), U64[:, :-1]], 1) - U64
        right = np.concatenate([U64[:, 1:] - U64[:, :-1], np.zeros((n, 1))], 1)
        du = _thomas32(*wl, (left + right + gs * (D64 - U64 - vin[:, None])).astype(f32))
        U = (U + du).astype(f32)
        U64 = U.astype(np.float64)
        up = np.concatenate([np.zeros((1, m)), D64[:-1, :] - D64[1:, :]], 0)
        down = np.concatenate([D64[1:, :], np.zeros((1, m))], 0) - D64
        dd = _thomas32(*bl, (up + down + gs * (U64 + vin[:, None] - D64)).T.astype(f32)).T
        D = (D + dd).astype(f32)
        delta = float(max(np.abs(du).max(), np.abs(dd).max())) + pem
        vm = float(max(np.abs(U).max(), np.abs(D).max()))
        if fp32_limit_update(stop, delta, vm, 2e-11, 0.2):
            return GW * D[-1].astype(np.float64), it
        Rc = Pr.T @ (gs * dd) @ Pc
        Pe = (Pr @ (Zr @ ((Zr.T @ Rc @ Zc) / (lr[:, None] + lc[None, :])) @ Zc.T) @ Pc.T).astype(f32)
        U, D = U + Pe, D + Pe
        pem = float(np.abs(Pe).max())
    raise AssertionError("no stall in %d iterations" % max_iters)


@pytest.mark.parametrize("r", [0, 127])
def test_unit_responses_to_the_fp32_limit(r):
    """The superposition's unit responses: the plain stop test ends where the
    largest node reaches its FP32 floor, which leaves a unit response's bitline
    currents ~1e-5..3e-4 of themselves off (the bitline ends are small nodes);
    run to the FP32 limit they are within ~1e-7."""
    g = mlp_slice(np.random.default_rng(5), 128, 0)
    vin = np.zeros(128)
    vin[r] = 0.2
    _, d_ref = nodal.solve(g, GW, vin)
    I_ref = GW * d_ref[-1]
    I, it = unit_response_fp32(g, r)
    assert np.abs(I - I_ref).max() <= 5e-7 * np.abs(I_ref).max()
    assert it <= 30
