"""The closed-form pieces the kernels use, checked in numpy: the series for
sinh(t)/t below t = 1 and the one-division form of the sinh cell's chord
conductance (csrc/common.cuh); the error-free transforms of the precise
residual and of the float-float pivots (csrc/line_common.cuh), restated in
float32 arithmetic and checked against exact rationals.  The restatements
mirror the device code; a change there must be mirrored here."""
import math

import numpy as np

COEF = [1 / math.factorial(2 * k + 1) for k in range(7)]   # 1/1!, 1/3!, ..., 1/13!


def sinhc_series(t, dtype):
    u = (t * t).astype(dtype)
    p = dtype(COEF[6])
    for c in reversed(COEF[:6]):
        p = (p * u + dtype(c)).astype(dtype)
    return p


def test_series_truncation_and_fp32_rounding():
    t = np.linspace(0.0, 1.0, 20001)
    exact = np.where(t > 0, np.sinh(t) / np.where(t > 0, t, 1), 1.0)
    assert np.abs(sinhc_series(t, np.float64) / exact - 1).max() < 1e-12     # truncation
    t32 = t.astype(np.float32)
    got = sinhc_series(t32, np.float32).astype(np.float64)
    ref = np.where(t32 > 0, np.sinh(t32.astype(np.float64)) / np.where(t32 > 0, t32, 1), 1.0)
    assert np.abs(got / ref - 1).max() < 4 * 2.0 ** -24                      # a few FP32 ulps


def test_chord_conductance_one_division_form():
    rng = np.random.default_rng(0)
    z = rng.random(1000)
    x = rng.random(1000) * 0.5
    a_on, b_on, a_off, b_off = 2.0, 1e-4, 2.0, 1e-6
    r0_on, r0_off = 1 / (a_on * b_on), 1 / (a_off * b_off)
    s_on = np.sinh(a_on * x) / (a_on * x)
    s_off = np.sinh(a_off * x) / (a_off * x)
    three = 1 / ((1 - z) * r0_on / s_on + z * r0_off / s_off)
    one = s_on * s_off / ((1 - z) * r0_on * s_off + z * r0_off * s_on)
    np.testing.assert_allclose(one, three, rtol=1e-14)
    # and the cell law itself: I = (1-z)-weighted series of the on and off sinh branches
    V = x
    R = (1 - z) * V / (b_on * np.sinh(a_on * V)) + z * V / (b_off * np.sinh(a_off * V))
    np.testing.assert_allclose(one, 1 / R, rtol=1e-13)


# ---- error-free transforms of the precise residual and the pivots
# (csrc/line_common.cuh two_sum, lap_exact, ff_pivot_step), restated in float32
# numpy arithmetic (IEEE round-to-nearest, as the kernels' __fadd_rn etc.) and
# checked against exact rational arithmetic.
from fractions import Fraction  # noqa: E402

F = np.float32


def rn32(q):
    """Round an exact rational to the nearest float32, ties to even."""
    if q == 0:
        return F(0)
    f = F(float(q))
    best = None
    for c in (np.nextafter(f, F(-np.inf)), f, np.nextafter(f, F(np.inf))):
        d = abs(Fraction(float(c)) - q)
        if best is None or d < best[0] or (d == best[0] and int(c.view(np.uint32)) % 2 == 0):
            best = (d, c)
    return best[1]


def fma32(a, b, c):
    return rn32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def two_sum(a, b):
    s = F(a + b)
    bb = F(s - a)
    return s, F(F(a - F(s - bb)) + F(b - bb))


def lap_exact(prev, cur, nxt, has_l, has_r):
    sh, sl = two_sum(prev if has_l else F(0), nxt if has_r else F(0))
    k = F(2) * cur if (has_l and has_r) else (cur if (has_l or has_r) else F(0))
    th, tl = two_sum(sh, -k)
    return th, F(tl + sl)


def ff_pivot_step(base, gs, first, rh, rl):
    dh, dl = two_sum(base, gs)
    ph, pl = dh, dl
    if not first:
        sh, sl = two_sum(dh, -rh)
        sl = F(sl + F(dl - rl))
        ph = F(sh + sl)
        pl = F(sl - F(ph - sh))
    r = F(F(1) / ph)
    e = fma32(-ph, r, F(1))
    e = fma32(-pl, r, e)
    return F(r + F(e * r)), r, F(e * r)


def ulp32(x):
    return float(np.spacing(np.abs(F(x))))


def test_two_sum_is_error_free():
    rng = np.random.default_rng(1)
    a = (rng.standard_normal(4000) * 10.0 ** rng.integers(-8, 3, 4000)).astype(F)
    b = (rng.standard_normal(4000) * 10.0 ** rng.integers(-8, 3, 4000)).astype(F)
    for x, y in zip(a, b):
        s, e = two_sum(x, y)
        assert Fraction(float(s)) + Fraction(float(e)) == Fraction(float(x)) + Fraction(float(y))


def test_line_part_exact_up_to_one_rounding_of_its_low_part():
    """(prev - cur) + (nxt - cur) as hi + lo: the error is the rounding of lo
    alone, for neighbouring node values (the cancellation the residual sees)."""
    rng = np.random.default_rng(2)
    for _ in range(3000):
        cur = F(rng.uniform(-0.2, 0.2))
        prev = F(cur + F(rng.standard_normal() * 10.0 ** rng.integers(-9, -2)))
        nxt = F(cur + F(rng.standard_normal() * 10.0 ** rng.integers(-9, -2)))
        has_l, has_r = bool(rng.integers(0, 4)), bool(rng.integers(0, 4))
        hi, lo = lap_exact(prev, cur, nxt, has_l, has_r)
        exact = ((Fraction(float(prev)) - Fraction(float(cur))) if has_l else 0) + \
                ((Fraction(float(nxt)) - Fraction(float(cur))) if has_r else 0)
        err = abs(Fraction(float(hi)) + Fraction(float(lo)) - exact)
        assert err <= Fraction(ulp32(lo)) / 2


def test_float_float_pivots_match_exact_recurrence():
    """Chain multipliers 1/P_q of P_q = D_q - 1/P_(q-1), D_q = (1 or 2) + g/gw,
    along 128-node wordlines and bitlines with 1 kohm - 1 Mohm cells and 2.93
    ohm wires: correctly rounded against the exact rational recurrence (a
    plain FP32 recurrence is hundreds of ulps off)."""
    rng = np.random.default_rng(3)
    L, gw = 128, 1 / 2.93
    plain_worst = 0
    for word in (True, False):
        for _ in range(3):
            gs = (1.0 / rng.choice([1e3, 2e4, 3e5, 1e6], L) / gw).astype(F)
            rh = rl = F(0)
            P = pf = None
            for q in range(L):
                base = F((2 if q + 1 < L else 1) if word else (2 if q > 0 else 1))
                cf, rh, rl = ff_pivot_step(base, gs[q], q == 0, rh, rl)
                D = Fraction(int(base)) + Fraction(float(gs[q]))
                P = D if q == 0 else D - 1 / P
                assert abs(Fraction(float(cf)) - 1 / P) <= Fraction(ulp32(cf)) / 2, (word, q)
                pf = F(base + gs[q]) if q == 0 else F(F(base + gs[q]) - F(F(1) / pf))
                plain_worst = max(plain_worst, abs(Fraction(float(F(F(1) / pf))) - 1 / P) / Fraction(ulp32(cf)))
    assert plain_worst > 50


# cluster kernels (csrc/cluster_impl.cuh ff_norm, ff_mul_sub, ff_dot2, cl_pivots):
# a bitline column spans C bands of RPC rows, one per CTA; each band's map
# P -> D - 1/P is a product of [[D, -1], [1, 0]] in float-float, rescaled by a
# power of two; the state entering a band composes the maps above it.
def ff_norm(s, e):
    h = F(s + e)
    return h, F(e - F(h - s))


def ff_mul_sub(x, y, z):
    ph = F(x[0] * y[0])
    pl = F(fma32(x[0], y[0], -ph) + F(F(x[0] * y[1]) + F(x[1] * y[0])))
    sh, sl = two_sum(ph, -z[0])
    return ff_norm(sh, F(sl + F(pl - z[1])))


def ff_dot2(x, y, z, w):
    ph, qh = F(x[0] * y[0]), F(z[0] * w[0])
    pl = F(fma32(x[0], y[0], -ph) + F(F(x[0] * y[1]) + F(x[1] * y[0])))
    ql = F(fma32(z[0], w[0], -qh) + F(F(z[0] * w[1]) + F(z[1] * w[0])))
    sh, sl = two_sum(ph, qh)
    return ff_norm(sh, F(sl + F(pl + ql)))


def inv_binade(v):
    _, e = np.frexp(np.float64(v))
    return F(2.0 ** (1 - e))


def band_pivots(gs, C, RPC):
    scale = lambda x, k: (F(x[0] * k), F(x[1] * k))
    mobs = []
    for r in range(C):
        a, b, c, d = (F(1), F(0)), (F(0), F(0)), (F(0), F(0)), (F(1), F(0))
        for lr in range(RPC):
            q = r * RPC + lr
            D = two_sum(F(2 if q > 0 else 1), gs[q])
            a, b, c, d = ff_mul_sub(D, a, c), ff_mul_sub(D, b, d), a, b
        k = inv_binade(max(abs(a[0]), abs(b[0]), abs(c[0]), abs(d[0])))
        mobs.append([scale(v, k) for v in (a, b, c, d)])
    out = []
    for rank in range(C):
        num, den = (F(1), F(0)), (F(0), F(0))
        for a, b, c, d in mobs[:rank]:
            nn, dd = ff_dot2(a, num, b, den), ff_dot2(c, num, d, den)
            k = inv_binade(max(abs(nn[0]), abs(dd[0])))
            num, den = scale(nn, k), scale(dd, k)
        rh = rl = F(0)
        if rank > 0 and num[0] != 0:
            rh = F(den[0] / num[0])
            rl = F(F(fma32(-num[0], rh, den[0]) + F(den[1] - F(rh * num[1]))) / num[0])
        for lr in range(RPC):
            q = rank * RPC + lr
            cf, rh, rl = ff_pivot_step(F(2 if q > 0 else 1), gs[q], q == 0, rh, rl)
            out.append(cf)
    return out


def test_cluster_band_pivots_match_exact_recurrence():
    """Bitline multipliers of the 256-row (4 bands of 64) and 512-row (16 bands
    of 32) cluster layouts, through the band products: correctly rounded against
    the exact recurrence, for mixed and for all-1-kohm columns."""
    rng = np.random.default_rng(4)
    gw = 1 / 2.93
    for L, C, RPC in ((256, 4, 64), (512, 16, 32)):
        for cells in ([1e3, 2e4, 3e5, 1e6], [1e3], [1e6]):
            gs = (1.0 / rng.choice(cells, L) / gw).astype(F)
            cfs = band_pivots(gs, C, RPC)
            P = None
            for q in range(L):
                D = Fraction(2 if q > 0 else 1) + Fraction(float(gs[q]))
                P = D if q == 0 else D - 1 / P
                assert abs(Fraction(float(cfs[q])) - 1 / P) <= Fraction(ulp32(cfs[q])) / 2, (L, cells, q)


def line_residual(RES, word, prev, cur, nxt, gs, o, vin):
    """line_residual_s (csrc/line_common.cuh) for an interior node, RES 0 (FP32),
    2 (float-float) and 3 (exact line part, FP32 cell term), in gw units."""
    if RES == 2:
        sh, sl = two_sum(o, -vin if word else vin)
        th, tl = two_sum(sh, -cur)
        lh, lap_lo = lap_exact(prev, cur, nxt, True, True)
        ph = F(gs * th)
        pl = fma32(gs, th, -ph)
        rh, rl = two_sum(lh, ph)
        return F(rh + F(F(rl + F(lap_lo + pl)) + F(gs * F(tl + sl))))
    src = F(F(o - vin) - cur) if word else F(F(o + vin) - cur)
    if RES == 3:
        lh, lap_lo = lap_exact(prev, cur, nxt, True, True)
        return F(lh + fma32(gs, src, lap_lo))
    return fma32(gs, src, F(F(prev - cur) + F(nxt - cur)))


def test_residual_forms_near_convergence():
    """Near convergence the residual is ~1e-10 V while its terms are ~1e-4: the
    float-float form (RES 2) stays within a few units of 2^-46 of the terms,
    orders of magnitude under the FP32 form (RES 0); the semi-precise form
    (RES 3) is held to one FP32 rounding of the cell term, which the kernels
    allow only where that rounding stays far under the tolerance."""
    rng = np.random.default_rng(5)
    q = lambda v: Fraction(float(v))
    err0, err2 = [], []
    for _ in range(1500):
        word = bool(rng.integers(0, 2))
        vin = F(rng.choice([0.0, 0.2, 1.0]))
        cur = F(-rng.uniform(0, 0.05)) if word else F(rng.uniform(0, 0.05))
        o = F(rng.uniform(0, 0.05)) if word else F(-rng.uniform(0, 0.05))
        gs = F(2.93 / rng.choice([1e3, 2e4, 3e5, 1e6]))
        nxt = F(cur + F(rng.standard_normal() * 1e-4))
        srcv = (float(o) - float(vin) - float(cur)) if word else (float(o) + float(vin) - float(cur))
        prev = F(2 * float(cur) - float(nxt) - float(gs) * srcv + rng.standard_normal() * 1e-10)
        src = (q(o) - q(vin) - q(cur)) if word else (q(o) + q(vin) - q(cur))
        exact = (q(prev) - q(cur)) + (q(nxt) - q(cur)) + q(gs) * src
        mag = max(abs(float(prev)), abs(float(cur)), abs(float(nxt)), abs(float(o)) + abs(float(vin)))
        r2 = line_residual(2, word, prev, cur, nxt, gs, o, vin)
        e2 = abs(q(r2) - exact)
        assert e2 <= Fraction(ulp32(r2)) / 2 + Fraction(mag) * Fraction(2) ** -46
        r3 = line_residual(3, word, prev, cur, nxt, gs, o, vin)
        assert abs(q(r3) - exact) <= Fraction(ulp32(r3)) + 4 * q(gs) * Fraction(mag + 1.0) * Fraction(2) ** -23
        r0 = line_residual(0, word, prev, cur, nxt, gs, o, vin)
        err0.append(float(abs(q(r0) - exact)))
        err2.append(float(e2))
    assert np.median(err0) > 1000 * np.median(err2)


def widen_f64(bits):
    """csrc/line_common.cuh widen_f64 on uint32 float bit patterns -> float64."""
    b = bits.astype(np.uint64)
    mag = b & np.uint64(0x7FFFFFFF)
    sign = b & np.uint64(0x80000000)
    normal = sign | ((mag >> np.uint64(3)) + np.uint64(896 << 20))
    special = sign | np.uint64(0x7FF00000) | ((mag & np.uint64(0x007FFFFF)) >> np.uint64(3)) | \
        np.where(mag > np.uint64(0x7F800000), np.uint64(0x00080000), np.uint64(0))
    hi = np.where(mag == 0, b, np.where(mag >= np.uint64(0x7F800000), special, normal))
    lo = (b & np.uint64(7)) << np.uint64(29)
    return ((hi << np.uint64(32)) | lo).view(np.float64)


def test_widen_to_fp64_on_the_integer_pipe():
    """The FP64 residual's float -> double conversion by bit manipulation: exact
    for normal numbers, signed zeros and infinities, NaN stays NaN; over every
    exponent and random mantissas and signs."""
    rng = np.random.default_rng(6)
    exps = np.repeat(np.arange(1, 255, dtype=np.uint32), 2000)
    bits = (rng.integers(0, 2, exps.size, dtype=np.uint32) << np.uint32(31)) | (exps << np.uint32(23)) | \
        rng.integers(0, 1 << 23, exps.size, dtype=np.uint32)
    bits = np.concatenate([bits, np.array([0, 0x80000000, 0x7F800000, 0xFF800000, 0x00800000, 0x7F7FFFFF],
                                          np.uint32)])
    got = widen_f64(bits)
    ref = bits.view(np.float32).astype(np.float64)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    nan = widen_f64(np.array([0x7FC00000, 0xFFC00001, 0x7F800001], np.uint32))
    assert np.isnan(nan).all()
