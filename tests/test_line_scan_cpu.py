"""The parallel Thomas solve of one line, as the kernels split it, restated on
the CPU: each lane folds its segment of SEG nodes into affine maps (forward
chain y -> C y + Y, backward chain x -> C x + X; csrc/cluster_impl.cuh
seg_fold_fwd, seg_apply_fwd_fold_bwd, seg_apply_bwd), the NSEG lanes of a line
join them by a doubling scan over shuffles (scan_up, scan_down), and on a
cluster the CTAs' totals are composed through distributed shared memory in
batches of K with identity padding (compose_above, compose_below).  Against a
dense solve of the same system, in FP64 (the decomposition is exact algebra)
and in FP32 (no worse than the sequential FP32 recurrence).  The restatement
mirrors the device code; a change there must be mirrored here.
"""
import numpy as np
import pytest


def seg_fold_fwd(x, c):
    Y = x.dtype.type(0)
    for k in range(len(x)):
        x[k] = x[k] * c[k]
        Y = c[k] * Y + x[k]
    return Y


def seg_apply_fwd_fold_bwd(x, c, y):
    for k in range(len(x)):
        y = c[k] * y + x[k]
        x[k] = y
    X = x.dtype.type(0)
    for k in range(len(x) - 1, -1, -1):
        X = c[k] * X + x[k]
    return X


def seg_apply_bwd(x, c, X):
    for k in range(len(x) - 1, -1, -1):
        X = c[k] * X + x[k]
        x[k] = X


def scan(C, Y, up):
    """scan_up / scan_down over the NSEG lanes of one line: inclusive and
    exclusive compositions (lanes read their partner's value before any lane
    writes, as a shuffle does)."""
    nseg = len(C)
    Ci, Yi = C.copy(), Y.copy()
    off = 1
    while off < nseg:
        Cp, Yp = Ci.copy(), Yi.copy()
        for s in range(nseg):
            src = s - off if up else s + off
            if 0 <= src < nseg:
                Yi[s] = Ci[s] * Yp[src] + Yi[s]
                Ci[s] = Ci[s] * Cp[src]
        off <<= 1
    one, zero = C.dtype.type(1), C.dtype.type(0)
    Cx = np.array([(Ci[s - 1] if up else Ci[s + 1]) if (s > 0 if up else s < nseg - 1) else one
                   for s in range(nseg)], C.dtype)
    Yx = np.array([(Yi[s - 1] if up else Yi[s + 1]) if (s > 0 if up else s < nseg - 1) else zero
                   for s in range(nseg)], C.dtype)
    return Ci, Yi, Cx, Yx


def compose(maps, rank, C, above):
    """compose_above / compose_below: the CTAs' (c, y) totals applied onto 0 in
    batches of K, entries past the end replaced by the identity."""
    K = 8 if C > 8 else 4
    one, zero = maps[0][0].dtype.type(1), maps[0][0].dtype.type(0)
    v = zero
    if above:
        for r0 in range(0, rank, K):
            for t in range(K):
                r = r0 + t
                c, y = maps[r] if (r < C and r < rank) else (one, zero)
                v = c * v + y
    else:
        for r0 in range(C - 1, rank, -K):
            for t in range(K):
                r = r0 - t
                c, y = maps[r] if (r >= 0 and r > rank) else (one, zero)
                v = c * v + y
    return v


def solve_line(r, cmul, C, NSEG, SEG, dt):
    """Correction of one line of C * NSEG * SEG nodes: CTAs of NSEG lanes of SEG nodes."""
    x = [[r[(q * NSEG + s) * SEG:(q * NSEG + s + 1) * SEG].astype(dt) for s in range(NSEG)] for q in range(C)]
    c = [[cmul[(q * NSEG + s) * SEG:(q * NSEG + s + 1) * SEG].astype(dt) for s in range(NSEG)] for q in range(C)]
    segprod = [np.array([np.prod(c[q][s], dtype=dt) for s in range(NSEG)], dt) for q in range(C)]
    # forward: fold, scan inside each CTA, publish the CTA's total, compose the CTAs above
    Y = [np.array([seg_fold_fwd(x[q][s], c[q][s]) for s in range(NSEG)], dt) for q in range(C)]
    fw = [scan(segprod[q], Y[q], True) for q in range(C)]
    aggF = [(fw[q][0][NSEG - 1], fw[q][1][NSEG - 1]) for q in range(C)]
    X = []
    for q in range(C):
        yent = compose(aggF, q, C, True)
        Cx, Yx = fw[q][2], fw[q][3]
        X.append(np.array([seg_apply_fwd_fold_bwd(x[q][s], c[q][s], Cx[s] * yent + Yx[s]) for s in range(NSEG)], dt))
    # backward: scan inside each CTA, publish, compose the CTAs below, apply
    bw = [scan(segprod[q], X[q], False) for q in range(C)]
    aggB = [(bw[q][0][0], bw[q][1][0]) for q in range(C)]
    for q in range(C):
        xent = compose(aggB, q, C, False)
        Cbx, Xbx = bw[q][2], bw[q][3]
        for s in range(NSEG):
            seg_apply_bwd(x[q][s], c[q][s], Cbx[s] * xent + Xbx[s])
    return np.concatenate([np.concatenate(x[q]) for q in range(C)])


def system(rng, L, word):
    """T' = tridiag(-1, D, -1) in units of gw, D = links + g/gw, and the
    multipliers c = 1/P of its pivots."""
    gs = 2.93 / rng.choice([1e3, 2e4, 3e5, 1e6], L)
    links = np.where(np.arange(L) < L - 1, 2.0, 1.0) if word else np.where(np.arange(L) > 0, 2.0, 1.0)
    D = links + gs
    P = np.empty(L)
    P[0] = D[0]
    for k in range(1, L):
        P[k] = D[k] - 1 / P[k - 1]
    T = np.diag(D) - np.diag(np.ones(L - 1), 1) - np.diag(np.ones(L - 1), -1)
    return T, 1 / P


# (C, NSEG, SEG): the 128 kernel's lines (4 lanes of 32), the 256 cluster's
# bitlines (4 CTAs x 2 lanes) and wordlines (8 lanes), the 512 cluster's
# bitlines (16 CTAs x 1 lane) and wordlines (16 lanes)
LAYOUTS = [(1, 4, 32), (4, 2, 32), (1, 8, 32), (16, 1, 32), (1, 16, 32), (3, 4, 8)]


@pytest.mark.parametrize("C,NSEG,SEG", LAYOUTS)
def test_segmented_thomas_equals_dense_solve(C, NSEG, SEG):
    rng = np.random.default_rng(C * 100 + NSEG * 10 + SEG)
    L = C * NSEG * SEG
    for word in (True, False):
        T, cmul = system(rng, L, word)
        r = rng.standard_normal(L) * 1e-3
        exact = np.linalg.solve(T, r)
        got = solve_line(r, cmul, C, NSEG, SEG, np.float64)
        assert np.abs(got - exact).max() <= 1e-10 * np.abs(exact).max()
        # FP32: the split costs no accuracy against the sequential FP32 recurrence
        got32 = solve_line(r, cmul, C, NSEG, SEG, np.float32).astype(np.float64)
        seq32 = solve_line(r, cmul, 1, 1, L, np.float32).astype(np.float64)
        e_split = np.abs(got32 - exact).max()
        e_seq = np.abs(seq32 - exact).max()
        assert e_split <= 4 * e_seq + 1e-7 * np.abs(exact).max(), (e_split, e_seq)


@pytest.mark.parametrize("C,NSEG,SEG", [(1, 4, 16), (1, 8, 32), (1, 16, 32)])
def test_first_wordline_pass_from_unit_response(C, NSEG, SEG):
    """The first wordline pass from the ideal state (csrc/line_impl.cuh
    line_word_zero_unit; cluster_impl.cuh cl_word_pass modes 5 and 6): with
    both planes zero its residual is -vin g / gw on every node, so its
    correction equals -vin times the line's unit response T'^-1 (g / gw),
    solved once per tile.  In FP32, through the kernels' segmented Thomas
    split, the two agree to a few ulps of the correction."""
    rng = np.random.default_rng(C * 7 + NSEG * 3 + SEG)
    L = C * NSEG * SEG
    T, cmul = system(rng, L, True)
    gs = (np.diag(T) - np.where(np.arange(L) < L - 1, 2.0, 1.0)).astype(np.float32)
    for vin in (0.2, 0.1375, 1.0):
        direct = solve_line((np.float32(-vin) * gs).astype(np.float32), cmul, C, NSEG, SEG, np.float32)
        unit = solve_line(gs.copy(), cmul, C, NSEG, SEG, np.float32)
        via_unit = np.float32(-vin) * unit
        exact = np.linalg.solve(T, -vin * gs.astype(np.float64))
        scale = np.abs(exact).max()
        assert np.abs(via_unit.astype(np.float64) - direct.astype(np.float64)).max() <= 1e-6 * scale
        assert np.abs(via_unit.astype(np.float64) - exact).max() <= 1e-5 * scale
