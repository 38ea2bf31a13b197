"""numpy restatement of the reference's sweep-order Gauss-Seidel/SOR solve.

Test infrastructure only: see ``oracle/__init__.py``.

This is the order PimTorch runs through its CUDA extension and its
``batchBybatch`` fallback, which are identical in order:

* one sweep = every wordline row relaxed left -> right using the NEW left
  neighbour, the OLD right neighbour and the OLD bitline node
  (split_arr_matmul.cu:75-119; ir_drop_solve.py:256-265), then every bitline
  column relaxed bottom -> top using the OLD upper neighbour, the NEW lower
  neighbour and the NEW wordline node (split_arr_matmul.cu:27-73;
  ir_drop_solve.py:267-276);
* the first wordline node couples to the input through g_load_left = g_wire
  and the bottom bitline node to 0 V through g_load_down = g_wire
  (split_arr_matmul.cu:275,290);
* initial state: wordline nodes = input voltage, bitline nodes = 0
  (split_arr_matmul.cu:231-235);
* optional break when no node moved by more than the threshold in a sweep
  (split_arr_matmul.cu:297-306);
* output: bitline currents from the last iterate, or the cell voltage
  u - d when ``ret_V`` (split_arr_matmul.cu:310-332).
"""
import numpy as np


def ir_drop_gs(input_v, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire, beta,
               enable_break=False, break_threshold=0.0, ret_V=False, return_iters=False):
    """Same arguments and layouts as the reference's ``ir_drop_gs`` (linear cells).

    input_v [B, numX, rows]; G [numX, rows, numY*cols]; returns
    [B, numX, numY*cols] currents, or [B, numX, numY, rows, cols] if ret_V.
    Arithmetic is done in the dtype of ``G`` (float32 or float64).
    """
    dt = np.asarray(G).dtype
    one = dt.type(1)
    w = dt.type(beta)
    gw = dt.type(g_wire)
    B, X, Y, n, m = batch_size, numX, numY, row_size, col_size
    inp = np.asarray(input_v, dt).reshape(B, X, n)
    g = np.asarray(G, dt).reshape(X, n, Y, m).transpose(0, 2, 1, 3)[None]  # [1, X, Y, n, m]
    up = np.broadcast_to(inp[:, :, None, :, None], (B, X, Y, n, m)).copy()
    dn = np.zeros((B, X, Y, n, m), dt)
    iters = 0
    for _ in range(iter_times):
        up_old = up.copy()
        dn_old = dn.copy()
        # wordlines, left -> right
        left = inp[:, :, None, :]
        for j in range(m):
            gj = g[..., j]
            if j == m - 1:
                sumg = gw + gj
                num = gw * left + gj * dn_old[..., j]
            else:
                sumg = gw + gw + gj
                num = gw * left + gw * up_old[..., j + 1] + gj * dn_old[..., j]
            up[..., j] = w * num / sumg + (one - w) * up_old[..., j]
            left = up[..., j]
        # bitlines, bottom -> top
        below = np.zeros((B, X, Y, m), dt)
        for i in range(n - 1, -1, -1):
            gi = g[..., i, :]
            if i == 0:
                sumg = gw + gi
                num = gw * below + gi * up[..., i, :]
            else:
                sumg = gw + gw + gi
                num = gw * dn_old[..., i - 1, :] + gw * below + gi * up[..., i, :]
            dn[..., i, :] = w * num / sumg + (one - w) * dn_old[..., i, :]
            below = dn[..., i, :]
        iters += 1
        if enable_break:
            moved_u = int((np.abs(up - up_old) > break_threshold).sum())
            moved_d = int((np.abs(dn - dn_old) > break_threshold).sum())
            if moved_u == 0 and moved_d == 0:
                break
    if ret_V:
        res = up - dn
    else:
        res = ((up - dn) * g).sum(axis=3).reshape(B, X, Y * m)
    if return_iters:
        return res, iters
    return res


def ir_drop_gs_nonlinear(input_v, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire, beta, params):
    """The reference's nonlinear sweeps (split_arr_matmul.cu:241-262), FP64.

    Before every sweep the cell conductances are recomputed from the cell
    voltages held in the buffers the sweep is about to overwrite -- after the
    ping-pong swap those hold the state from two sweeps back -- with |V| < 1e-5
    clamped to +-1e-5 (deal_v) and z from the linear conductances.  Returns the
    currents computed with the last conductances, as get_current does.
    """
    import numpy as _np
    R_on, R_off, a_on, b_on, a_off, b_off = [float(p) for p in params]
    B, X, Y, n, m = batch_size, numX, numY, row_size, col_size
    gw = float(g_wire)
    w = float(beta)
    inp = _np.asarray(input_v, _np.float64).reshape(B, X, n)
    glin = _np.asarray(G, _np.float64).reshape(X, n, Y, m).transpose(0, 2, 1, 3)[None]
    z = (1.0 / glin - R_on) / (R_off - R_on)
    z = _np.where(z < 0, 0.0, z)
    cur_u = _np.broadcast_to(inp[:, :, None, :, None], (B, X, Y, n, m)).copy()   # "voltage_up"
    cur_d = _np.zeros((B, X, Y, n, m))
    prev_u, prev_d = cur_u.copy(), cur_d.copy()                                  # "..._prev" (newest)
    g = _np.broadcast_to(glin, (B, X, Y, n, m))
    for _ in range(iter_times):
        V = cur_u - cur_d
        small = (V < 1e-5) & (V > -1e-5)
        V = _np.where(small, _np.where(V > 0, 1e-5, -1e-5), V)
        Va = _np.abs(V)
        g = 1.0 / ((1 - z) * Va / (b_on * _np.sinh(a_on * Va)) + z * Va / (b_off * _np.sinh(a_off * Va)))
        # one sweep in the reference order, writing cur_* from prev_*
        left = inp[:, :, None, :]
        for j in range(m):
            gj = g[..., j]
            if j == m - 1:
                num = gw * left + gj * prev_d[..., j]
                sumg = gw + gj
            else:
                num = gw * left + gw * prev_u[..., j + 1] + gj * prev_d[..., j]
                sumg = 2 * gw + gj
            cur_u[..., j] = w * num / sumg + (1 - w) * prev_u[..., j]
            left = cur_u[..., j]
        below = _np.zeros((B, X, Y, m))
        for i in range(n - 1, -1, -1):
            gi = g[..., i, :]
            if i == 0:
                num = gw * below + gi * cur_u[..., i, :]
                sumg = gw + gi
            else:
                num = gw * prev_d[..., i - 1, :] + gw * below + gi * cur_u[..., i, :]
                sumg = 2 * gw + gi
            cur_d[..., i, :] = w * num / sumg + (1 - w) * prev_d[..., i, :]
            below = cur_d[..., i, :]
        cur_u, prev_u = prev_u, cur_u
        cur_d, prev_d = prev_d, cur_d
    return ((prev_u - prev_d) * g).sum(axis=3).reshape(B, X, Y * m)


def ir_family(input_v, G, batch_size, row_size, col_size, numX, numY, iter_times, wire, mode, ou=None, loads=None,
              beta=1.0, enable_break=False, break_threshold=0.0, ret_V=False, nonlinear=None):
    """The reference extension's IR2S and operation-unit (OU) solvers
    (split_arr_matmul.cu:336-1327), in the dtype of ``G``.

    mode "gs": the ir_drop_gs sweep (wire = g_wire) -- ir_gs_ou_local with
    ``loads`` = (g_load_left, g_load_down), ir_gs_ou with ``ou`` = (ou_rows,
    ou_cols), each OU's source load g_wire / (first column + 1) and ground load
    g_wire / (rows - last row) (:1086-1150).
    mode "ir2s": the IR-drop-to-source iteration (wire = r_wire; :336-410,
    816-930): Jacobi from the previous planes, per-segment line current sums
    that persist between iterations, source and ground loads r_wire (ir2s),
    ``loads`` = (r_load_left, r_load_down) (ir2s_ou_local) or, per OU,
    r_wire * (first column + 1) and r_wire * (rows - last row) (ir2s_ou).
    Returns currents [B, numX * rows / ou_rows, numY * cols] (one row group
    without OUs), or cell voltages [B, numX, numY, rows, cols] with ret_V.

    ``nonlinear`` = [R_on, R_off, a_on, b_on, a_off, b_off]: sinh cells as in
    all five host functions (:455-475, 603-622, 727-746, 996-1016,
    1241-1260).  Before every iteration the conductances are recomputed, in the
    dtype of ``G``, from u - d of the buffers that iteration overwrites -- after
    the ping-pong swap those hold the iterate before the newest one, so
    iterations 0 and 1 both see the initial planes -- with |V| < 1e-5 set to
    +-1e-5 (deal_v) and z from the linear conductances, negative z set to 0.
    The currents are taken with the last conductances (get_current).
    """
    dt = np.asarray(G).dtype
    S = dt.type
    B, X, Y, n, m = batch_size, numX, numY, row_size, col_size
    on, om = ou if ou is not None else (n, m)
    nox, noy = n // on, m // om
    w, b = S(wire), S(beta)
    one = S(1)
    inp = np.asarray(input_v, dt).reshape(B, X, n)
    g = np.asarray(G, dt).reshape(X, n, Y, m).transpose(0, 2, 1, 3)[None]  # [1, X, Y, n, m]
    U = np.broadcast_to(inp[:, :, None, :, None], (B, X, Y, n, m)).copy()
    D = np.zeros((B, X, Y, n, m), dt)
    scol = np.arange(noy) * om                       # first column of each OU column
    srow = np.arange(nox) * on                       # first row of each OU row
    if mode == "gs":
        if ou is not None:
            gl = np.array([w / S(s + 1) for s in scol], dt)
            gd = np.array([w / S(n - (s + on - 1)) for s in srow], dt)
        else:
            gl = np.array([S(loads[0]) if loads else w], dt)
            gd = np.array([S(loads[1]) if loads else w], dt)
    else:
        if ou is not None:
            rl = np.array([w * S(s + 1) for s in scol], dt)
            rd = np.array([w * S(n - (s + on - 1)) for s in srow], dt)
        else:
            rl = np.array([S(loads[0]) if loads else w], dt)
            rd = np.array([S(loads[1]) if loads else w], dt)
        Rs = np.zeros((B, X, Y, n, noy), dt)
        Cs = np.zeros((B, X, Y, m, nox), dt)
    src = inp[:, :, None, :, None]                    # [B, X, 1, n, 1]
    if nonlinear is not None:
        R_on, R_off, a_on, b_on, a_off, b_off = (S(p) for p in nonlinear)
        z = (one / g - R_on) / S(float(nonlinear[1]) - float(nonlinear[0]))
        z = np.where(z < 0, S(0), z).astype(dt)
        U_lag, D_lag = U.copy(), D.copy()            # the iterate before the newest
    for _ in range(iter_times):
        if nonlinear is not None:
            V = U_lag - D_lag
            eps = S(1e-5)
            V = np.where((V < eps) & (V > -eps), np.where(V > 0, eps, -eps), V).astype(dt)
            Va = np.abs(V)
            I_on = b_on * np.sinh(Va * a_on)
            I_off = b_off * np.sinh(Va * a_off)
            g = (one / ((one - z) * Va / I_on + z * Va / I_off)).astype(dt)
            U_lag, D_lag = U.copy(), D.copy()
        U0, D0 = U.copy(), D.copy()
        if mode == "gs":
            for t in range(om):
                c = scol + t
                gj = g[..., c]
                old = U[..., c]
                other = D[..., c]
                if t == 0:
                    num = gl * src + w * U[..., c + 1] + gj * other
                    sumg = w + gl + gj
                elif t < om - 1:
                    num = w * (U[..., c - 1] + U[..., c + 1]) + gj * other
                    sumg = w * S(2) + gj
                else:
                    num = w * U[..., c - 1] + gj * other
                    sumg = w + gj
                U[..., c] = b * num / sumg + (one - b) * old
            for t in range(on - 1, -1, -1):
                r = srow + t
                gi = g[..., r, :]
                old = D[..., r, :]
                other = U[..., r, :]
                if t == on - 1:
                    gdd = gd[:, None]
                    num = w * D[..., r - 1, :] + gdd * S(0) + gi * other
                    sumg = w + gdd + gi
                elif t > 0:
                    num = w * (D[..., r - 1, :] + D[..., r + 1, :]) + gi * other
                    sumg = w * S(2) + gi
                else:
                    num = w * D[..., r + 1, :] + gi * other
                    sumg = w + gi
                D[..., r, :] = b * num / sumg + (one - b) * old
        else:
            cur = (U0 - D0) * g                       # cell currents from the previous iterate
            Un = np.empty_like(U)
            Dn = np.empty_like(D)
            for t in range(om):
                Rs += cur[..., scol + t].transpose(0, 1, 2, 3, 4)
            for t in range(om):
                c = scol + t
                if t == 0:
                    Un[..., c] = src - Rs * rl
                else:
                    Un[..., c] = Un[..., c - 1] - Rs * w
                Rs -= cur[..., c]
            for t in range(on):
                Cs += np.moveaxis(cur[..., srow + t, :], 3, 4)
            for t in range(on - 1, -1, -1):
                r = srow + t
                if t == on - 1:
                    Dn[..., r, :] = np.moveaxis(Cs * rd, 4, 3)
                else:
                    Dn[..., r, :] = Dn[..., r + 1, :] + np.moveaxis(Cs * w, 4, 3)
                Cs -= np.moveaxis(cur[..., r, :], 3, 4)
            U, D = Un, Dn
        if enable_break:
            moved = int((np.abs(U - U0) > break_threshold).sum()) + int((np.abs(D - D0) > break_threshold).sum())
            if moved == 0:
                break
    if ret_V:
        return U - D
    cur = (U - D) * g                                  # [B, X, Y, n, m]
    out = np.zeros((B, X, nox, Y, m), dt)
    for t in range(on):
        out += cur[..., srow + t, :].transpose(0, 1, 3, 2, 4)
    return out.reshape(B, X * nox, Y * m)
