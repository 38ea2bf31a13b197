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
