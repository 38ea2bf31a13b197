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
