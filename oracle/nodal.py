"""FP64 direct solve of the crossbar nodal system (the accuracy oracle).

Test infrastructure only: see ``oracle/__init__.py``.

The system restates the node equations the reference relaxes:

* wordline node (i, j), unknown u[i, j]:
  (gL + gR + g[i, j]) u = gL * (vin[i] if j == 0 else u[i, j-1]) + gR * u[i, j+1] + g[i, j] d[i, j]
  with gL = g_wire and gR = g_wire for j < m-1, 0 at the open right end
  (crossbarHspice/2dArray.cc:1563-1574; split_arr_matmul.cu:75-119 where the
  first node couples to the input through g_load_left = g_wire, :275).
* bitline node (i, j), unknown d[i, j]:
  (gU + gD + g[i, j]) d = gU * d[i-1, j] + gD * (vout[j] if i == n-1 else d[i+1, j]) + g[i, j] u[i, j]
  with gU = 0 at the open top (i == 0), gD = g_wire
  (crossbarHspice/2dArray.cc:1576-1588; split_arr_matmul.cu:27-73, :290).
* bitline current I[j] = sum_i (u[i, j] - d[i, j]) * g[i, j]
  (crossbarHspice/2dArray.cc:1670-1674; split_arr_matmul.cu:121-140).

The matrix is the conductance Laplacian with Dirichlet terminals (symmetric
positive definite).  The reference's own dense direct solve,
``ir_drop_accurate_math`` (pimtorch/.../nn/ir_drop_solve.py:75-186), builds the
same system with the terminal nodes kept as extra unknowns; here they are
eliminated into the right-hand side.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def assemble(g, g_wire, vin, vout=None):
    """Sparse SPD matrix and right-hand side for one tile and one input vector.

    Unknowns are interleaved per cell: index 2*(i*m+j) is u[i,j], +1 is d[i,j].
    ``g`` is [n, m] cell conductance, ``vin`` [n] wordline drive, ``vout`` [m]
    bitline terminal voltage (0 V when None).
    """
    g = np.asarray(g, dtype=np.float64)
    n, m = g.shape
    vin = np.asarray(vin, dtype=np.float64).reshape(n)
    vout = np.zeros(m) if vout is None else np.asarray(vout, dtype=np.float64).reshape(m)
    gw = float(g_wire)
    N = 2 * n * m
    I, J = np.meshgrid(np.arange(n), np.arange(m), indexing="ij")
    I = I.ravel()
    J = J.ravel()
    G = g.ravel()
    u = 2 * (I * m + J)
    d = u + 1
    gR = np.where(J < m - 1, gw, 0.0)
    gU = np.where(I > 0, gw, 0.0)
    rows = [u, d, u, d]
    cols = [u, d, d, u]
    vals = [gw + gR + G, gU + gw + G, -G, -G]
    mk = J < m - 1
    k = int(mk.sum())
    rows += [u[mk], u[mk] + 2]
    cols += [u[mk] + 2, u[mk]]
    vals += [np.full(k, -gw), np.full(k, -gw)]
    mk = I < n - 1
    k = int(mk.sum())
    rows += [d[mk], d[mk] + 2 * m]
    cols += [d[mk] + 2 * m, d[mk]]
    vals += [np.full(k, -gw), np.full(k, -gw)]
    A = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    b = np.zeros(N)
    b[2 * (np.arange(n) * m)] += gw * vin
    b[2 * ((n - 1) * m + np.arange(m)) + 1] += gw * vout
    return A, b


def solve(g, g_wire, vin, vout=None, dense=False):
    """Node voltages (u, d), each [n, m], from a direct FP64 solve.

    ``vin`` may be [n] or [V, n] (V input vectors against one conductance map);
    the result is then [V, n, m].  ``dense=True`` uses a dense LU (numpy), the
    form the reference's ``ir_drop_accurate_math`` uses; practical up to 64x64.
    """
    g = np.asarray(g, dtype=np.float64)
    n, m = g.shape
    vin = np.asarray(vin, dtype=np.float64)
    single = vin.ndim == 1
    V = vin.reshape(-1, n)
    A, _ = assemble(g, g_wire, V[0], vout)
    B = np.zeros((2 * n * m, V.shape[0]))
    B[2 * (np.arange(n) * m), :] = float(g_wire) * V.T
    if vout is not None:
        B[2 * ((n - 1) * m + np.arange(m)) + 1, :] += float(g_wire) * np.asarray(vout, np.float64)[:, None]
    if dense:
        X = np.linalg.solve(A.toarray(), B)
    else:
        X = spla.splu(A).solve(B)
    u = X[0::2].T.reshape(-1, n, m)
    d = X[1::2].T.reshape(-1, n, m)
    if single:
        return u[0], d[0]
    return u, d


def currents(g, u, d):
    """Bitline currents I[..., j] = sum_i (u - d) * g (split_arr_matmul.cu:121-140)."""
    return ((u - d) * np.asarray(g, np.float64)).sum(axis=-2)


def solve_layer(input_v, G, rows, cols, numX, numY, g_wire, return_planes=False):
    """Oracle for the ``ir_drop_gs`` boundary layout.

    ``input_v`` is [B, numX, rows] wordline voltages, ``G`` is
    [numX, rows, numY*cols] (split_arr_matmul.cu:200-203,238).  Returns currents
    [B, numX, numY*cols]; with ``return_planes`` also u and d as
    [B, numX, numY, rows, cols].
    """
    input_v = np.asarray(input_v, np.float64)
    G = np.asarray(G, np.float64).reshape(numX, rows, numY, cols)
    B = input_v.shape[0]
    out = np.zeros((B, numX, numY, cols))
    U = np.zeros((B, numX, numY, rows, cols)) if return_planes else None
    D = np.zeros_like(U) if return_planes else None
    for x in range(numX):
        for y in range(numY):
            g = G[x, :, y, :]
            u, d = solve(g, g_wire, input_v[:, x, :])
            out[:, x, y, :] = currents(g, u, d)
            if return_planes:
                U[:, x, y] = u
                D[:, x, y] = d
    out = out.reshape(B, numX, numY * cols)
    if return_planes:
        return out, U, D
    return out


def min_eigen_bound(n, m, g_wire):
    """Lower bound on the smallest eigenvalue of the nodal matrix.

    Every line is a path Laplacian with one Dirichlet end; the cell terms add a
    positive semi-definite coupling, so lambda_min >= g_wire*4*sin^2(pi/(2(2L+1)))
    with L the longer line.
    """
    L = max(n, m)
    return float(g_wire) * 4.0 * np.sin(np.pi / (2.0 * (2 * L + 1))) ** 2


def nonlinear_z(g_lin, R_on, R_off):
    """Cell position between the on and off states from its linear conductance,
    z = (1/g - R_on) / (R_off - R_on), negative z set to 0
    (split_arr_matmul.cu:176-182 get_nonlinear_ratio_z, called at :244)."""
    z = (1.0 / np.asarray(g_lin, np.float64) - R_on) / (R_off - R_on)
    return np.where(z < 0, 0.0, z)


def nonlinear_conductance(V, z, params):
    """Chord conductance I(V)/V of the sinh cell: 1/R(V) with
    R(V) = (1-z) |V| / (b_on sinh(a_on |V|)) + z |V| / (b_off sinh(a_off |V|))
    (split_arr_matmul.cu:184-196 nonlinear_R_tensor), evaluated without the
    reference's |V| < 1e-5 clamp (deal_v, :142-166) by the limit sinh(x)/x -> 1."""
    R_on, R_off, a_on, b_on, a_off, b_off = [float(p) for p in params]
    x = np.abs(np.asarray(V, np.float64))

    def r(a, b):
        ax = a * x
        f = np.where(ax < 1e-4, 1.0 + ax * ax / 6.0, np.sinh(np.maximum(ax, 1e-300)) / np.maximum(ax, 1e-300))
        return 1.0 / (a * b * f)

    return 1.0 / ((1.0 - z) * r(a_on, b_on) + z * r(a_off, b_off))


def solve_nonlinear(g_lin, g_wire, vin, params, tol=1e-14, max_iter=200, reuse_factor=False):
    """FP64 fixed point of the nonlinear nodal system by Picard iteration: the
    cell conductances are re-evaluated at the current cell voltages and the
    linear system is solved exactly (sparse LU) until the node voltages move
    less than ``tol``.  Returns (u, d, iterations).

    ``reuse_factor=True`` keeps the factorisation of the linear-cell matrix and
    iterates x += A0^-1 (b - A(x) x) instead (the same fixed point, a few more
    but far cheaper iterations: for 512 x 512 tiles one triangular solve per
    iteration instead of a new factorisation); it stops at ``tol`` or where the
    corrections stop shrinking below 1e-10 V, the FP64 rounding floor of the
    residual b - A(x) x (~4e-13 V at 512 x 512)."""
    z = nonlinear_z(g_lin, params[0], params[1])
    g = np.asarray(g_lin, np.float64).copy()
    if reuse_factor:
        n, m = g.shape
        vin = np.asarray(vin, np.float64).reshape(n)
        A0, b = assemble(g, g_wire, vin)
        lu = spla.splu(A0)
        x = lu.solve(b)
        prev = np.inf
        for it in range(1, max_iter + 1):
            gv = nonlinear_conductance(x[0::2].reshape(n, m) - x[1::2].reshape(n, m), z, params)
            A, _ = assemble(gv, g_wire, vin)
            dx = lu.solve(b - A @ x)
            x += dx
            step = np.abs(dx).max()
            if step < tol or (step < 1e-10 and step > 0.5 * prev):
                return x[0::2].reshape(n, m), x[1::2].reshape(n, m), it
            prev = step
        raise RuntimeError("nonlinear oracle did not converge")
    u, d = solve(g, g_wire, vin)
    for it in range(1, max_iter + 1):
        g = nonlinear_conductance(u - d, z, params)
        u2, d2 = solve(g, g_wire, vin)
        delta = max(np.abs(u2 - u).max(), np.abs(d2 - d).max())
        u, d = u2, d2
        if delta < tol:
            return u, d, it
    raise RuntimeError("nonlinear oracle did not converge")


def nonlinear_currents(g_lin, u, d, params):
    z = nonlinear_z(g_lin, params[0], params[1])
    V = u - d
    return (nonlinear_conductance(V, z, params) * V).sum(axis=-2)


def sinh_params(R_on, R_off, a=2.0):
    """[R_on, R_off, a_on, b_on, a_off, b_off] for I = (V/R) sinh(aV)/(aV), i.e.
    b = 1/(a R): the cell law of the large-tile non-ideal configuration written
    in the reference's parameterisation (commonConst.py:200-207)."""
    return [R_on, R_off, a, 1.0 / (a * R_on), a, 1.0 / (a * R_off)]
