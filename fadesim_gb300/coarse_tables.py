"""Tables of the coarse correction of the two-level line relaxation.

The block line relaxation converges slowly when the cells couple the two
planes strongly (1 kOhm cells on 128-node lines): the slow error is smooth and
equal on both planes.  The two-level method corrects it on a coarse grid after
every iteration, with the same bilinear interpolation Phi for the wordline and
the bitline plane, P = [Phi; Phi].  The coarse operator P^T A P then holds no
cell conductance at all (the cell terms g (u - d)^2 vanish for u = d): it is
the wire part only, in units of the wire conductance,

    A_c = M_r (x) K_c + K_r (x) M_c,
    M_r = Pr^T Pr,  K_r = Pr^T Lv Pr,  M_c = Pc^T Pc,  K_c = Pc^T Lh Pc,

with Lh a wordline's chain (driven end at column 0, open at the last column)
and Lv a bitline's (open at row 0, grounded below the last row).  A coarse
solve A_c vec(E) = vec(R) is then E = Zr ((Zr^T R Zc) / (lr_a + lc_b)) Zc^T
from the generalised eigenpairs K Z = M Z diag(l), Z^T M Z = I, of each side.
These depend on the tile shape only, so they are computed here once (FP64)
and compiled into the kernel as FP32 tables (``csrc/coarse_tables.h``):

    python -m fadesim_gb300.coarse_tables     # rewrites csrc/coarse_tables.h
"""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "csrc", "coarse_tables.h")
LD, C = 128, 8  # tile size and fine nodes per coarse cell: a 16 x 16 coarse grid


def hat(L, c):
    """[L, L/c] bilinear interpolation from cell-centred coarse nodes (node I at
    fine position c I + c/2 - 1/2), constant beyond the first and last."""
    Lc = -(-L // c)
    P = np.zeros((L, Lc))
    for i in range(L):
        f = (i + 0.5) / c - 0.5
        i0 = int(math.floor(f))
        t = f - i0
        for k, w in ((i0, 1.0 - t), (i0 + 1, t)):
            P[i, min(max(k, 0), Lc - 1)] += w
    return P


def chain(L, open_end):
    """A line's wire Laplacian in units of the wire conductance: 2 on the
    diagonal (1 at the open end), -1 off it."""
    K = 2.0 * np.eye(L) - np.eye(L, k=1) - np.eye(L, k=-1)
    K[open_end, open_end] = 1.0
    return K


def gen_eig(K, M):
    """K Z = M Z diag(l) with Z^T M Z = I (M symmetric positive definite)."""
    Lm = np.linalg.cholesky(M)
    Li = np.linalg.inv(Lm)
    S = Li @ K @ Li.T
    lam, Q = np.linalg.eigh((S + S.T) / 2)
    return lam, Li.T @ Q


def factors(n=LD, m=LD, c=C):
    """(Pr, Pc, Zr, Zc, lr, lc) of an n x m tile."""
    Pr, Pc = hat(n, c), hat(m, c)
    Lv, Lh = chain(n, 0), chain(m, m - 1)
    lr, Zr = gen_eig(Pr.T @ Lv @ Pr, Pr.T @ Pr)
    lc, Zc = gen_eig(Pc.T @ Lh @ Pc, Pc.T @ Pc)
    return Pr, Pc, Zr, Zc, lr, lc


def coarse_matrix(n=LD, m=LD, c=C):
    """A_c (row-major coarse index I * mc + J), for checks."""
    Pr, Pc = hat(n, c), hat(m, c)
    Lv, Lh = chain(n, 0), chain(m, m - 1)
    return np.kron(Pr.T @ Pr, Pc.T @ Lh @ Pc) + np.kron(Pr.T @ Lv @ Pr, Pc.T @ Pc)


def table(n=LD, m=LD, c=C):
    """The kernel's table: Zr, Zc row-major ([fine-coarse index][eigen index]),
    then lr, lc, as FP32."""
    _, _, Zr, Zc, lr, lc = factors(n, m, c)
    return np.concatenate([Zr.ravel(), Zc.ravel(), lr, lc]).astype(np.float32)


def header_text():
    t = table()
    nc = LD // C
    lines = ["// Generated by fadesim_gb300/coarse_tables.py: the coarse correction of the",
             "// two-level line relaxation on %d x %d tiles, %d x %d coarse grid (see there)." % (LD, LD, nc, nc),
             "// Layout: Zr[%d][%d], Zc[%d][%d] (row: coarse node, column: eigenvector), lr[%d], lc[%d]."
             % (nc, nc, nc, nc, nc, nc),
             "#pragma once", "", "namespace fadesim {", "",
             "constexpr int COARSE_LD = %d, COARSE_C = %d, COARSE_N = %d, COARSE_TABLE = %d;" % (LD, C, nc, t.size),
             "", "static __device__ const float coarse_table_128[COARSE_TABLE] = {"]
    vals = ["%.9e" % float(v) for v in t]
    for k in range(0, len(vals), 6):
        lines.append("    " + ", ".join(v + "f" for v in vals[k:k + 6]) + ",")
    lines += ["};", "", "}  // namespace fadesim", ""]
    return "\n".join(lines)


if __name__ == "__main__":
    with open(HEADER, "w") as f:
        f.write(header_text())
    print(HEADER)
