"""Effective conductance matrices of crossbar tiles and the datasets built on them.

The bitline currents of a tile with linear cells are a linear map of its
wordline voltages, I = v G_eff, G_eff[i, j] the current into bitline j per volt
on wordline i with the other wordlines at 0 V.  It is the reference's FCM
"non-ideal conductance" (crossbarHspice/2dArray.cc:949-1011: one unit-voltage
solve per wordline, then I_j = sum_i g_non_ideal[i][j] v_i) and the target of its
SCN surrogate dataset (pimtorch/pimfixedpoint/SCN_data_gen.py:66-180: one-hot
inputs at the DAC step, labels (I - 1/HRS) / (dG * dV)).  Here the unit
responses of every tile come from one batched line solve on the GPU.

  python -m fadesim_gb300.geff scn --data-num 100 --out data.binlog
"""
import argparse
import pickle

import numpy as np
import torch

from . import cpp_ir_drop_accelerate as acc


def effective_conductance(G, g_wire, v_unit=1.0, tol_v=None):
    """G [T, n, m] tiles (CUDA, float32 or float64) -> G_eff [T, n, m] in A/V.

    Row i of tile t is driven at ``v_unit`` volts with every other row at 0 V;
    the bitline currents divided by ``v_unit`` form G_eff[t, i]."""
    if G.dim() != 3:
        raise ValueError("G must be [tiles, rows, cols]")
    T, n, m = G.shape
    unit = torch.zeros((n, T, n), dtype=G.dtype, device=G.device)
    r = torch.arange(n, device=G.device)
    unit[r, :, r] = v_unit
    cur, _, _ = acc.ir_drop_gs_ex(unit, G.contiguous(), n, n, m, T, 1, g_wire=g_wire, tol_v=tol_v,
                                  return_stats=False)
    return cur.permute(1, 0, 2).contiguous() / v_unit  # [T, n, m]


def fcm_text(states, Rset, g_eff):
    """The reference's FCM output file (2dArray.cc:986-1008): "n m cellR_num", the
    cell resistance states, the state index of every cell, then G_eff, all in
    C++ scientific notation with 12 digits, space separated."""
    states = np.asarray(states)
    g_eff = np.asarray(g_eff, dtype=np.float64)
    n, m = states.shape
    f = lambda v: "%.12e" % v
    out = ["", "%d %d %d" % (n, m, len(Rset))]
    out.append("".join(f(r) + " " for r in Rset))
    for i in range(n):
        out.append("".join(str(int(states[i, j])) + " " for j in range(m)))
    for i in range(n):
        out.append("".join(f(g_eff[i, j]) + " " for j in range(m)))
    return "\n".join(out[1:]) + "\n"


def fcm_currents(g_eff, vin):
    """I_j = sum_i G_eff[i, j] v_i (2dArray.cc:966-973), FP64."""
    return np.asarray(vin, np.float64) @ np.asarray(g_eff, np.float64)


def scn_dataset(path, data_num=50000, cbsize=(128, 128), inputV=1.0, dacBits=1, HRS=74867.0, LRS=16.9e3,
                cellBits=1, r_wire=2.93, sigma=0.0, seed=959595, batch=64, tol_v=None):
    """Write the SCN surrogate dataset in the reference's pickle stream layout
    (SCN_data_gen.py:112-180): a header [rows, cols, inputV, dacBits, HRS, LRS,
    cellBits, r_wire, sigma], then per instance the cell states (flattened list)
    and the labels (G_eff * dV - 1/HRS) / (dG * dV) (flattened list).  Cell
    states are drawn with torch.manual_seed(seed) and one torch.randint per
    instance, as the reference does, so the instances are the same; the labels
    come from converged solves (``batch`` instances per GPU call)."""
    rows, cols = cbsize
    inDeltaV = inputV / (2 ** dacBits - 1)
    cellNum = 2 ** cellBits
    dG = (1 / LRS - 1 / HRS) / (cellNum - 1)
    torch.manual_seed(seed)
    with open(path, "wb") as f:
        pickle.dump([rows, cols, inputV, dacBits, HRS, LRS, cellBits, r_wire, sigma], f)
        done = 0
        while done < data_num:
            k = min(batch, data_num - done)
            wq = [torch.randint(0, cellNum, (1, rows, cols)) for _ in range(k)]
            G = torch.cat([w * dG + 1 / HRS for w in wq]).to(device="cuda", dtype=torch.float64)
            Y = effective_conductance(G, 1 / r_wire, v_unit=inDeltaV, tol_v=tol_v) * inDeltaV  # currents
            Y = Y.cpu()
            for t in range(k):
                pickle.dump(wq[t].view(-1).tolist(), f)
                pickle.dump((Y[t].view(-1) - 1 / HRS).div(dG * inDeltaV).tolist(), f)
            done += k
    return done


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    sc = sub.add_parser("scn", help="SCN surrogate dataset (pickle stream)")
    sc.add_argument("--out", required=True)
    sc.add_argument("--data-num", type=int, default=50000)
    sc.add_argument("--cbsize", type=int, nargs=2, default=[128, 128])
    sc.add_argument("--inputV", type=float, default=1.0)
    sc.add_argument("--dacBits", type=int, default=1)
    sc.add_argument("--HRS", type=float, default=74867.0)
    sc.add_argument("--LRS", type=float, default=16.9e3)
    sc.add_argument("--cellBits", type=int, default=1)
    sc.add_argument("--r-wire", type=float, default=2.93)
    sc.add_argument("--seed", type=int, default=959595)
    a = ap.parse_args()
    if a.cmd == "scn":
        n = scn_dataset(a.out, a.data_num, tuple(a.cbsize), a.inputV, a.dacBits, a.HRS, a.LRS, a.cellBits, a.r_wire,
                        0.0, a.seed)
        print("wrote %d instances to %s" % (n, a.out))


if __name__ == "__main__":
    main()
