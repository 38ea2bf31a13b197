// Block line relaxation for tiles larger than 128 x 128, cluster-resident.
//
// Same method as linegs.cu (wordline rows then bitline columns, each line's
// tridiagonal system solved in residual form, in units of the wire
// conductance, with an adaptive residual precision), for tiles up to 256 x 256
// on a 4-CTA cluster and up to 512 x 512 on a 16-CTA cluster.  Each CTA keeps a
// band of RPC consecutive rows of the conductances and of both deviation planes
// in its shared memory (3 x RPC x LDM floats, XOR-swizzled like the 128 kernel).
// 512 threads per CTA, each holding a 32-node segment of a line in registers.
//
// * Wordline pass: rows are local to a CTA; identical to the 128 kernel's pass.
// * Bitline pass: a column crosses all C CTAs.  Each CTA folds its part of the
//   Thomas recurrences into an affine map per column (value entering its first
//   row -> value at its last row, and the mirror map for back substitution),
//   publishes it in shared memory, and after a cluster barrier composes the maps
//   of the CTAs above (forward) or below (backward) through distributed shared
//   memory (ld.shared::cluster via cooperative_groups::map_shared_rank).  The
//   bitline residual needs one row above and below the band: those halo rows
//   are read from the neighbouring CTAs before anyone updates them.
// * Pivots of bitline columns: the recurrence p_r = diag_r - gw^2 / p_{r-1} is
//   a product of 2x2 matrices; each CTA multiplies its rows' matrices (float-
//   float, normalised), the products are exchanged once, and each CTA continues from
//   the state entering its band.
// * The stop and precision decisions read every CTA's partial maxima after a
//   cluster barrier and are therefore identical in all CTAs: every CTA of a
//   cluster runs the same number of iterations, vectors and work items, so all
//   cluster barriers match.
//
// This header holds the templates; linegs_cluster_256.cu and
// linegs_cluster_512.cu instantiate one size each and linegs_cluster.cu
// dispatches.  FP32 or FP64 I/O is a run-time property of the launch.
#pragma once
#include <cooperative_groups.h>
#include <math.h>

#include "kernels.h"
#include "line_common.cuh"

namespace cg = cooperative_groups;

namespace fadesim {

// Per-size shape: C CTAs of RPC rows; the wordline pass puts LPW_W rows x
// NSEG_W segments in a warp, the bitline pass LPW_B columns x NSEG_B segments;
// along a bitline segment the swizzle varies with the row only through row % V.
template <int LDM>
struct CCfg;
template <>
struct CCfg<256> {
    static constexpr int C = 4, RPC = 64, NSEG_W = 8, LPW_W = 4, NSEG_B = 2, LPW_B = 16, V = 4;
};
template <>
struct CCfg<512> {
    static constexpr int C = 16, RPC = 32, NSEG_W = 16, LPW_W = 2, NSEG_B = 1, LPW_B = 32, V = 2;
};
constexpr int CL_T = 512, CL_SEG = 32, CL_NW = 16;

// Node (local row lr, column c) of a band in shared memory.  The XOR term
// touches the low 5 bits of c and depends on c only through c >> 5, so node k
// of a wordline segment sits at (its first node) ^ k; it is chosen so that one
// step of either walk -- LPW_W rows x NSEG_W segments, or LPW_B columns x
// NSEG_B segments -- hits 32 distinct banks (checked exhaustively).
template <int LDM>
__device__ __forceinline__ int cswz(int lr, int c) {
    int x;
    if (LDM == 256) x = (lr & 3) | (((c >> 5) & 3) << 2) | ((((c >> 7) ^ (lr >> 5)) & 1) << 4);
    else x = (lr & 1) | (((c >> 5) & 15) << 1);
    return lr * LDM + (c ^ x);
}

template <int LDM>
constexpr size_t cl_smem_floats() {
    return (size_t)3 * CCfg<LDM>::RPC * LDM + 2 * LDM + CCfg<LDM>::RPC + 8 * LDM + 4 * CL_NW + 8;
}

// Affine-map scans over the NSEG segments of a line held by lanes LPW apart:
// inclusive and exclusive compositions, forward (up) and backward (down).
template <int NSEG, int LPW>
__device__ __forceinline__ void scan_up(float C, float Y, int s, float &Cinc, float &Yinc, float &Cexc, float &Yexc) {
    float Ci = C, Yi = Y;
#pragma unroll
    for (int off = 1; off < NSEG; off <<= 1) {
        const float Cp = __shfl_up_sync(0xffffffffu, Ci, LPW * off);
        const float Yp = __shfl_up_sync(0xffffffffu, Yi, LPW * off);
        if (s >= off) {
            Yi = fmaf(Ci, Yp, Yi);
            Ci *= Cp;
        }
    }
    Cinc = Ci;
    Yinc = Yi;
    Cexc = 1.f;
    Yexc = 0.f;
    if (NSEG > 1) {
        Cexc = __shfl_up_sync(0xffffffffu, Ci, LPW);
        Yexc = __shfl_up_sync(0xffffffffu, Yi, LPW);
        if (s == 0) {
            Cexc = 1.f;
            Yexc = 0.f;
        }
    }
}

template <int NSEG, int LPW>
__device__ __forceinline__ void scan_down(float C, float X, int s, float &Cinc, float &Xinc, float &Cexc, float &Xexc) {
    float Ci = C, Xi = X;
#pragma unroll
    for (int off = 1; off < NSEG; off <<= 1) {
        const float Cn = __shfl_down_sync(0xffffffffu, Ci, LPW * off);
        const float Xn = __shfl_down_sync(0xffffffffu, Xi, LPW * off);
        if (s + off < NSEG) {
            Xi = fmaf(Ci, Xn, Xi);
            Ci *= Cn;
        }
    }
    Cinc = Ci;
    Xinc = Xi;
    Cexc = 1.f;
    Xexc = 0.f;
    if (NSEG > 1) {
        Cexc = __shfl_down_sync(0xffffffffu, Ci, LPW);
        Xexc = __shfl_down_sync(0xffffffffu, Xi, LPW);
        if (s == NSEG - 1) {
            Cexc = 1.f;
            Xexc = 0.f;
        }
    }
}

// Thomas in the multiplier form c = gw / pivot on a segment held in x[] (the
// residual on entry, the correction on exit), the incoming values of the
// forward and backward chains supplied by the caller's scans.
template <int SEG>
__device__ __forceinline__ float seg_fold_fwd(float (&x)[SEG], const float (&c)[SEG]) {
    float Y = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        x[k] *= c[k];
        Y = fmaf(c[k], Y, x[k]);
    }
    return Y;
}
template <int SEG>
__device__ __forceinline__ float seg_apply_fwd_fold_bwd(float (&x)[SEG], const float (&c)[SEG], float y) {
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        y = fmaf(c[k], y, x[k]);
        x[k] = y;
    }
    float X = 0.f;
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) X = fmaf(c[k], X, x[k]);
    return X;
}
template <int SEG>
__device__ __forceinline__ void seg_apply_bwd(float (&x)[SEG], const float (&c)[SEG], float X) {
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) {
        X = fmaf(c[k], X, x[k]);
        x[k] = X;
    }
}

// The value entering this CTA's part of a bitline: the affine maps (c, y) the
// CTAs above published, composed in order onto 0 (forward), or those of the
// CTAs below, bottom up (backward).  Remote maps are fetched four (16-CTA
// clusters: eight) at a time so that their latencies overlap.
template <int C>
__device__ __forceinline__ float compose_above(cg::cluster_group &cluster, const float *agg, int col, int rank) {
    constexpr int K = C > 8 ? 8 : 4;
    float v = 0.f;
#pragma unroll 1
    for (int r0 = 0; r0 < rank; r0 += K) {
        float2 mp[K];
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int r = r0 + t;
            mp[t] = (r < C && r < rank) ? *reinterpret_cast<const float2 *>(cluster.map_shared_rank(agg, r) + 2 * col)
                                        : make_float2(1.f, 0.f);
        }
#pragma unroll
        for (int t = 0; t < K; ++t) v = fmaf(mp[t].x, v, mp[t].y);
    }
    return v;
}
template <int C>
__device__ __forceinline__ float compose_below(cg::cluster_group &cluster, const float *agg, int col, int rank) {
    constexpr int K = C > 8 ? 8 : 4;
    float v = 0.f;
#pragma unroll 1
    for (int r0 = C - 1; r0 > rank; r0 -= K) {
        float2 mp[K];
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int r = r0 - t;
            mp[t] = (r >= 0 && r > rank) ? *reinterpret_cast<const float2 *>(cluster.map_shared_rank(agg, r) + 2 * col)
                                         : make_float2(1.f, 0.f);
        }
#pragma unroll
        for (int t = 0; t < K; ++t) v = fmaf(mp[t].x, v, mp[t].y);
    }
    return v;
}

// Residual of the wordline pass over the CTA's rows (lines local to the CTA)
// into x[], one 32-node segment per thread.  Gs holds g / gw (or the sinh
// cells' positions z); ZOWN / ZOTH: the own / other plane is known to be zero
// (first iteration).  FULL: every row of the band and every column present
// (bounds tests fold away).
template <int LDM, int RES, bool NL, bool ZOWN, bool ZOTH, bool FULL>
__device__ __forceinline__ void cl_word_residual(float (&x)[CL_SEG], const float *__restrict__ U,
                                                 const float *__restrict__ D, const float *__restrict__ Gs,
                                                 const float *__restrict__ vin, int nloc, int m, float inv_gw,
                                                 const SolveCtl &ctl) {
    constexpr int LPW = CCfg<LDM>::LPW_W, SEG = CL_SEG;
    const int tid = threadIdx.x, lane = tid & 31, s = lane / LPW;
    const int line = (tid >> 5) * LPW + (lane % LPW);  // < RPC by the shape
    const bool ok = FULL || line < nloc;
    const int p0 = s * SEG;
    const int Bw = cswz<LDM>(line, p0);  // node p0 + k sits at Bw ^ k
    const float vl = ok ? vin[line] : 0.f;
    float prev = (!ZOWN && ok && p0 > 0 && (FULL || p0 - 1 < m)) ? U[cswz<LDM>(line, p0 - 1)] : 0.f;
    float cur = (!ZOWN && ok && (FULL || p0 < m)) ? U[Bw] : 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        const int p = p0 + k;
        const bool has_next = (FULL && k + 1 < SEG) || (ok && p + 1 < m);
        const float nxt = (!ZOWN && has_next) ? U[k + 1 < SEG ? (Bw ^ (k + 1)) : cswz<LDM>(line, p + 1)] : 0.f;
        float r = 0.f;
        if (FULL || (ok && p < m)) {
            const int q = Bw ^ k;
            const float o = ZOTH ? 0.f : D[q];
            const float gs = NL ? nl_gs(Gs[q], (cur + vl) - o, ctl, inv_gw) : Gs[q];
            r = line_residual_s<true, RES>(prev, cur, nxt, gs, o, vl, true, (FULL && k + 1 < SEG) || p + 1 < m);
        }
        x[k] = r;
        prev = cur;
        cur = nxt;
    }
}

// Wordline pass: the residual form selected by mode (4: both planes zero, 0:
// FP32, 3: exact line differences with an FP32 cell term, 2: float-float, 1:
// FP64; uniform across the cluster), then one shared Thomas solve and update
// in the multiplier form (cm the chain multipliers gw / pivot), so that the
// kernel carries a single copy of the solve whatever the residual forms.
// Modes beyond the residual forms (linear cells): 5 computes the band's
// wordline unit response T'^-1 (g / gw) into w1[k * CL_T + tid]; 6 is the
// first iteration from the ideal state taken from it (its residual is -vin
// g / gw on every node, so its correction is -vin times the unit response).
template <int LDM, bool NL, bool FULL>
__device__ __forceinline__ void cl_word_pass(int mode, float *__restrict__ U, const float *__restrict__ D,
                                             const float *__restrict__ Gs, const float *__restrict__ vin,
                                             const float *__restrict__ cm, const float *__restrict__ segprod,
                                             int nloc_in, int m_in, float inv_gw, float omega, float &dmax,
                                             float &vmax, const SolveCtl &ctl, float *__restrict__ w1 = nullptr) {
    constexpr int NSEG = CCfg<LDM>::NSEG_W, LPW = CCfg<LDM>::LPW_W, SEG = CL_SEG;
    const int nloc = FULL ? CCfg<LDM>::RPC : nloc_in, m = FULL ? LDM : m_in;
    const int tid = threadIdx.x, lane = tid & 31, s = lane / LPW;
    const int line = (tid >> 5) * LPW + (lane % LPW);
    const bool ok = FULL || line < nloc;
    const int p0 = s * SEG;
    const int Bw = cswz<LDM>(line, p0);
    if constexpr (!NL) {
        if (mode == 6) {
            const float sc = ok ? -vin[line] : 0.f;
            float dm = 0.f;
#pragma unroll
            for (int k = 0; k < SEG; ++k) {
                if (FULL || (ok && p0 + k < m)) {
                    const float xk = sc * w1[k * CL_T + tid];
                    const float nv = omega * xk;
                    U[Bw ^ k] = nv;
                    dm = fmaxf(dm, fabsf(xk));
                    vmax = fmaxf(vmax, fabsf(nv));
                }
            }
            dmax = fmaxf(dmax, omega * dm);
            return;
        }
    }
    float x[SEG];
    if (!NL && mode == 5) {
#pragma unroll
        for (int k = 0; k < SEG; ++k) x[k] = (FULL || (ok && p0 + k < m)) ? Gs[Bw ^ k] : 0.f;
    } else
    switch (mode) {
        case 4: cl_word_residual<LDM, 0, NL, true, true, FULL>(x, U, D, Gs, vin, nloc, m, inv_gw, ctl); break;
        case 0: cl_word_residual<LDM, 0, NL, false, false, FULL>(x, U, D, Gs, vin, nloc, m, inv_gw, ctl); break;
        case 3:
            if constexpr (!NL) {  // (sinh cells never take the FP32 cell term)
                cl_word_residual<LDM, 3, NL, false, false, FULL>(x, U, D, Gs, vin, nloc, m, inv_gw, ctl);
                break;
            }
        case 2: cl_word_residual<LDM, 2, NL, false, false, FULL>(x, U, D, Gs, vin, nloc, m, inv_gw, ctl); break;
        default: cl_word_residual<LDM, 1, NL, false, false, FULL>(x, U, D, Gs, vin, nloc, m, inv_gw, ctl); break;
    }
    const bool zown = mode == 4;
    float c[SEG];
#pragma unroll
    for (int k = 0; k < SEG; ++k) c[k] = cm[k * CL_T + tid];
    const float C = segprod[tid];
    const float Y = seg_fold_fwd<SEG>(x, c);
    float Ci, Yi, Cx, Yx;
    scan_up<NSEG, LPW>(C, Y, s, Ci, Yi, Cx, Yx);
    const float X = seg_apply_fwd_fold_bwd<SEG>(x, c, Yx);  // entering value 0 at the line start
    float Cb, Xb, Cbx, Xbx;
    scan_down<NSEG, LPW>(C, X, s, Cb, Xb, Cbx, Xbx);
    seg_apply_bwd<SEG>(x, c, Xbx);
    if (!NL && mode == 5) {
#pragma unroll
        for (int k = 0; k < SEG; ++k) w1[k * CL_T + tid] = x[k];
        return;
    }
    float dm = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        if (FULL || (ok && p0 + k < m)) {
            const int q = Bw ^ k;
            const float nv = zown ? omega * x[k] : fmaf(omega, x[k], U[q]);
            U[q] = nv;
            dm = fmaxf(dm, fabsf(x[k]));
            vmax = fmaxf(vmax, fabsf(nv));
        }
    }
    dmax = fmaxf(dmax, omega * dm);
}

// Residual of the bitline pass into x[] (columns cross the cluster; hup / hdn
// the halo rows above and below the band).  ZOWN: the bitline plane (and so
// the halos) is known to be zero.
template <int LDM, int RES, bool NL, bool ZOWN, bool FULL>
__device__ __forceinline__ void cl_bit_residual(float (&x)[CL_SEG], const float *__restrict__ D,
                                                const float *__restrict__ U, const float *__restrict__ Gs,
                                                const float *__restrict__ vin, const float *__restrict__ hup,
                                                const float *__restrict__ hdn, int row0, int nloc, int m,
                                                float inv_gw, const SolveCtl &ctl) {
    constexpr int LPW = CCfg<LDM>::LPW_B, SEG = CL_SEG, V = CCfg<LDM>::V;
    const int tid = threadIdx.x, lane = tid & 31, s = lane / LPW;
    const int col = (tid >> 5) * LPW + (lane % LPW);  // < LDM by the shape
    const bool ok = FULL || col < m;
    const int p0 = s * SEG;  // first local row of the segment
    int Rb[V];               // node p0 + k sits at Rb[k % V] + k * LDM
#pragma unroll
    for (int t = 0; t < V; ++t) Rb[t] = cswz<LDM>(p0 + t, col) - t * LDM;
    auto qk = [&](int k) { return Rb[k % V] + k * LDM; };
    float prev = ZOWN ? 0.f
                      : ((p0 > 0) ? ((ok && (FULL || p0 - 1 < nloc)) ? D[cswz<LDM>(p0 - 1, col)] : 0.f)
                                  : (ok ? hup[col] : 0.f));
    float cur = (!ZOWN && ok && (FULL || p0 < nloc)) ? D[qk(0)] : 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        const int lr = p0 + k;
        float nxt = 0.f;
        if (!ZOWN && ok)
            nxt = ((FULL && k + 1 < SEG) || lr + 1 < nloc) ? D[k + 1 < SEG ? qk(k + 1) : cswz<LDM>(lr + 1, col)]
                                                           : hdn[col];
        float r = 0.f;
        if (FULL || (ok && lr < nloc)) {
            const int q = qk(k);
            const float o = U[q];
            const float gs = NL ? nl_gs(Gs[q], (o + vin[lr]) - cur, ctl, inv_gw) : Gs[q];
            r = line_residual_s<false, RES>(prev, cur, nxt, gs, o, vin[lr], k > 0 || p0 > 0 || row0 > 0, true);
        }
        x[k] = r;
        prev = cur;
        cur = nxt;
    }
}

// Bitline pass: the residual form selected by mode (as the wordline pass),
// then one shared cross-cluster Thomas solve and update.  Contains two cluster
// barriers.
template <int LDM, bool NL, bool FULL>
__device__ __forceinline__ void cl_bit_pass(int mode, cg::cluster_group &cluster, int rank, float *__restrict__ D,
                                            const float *__restrict__ U, const float *__restrict__ Gs,
                                            const float *__restrict__ vin, const float *__restrict__ cm,
                                            const float *__restrict__ segprod, const float *__restrict__ hup,
                                            const float *__restrict__ hdn, float *__restrict__ aggF,
                                            float *__restrict__ aggB, int row0, int nloc_in, int m_in, float inv_gw,
                                            float omega, float &dmax, float &vmax, const SolveCtl &ctl) {
    constexpr int C = CCfg<LDM>::C, NSEG = CCfg<LDM>::NSEG_B, LPW = CCfg<LDM>::LPW_B, SEG = CL_SEG;
    constexpr int V = CCfg<LDM>::V;
    const int nloc = FULL ? CCfg<LDM>::RPC : nloc_in, m = FULL ? LDM : m_in;
    const int tid = threadIdx.x, lane = tid & 31, s = lane / LPW;
    const int col = (tid >> 5) * LPW + (lane % LPW);
    const bool ok = FULL || col < m;
    const int p0 = s * SEG;
    float x[SEG];
    switch (mode) {
        case 4: cl_bit_residual<LDM, 0, NL, true, FULL>(x, D, U, Gs, vin, hup, hdn, row0, nloc, m, inv_gw, ctl); break;
        case 0: cl_bit_residual<LDM, 0, NL, false, FULL>(x, D, U, Gs, vin, hup, hdn, row0, nloc, m, inv_gw, ctl); break;
        case 3:
            if constexpr (!NL) {
                cl_bit_residual<LDM, 3, NL, false, FULL>(x, D, U, Gs, vin, hup, hdn, row0, nloc, m, inv_gw, ctl);
                break;
            }
        case 2: cl_bit_residual<LDM, 2, NL, false, FULL>(x, D, U, Gs, vin, hup, hdn, row0, nloc, m, inv_gw, ctl); break;
        default: cl_bit_residual<LDM, 1, NL, false, FULL>(x, D, U, Gs, vin, hup, hdn, row0, nloc, m, inv_gw, ctl); break;
    }
    const bool zown = mode == 4;
    int Rb[V];
#pragma unroll
    for (int t = 0; t < V; ++t) Rb[t] = cswz<LDM>(p0 + t, col) - t * LDM;
    auto qk = [&](int k) { return Rb[k % V] + k * LDM; };
    float c[SEG];
#pragma unroll
    for (int k = 0; k < SEG; ++k) c[k] = cm[k * CL_T + tid];
    const float Cs = segprod[tid];
    // ---- forward: fold, scan within the CTA, compose the CTAs above ---------
    const float Y = seg_fold_fwd<SEG>(x, c);
    float Ci, Yi, Cx, Yx;
    scan_up<NSEG, LPW>(Cs, Y, s, Ci, Yi, Cx, Yx);
    if (s == NSEG - 1) {
        aggF[2 * col] = Ci;
        aggF[2 * col + 1] = Yi;
    }
    cluster.sync();
    float yent = 0.f;
    if (s == 0) yent = compose_above<C>(cluster, aggF, col, rank);
    if (NSEG > 1) yent = __shfl_sync(0xffffffffu, yent, lane % LPW);
    // ---- backward: fold, scan within the CTA, compose the CTAs below --------
    const float X = seg_apply_fwd_fold_bwd<SEG>(x, c, fmaf(Cx, yent, Yx));
    float Cb, Xb, Cbx, Xbx;
    scan_down<NSEG, LPW>(Cs, X, s, Cb, Xb, Cbx, Xbx);
    if (s == 0) {
        aggB[2 * col] = Cb;
        aggB[2 * col + 1] = Xb;
    }
    cluster.sync();
    float xent = 0.f;
    if (s == 0) xent = compose_below<C>(cluster, aggB, col, rank);
    if (NSEG > 1) xent = __shfl_sync(0xffffffffu, xent, lane % LPW);
    seg_apply_bwd<SEG>(x, c, fmaf(Cbx, xent, Xbx));
    float dm = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        const int lr = p0 + k;
        if (FULL || (ok && lr < nloc)) {
            const int q = qk(k);
            const float nv = zown ? omega * x[k] : fmaf(omega, x[k], D[q]);
            D[q] = nv;
            dm = fmaxf(dm, fabsf(x[k]));
            vmax = fmaxf(vmax, fabsf(nv));
        }
    }
    dmax = fmaxf(dmax, omega * dm);
}

// Float-float helpers for the band products below (error-free FP32 transforms).
struct FF {
    float h, l;
};
__device__ __forceinline__ FF ff_norm(float s, float e) {
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
// x * y - z
__device__ __forceinline__ FF ff_mul_sub(FF x, FF y, FF z) {
    const float ph = __fmul_rn(x.h, y.h);
    const float pl = __fmaf_rn(x.h, y.h, -ph) + (__fmul_rn(x.h, y.l) + __fmul_rn(x.l, y.h));
    float sh, sl;
    two_sum(ph, -z.h, sh, sl);
    return ff_norm(sh, __fadd_rn(sl, __fsub_rn(pl, z.l)));
}
// x * y + z * w
__device__ __forceinline__ FF ff_dot2(FF x, FF y, FF z, FF w) {
    const float ph = __fmul_rn(x.h, y.h), qh = __fmul_rn(z.h, w.h);
    const float pl = __fmaf_rn(x.h, y.h, -ph) + (__fmul_rn(x.h, y.l) + __fmul_rn(x.l, y.h));
    const float ql = __fmaf_rn(z.h, w.h, -qh) + (__fmul_rn(z.h, w.l) + __fmul_rn(z.l, w.h));
    float sh, sl;
    two_sum(ph, qh, sh, sl);
    return ff_norm(sh, __fadd_rn(sl, __fadd_rn(pl, ql)));
}
// x * 2^k (exact)
__device__ __forceinline__ FF ff_scale(FF x, float p2) { return {x.h * p2, x.l * p2}; }
// 2^-e with 2^e the binade of |v| (v finite, nonzero): keeps composed states near 1
__device__ __forceinline__ float inv_binade(float v) {
    const int e = ((__float_as_int(v) >> 23) & 0xff) - 127;
    return __int_as_float((127 - e) << 23);
}

// Chain multipliers gw / pivot of the CTA's wordline rows and of its part of
// every bitline column, written in the order the pass threads read them, with
// each segment's product; uses mob (8 floats per column) as scratch read by the
// other CTAs.  Everything in units of gw and in float-float (FP64-class
// precision on the FP32 pipe; the FP64 pipe of this part is slow): the row
// recurrences step by ff_pivot_step; a bitline's pivot entering a band comes
// from the bands above as a product of Moebius maps P -> D - 1 / P, i.e.
// [num; den] <- [[D, -1], [1, 0]] [num; den] with P = num / den.
template <int LDM>
__device__ void cl_pivots(cg::cluster_group &cluster, int rank, const float *__restrict__ Gs, float *__restrict__ piv,
                          float *__restrict__ mob, int row0, int nloc, int n, int m, float gw) {
    constexpr int RPC = CCfg<LDM>::RPC, SEG = CL_SEG, LPW_W = CCfg<LDM>::LPW_W, LPW_B = CCfg<LDM>::LPW_B;
    float *pivW = piv, *pivB = piv + SEG * CL_T, *prodW = piv + 2 * SEG * CL_T, *prodB = prodW + CL_T;
    // 1. each column's 2x2 product over the band (jobs < LDM) and the wordline
    //    rows' multipliers (jobs LDM .. LDM + RPC - 1)
    for (int job = threadIdx.x; job < LDM + RPC; job += CL_T) {
        if (job >= LDM) {
            const int lr = job - LDM;
            const int tw_base = (lr / LPW_W) * 32 + (lr % LPW_W);
            float rh = 0.f, rl = 0.f, sp = 1.f;
            for (int c = 0; c < LDM; ++c) {
                float f = 0.f;
                if (lr < nloc && c < m) {
                    // source link + right link (absent at the end) + cell
                    const float gs = __fdiv_rn(Gs[cswz<LDM>(lr, c)], gw);
                    f = ff_pivot_step(c + 1 < m ? 2.f : 1.f, gs, c == 0, rh, rl);
                }
                const int tw = tw_base + (c / SEG) * LPW_W;
                pivW[(c % SEG) * CL_T + tw] = f;
                sp *= f;
                if (c % SEG == SEG - 1) {
                    prodW[tw] = sp;
                    sp = 1.f;
                }
            }
        } else {
            // the band's map: the product of its rows' [[D, -1], [1, 0]], from
            // the identity; entries grow at most ~linearly with the rows for
            // D near 2, so the band needs no rescaling until its end
            const int jb = job;
            FF a = {1.f, 0.f}, b = {0.f, 0.f}, c = {0.f, 0.f}, d = {1.f, 0.f};
            if (jb < m) {
                for (int lr = 0; lr < nloc; ++lr) {
                    // upper link (absent at the top) + lower link + cell
                    FF D;
                    two_sum(row0 + lr > 0 ? 2.f : 1.f, __fdiv_rn(Gs[cswz<LDM>(lr, jb)], gw), D.h, D.l);
                    const FF na = ff_mul_sub(D, a, c), nb = ff_mul_sub(D, b, d);
                    c = a;
                    d = b;
                    a = na;
                    b = nb;
                }
                const float k = inv_binade(fmaxf(fmaxf(fabsf(a.h), fabsf(b.h)), fmaxf(fabsf(c.h), fabsf(d.h))));
                a = ff_scale(a, k);
                b = ff_scale(b, k);
                c = ff_scale(c, k);
                d = ff_scale(d, k);
            }
            float *M = mob + 8 * jb;
            M[0] = a.h; M[1] = a.l; M[2] = b.h; M[3] = b.l;
            M[4] = c.h; M[5] = c.l; M[6] = d.h; M[7] = d.l;
        }
    }
    cluster.sync();
    for (int jb = threadIdx.x; jb < LDM; jb += CL_T) {
        // state entering this band: [1; 0] (no row above the first) through the bands above
        FF num = {1.f, 0.f}, den = {0.f, 0.f};
        for (int r = 0; r < rank; ++r) {
            const float *M = cluster.map_shared_rank(mob, r) + 8 * jb;
            const FF nn = ff_dot2({M[0], M[1]}, num, {M[2], M[3]}, den);
            const FF dd = ff_dot2({M[4], M[5]}, num, {M[6], M[7]}, den);
            const float k = inv_binade(fmaxf(fabsf(nn.h), fabsf(dd.h)));
            num = ff_scale(nn, k);
            den = ff_scale(dd, k);
        }
        // 1 / P of the row above the band: den / num in float-float
        float rh = 0.f, rl = 0.f;
        if (rank > 0 && num.h != 0.f) {
            rh = __fdiv_rn(den.h, num.h);
            const float e = __fmaf_rn(-num.h, rh, den.h) + __fsub_rn(den.l, __fmul_rn(rh, num.l));
            rl = __fdiv_rn(e, num.h);
        }
        const int tb_base = (jb / LPW_B) * 32 + (jb % LPW_B);
        float sp = 1.f;
        for (int lr = 0; lr < RPC; ++lr) {
            float f = 0.f;
            if (jb < m && lr < nloc) {
                const float gs = __fdiv_rn(Gs[cswz<LDM>(lr, jb)], gw);
                f = ff_pivot_step(row0 + lr > 0 ? 2.f : 1.f, gs, row0 + lr == 0, rh, rl);
            }
            const int tb = tb_base + (lr / SEG) * LPW_B;
            pivB[(lr % SEG) * CL_T + tb] = f;
            sp *= f;
            if (lr % SEG == SEG - 1) {
                prodB[tb] = sp;
                sp = 1.f;
            }
        }
    }
    cluster.sync();  // the band products are read remotely until here
}

// Outputs of one solve (see line_outputs in line_impl.cuh): planes, or bitline
// currents summed over the bands through distributed shared memory.  Contains
// cluster barriers: every CTA of the cluster calls it.
template <int LDM, typename TIO, bool NL>
__device__ __forceinline__ void cl_outputs(cg::cluster_group &cluster, int rank, const SolveArgs &a, const float *Gs,
                                           const float *U, const float *D, const float *vin, float *part, int n,
                                           int m, int nloc, int row0, int b, int x, int y, float gw,
                                           int &nonfinite_flag) {
    constexpr int C = CCfg<LDM>::C, SEG = CL_SEG, LPW_B = CCfg<LDM>::LPW_B;
    const int tid = threadIdx.x;
    TIO *out = static_cast<TIO *>(a.out);
    const int ldG = a.numY * m;
    if (a.ret_V) {
        for (int e = tid; e < nloc * m; e += CL_T) {
            const int lr = e / m, j = e - lr * m;
            const int q = cswz<LDM>(lr, j);
            const TIO uu = (TIO)U[q] + vin_exact<TIO>(a.input, ((size_t)b * a.numX + x) * n + row0 + lr, a.f64,
                                                      vin[lr]);
            if (!isfinite((float)uu) || !isfinite(D[q])) nonfinite_flag = 1;
            const size_t sol = ((size_t)b * a.numX + x) * a.numY + y;
            const size_t i = (size_t)row0 + lr;
            if (a.ret_V == 2) {
                out[(sol * 2 + 0) * n * m + i * m + j] = uu;
                out[(sol * 2 + 1) * n * m + i * m + j] = (TIO)D[q];
            } else {
                out[(sol * n + i) * m + j] = uu - (TIO)D[q];
            }
        }
        __syncthreads();
        cluster.sync();
    } else {
        // partial currents over the band, then each CTA finishes LDM/C columns
        const int lane = tid & 31, s = lane / LPW_B, j = (tid >> 5) * LPW_B + (lane % LPW_B);
        float acc = 0.f;
        if (j < m) {
            for (int k = 0; k < SEG; ++k) {
                const int lr = s * SEG + k;
                if (lr < nloc) {
                    const int q = cswz<LDM>(lr, j);
                    const float V = (U[q] + vin[lr]) - D[q];
                    float Ic = (NL ? nl_g(Gs[q], V, a.ctl, gw) : Gs[q] * gw) * V;
                    if (a.ctl.noise_sigma > 0.f)
                        Ic *= 1.f + a.ctl.noise_sigma * normal_from(a.ctl.noise_seed,
                                                                    ((unsigned long long)b * a.numX + x) * a.numY + y,
                                                                    (unsigned long long)(row0 + lr) * m + j);
                    acc += Ic;
                }
            }
        }
#pragma unroll
        for (int off = LPW_B; off < 32; off <<= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (s == 0) part[j] = acc;
        cluster.sync();
        constexpr int CPC = LDM / C;
        if (tid < CPC) {
            const int jj = rank * CPC + tid;
            if (jj < m) {
                TIO tot = 0;
                for (int r = 0; r < C; ++r) tot += (TIO)cluster.map_shared_rank(part, r)[jj];
                out[((size_t)b * a.numX + x) * ldG + (size_t)y * m + jj] = tot;
                if (!isfinite((float)tot)) nonfinite_flag = 1;
            }
        }
        __syncthreads();
        cluster.sync();  // partial currents read remotely until here
    }
}

template <int LDM, bool NL, bool FULL>
__global__ void __launch_bounds__(CL_T, 1) line_relax_cluster_kernel(SolveArgs a) {
    constexpr int C = CCfg<LDM>::C, RPC = CCfg<LDM>::RPC, SEG = CL_SEG;
    // Full tiles drop the bounds tests of both passes.  (With one pass body per
    // residual form, a bounds-free wordline pass made the compiler hoist a whole
    // segment's loads and spill 650 bytes; with the residual forms sharing one
    // Thomas solve it does not, and the 256 x 256 solve is 15% faster.)
    constexpr bool WFULL = FULL;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    extern __shared__ float4 smem4[];
    float *Gs = reinterpret_cast<float *>(smem4);
    float *U = Gs + RPC * LDM;
    float *D = U + RPC * LDM;
    float *hup = D + RPC * LDM;
    float *hdn = hup + LDM;
    float *vin = hdn + LDM;
    float *aux = vin + RPC;         // 8 * LDM floats: 2x2 float-float band products, or aggF/aggB/partial currents
    float *red = aux + 8 * LDM;     // [2][2][CL_NW]
    float *cred = red + 4 * CL_NW;  // [2][2] this CTA's maxima, read by the cluster
    float *aggF = aux, *aggB = aux + 2 * LDM, *part = aux + 4 * LDM;
    __shared__ unsigned long long st_solves, st_iters, st_rej;
    __shared__ int st_max, st_or, nonfinite_flag;
    __shared__ float bmax_scratch[CL_NW];
    __shared__ float band_gsmax, band_vmax;  // this CTA's maxima, read by the cluster
    __shared__ float cl_bcast[2];            // cluster-wide values, gathered by warp 0

    const int tid = threadIdx.x;
    const int n = FULL ? LDM : a.n, m = FULL ? LDM : a.m, ldG = a.numY * m;
    const int row0 = rank * RPC;
    const int nloc = FULL ? RPC : max(0, min(RPC, n - row0));
    const bool f64 = a.f64 != 0;
    // per CTA: the chain multipliers of both passes, their segment products and
    // the band's wordline unit response (linear cells)
    float *piv = a.scratch + (size_t)blockIdx.x * (3 * SEG * CL_T + 2 * CL_T);
    float *w1 = piv + 2 * SEG * CL_T + 2 * CL_T;
    const float gw = a.gw, tol = a.ctl.tol_v;
    const float inv_gw = 1.f / gw;
    const int kres = a.ctl.residual_period, maxit = a.ctl.max_iters;
    const bool ff = a.ctl.residual_ff != 0;
    const bool precise_first = kres == 1;
    const long long cid = blockIdx.x / C, ncl = gridDim.x / C;
    if (tid == 0) {
        st_solves = 0;
        st_iters = 0;
        st_rej = 0;
        st_max = 0;
        st_or = 0;
    }
    long long cached_tile = -1;
    float rate_hint = 0.f;  // first-step rate of the previous vector of this tile (cluster-uniform)
    float omega_prev = 0.f; // final relaxation factor of that vector (cluster-uniform)
    float gs_max = 0.f;     // largest g / gw of the tile (cluster-uniform, linear cells)
    // work queue: rank 0 of every cluster claims the cluster's next (tile,
    // vector chunk) item from the call's counter and the cluster reads it after
    // a cluster barrier (rank 0 claims again only after the item's own cluster
    // barriers, which every CTA reaches after reading the claim)
    __shared__ long long s_item;
    long long next_static = cid;
    auto claim = [&]() -> long long {
        if (rank == 0 && tid == 0) {
            if (a.stats) {
                s_item = (long long)atomicAdd(&a.stats->queue_head, 1ull);
            } else {
                s_item = next_static;
                next_static += ncl;
            }
        }
        cluster.sync();
        return *cluster.map_shared_rank(&s_item, 0);
    };
    for (long long item = claim(); item < a.nitems; item = claim()) {
        const long long tile = item / a.nchunks;
        const int chunk = (int)(item % a.nchunks);
        const int x = (int)(tile / a.numY), y = (int)(tile % a.numY);
        const int b0 = chunk * a.vchunk, b1 = min(a.B, b0 + a.vchunk);
        if (tile != cached_tile) {
            __syncthreads();
            for (int e = tid; e < RPC * LDM; e += CL_T) {
                const int lr = e / LDM, c = e - lr * LDM;
                Gs[cswz<LDM>(lr, c)] =
                    (lr < nloc && c < m) ? load_io(a.G, ((size_t)x * n + row0 + lr) * ldG + (size_t)y * m + c, f64)
                                         : 0.f;
            }
            __syncthreads();
            cl_pivots<LDM>(cluster, rank, Gs, piv, aux, row0, nloc, n, m, gw);
            __syncthreads();
            if (!NL) {
                // the passes work in units of gw: g / gw
                float gm = 0.f;
                for (int e = tid; e < RPC * LDM; e += CL_T) {
                    const int q = cswz<LDM>(e / LDM, e % LDM);
                    const float gsv = __fdiv_rn(Gs[q], gw);
                    Gs[q] = gsv;
                    gm = fmaxf(gm, fabsf(gsv));
                }
                gm = warp_max(gm);
                if ((tid & 31) == 0) bmax_scratch[tid >> 5] = gm;
                __syncthreads();
                if (tid == 0) {
                    float v = 0.f;
                    for (int w = 0; w < CL_NW; ++w) v = fmaxf(v, bmax_scratch[w]);
                    band_gsmax = v;
                }
                cluster.sync();
                if (tid < 32) {
                    const float v = warp_max(tid < C ? *cluster.map_shared_rank(&band_gsmax, tid) : 0.f);
                    if (tid == 0) cl_bcast[0] = v;
                }
                __syncthreads();
                gs_max = cl_bcast[0];
                // the band's wordline unit response (each thread writes and later
                // reads only its own entries)
                float dn0 = 0.f, dn1 = 0.f;
                cl_word_pass<LDM, NL, WFULL>(5, U, D, Gs, vin, piv, piv + 2 * SEG * CL_T, nloc, m, inv_gw, 1.f, dn0,
                                             dn1, a.ctl, w1);
            } else {
                // the sinh cells keep their on/off position; the linear values served the pivots
                for (int e = tid; e < RPC * LDM; e += CL_T) {
                    const int q = cswz<LDM>(e / LDM, e % LDM);
                    Gs[q] = nl_cell(Gs[q], a.ctl, inv_gw);
                }
                __syncthreads();
            }
            cached_tile = tile;
            rate_hint = 0.f;
            omega_prev = 0.f;
        }
        for (int b = b0; b < b1; ++b) {
            __syncthreads();
            // From the ideal state the planes are zero: the first iteration reads
            // neither plane nor the halos, so they need no clearing -- unless every
            // iteration must be precise (then they are cleared).  (Clearing them for
            // sinh cells too, so that two pass bodies alternate instead of three,
            // measured 2% slower on the 512x512 sinh-cell workload.)  A warm start
            // loads this band's rows of the initial deviation planes [2][n][m].
            bool warm = a.init != nullptr, rejected = false;
            bool zero = !warm && !precise_first;
            if (warm) {
                const float *w0 = a.init + (((size_t)b * a.numX + x) * a.numY + y) * 2 * n * m;
                for (int e = tid; e < RPC * LDM; e += CL_T) {
                    const int lr = e / LDM, c = e - lr * LDM;
                    const bool in = lr < nloc && c < m;
                    const size_t o = (size_t)(row0 + lr) * m + c;
                    U[cswz<LDM>(lr, c)] = in ? w0[o] : 0.f;
                    D[cswz<LDM>(lr, c)] = in ? w0[(size_t)n * m + o] : 0.f;
                }
            } else if (precise_first) {
                for (int e = tid; e < RPC * LDM; e += CL_T) {
                    U[e] = 0.f;
                    D[e] = 0.f;
                }
            }
            float vabs = 0.f;
            if (tid < RPC) {
                const float v = (tid < nloc) ? load_io(a.input, ((size_t)b * a.numX + x) * n + row0 + tid, f64) : 0.f;
                vin[tid] = v;
                vabs = fabsf(v);
            }
            vabs = warp_max(vabs);
            if ((tid & 31) == 0) bmax_scratch[tid >> 5] = vabs;
            __syncthreads();
            if (tid == 0) {
                float v = 0.f;
                for (int w = 0; w < CL_NW; ++w) v = fmaxf(v, bmax_scratch[w]);
                band_vmax = v;
            }
            cluster.sync();  // every band initialised (and its maxima published) before halos are read
            if (tid < 32) {
                const float v = warp_max(tid < C ? *cluster.map_shared_rank(&band_vmax, tid) : 0.f);
                if (tid == 0) cl_bcast[1] = v;
            }
            __syncthreads();
            const float vin_max = cl_bcast[1];
            // precise iterations may keep the cell term in FP32 (RES 3) when its
            // rounding, amplified by at most L^2/2 through a line solve, stays 8x
            // under the tolerance (cluster-uniform: from cluster-wide maxima)
            const float Lmax = (float)max(n, m);
            const bool semi = !NL && ff &&
                              gs_max * 3.f * vin_max * 1.1920929e-07f * 0.5f * Lmax * Lmax <= 0.125f * tol;
            LineStop stop;
            stop.init(a.ctl.omega, rate_hint, omega_prev);
            float omega = stop.omega, omega_last = omega;
            bool res64 = precise_first;
            int status = 0, it = 0, par = 0;
            while (true) {
                float dmax = 0.f, vmax = 0.f;
                omega_last = omega;
                const int mode = zero ? 4 : (!res64 ? 0 : (semi ? 3 : (ff ? 2 : 1)));
                const float *pW = piv, *sW = piv + 2 * SEG * CL_T;
                cl_word_pass<LDM, NL, WFULL>(!NL && mode == 4 ? 6 : mode, U, D, Gs, vin, pW, sW, nloc, m, inv_gw,
                                             omega, dmax, vmax, a.ctl, w1);
                __syncthreads();
                for (int j = tid; j < LDM; j += CL_T) {
                    // halo rows: the row above the band and the row below it (0 V ground below the last row)
                    hup[j] = (!zero && row0 > 0 && nloc > 0 && j < m)
                                 ? cluster.map_shared_rank(D, rank - 1)[cswz<LDM>(RPC - 1, j)]
                                 : 0.f;
                    hdn[j] = (!zero && row0 + nloc < n && j < m) ? cluster.map_shared_rank(D, rank + 1)[cswz<LDM>(0, j)]
                                                                 : 0.f;
                }
                __syncthreads();
                const float *pB = piv + SEG * CL_T, *sB = piv + 2 * SEG * CL_T + CL_T;
                cl_bit_pass<LDM, NL, FULL>(mode, cluster, rank, D, U, Gs, vin, pB, sB, hup, hdn, aggF, aggB, row0, nloc, m,
                                           inv_gw, omega, dmax, vmax, a.ctl);
                zero = false;
                dmax = warp_max(dmax);
                vmax = warp_max(vmax);
                if ((tid & 31) == 0) {
                    red[(par * 2 + 0) * CL_NW + (tid >> 5)] = dmax;
                    red[(par * 2 + 1) * CL_NW + (tid >> 5)] = vmax;
                }
                __syncthreads();
                if (tid < 32) {
                    const float d0 = warp_max(tid < CL_NW ? red[(par * 2 + 0) * CL_NW + tid] : 0.f);
                    const float v0 = warp_max(tid < CL_NW ? red[(par * 2 + 1) * CL_NW + tid] : 0.f);
                    if (tid == 0) {
                        cred[par * 2 + 0] = d0;
                        cred[par * 2 + 1] = v0;
                    }
                }
                cluster.sync();
                // the same C values in every CTA: an identical decision.  Warp 0
                // gathers them; the pair is then read from this CTA's memory.
                if (tid < 32) {
                    const float *cr = cluster.map_shared_rank(cred, tid < C ? tid : 0);
                    const float d0 = warp_max(tid < C ? cr[par * 2 + 0] : 0.f);
                    const float v0 = warp_max(tid < C ? cr[par * 2 + 1] : 0.f);
                    if (tid == 0) {
                        red[(par * 2 + 0) * CL_NW] = d0;
                        red[(par * 2 + 1) * CL_NW] = v0;
                    }
                }
                __syncthreads();
                const float delta = red[(par * 2 + 0) * CL_NW], vm = red[(par * 2 + 1) * CL_NW];
                par ^= 1;
                ++it;
                if (!isfinite(delta) || !isfinite(vm)) {
                    // the same cluster-wide values in every CTA: every CTA leaves here
                    status = FADESIM_ST_NONFINITE;
                    break;
                }
                if (warm && it == 1 && !(delta < vm)) {
                    // the prediction moved as much as the solution is large: discard
                    // it and start again from the ideal state (cluster-uniform)
                    if (precise_first) {
                        __syncthreads();
                        for (int e = tid; e < RPC * LDM; e += CL_T) {
                            U[e] = 0.f;
                            D[e] = 0.f;
                        }
                    }
                    cluster.sync();  // every band restarted before any halo is read again
                    zero = !precise_first;
                    warm = false;
                    rejected = true;
                    stop.init(a.ctl.omega, rate_hint, omega_prev);
                    omega = stop.omega;
                    res64 = precise_first;
                    continue;
                }
                const bool small = stop.update(delta, vm, tol);
                omega = stop.omega;
                if (small) {
                    if (res64 || kres < 0) {
                        status = FADESIM_ST_CONVERGED;
                        break;
                    }
                    res64 = true;
                } else {
                    res64 = kres > 0 ? (it % kres == 0) : (kres == 0 && stop.want_precise(tol, vm, a.ctl.precise_margin));
                }
                if (it >= maxit) {
                    status = FADESIM_ST_MAXITER;
                    break;
                }
            }
            if (rejected) status |= FADESIM_ST_WARM_REJECTED;
            rate_hint = stop.final_rate();
            omega_prev = stop.omega;
            // ---- outputs --------------------------------------------------------
            if (!NL && !a.ret_V && !(a.ctl.noise_sigma > 0.f) && omega_last == 1.f) {
                // After a bitline pass at omega 1 the bitline equations hold, and a
                // column's equations telescope to sum_i g_ij (u_ij - d_ij) = gw d_(n-1)j:
                // the CTA holding the last row writes every current from its band
                // alone (no cluster exchange); it records a non-finite value itself.
                if (row0 <= n - 1 && n - 1 < row0 + nloc) {
                    const int lr = n - 1 - row0;
                    bool bad = false;
                    for (int j = tid; j < m; j += CL_T) {
                        const float dl = D[cswz<LDM>(lr, j)];
                        const size_t o = ((size_t)b * a.numX + x) * ldG + (size_t)y * m + j;
                        if (f64) static_cast<double *>(a.out)[o] = (double)gw * (double)dl;
                        else static_cast<float *>(a.out)[o] = gw * dl;
                        bad |= !isfinite(dl);
                    }
                    if (bad) atomicOr(&st_or, FADESIM_ST_NONFINITE);
                }
            } else {
                if (tid == 0) nonfinite_flag = 0;
                __syncthreads();
                if (f64)
                    cl_outputs<LDM, double, NL>(cluster, rank, a, Gs, U, D, vin, part, n, m, nloc, row0, b, x, y, gw,
                                                nonfinite_flag);
                else
                    cl_outputs<LDM, float, NL>(cluster, rank, a, Gs, U, D, vin, part, n, m, nloc, row0, b, x, y, gw,
                                               nonfinite_flag);
                if (nonfinite_flag) status |= FADESIM_ST_NONFINITE;
            }
            if (tid == 0 && rank == 0) {
                if (a.iters_out) a.iters_out[((long long)b * a.numX + x) * a.numY + y] = it;
                st_solves += 1;
                st_iters += it;
                st_max = max(st_max, it);
                if (status & FADESIM_ST_WARM_REJECTED) st_rej += 1;
                atomicOr(&st_or, status);  // the last row's CTA may flag it too
            }
        }
    }
    __syncthreads();
    cluster.sync();  // no CTA leaves while another may still read its shared memory
    if (tid == 0 && a.stats) {
        if (rank == 0 && st_solves) {
            atomicAdd(&a.stats->solves, st_solves);
            atomicAdd(&a.stats->iters_sum, st_iters);
            atomicMax(&a.stats->iters_max, st_max);
            if (st_rej) atomicAdd(&a.stats->warm_rejected, st_rej);
        }
        if (st_or) atomicOr(&a.stats->status_or, st_or);  // rank 0's, or a flag of the last row's CTA
    }
}

// Launch helpers for one size and cell law (instantiated by linegs_cluster_<LDM>[nl].cu).
template <int LDM, bool NL>
cudaError_t cl_launch_cfg_t(int *clusters, const SolveArgs *a, int grid, cudaStream_t st) {
    // full tiles (n = m = LDM) run the bounds-free bitline pass
    const bool full = a && a->n == LDM && a->m == LDM;
    void (*kern)(SolveArgs) =
        full ? line_relax_cluster_kernel<LDM, NL, true> : line_relax_cluster_kernel<LDM, NL, false>;
    const size_t smem = cl_smem_floats<LDM>() * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (CCfg<LDM>::C > 8) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CCfg<LDM>::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(CL_T);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (clusters) {
        cfg.gridDim = dim3(CCfg<LDM>::C);
        return cudaOccupancyMaxActiveClusters(clusters, kern, &cfg);
    }
    cfg.gridDim = dim3(grid);
    e = cudaLaunchKernelEx(&cfg, kern, *a);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace fadesim
