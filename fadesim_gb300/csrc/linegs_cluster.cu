// Block line relaxation for tiles larger than 128 x 128, cluster-resident.
//
// Same method as linegs.cu (wordline rows then bitline columns, each line's
// tridiagonal system solved in residual form), for tiles up to 256 x 256 on a
// 4-CTA cluster and up to 512 x 512 on a 16-CTA cluster.  Each CTA keeps a band
// of RPC consecutive rows of the conductances and of both deviation planes in
// its shared memory (3 x RPC x LDM floats, padded one word per 16 columns).
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
//   a product of 2x2 matrices; each CTA multiplies its rows' matrices (FP64,
//   normalised), the products are exchanged once, and each CTA continues from
//   the state entering its band.
// * The stop decision reads every CTA's partial maxima after a cluster barrier
//   and is therefore identical in all CTAs: every CTA of a cluster runs the
//   same number of iterations, vectors and work items, so all cluster barriers
//   match.
#include <cooperative_groups.h>
#include <math.h>

#include "kernels.h"
#include "line_common.cuh"

namespace cg = cooperative_groups;

namespace fadesim {

template <int LDM>
struct CCfg;
template <>
struct CCfg<256> {
    static constexpr int C = 4, RPC = 64, S = 273, NSEG_W = 16, LPW_W = 2, NSEG_B = 4, LPW_B = 8;
};
template <>
struct CCfg<512> {
    static constexpr int C = 16, RPC = 32, S = 545, NSEG_W = 32, LPW_W = 1, NSEG_B = 2, LPW_B = 16;
};
constexpr int CL_T = 1024, CL_SEG = 16, CL_NW = 32;

// local row lr, column c; one pad word per 16 columns (bank spread of the walks)
template <int LDM>
__device__ __forceinline__ int cidx(int lr, int c) {
    return lr * CCfg<LDM>::S + c + (c >> 4);
}

template <int LDM>
constexpr size_t cl_smem_floats() {
    return (size_t)3 * CCfg<LDM>::RPC * CCfg<LDM>::S + 2 * LDM + CCfg<LDM>::RPC + 8 * LDM + 4 * CL_NW + 8;
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
    Cexc = __shfl_up_sync(0xffffffffu, Ci, LPW);
    Yexc = __shfl_up_sync(0xffffffffu, Yi, LPW);
    if (s == 0) {
        Cexc = 1.f;
        Yexc = 0.f;
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
    Cexc = __shfl_down_sync(0xffffffffu, Ci, LPW);
    Xexc = __shfl_down_sync(0xffffffffu, Xi, LPW);
    if (s == NSEG - 1) {
        Cexc = 1.f;
        Xexc = 0.f;
    }
}

// Wordline pass over the CTA's rows (lines local to the CTA).
template <int LDM, int RES, bool NL>
__device__ __forceinline__ void cl_word_pass(float *__restrict__ U, const float *__restrict__ D,
                                             const float *__restrict__ Gs, const float *__restrict__ vin,
                                             const float *__restrict__ piv, const float *__restrict__ segprod,
                                             int nloc, int m, float gw, float omega, float &dmax, float &vmax,
                                             const SolveCtl &ctl) {
    constexpr int NSEG = CCfg<LDM>::NSEG_W, LPW = CCfg<LDM>::LPW_W, SEG = CL_SEG, S = CCfg<LDM>::S;
    const int tid = threadIdx.x, lane = tid & 31, s = lane / LPW;
    const int line = (tid >> 5) * LPW + (lane % LPW);
    const bool ok = line < nloc;
    const int p0 = s * SEG;
    const int base = line * S + p0 + s;  // node p0 + k sits at base + k
    float x[SEG];
    {
        const float vl = ok ? vin[line] : 0.f;
        float prev = (ok && p0 > 0 && p0 - 1 < m) ? U[base - 2] : 0.f;  // column p0 - 1 (previous pad group)
        float cur = (ok && p0 < m) ? U[base] : 0.f;
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            const int p = p0 + k;
            const float nxt = (ok && p + 1 < m) ? U[k + 1 < SEG ? base + k + 1 : base + SEG + 1] : 0.f;
            float r = 0.f;
            if (ok && p < m) {
                const float o = D[base + k];
                const float g = NL ? nl_geff(Gs[base + k], (cur + vl) - o, ctl) : Gs[base + k];
                r = line_residual<true, RES>(prev, cur, nxt, g, o, vl, true, p + 1 < m, gw);
            }
            x[k] = r;
            prev = cur;
            cur = nxt;
        }
    }
    float ip[SEG];
#pragma unroll
    for (int k = 0; k < SEG; ++k) ip[k] = piv[k * CL_T + tid];
    const float C = segprod[tid];
    float Y = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) Y = ip[k] * fmaf(gw, Y, x[k]);
    float Ci, Yi, Cx, Yx;
    scan_up<NSEG, LPW>(C, Y, s, Ci, Yi, Cx, Yx);
    float y = Yx;  // entering value 0 at the line start
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        y = ip[k] * fmaf(gw, y, x[k]);
        x[k] = y;
    }
    float X = 0.f;
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) X = fmaf(gw * ip[k], X, x[k]);
    float Cb, Xb, Cbx, Xbx;
    scan_down<NSEG, LPW>(C, X, s, Cb, Xb, Cbx, Xbx);
    X = Xbx;
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) {
        X = fmaf(gw * ip[k], X, x[k]);
        x[k] = X;
    }
    float dm = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        if (ok && p0 + k < m) {
            const float nv = fmaf(omega, x[k], U[base + k]);
            U[base + k] = nv;
            dm = fmaxf(dm, fabsf(x[k]));
            vmax = fmaxf(vmax, fabsf(nv));
        }
    }
    dmax = fmaxf(dmax, omega * dm);
}

// Bitline pass: columns cross the cluster.  Contains two cluster barriers.
template <int LDM, int RES, bool NL>
__device__ __forceinline__ void cl_bit_pass(cg::cluster_group &cluster, int rank, float *__restrict__ D,
                                            const float *__restrict__ U, const float *__restrict__ Gs,
                                            const float *__restrict__ vin, const float *__restrict__ piv,
                                            const float *__restrict__ segprod, const float *__restrict__ hup,
                                            const float *__restrict__ hdn, float *__restrict__ aggF,
                                            float *__restrict__ aggB, int row0, int nloc, int m, float gw,
                                            float omega, float &dmax, float &vmax, const SolveCtl &ctl) {
    constexpr int C = CCfg<LDM>::C, NSEG = CCfg<LDM>::NSEG_B, LPW = CCfg<LDM>::LPW_B, SEG = CL_SEG;
    constexpr int S = CCfg<LDM>::S;
    const int tid = threadIdx.x, lane = tid & 31, s = lane / LPW;
    const int col = (tid >> 5) * LPW + (lane % LPW);
    const bool ok = col < m;
    const int p0 = s * SEG;                 // first local row of the segment
    const int cb = col + (col >> 4);        // node (p0 + k) sits at (p0 + k) * S + cb
    float x[SEG];
    {
        float prev = (p0 > 0) ? ((ok && p0 - 1 < nloc) ? D[(p0 - 1) * S + cb] : 0.f) : (ok ? hup[col] : 0.f);
        float cur = (ok && p0 < nloc) ? D[p0 * S + cb] : 0.f;
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            const int lr = p0 + k;
            float nxt = 0.f;
            if (ok) nxt = (lr + 1 < nloc) ? D[(lr + 1) * S + cb] : hdn[col];
            float r = 0.f;
            if (ok && lr < nloc) {
                const float o = U[lr * S + cb];
                const float g = NL ? nl_geff(Gs[lr * S + cb], (o + vin[lr]) - cur, ctl) : Gs[lr * S + cb];
                r = line_residual<false, RES>(prev, cur, nxt, g, o, vin[lr], row0 + lr > 0, true, gw);
            }
            x[k] = r;
            prev = cur;
            cur = nxt;
        }
    }
    float ip[SEG];
#pragma unroll
    for (int k = 0; k < SEG; ++k) ip[k] = piv[k * CL_T + tid];
    const float Cs = segprod[tid];
    // ---- forward: fold, scan within the CTA, compose the CTAs above ---------
    float Y = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) Y = ip[k] * fmaf(gw, Y, x[k]);
    float Ci, Yi, Cx, Yx;
    scan_up<NSEG, LPW>(Cs, Y, s, Ci, Yi, Cx, Yx);
    if (s == NSEG - 1 && col < LDM) {
        aggF[2 * col] = Ci;
        aggF[2 * col + 1] = Yi;
    }
    cluster.sync();
    float yent = 0.f;
    if (s == 0 && col < LDM) {
        for (int r = 0; r < rank; ++r) {
            const float *agg = cluster.map_shared_rank(aggF, r);
            yent = fmaf(agg[2 * col], yent, agg[2 * col + 1]);
        }
    }
    yent = __shfl_sync(0xffffffffu, yent, lane % LPW);
    float y = fmaf(Cx, yent, Yx);
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        y = ip[k] * fmaf(gw, y, x[k]);
        x[k] = y;
    }
    // ---- backward: fold, scan within the CTA, compose the CTAs below --------
    float X = 0.f;
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) X = fmaf(gw * ip[k], X, x[k]);
    float Cb, Xb, Cbx, Xbx;
    scan_down<NSEG, LPW>(Cs, X, s, Cb, Xb, Cbx, Xbx);
    if (s == 0 && col < LDM) {
        aggB[2 * col] = Cb;
        aggB[2 * col + 1] = Xb;
    }
    cluster.sync();
    float xent = 0.f;
    if (s == 0 && col < LDM) {
        for (int r = C - 1; r > rank; --r) {
            const float *agg = cluster.map_shared_rank(aggB, r);
            xent = fmaf(agg[2 * col], xent, agg[2 * col + 1]);
        }
    }
    xent = __shfl_sync(0xffffffffu, xent, lane % LPW);
    X = fmaf(Cbx, xent, Xbx);
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) {
        X = fmaf(gw * ip[k], X, x[k]);
        x[k] = X;
    }
    float dm = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        const int lr = p0 + k;
        if (ok && lr < nloc) {
            const int q = lr * S + cb;
            const float nv = fmaf(omega, x[k], D[q]);
            D[q] = nv;
            dm = fmaxf(dm, fabsf(x[k]));
            vmax = fmaxf(vmax, fabsf(nv));
        }
    }
    dmax = fmaxf(dmax, omega * dm);
}

// Pivots of the CTA's wordline rows and of its part of every bitline column,
// written in the order the pass threads read them; uses aux as FP64 scratch.
template <int LDM>
__device__ void cl_pivots(cg::cluster_group &cluster, int rank, const float *__restrict__ Gs, float *__restrict__ piv,
                          double *__restrict__ mob, int row0, int nloc, int n, int m, float gwf) {
    constexpr int RPC = CCfg<LDM>::RPC, SEG = CL_SEG, LPW_W = CCfg<LDM>::LPW_W, LPW_B = CCfg<LDM>::LPW_B;
    const double gw = gwf, gw2 = (double)gwf * (double)gwf;
    const int tid = threadIdx.x;
    float *pivW = piv, *pivB = piv + SEG * CL_T, *prodW = piv + 2 * SEG * CL_T, *prodB = prodW + CL_T;
    const int jb = tid;  // bitline column handled by this thread (tid < LDM)
    // 1. wordline rows (threads LDM .. LDM+RPC-1) and each column's 2x2 product over the band
    if (tid >= LDM && tid < LDM + RPC) {
        const int lr = tid - LDM;
        const int tw_base = (lr / LPW_W) * 32 + (lr % LPW_W);
        double p = 1.0, ipp = 0.0;
        float sp = 1.f;
        for (int c = 0; c < LDM; ++c) {
            double ipv = 0.0;
            if (lr < nloc && c < m) {
                const double diag = gw + (c + 1 < m ? gw : 0.0) + (double)Gs[cidx<LDM>(lr, c)];
                p = (c == 0) ? diag : fma(-gw2, ipp, diag);
                const double r0 = (double)__frcp_rn((float)p);
                ipv = r0 * fma(-p, r0, 2.0);
                ipp = ipv;
            }
            const int tw = tw_base + (c / SEG) * LPW_W;
            const float f = (float)ipv;
            pivW[(c % SEG) * CL_T + tw] = f;
            sp *= gwf * f;
            if (c % SEG == SEG - 1) {
                prodW[tw] = sp;
                sp = 1.f;
            }
        }
    }
    if (tid < LDM) {
        // p_r = num/den with [num; den] <- [[diag_r, -gw^2], [1, 0]] [num; den]
        double a = 1, b = 0, c = 0, d = 1;  // band product, starts as identity
        if (jb < m) {
            for (int lr = 0; lr < nloc; ++lr) {
                const double diag = (row0 + lr > 0 ? gw : 0.0) + gw + (double)Gs[cidx<LDM>(lr, jb)];
                const double na = diag * a - gw2 * c, nb = diag * b - gw2 * d;
                c = a;
                d = b;
                a = na;
                b = nb;
                const double sc = 1.0 / fmax(fmax(fabs(a), fabs(b)), fmax(fabs(c), fabs(d)));
                a *= sc;
                b *= sc;
                c *= sc;
                d *= sc;
            }
        }
        mob[4 * jb + 0] = a;
        mob[4 * jb + 1] = b;
        mob[4 * jb + 2] = c;
        mob[4 * jb + 3] = d;
    }
    cluster.sync();
    if (tid < LDM) {
        // state entering this band: [1; 0] (no row above the first) through the bands above
        double num = 1.0, den = 0.0;
        for (int r = 0; r < rank; ++r) {
            const double *M = cluster.map_shared_rank(mob, r) + 4 * jb;
            const double nn = M[0] * num + M[1] * den, dd = M[2] * num + M[3] * den;
            const double sc = 1.0 / fmax(fabs(nn), fabs(dd));
            num = nn * sc;
            den = dd * sc;
        }
        const int tb_base = (jb / LPW_B) * 32 + (jb % LPW_B);
        double ipp = (rank > 0 && num != 0.0) ? den / num : 0.0;  // 1 / p of the row above the band
        float sp = 1.f;
        for (int lr = 0; lr < RPC; ++lr) {
            double ipv = 0.0;
            if (jb < m && lr < nloc) {
                const double diag = (row0 + lr > 0 ? gw : 0.0) + gw + (double)Gs[cidx<LDM>(lr, jb)];
                const double p = (row0 + lr == 0) ? diag : fma(-gw2, ipp, diag);
                const double r0 = (double)__frcp_rn((float)p);
                ipv = r0 * fma(-p, r0, 2.0);
                ipp = ipv;
            }
            const int tb = tb_base + (lr / SEG) * LPW_B;
            const float f = (float)ipv;
            pivB[(lr % SEG) * CL_T + tb] = f;
            sp *= gwf * f;
            if (lr % SEG == SEG - 1) {
                prodB[tb] = sp;
                sp = 1.f;
            }
        }
    }
    cluster.sync();  // the band products are read remotely until here
}

template <int LDM, typename TIO, bool NL>
__global__ void __launch_bounds__(CL_T, 1) line_relax_cluster_kernel(SolveArgs a) {
    constexpr int C = CCfg<LDM>::C, RPC = CCfg<LDM>::RPC, S = CCfg<LDM>::S, SEG = CL_SEG;
    constexpr int LPW_B = CCfg<LDM>::LPW_B, NSEG_B = CCfg<LDM>::NSEG_B;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    extern __shared__ float4 smem4[];
    float *Gs = reinterpret_cast<float *>(smem4);
    float *U = Gs + RPC * S;
    float *D = U + RPC * S;
    float *hup = D + RPC * S;
    float *hdn = hup + LDM;
    float *vin = hdn + LDM;
    float *aux = vin + RPC;  // 8 * LDM floats: 2x2 FP64 products, or aggF/aggB/partial currents
    float *red = aux + 8 * LDM;  // [2][2][CL_NW]
    float *cred = red + 4 * CL_NW;  // [2][2] this CTA's maxima, read by the cluster
    float *aggF = aux, *aggB = aux + 2 * LDM, *part = aux + 4 * LDM;
    __shared__ unsigned long long st_solves, st_iters;
    __shared__ int st_max, st_or, nonfinite_flag;

    const int tid = threadIdx.x;
    const int n = a.n, m = a.m, ldG = a.numY * m;
    const int row0 = rank * RPC;
    const int nloc = max(0, min(RPC, n - row0));
    const TIO *inp = static_cast<const TIO *>(a.input);
    const TIO *Gg = static_cast<const TIO *>(a.G);
    TIO *out = static_cast<TIO *>(a.out);
    float *piv = a.scratch + (size_t)blockIdx.x * (2 * SEG * CL_T + 2 * CL_T);
    const float gw = a.gw, tol = a.ctl.tol_v;
    const int kres = a.ctl.residual_period, maxit = a.ctl.max_iters;
    const bool ff = a.ctl.residual_ff != 0;
    const long long cid = blockIdx.x / C, ncl = gridDim.x / C;
    if (tid == 0) {
        st_solves = 0;
        st_iters = 0;
        st_max = 0;
        st_or = 0;
    }
    long long cached_tile = -1;
    float rate_hint = 0.f;  // final rate of the previous vector of this tile (cluster-uniform)
    for (long long item = cid; item < a.nitems; item += ncl) {
        const long long tile = item / a.nchunks;
        const int chunk = (int)(item % a.nchunks);
        const int x = (int)(tile / a.numY), y = (int)(tile % a.numY);
        const int b0 = chunk * a.vchunk, b1 = min(a.B, b0 + a.vchunk);
        if (tile != cached_tile) {
            __syncthreads();
            for (int e = tid; e < RPC * LDM; e += CL_T) {
                const int lr = e / LDM, c = e - lr * LDM;
                Gs[cidx<LDM>(lr, c)] =
                    (lr < nloc && c < m) ? (float)Gg[((size_t)x * n + row0 + lr) * ldG + (size_t)y * m + c] : 0.f;
            }
            __syncthreads();
            cl_pivots<LDM>(cluster, rank, Gs, piv, reinterpret_cast<double *>(aux), row0, nloc, n, m, gw);
            __syncthreads();
            if (NL) {
                for (int e = tid; e < RPC * LDM; e += CL_T) {
                    const int lr = e / LDM, c = e - lr * LDM;
                    Gs[cidx<LDM>(lr, c)] = nl_z(Gs[cidx<LDM>(lr, c)], a.ctl);
                }
                __syncthreads();
            }
            cached_tile = tile;
            rate_hint = 0.f;
        }
        for (int b = b0; b < b1; ++b) {
            __syncthreads();
            for (int e = tid; e < RPC * S; e += CL_T) {
                U[e] = 0.f;
                D[e] = 0.f;
            }
            if (tid < RPC) vin[tid] = (tid < nloc) ? (float)inp[((size_t)b * a.numX + x) * n + row0 + tid] : 0.f;
            __syncthreads();
            cluster.sync();  // every band initialised before halos are read
            LineStop stop;
            stop.init(a.ctl.omega, rate_hint);
            float omega = stop.omega;
            bool res64 = kres == 1;
            int status = 0, it = 0, par = 0;
            while (true) {
                float dmax = 0.f, vmax = 0.f;
                if (!res64) cl_word_pass<LDM, 0, NL>(U, D, Gs, vin, piv, piv + 2 * SEG * CL_T, nloc, m, gw, omega, dmax, vmax, a.ctl);
                else if (ff) cl_word_pass<LDM, 2, NL>(U, D, Gs, vin, piv, piv + 2 * SEG * CL_T, nloc, m, gw, omega, dmax, vmax, a.ctl);
                else cl_word_pass<LDM, 1, NL>(U, D, Gs, vin, piv, piv + 2 * SEG * CL_T, nloc, m, gw, omega, dmax, vmax, a.ctl);
                __syncthreads();
                if (tid < LDM) {
                    // halo rows: the row above the band and the row below it (0 V ground below the last row)
                    hup[tid] = (row0 > 0 && nloc > 0 && tid < m)
                                   ? cluster.map_shared_rank(D, rank - 1)[cidx<LDM>(RPC - 1, tid)]
                                   : 0.f;
                    hdn[tid] = (row0 + nloc < n && tid < m) ? cluster.map_shared_rank(D, rank + 1)[cidx<LDM>(0, tid)]
                                                            : 0.f;
                }
                __syncthreads();
                float *pB = piv + SEG * CL_T, *sB = piv + 2 * SEG * CL_T + CL_T;
                if (!res64)
                    cl_bit_pass<LDM, 0, NL>(cluster, rank, D, U, Gs, vin, pB, sB, hup, hdn, aggF, aggB, row0, nloc, m, gw,
                                        omega, dmax, vmax, a.ctl);
                else if (ff)
                    cl_bit_pass<LDM, 2, NL>(cluster, rank, D, U, Gs, vin, pB, sB, hup, hdn, aggF, aggB, row0, nloc, m, gw,
                                        omega, dmax, vmax, a.ctl);
                else
                    cl_bit_pass<LDM, 1, NL>(cluster, rank, D, U, Gs, vin, pB, sB, hup, hdn, aggF, aggB, row0, nloc, m, gw,
                                        omega, dmax, vmax, a.ctl);
                dmax = warp_max(dmax);
                vmax = warp_max(vmax);
                if ((tid & 31) == 0) {
                    red[(par * 2 + 0) * CL_NW + (tid >> 5)] = dmax;
                    red[(par * 2 + 1) * CL_NW + (tid >> 5)] = vmax;
                }
                __syncthreads();
                if (tid < 32) {
                    const float d0 = warp_max(red[(par * 2 + 0) * CL_NW + tid]);
                    const float v0 = warp_max(red[(par * 2 + 1) * CL_NW + tid]);
                    if (tid == 0) {
                        cred[par * 2 + 0] = d0;
                        cred[par * 2 + 1] = v0;
                    }
                }
                cluster.sync();
                // the same C values in the same order in every CTA: an identical decision
                float delta = 0.f, vm = 0.f;
                for (int r = 0; r < C; ++r) {
                    const float *cr = cluster.map_shared_rank(cred, r);
                    delta = fmaxf(delta, cr[par * 2 + 0]);
                    vm = fmaxf(vm, cr[par * 2 + 1]);
                }
                par ^= 1;
                ++it;
                const bool small = stop.update(delta, vm, tol);
                omega = stop.omega;
                if (small) {
                    if (res64 || kres < 0) {
                        status = FADESIM_ST_CONVERGED;
                        break;
                    }
                    res64 = true;
                } else {
                    res64 = kres > 0 ? (it % kres == 0) : (kres == 0 && stop.want_precise(tol, vm));
                }
                if (it >= maxit) {
                    status = FADESIM_ST_MAXITER;
                    break;
                }
            }
            rate_hint = stop.final_rate();
            // ---- outputs --------------------------------------------------------
            if (tid == 0) nonfinite_flag = 0;
            __syncthreads();
            if (a.ret_V) {
                for (int e = tid; e < nloc * m; e += CL_T) {
                    const int lr = e / m, j = e - lr * m;
                    const int q = cidx<LDM>(lr, j);
                    const TIO uu = (TIO)U[q] + (TIO)vin[lr];
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
                            const int q = cidx<LDM>(lr, j);
                            const float V = (U[q] + vin[lr]) - D[q];
                            float Ic = (NL ? nl_geff(Gs[q], V, a.ctl) : Gs[q]) * V;
                            if (a.ctl.noise_sigma > 0.f)
                                Ic *= 1.f + a.ctl.noise_sigma *
                                                normal_from(a.ctl.noise_seed,
                                                            ((unsigned long long)b * a.numX + x) * a.numY + y,
                                                            (unsigned long long)(row0 + lr) * m + j);
                            acc += Ic;
                        }
                    }
                }
#pragma unroll
                for (int off = LPW_B; off < 32; off <<= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
                if (s == 0 && j < LDM) part[j] = acc;
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
            if (nonfinite_flag) status |= FADESIM_ST_NONFINITE;
            if (tid == 0 && rank == 0) {
                if (a.iters_out) a.iters_out[((long long)b * a.numX + x) * a.numY + y] = it;
                st_solves += 1;
                st_iters += it;
                st_max = max(st_max, it);
                st_or |= status;
            }
        }
    }
    __syncthreads();
    cluster.sync();  // no CTA leaves while another may still read its shared memory
    if (tid == 0 && rank == 0 && a.stats && st_solves) {
        atomicAdd(&a.stats->solves, st_solves);
        atomicAdd(&a.stats->iters_sum, st_iters);
        atomicMax(&a.stats->iters_max, st_max);
        atomicOr(&a.stats->status_or, st_or);
    }
}

int cluster_relax_ld(int n, int m) {
    const int L = n > m ? n : m;
    if (L <= 128) return 0;
    if (L <= 256) return 256;
    if (L <= 512) return 512;
    return 0;
}

int cluster_relax_size(int ld) { return ld == 256 ? CCfg<256>::C : CCfg<512>::C; }

size_t cluster_relax_scratch_floats_per_cta(int) { return (size_t)2 * CL_SEG * CL_T + 2 * CL_T; }

template <int LDM, typename TIO>
static cudaError_t cl_launch_cfg(int *clusters, const SolveArgs *a, int grid, cudaStream_t st) {
    auto kern = (a && a->ctl.nl) ? line_relax_cluster_kernel<LDM, TIO, true> : line_relax_cluster_kernel<LDM, TIO, false>;
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

cudaError_t cluster_relax_occupancy(int ld, int dtype, int *clusters) {
    if (ld == 256) return dtype == FADESIM_F64 ? cl_launch_cfg<256, double>(clusters, nullptr, 0, 0)
                                               : cl_launch_cfg<256, float>(clusters, nullptr, 0, 0);
    if (ld == 512) return dtype == FADESIM_F64 ? cl_launch_cfg<512, double>(clusters, nullptr, 0, 0)
                                               : cl_launch_cfg<512, float>(clusters, nullptr, 0, 0);
    return cudaErrorInvalidValue;
}

cudaError_t launch_cluster_relax(const SolveArgs &a, int ld, int dtype, int grid, cudaStream_t st) {
    if (ld == 256) return dtype == FADESIM_F64 ? cl_launch_cfg<256, double>(nullptr, &a, grid, st)
                                               : cl_launch_cfg<256, float>(nullptr, &a, grid, st);
    if (ld == 512) return dtype == FADESIM_F64 ? cl_launch_cfg<512, double>(nullptr, &a, grid, st)
                                               : cl_launch_cfg<512, float>(nullptr, &a, grid, st);
    return cudaErrorInvalidValue;
}

}  // namespace fadesim
