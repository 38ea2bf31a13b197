// Block line relaxation for the crossbar nodal system (sm_103a).
//
// The reference relaxes one node at a time (split_arr_matmul.cu:27-119,
// crossbarHspice/2dArray.cc:1551-1590).  Its two planes are coupled only
// through the cell conductance, which is 1e-6..1e-3 of the wire conductance,
// so the natural blocks are whole lines: every wordline row is a tridiagonal
// system in its own unknowns once the bitline plane is fixed, and every
// bitline column is one once the wordline plane is fixed.  One iteration here
// solves all wordlines exactly, then all bitlines exactly (block Gauss-Seidel,
// optionally over-relaxed).  It converges to the same fixed point as the
// reference's point sweeps: the nodal solution.
//
// Numerics.  Unknowns are deviations from the ideal state (wordline u - vin,
// bitline d), so FP32 resolves ~1e-9 V.  Each line solve is a correction
// x += omega * T^-1 r with r the line's residual computed from differences of
// neighbouring values (FP32, or precise -- float-float or FP64 -- on the
// iterations an adaptive schedule or residual_period picks, and always for the
// final convergence test) and T the line's tridiagonal matrix factored
// once per tile (float-float pivots rounded to FP32).  Forming T's diagonal in FP32
// loses the cell term, so a direct (non-residual) FP32 line solve would stall
// near 1e-5 V; in residual form that rounding only slows convergence.
//
// Mapping.  One CTA owns one tile at a time and solves its input vectors one
// after another with the tile's conductances and both deviation planes in
// shared memory (3 x LD x LD floats).  A warp handles 8 lines x 4 segments of
// SEG = LD/4 nodes; a thread keeps its segment in registers, folds the Thomas
// recurrences locally and joins segments with a 2-step affine scan over the
// 4 lanes of its line (__shfl at stride 8).  Planes are stored row-major with
// an XOR swizzle so that both the row walk (wordline pass) and the column walk
// (bitline pass) hit 32 distinct banks.
//
// This header holds the kernel templates; linegs_32.cu, linegs_64.cu and
// linegs_128.cu instantiate one tile size each (parallel compilation), and
// linegs.cu dispatches between them.  Input and output types (FP32 or FP64)
// are a run-time property of the launch: only the load and store code differs.
#pragma once
#include <math.h>

#include "coarse_impl.cuh"
#include "kernels.h"
#include "line_common.cuh"

namespace fadesim {

// Per-size launch shape.  A warp holds LPW lines x NSEG segments of SEG nodes;
// T threads cover all LD lines of one pass with one segment each.
template <int LD>
struct LineCfg;
template <>
struct LineCfg<128> {
    static constexpr int NSEG = 4, SEG = 32, LPW = 8, T = 512, NW = 16, MINB = 1;
};
template <>
struct LineCfg<64> {
    static constexpr int NSEG = 4, SEG = 16, LPW = 8, T = 256, NW = 8, MINB = 3;
};
template <>
struct LineCfg<32> {
    static constexpr int NSEG = 4, SEG = 8, LPW = 8, T = 128, NW = 4, MINB = 8;
};

// Node (r, c) of an LD x LD plane in shared memory.  The XOR term touches only
// the low 5 bits of c and depends on c only through c >> 5, so it permutes
// every 32-column block of a row.  For each size it is chosen so that both
// walks -- LPW rows x NSEG segments at one step of the wordline pass, LPW
// columns x NSEG segments at one step of the bitline pass -- hit 32 distinct
// banks (checked exhaustively when the layouts were designed).
template <int LD>
__device__ __forceinline__ int swz(int r, int c) {
    int x;
    if (LD == 128) x = (r & 7) | ((((c >> 5) ^ (r >> 5)) & 3) << 3);
    else if (LD == 64) x = (r & 7) | (((((c >> 5) & 1) ^ ((r >> 4) & 1))) << 3) | (((r >> 5) & 1) << 4);
    else x = r & 31;
    return r * LD + (c ^ x);
}

// Input voltages in shared memory, one pad word per 16 rows: the bitline pass
// reads rows 16s + k for NSEG segments s at once, which would otherwise share banks.
__device__ __forceinline__ int vpad(int p) { return p + (p >> 4); }

// One pass over all lines of one plane.  WORD: wordline rows (own plane = U
// deviations, other = D); else bitline columns (own = D, other = U).
// FULL: an LD x LD tile, every line and node present (the bounds tests fold away).
// Gs holds g / gw (linear cells) or the sinh cells' positions z (NL); cm the
// chain multipliers gw / pivot; the pass solves T' d = r' (both divided by gw).
// ZOWN / ZOTH: the own / other plane is known to be zero (the first iteration
// from the ideal state): its loads are skipped and the planes need no clearing.
// UNIT: instead, the response of every line to its own cell conductances,
// T'^-1 (g / gw), written to own[k * T + tid] in the pass threads' order (the
// first wordline pass from the ideal state is -vin times it, linear cells).
// RST (bitline pass of a full 128 x 128 tile, linear cells): also restrict the
// wordline residual the correction leaves, g / gw times it, onto the coarse
// grid of the two-level method (accumulated into crs).
template <int LD, bool WORD, int RES, bool NL, bool FULL, bool ZOWN, bool ZOTH, bool UNIT = false, bool RST = false>
__device__ __forceinline__ void line_pass(float *__restrict__ own, const float *__restrict__ oth,
                                          const float *__restrict__ Gs, const float *__restrict__ vin_s,
                                          const float *__restrict__ cm, const float *__restrict__ segprod,
                                          int L_in, int NLINES_in, float inv_gw, float omega, float &dmax, float &vmax,
                                          const SolveCtl &ctl, float *__restrict__ crs = nullptr) {
    static_assert(!RST || (LD == 128 && !WORD && !NL && FULL && !UNIT), "coarse restriction: 128 bitline pass");
    const int L = FULL ? LD : L_in;
    const int NLINES = FULL ? LD : NLINES_in;
    constexpr int SEG = LineCfg<LD>::SEG;
    constexpr int T = LineCfg<LD>::T;
    constexpr int LPW = LineCfg<LD>::LPW;
    constexpr int NSEG = LineCfg<LD>::NSEG;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int s = lane / LPW;
    const int line = (tid >> 5) * LPW + (lane % LPW);
    const bool line_ok = FULL || line < NLINES;
    const int p0 = s * SEG;
    auto at = [&](int p) { return WORD ? swz<LD>(line, p) : swz<LD>(p, line); };
    // Addresses of this segment's nodes.  The swizzle term is constant along a
    // wordline segment, so node k sits at Bw ^ k; along a bitline segment it
    // depends on k only through k % V, so node k sits at Rb[k % V] + k * LD
    // (an immediate offset from one of V registers).
    constexpr int V = 8;
    const int Bw = swz<LD>(line & (LD - 1), p0);
    int Rb[V];
#pragma unroll
    for (int t = 0; t < V; ++t) Rb[t] = swz<LD>(p0 + t, line & (LD - 1)) - t * LD;
    auto qk = [&](int k) { return WORD ? (Bw ^ k) : (Rb[k % V] + k * LD); };

    float x[SEG];
    // ---- residual of the line equations at the current iterate -------------
    // WORD: left link always present (the source at p == 0, deviation 0), right
    //       link absent at the open end.
    // BIT:  upper link absent at the open top, lower link always present
    //       (ground below the last node, deviation 0).
    if constexpr (UNIT) {
#pragma unroll
        for (int k = 0; k < SEG; ++k) x[k] = (FULL || (line_ok && p0 + k < L)) ? Gs[qk(k)] : 0.f;
    } else {
        const float vl = (WORD && line_ok) ? vin_s[vpad(line)] : 0.f;
        float prev = (!ZOWN && line_ok && p0 > 0 && (FULL || p0 - 1 < L)) ? own[at(p0 - 1)] : 0.f;
        float cur = (!ZOWN && line_ok && (FULL || p0 < L)) ? own[at(p0)] : 0.f;
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            const int p = p0 + k;
            const bool valid = FULL || (line_ok && p < L);
            const bool has_next = (FULL && k + 1 < SEG) || (line_ok && p + 1 < L);
            const float nxt = (!ZOWN && has_next) ? own[k + 1 < SEG ? qk(k + 1) : at(p + 1)] : 0.f;
            float r = 0.f;
            if (valid) {
                const int q = qk(k);
                const float o = ZOTH ? 0.f : oth[q], vv = WORD ? vl : vin_s[vpad(p)];
                // g / gw: stored, or the sinh cell's at the present cell voltage
                const float gs =
                    NL ? nl_gs(Gs[q], WORD ? (cur + vv) - o : (o + vv) - cur, ctl, inv_gw) : Gs[q];
                const bool has_l = WORD || k > 0 || p0 > 0;
                const bool has_r = !WORD || (FULL && k + 1 < SEG) || p + 1 < L;
                r = line_residual_s<WORD, RES>(prev, cur, nxt, gs, o, vv, has_l, has_r);
            }
            x[k] = r;
            prev = cur;
            cur = nxt;
        }
    }
    // ---- T'^-1 r' by Thomas, segmented over NSEG lanes ----------------------
    // With c_p = gw / pivot_p:  y_p = c_p r'_p + c_p y_{p-1},  d_p = y_p + c_p d_{p+1}.
    // A segment maps its incoming value v to (prod_seg c) v + (result with
    // v = 0); the product is a tile constant (segprod).  Padding nodes carry
    // c = 0 and r' = 0, which breaks both chains at the line end; the first
    // segment's incoming y and the last segment's incoming d are zero.
    float c[SEG];
#pragma unroll
    for (int k = 0; k < SEG; ++k) c[k] = cm[k * T + tid];
    const float C = segprod[tid];
    float Y = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        x[k] *= c[k];
        Y = fmaf(c[k], Y, x[k]);
    }
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
    float y = __shfl_up_sync(0xffffffffu, Yi, LPW);
    if (s == 0) y = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        y = fmaf(c[k], y, x[k]);
        x[k] = y;
    }
    float X = 0.f;
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) X = fmaf(c[k], X, x[k]);
    Ci = C;
    float Xi = X;
#pragma unroll
    for (int off = 1; off < NSEG; off <<= 1) {
        const float Cn = __shfl_down_sync(0xffffffffu, Ci, LPW * off);
        const float Xn = __shfl_down_sync(0xffffffffu, Xi, LPW * off);
        if (s + off < NSEG) {
            Xi = fmaf(Ci, Xn, Xi);
            Ci *= Cn;
        }
    }
    X = __shfl_down_sync(0xffffffffu, Xi, LPW);
    if (s == NSEG - 1) X = 0.f;
#pragma unroll
    for (int k = SEG - 1; k >= 0; --k) {
        X = fmaf(c[k], X, x[k]);
        x[k] = X;
    }
    if constexpr (UNIT) {
#pragma unroll
        for (int k = 0; k < SEG; ++k) own[k * T + tid] = x[k];
        return;
    }
    // ---- apply the correction ----------------------------------------------
    // (a NaN correction is not seen by fmaxf; the output stage flags it)
    float dm = 0.f;
    float S[COARSE_SLOTS];
    if constexpr (RST) {
#pragma unroll
        for (int a = 0; a < COARSE_SLOTS; ++a) S[a] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        const int p = p0 + k;
        if (FULL || (line_ok && p < L)) {
            const int q = qk(k);
            const float nv = ZOWN ? omega * x[k] : fmaf(omega, x[k], own[q]);
            own[q] = nv;
            dm = fmaxf(dm, fabsf(x[k]));
            vmax = fmaxf(vmax, fabsf(nv));
            if constexpr (RST) {
                const float r = Gs[q] * (omega * x[k]);
                const float t = coarse_t(k);
                S[coarse_lo_slot(k)] = fmaf(1.f - t, r, S[coarse_lo_slot(k)]);
                S[coarse_lo_slot(k) + 1] = fmaf(t, r, S[coarse_lo_slot(k) + 1]);
                // hand each slot on as soon as it is complete (fewer live registers)
                if (coarse_slot_done_after(k)) coarse_restrict_slot(S[k >> 3], k >> 3, crs, line, s);
            }
        }
    }
    dmax = fmaxf(dmax, omega * dm);
    if constexpr (RST) {
        coarse_restrict_slot(S[4], 4, crs, line, s);
        coarse_restrict_slot(S[5], 5, crs, line, s);
    }
}

// The coarse correction of the two-level method added to both planes: node
// (i, j) gets sum_I sum_J phi_I(i) phi_J(j) E[I][J] (E in shared memory, row
// stride COARSE_EST), threads in the bitline pass's layout.  Returns the
// thread's largest |correction|.
template <int LD>
__device__ __forceinline__ float line_coarse_apply(float *__restrict__ U, float *__restrict__ D,
                                                   const float *__restrict__ E) {
    static_assert(LD == 128, "the coarse correction is built for 128 x 128 tiles");
    constexpr int SEG = LineCfg<LD>::SEG;
    constexpr int LPW = LineCfg<LD>::LPW;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int s = lane / LPW;
    const int line = (tid >> 5) * LPW + (lane % LPW);
    const int p0 = s * SEG;
    constexpr int V = 8;
    int Rb[V];
#pragma unroll
    for (int t = 0; t < V; ++t) Rb[t] = swz<LD>(p0 + t, line) - t * LD;
    // the bitline's column weights, then its values on the segment's six coarse rows
    const int l = line & 7, w = line >> 3;
    const float tj = l < 4 ? ((float)l + 4.5f) * 0.125f : ((float)l - 3.5f) * 0.125f;
    const int J0 = coarse_clamp(l < 4 ? w - 1 : w), J1 = coarse_clamp(l < 4 ? w : w + 1);
    float Ej[COARSE_SLOTS];
#pragma unroll
    for (int a = 0; a < COARSE_SLOTS; ++a) {
        const int I = coarse_clamp(4 * s - 1 + a);
        Ej[a] = fmaf(1.f - tj, E[I * COARSE_EST + J0], tj * E[I * COARSE_EST + J1]);
    }
    float pm = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        const float t = coarse_t(k);
        const float pe = fmaf(1.f - t, Ej[coarse_lo_slot(k)], t * Ej[coarse_lo_slot(k) + 1]);
        const int q = Rb[k % V] + k * LD;
        U[q] += pe;
        D[q] += pe;
        pm = fmaxf(pm, fabsf(pe));
    }
    return pm;
}

// Chain multipliers gw / pivot of every line of the tile, written in the order
// each pass thread reads them (k * T + tid), and the product of each segment's
// multipliers as the pass forms it.  In units of gw the pivots follow
//   P_0 = D_0,  P_q = D_q - 1 / P_(q-1),  D_q = (1 or 2) + g_q / gw,  c_q = 1 / P_q,
// and g / gw is ~1e-6 of the link terms, so D and P are carried in float-float
// (ff_pivot_step) -- FP64 precision on the FP32 pipe: the FP64 pipe of this
// part is slow, and this recurrence is serial.  Matches an FP64 evaluation of
// the same recurrence to 1 ulp of the FP32 multipliers.
template <int LD>
__device__ void line_pivots(const float *__restrict__ Gs, float *__restrict__ piv, int n, int m, float gw) {
    constexpr int SEG = LineCfg<LD>::SEG;
    constexpr int T = LineCfg<LD>::T;
    constexpr int LPW = LineCfg<LD>::LPW;
    const int tid = threadIdx.x;
    if (tid < 2 * LD) {
        const bool word = tid < LD;
        const int line = word ? tid : tid - LD;
        const int L = word ? m : n;
        const int NL = word ? n : m;
        float *dst = word ? piv : piv + SEG * T;
        float *prod = piv + 2 * SEG * T + (word ? 0 : T);
        const int tw_base = (line / LPW) * 32 + (line % LPW);
        float rh = 0.f, rl = 0.f;  // 1 / P_(q-1) in float-float
        float seg_prod = 1.f;
        for (int q = 0; q < LD; ++q) {
            float cf = 0.f;
            if (line < NL && q < L) {
                const float gs = __fdiv_rn(word ? Gs[swz<LD>(line, q)] : Gs[swz<LD>(q, line)], gw);
                // wordline: source link + right link (absent at the end) + cell
                // bitline:  upper link (absent at the top) + lower link + cell
                const float base = word ? (q + 1 < L ? 2.f : 1.f) : (q > 0 ? 2.f : 1.f);
                cf = ff_pivot_step(base, gs, q == 0, rh, rl);
            }
            const int tw = tw_base + (q / SEG) * LPW;
            dst[(q % SEG) * T + tw] = cf;
            seg_prod *= cf;
            if (q % SEG == SEG - 1) {
                prod[tw] = seg_prod;
                seg_prod = 1.f;
            }
        }
    }
}

// The first wordline pass from the ideal state with linear cells: its
// residual is -vin g / gw on every node, so its correction is -vin times the
// tile's unit response w1 (line_pass UNIT) -- one load and a multiply per node
// instead of a residual and a Thomas solve.
template <int LD, bool FULL>
__device__ __forceinline__ void line_word_zero_unit(float *__restrict__ U, const float *__restrict__ vin_s,
                                                    const float *__restrict__ w1, int L_in, int NLINES_in,
                                                    float omega, float &dmax, float &vmax) {
    const int L = FULL ? LD : L_in;
    const int NLINES = FULL ? LD : NLINES_in;
    constexpr int SEG = LineCfg<LD>::SEG;
    constexpr int T = LineCfg<LD>::T;
    constexpr int LPW = LineCfg<LD>::LPW;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int s = lane / LPW;
    const int line = (tid >> 5) * LPW + (lane % LPW);
    const bool line_ok = FULL || line < NLINES;
    const int p0 = s * SEG;
    const int Bw = swz<LD>(line & (LD - 1), p0);
    const float sc = line_ok ? -vin_s[vpad(line)] : 0.f;
    float dm = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
        if (FULL || (line_ok && p0 + k < L)) {
            const float xk = sc * w1[k * T + tid];
            const float nv = omega * xk;
            U[Bw ^ k] = nv;
            dm = fmaxf(dm, fabsf(xk));
            vmax = fmaxf(vmax, fabsf(nv));
        }
    }
    dmax = fmaxf(dmax, omega * dm);
}

// Whether the first wordline pass uses the unit response: measured +7.7% on
// 64 x 64 tiles, -1.4% on 128 x 128 (the 128 kernel's registers are full and
// the extra path makes it spill), so 32 and 64 only.
template <int LD>
__host__ __device__ constexpr bool unit_first() { return LD < 128; }

// One iteration: every wordline, then every bitline.  ZERO: both planes are
// still zero (first iteration from the ideal state).
template <int LD, int RES, bool NL, bool FULL, bool ZERO, bool RST = false>
__device__ __forceinline__ void line_iteration(float *U, float *D, const float *Gs, const float *vin_s,
                                               const float *piv, int n, int m, float inv_gw, float omega,
                                               float &dmax, float &vmax, const SolveCtl &ctl, float *crs = nullptr) {
    constexpr int SEG = LineCfg<LD>::SEG;
    constexpr int T = LineCfg<LD>::T;
    if constexpr (ZERO && !NL && unit_first<LD>())
        line_word_zero_unit<LD, FULL>(U, vin_s, piv + 2 * SEG * T + 2 * T, m, n, omega, dmax, vmax);
    else
        line_pass<LD, true, RES, NL, FULL, ZERO, ZERO>(U, D, Gs, vin_s, piv, piv + 2 * SEG * T, m, n, inv_gw, omega,
                                                       dmax, vmax, ctl);
    __syncthreads();
    line_pass<LD, false, RES, NL, FULL, ZERO, false, false, RST>(D, U, Gs, vin_s, piv + SEG * T,
                                                                 piv + 2 * SEG * T + T, n, m, inv_gw, omega, dmax,
                                                                 vmax, ctl, crs);
}

// Largest of one value per thread, the same in every thread (two barriers).
template <int NW>
__device__ __forceinline__ float block_max(float v, float *scratch) {
    v = warp_max(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
    __syncthreads();
    return warp_max((threadIdx.x & 31) < NW ? scratch[threadIdx.x & 31] : 0.f);
}

// Outputs of one solve: both planes or cell voltages (ret_V), else the bitline
// currents I_j = sum_i g_ij (u_ij - d_ij) in the bitline mapping, in the I/O type.
template <int LD, typename TIO, bool NL>
__device__ __forceinline__ void line_outputs(const SolveArgs &a, const float *Gs, const float *U, const float *D,
                                             const float *vin_s, int n, int m, int b, int x, int y, float gw,
                                             int &nonfinite_flag) {
    constexpr int T = LineCfg<LD>::T;
    constexpr int SEG = LineCfg<LD>::SEG;
    const int tid = threadIdx.x;
    TIO *out = static_cast<TIO *>(a.out);
    const int ldG = a.numY * m;
    if (a.ret_V) {
        for (int e = tid; e < n * m; e += T) {
            const int i = e / m, j = e - i * m;
            const int q = swz<LD>(i, j);
            const TIO uu =
                (TIO)U[q] + vin_exact<TIO>(a.input, ((size_t)b * a.numX + x) * n + i, a.f64, vin_s[vpad(i)]);
            const size_t sol = ((size_t)b * a.numX + x) * a.numY + y;
            if (!isfinite((float)uu) || !isfinite(D[q])) nonfinite_flag = 1;
            if (a.ret_V == 2) {
                out[(sol * 2 + 0) * n * m + (size_t)i * m + j] = uu;
                out[(sol * 2 + 1) * n * m + (size_t)i * m + j] = (TIO)D[q];
            } else {
                out[(sol * n + i) * m + j] = uu - (TIO)D[q];
            }
        }
    } else {
        constexpr int LPW = LineCfg<LD>::LPW;
        const int lane = tid & 31;
        const int s = lane / LPW;
        const int j = (tid >> 5) * LPW + (lane % LPW);
        TIO acc = 0;
        if (j < m) {
            for (int k = 0; k < SEG; ++k) {
                const int i = s * SEG + k;
                if (i < n) {
                    const int q = swz<LD>(i, j);
                    const TIO V =
                        ((TIO)U[q] + vin_exact<TIO>(a.input, ((size_t)b * a.numX + x) * n + i, a.f64,
                                                    vin_s[vpad(i)])) - (TIO)D[q];
                    TIO Ic = (TIO)(NL ? nl_g(Gs[q], (float)V, a.ctl, gw) : Gs[q] * gw) * V;
                    if (a.ctl.noise_sigma > 0.f)
                        Ic *= (TIO)1 + (TIO)(a.ctl.noise_sigma *
                                             normal_from(a.ctl.noise_seed,
                                                         ((unsigned long long)b * a.numX + x) * a.numY + y,
                                                         (unsigned long long)i * m + j));
                    acc += Ic;
                }
            }
        }
#pragma unroll
        for (int off = LPW; off < 32; off <<= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (s == 0 && j < m) out[((size_t)b * a.numX + x) * ldG + (size_t)y * m + j] = acc;
        if (s == 0 && j < m && !isfinite((float)acc)) nonfinite_flag = 1;
    }
}

// TWO: the two-level method (coarse correction after every iteration) on the
// tiles whose cells couple the planes strongly (sum of g / gw over the tile at
// least 3); full 128 x 128 tiles with linear cells.
template <int LD, bool NL, bool FULL, bool TWO = false>
__global__ void __launch_bounds__(LineCfg<LD>::T, LineCfg<LD>::MINB) line_relax_kernel(SolveArgs a) {
    static_assert(!TWO || (LD == 128 && !NL && FULL), "the two-level method is built for full 128 x 128 tiles");
    constexpr int T = LineCfg<LD>::T;
    constexpr int NW = LineCfg<LD>::NW;
    constexpr int SEG = LineCfg<LD>::SEG;
    constexpr int NRED = TWO ? 3 : 2;  // per-warp maxima: correction, deviation (, coarse correction)
    extern __shared__ float4 smem4[];
    float *Gs = reinterpret_cast<float *>(smem4);
    float *U = Gs + LD * LD;
    float *D = U + LD * LD;
    float *vin_s = D + LD * LD;
    float *red = vin_s + LD + LD / 16;  // [2][NRED][NW]
    float *coarse_s = red + 2 * NRED * NW;  // TWO: the coarse step's tables and buffers
    __shared__ int nonfinite_flag;
    __shared__ float bmax_scratch[NW];

    const int tid = threadIdx.x;
    const int n = FULL ? LD : a.n, m = FULL ? LD : a.m;
    const int ldG = a.numY * m;
    const bool f64 = a.f64 != 0;
    // per CTA: the chain multipliers of both passes, their segment products and
    // (32 and 64 layouts) the wordline unit response of linear cells
    float *piv = a.scratch + (size_t)blockIdx.x * ((unit_first<LD>() ? 3 : 2) * SEG * T + 2 * T);
    const float gw = a.gw;
    const float inv_gw = 1.f / gw;
    const float tol = a.ctl.tol_v;
    const int kres = a.ctl.residual_period;
    const int maxit = a.ctl.max_iters;
    const bool ff = a.ctl.residual_ff != 0;  // precise residual in float-float instead of FP64
    const bool precise_first = kres == 1;    // every iteration precise
    long long cached_tile = -1;
    float rate_hint = 0.f;                   // final rate of the previous vector of this tile
    float omega_prev = 0.f;                  // final relaxation factor of that vector
    float gs_max = 0.f;                      // largest g / gw of the tile (linear cells)
    __shared__ unsigned long long st_solves, st_iters, st_rej;  // this CTA's counters (thread 0)
    __shared__ int st_max, st_or;
    if (tid == 0) {
        st_solves = 0;
        st_iters = 0;
        st_rej = 0;
        st_max = 0;
        st_or = 0;
        nonfinite_flag = 0;
    }
    bool two_tile = false;  // TWO: this tile takes the coarse correction
    if constexpr (TWO) coarse_load_tables(coarse_s);  // (the first claim's barrier orders it)

    // work queue: every CTA claims its next (tile, vector chunk) item from the
    // call's counter, so CTAs that finish early take more items
    __shared__ long long s_item;
    long long next_static = blockIdx.x;
    auto claim = [&]() -> long long {
        __syncthreads();  // every thread has read the previous claim
        if (tid == 0) {
            if (a.stats) {
                s_item = (long long)atomicAdd(&a.stats->queue_head, 1ull);
            } else {
                s_item = next_static;
                next_static += gridDim.x;
            }
        }
        __syncthreads();
        return s_item;
    };
    for (long long item = claim(); item < a.nitems; item = claim()) {
        const long long tile = item / a.nchunks;
        const int chunk = (int)(item % a.nchunks);
        const int x = (int)(tile / a.numY), y = (int)(tile % a.numY);
        const int b0 = chunk * a.vchunk;
        const int b1 = min(a.B, b0 + a.vchunk);
        if (tile != cached_tile) {
            __syncthreads();
            for (int e = tid; e < n * m; e += T) {
                const int i = e / m, j = e - i * m;
                Gs[swz<LD>(i, j)] = load_io(a.G, ((size_t)x * n + i) * ldG + (size_t)y * m + j, f64);
            }
            __syncthreads();
            line_pivots<LD>(Gs, piv, n, m, gw);
            __syncthreads();
            if (!NL) {
                // the passes work in units of gw: g / gw
                float gm = 0.f;
                for (int e = tid; e < n * m; e += T) {
                    const int i = e / m, j = e - i * m;
                    const float gsv = __fdiv_rn(Gs[swz<LD>(i, j)], gw);
                    Gs[swz<LD>(i, j)] = gsv;
                    gm = fmaxf(gm, fabsf(gsv));
                }
                gs_max = block_max<NW>(gm, bmax_scratch);
                if constexpr (TWO) {
                    // coupling strength: the sum of g / gw over the tile (mean g / gw times
                    // the square of the line length); the coarse correction pays from ~3
                    float gsum = 0.f;
                    for (int e = tid; e < n * m; e += T) gsum += Gs[swz<LD>(e / m, e - (e / m) * m)];
                    gsum = warp_sum(gsum);
                    __syncthreads();
                    if ((tid & 31) == 0) bmax_scratch[tid >> 5] = gsum;
                    __syncthreads();
                    two_tile = warp_sum((tid & 31) < NW ? bmax_scratch[tid & 31] : 0.f) >= 3.f;
                }
                if constexpr (unit_first<LD>()) {
                    // the wordline unit response w1 = T'^-1 (g / gw) of every row (each
                    // thread writes and later reads only its own entries)
                    float dn0 = 0.f, dn1 = 0.f;
                    line_pass<LD, true, 0, false, FULL, true, true, true>(piv + 2 * SEG * T + 2 * T, nullptr, Gs,
                                                                          vin_s, piv, piv + 2 * SEG * T, m, n, inv_gw,
                                                                          1.f, dn0, dn1, a.ctl);
                }
            }
            if (NL) {
                // the sinh cells keep their on/off position; the linear values served the pivots
                for (int e = tid; e < n * m; e += T) {
                    const int i = e / m, j = e - i * m;
                    Gs[swz<LD>(i, j)] = nl_cell(Gs[swz<LD>(i, j)], a.ctl, inv_gw);
                }
                __syncthreads();
            }
            cached_tile = tile;
            rate_hint = 0.f;
            omega_prev = 0.f;
        }
        for (int b = b0; b < b1; ++b) {
            // (the tile setup and the previous solve's outputs end with a barrier)
            // warm start: initial deviation planes [2][n][m] of this solve.  From
            // the ideal state the planes are zero: the first iteration is then a
            // ZERO iteration that reads neither plane, unless every iteration must
            // be precise (the planes are cleared instead).
            bool warm = a.init != nullptr;
            bool zero = !warm && !precise_first;
            if (!warm && precise_first) {
                for (int e = tid; e < LD * LD; e += T) {
                    U[e] = 0.f;
                    D[e] = 0.f;
                }
            }
            if (tid < LD)
                vin_s[vpad(tid)] = (tid < n) ? load_io(a.input, ((size_t)b * a.numX + x) * n + tid, f64) : 0.f;
            if constexpr (TWO) {
                // no coarse correction precedes the first iteration
                if (tid < 256) CoarseSmem(coarse_s).R[tid] = 0.f;
                if (tid < NW) red[2 * NW + tid] = red[(NRED + 2) * NW + tid] = 0.f;
            }
            __syncthreads();
            // precise iterations may keep the cell term in FP32 (RES 3) when its
            // rounding, amplified by at most L^2/2 through a line solve, stays 8x
            // under the tolerance: per node <= gs_max * 3 vin_max * 2^-23.  Every
            // warp takes the largest input from the shared copy itself, before
            // the first iteration only when that one is precise (otherwise after
            // its reduction barrier, where the warps wait anyway).
            auto semi_now = [&]() {
                float vmx = 0.f;
                for (int i = tid & 31; i < n; i += 32) vmx = fmaxf(vmx, fabsf(vin_s[vpad(i)]));
                const float Lmax = (float)max(n, m);
                return !NL && ff && gs_max * 3.f * warp_max(vmx) * 1.1920929e-07f * 0.5f * Lmax * Lmax <= 0.125f * tol;
            };
            bool semi = precise_first ? semi_now() : false;
            if (warm) {
                const float *w0 = a.init + (((size_t)b * a.numX + x) * a.numY + y) * 2 * n * m;
                for (int e = tid; e < n * m; e += T) {
                    const int i = e / m, j = e - i * m;
                    U[swz<LD>(i, j)] = w0[e];
                    D[swz<LD>(i, j)] = w0[(size_t)n * m + e];
                }
                __syncthreads();
            }
            // (the two-level method runs at omega 1: its error is no SOR mode)
            LineStop stop;
            stop.init((TWO && two_tile) ? 1.f : a.ctl.omega, rate_hint, omega_prev);
            float omega = stop.omega, omega_last = omega;
            bool res64 = precise_first;
            int status = 0, it = 0, par = 0;
            while (true) {
                float dmax = 0.f, vmax = 0.f;
                omega_last = omega;
                // (TWO: the bitline pass restricts the residual only on the tiles that
                // take the coarse correction; the others run the plain passes)
                float *crs = TWO ? CoarseSmem(coarse_s).R : nullptr;
                if (TWO && two_tile) {
                    if (zero) line_iteration<LD, 0, NL, FULL, true, TWO>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl, crs);
                    else if (!res64) line_iteration<LD, 0, NL, FULL, false, TWO>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl, crs);
                    else if (semi) line_iteration<LD, 3, NL, FULL, false, TWO>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl, crs);
                    else if (ff) line_iteration<LD, 2, NL, FULL, false, TWO>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl, crs);
                    else line_iteration<LD, 1, NL, FULL, false, TWO>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl, crs);
                } else {
                    if (zero) line_iteration<LD, 0, NL, FULL, true>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl);
                    else if (!res64) line_iteration<LD, 0, NL, FULL, false>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl);
                    else if (semi) line_iteration<LD, 3, NL, FULL, false>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl);
                    else if (ff) line_iteration<LD, 2, NL, FULL, false>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl);
                    else line_iteration<LD, 1, NL, FULL, false>(U, D, Gs, vin_s, piv, n, m, inv_gw, omega, dmax, vmax, a.ctl);
                }
                zero = false;
                dmax = warp_max(dmax);
                vmax = warp_max(vmax);
                if ((tid & 31) == 0) {
                    red[(par * NRED + 0) * NW + (tid >> 5)] = dmax;
                    red[(par * NRED + 1) * NW + (tid >> 5)] = vmax;
                }
                __syncthreads();
                // every warp reduces the NW partial maxima itself (no second barrier)
                const int ln = tid & 31;
                float delta = warp_max(ln < NW ? red[(par * NRED + 0) * NW + ln] : 0.f);
                float vm = warp_max(ln < NW ? red[(par * NRED + 1) * NW + ln] : 0.f);
                // the two-level method's step is the fine corrections plus the
                // coarse correction before them (its per-warp maxima, or zeros)
                if constexpr (TWO) delta += warp_max(ln < NW ? red[(par * NRED + 2) * NW + ln] : 0.f);
                if (it == 0 && !precise_first) semi = semi_now();
                par ^= 1;
                ++it;
                if (!isfinite(delta) || !isfinite(vm)) {
                    status |= FADESIM_ST_NONFINITE;
                    break;
                }
                if (warm && it == 1 && !(delta < vm)) {
                    // the prediction moved as much as the solution is large: discard
                    // it and start again from the ideal state
                    __syncthreads();
                    if constexpr (TWO) {
                        if (tid < 256) CoarseSmem(coarse_s).R[tid] = 0.f;
                        if (tid < NW) red[2 * NW + tid] = red[(NRED + 2) * NW + tid] = 0.f;
                    }
                    if (precise_first) {
                        for (int e = tid; e < LD * LD; e += T) {
                            U[e] = 0.f;
                            D[e] = 0.f;
                        }
                        __syncthreads();
                    }
                    zero = !precise_first;
                    warm = false;
                    status |= FADESIM_ST_WARM_REJECTED;
                    stop.init((TWO && two_tile) ? 1.f : a.ctl.omega, rate_hint, omega_prev);
                    omega = stop.omega;
                    res64 = precise_first;
                    continue;
                }
                // (two-level: the rate taken at least 0.2 -- its steps shrink by
                // ~0.1 per iteration, and a single small one can hide a larger error)
                bool small;
                if constexpr (TWO) small = stop.update<true>(delta, vm, tol, two_tile ? 0.2f : 0.f, a.fp32_limit != 0);
                else small = stop.update(delta, vm, tol);
                omega = stop.omega;
                if (small) {
                    // the final test must pass on an iteration whose residual was
                    // FP64 (kres < 0: FP32 only, the FP32 test is final)
                    if (res64 || kres < 0) {
                        status |= FADESIM_ST_CONVERGED;
                        break;
                    }
                    res64 = true;
                } else {
                    // kres 0: adaptive (precise when the next iteration should be
                    // the last or nears the FP32 residual noise); k > 0: every k
                    res64 = kres > 0 ? (it % kres == 0) : (kres == 0 && stop.want_precise(tol, vm, a.ctl.precise_margin));
                }
                if (it >= maxit) {
                    status |= FADESIM_ST_MAXITER;
                    break;
                }
                if constexpr (TWO) {
                    // another iteration follows: correct the smooth, plane-locked error
                    // on the coarse grid first (the reduction barrier completed R)
                    const CoarseSmem cc(coarse_s);
                    if (two_tile) {
                        coarse_solve(cc);
                        // its largest value joins the next iteration's step (par: that
                        // iteration's slots, read two iterations ago)
                        const float pm = warp_max(line_coarse_apply<LD>(U, D, cc.E));
                        if ((tid & 31) == 0) red[(par * NRED + 2) * NW + (tid >> 5)] = pm;
                        __syncthreads();
                    }
                }
            }
            rate_hint = stop.final_rate();
            omega_prev = stop.omega;
            // ---- outputs (the planes are complete: the last reduction barrier) --
            if (!NL && !a.ret_V && !(a.ctl.noise_sigma > 0.f) && omega_last == 1.f) {
                // After a bitline pass at omega 1 every bitline equation holds, and
                // summed down a column they telescope to
                //   sum_i g_ij (u_ij - d_ij) = gw d_(n-1)j :
                // the column current is the current through its last wire segment
                // to ground (to the FP32 rounding of that node, ~1e-7 relative).
                for (int j = tid; j < m; j += T) {
                    const float dl = D[swz<LD>(n - 1, j)];
                    const size_t o = ((size_t)b * a.numX + x) * ldG + (size_t)y * m + j;
                    if (f64) static_cast<double *>(a.out)[o] = (double)gw * (double)dl;
                    else static_cast<float *>(a.out)[o] = gw * dl;
                    if (!isfinite(dl)) nonfinite_flag = 1;
                }
            } else if (f64) {
                line_outputs<LD, double, NL>(a, Gs, U, D, vin_s, n, m, b, x, y, gw, nonfinite_flag);
            } else {
                line_outputs<LD, float, NL>(a, Gs, U, D, vin_s, n, m, b, x, y, gw, nonfinite_flag);
            }
            __syncthreads();
            if (tid == 0) {
                if (nonfinite_flag) status |= FADESIM_ST_NONFINITE;
                nonfinite_flag = 0;
                if (a.iters_out) a.iters_out[((long long)b * a.numX + x) * a.numY + y] = it;
                st_solves += 1;
                st_iters += it;
                st_max = max(st_max, it);
                st_or |= status;
                if (status & FADESIM_ST_WARM_REJECTED) st_rej += 1;
            }
        }
    }
    __syncthreads();
    if (tid == 0 && a.stats && st_solves) {
        atomicAdd(&a.stats->solves, st_solves);
        atomicAdd(&a.stats->iters_sum, st_iters);
        atomicMax(&a.stats->iters_max, st_max);
        atomicOr(&a.stats->status_or, st_or);
        if (st_rej) atomicAdd(&a.stats->warm_rejected, st_rej);
    }
}

// Launch helpers for one tile size (instantiated by linegs_<LD>.cu).
// Instantiations: linear cells on any tile, linear cells on a full LD x LD
// tile, sinh cells on any tile; for LD 128 also the two-level kernel on a full
// tile of linear cells (linegs_128c.cu).
inline size_t line_relax_smem_ld(int ld, int nw) { return (size_t)(3 * ld * ld + ld + ld / 16 + 4 * nw) * sizeof(float); }
// the two-level kernel: a third per-warp maximum and the coarse step's buffers
inline size_t line_relax_smem_two(int ld, int nw) {
    return line_relax_smem_ld(ld, nw) + (size_t)(2 * nw + COARSE_SMEM_FLOATS) * sizeof(float);
}
// The two-level kernel on full 128 x 128 tiles with linear cells (linegs_128c.cu).
cudaError_t line_relax_prepare_128_coarse();
cudaError_t launch_line_relax_128_coarse(const SolveArgs &a, int grid, cudaStream_t st);

template <int LD>
cudaError_t line_relax_prepare_t() {
    const int sm = (int)line_relax_smem_ld(LD, LineCfg<LD>::NW);
    cudaError_t e = cudaFuncSetAttribute(line_relax_kernel<LD, false, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(line_relax_kernel<LD, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(line_relax_kernel<LD, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if constexpr (LD == 128) {
        if (e == cudaSuccess) e = line_relax_prepare_128_coarse();
    }
    return e;
}

template <int LD>
cudaError_t line_relax_occupancy_t(int *n) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, line_relax_kernel<LD, false, false>, LineCfg<LD>::T,
                                                         line_relax_smem_ld(LD, LineCfg<LD>::NW));
}

template <int LD>
cudaError_t launch_line_relax_t(const SolveArgs &a, int grid, cudaStream_t st) {
    const size_t sm = line_relax_smem_ld(LD, LineCfg<LD>::NW);
    if constexpr (LD == 128) {
        if (!a.ctl.nl && a.two_level && a.n == LD && a.m == LD) return launch_line_relax_128_coarse(a, grid, st);
    }
    if (a.ctl.nl) line_relax_kernel<LD, true, false><<<grid, LineCfg<LD>::T, sm, st>>>(a);
    else if (a.n == LD && a.m == LD) line_relax_kernel<LD, false, true><<<grid, LineCfg<LD>::T, sm, st>>>(a);
    else line_relax_kernel<LD, false, false><<<grid, LineCfg<LD>::T, sm, st>>>(a);
    return cudaGetLastError();
}

}  // namespace fadesim
