// Device helpers shared by the line-relaxation kernels.
#pragma once
#include <cuda_runtime.h>

namespace fadesim {

// Knuth's error-free sum: s + e == a + b exactly (round-to-nearest).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// float -> double on the integer pipe (exact for normal numbers, zero, inf and
// NaN; FP32 subnormals, which the solve never produces, widen to ~2^-127).
__device__ __forceinline__ double widen_f64(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int mag = b & 0x7fffffffu;
    unsigned int hi;
    if (mag == 0u) hi = b;                                                // signed zero
    else if (mag >= 0x7f800000u) hi = (b & 0x80000000u) | 0x7ff00000u | (mag & 0x007fffffu) >> 3 | (mag > 0x7f800000u ? 0x00080000u : 0u);
    else hi = (b & 0x80000000u) | ((mag >> 3) + (896u << 20));
    return __hiloint2double((int)hi, (int)((b & 7u) << 29));
}

// One step of a line's pivot recurrence in units of gw, in float-float:
//   P = D - 1 / P_prev (P = D on the first node),  D = base + gs,
// base the node's link count (1 or 2) and gs = g / gw ~1e-6 of it, so D and P
// need more than FP32 (FP64-class precision on the FP32 pipe).  (rh, rl) holds
// 1 / P_prev on entry and 1 / P on return: the correctly rounded FP32
// reciprocal corrected by one float-float step.  Returns the chain multiplier
// gw / pivot = 1 / P rounded to FP32.
__device__ __forceinline__ float ff_pivot_step(float base, float gs, bool first, float &rh, float &rl) {
    float dh, dl;
    two_sum(base, gs, dh, dl);
    float ph = dh, pl = dl;
    if (!first) {
        float sh, sl;
        two_sum(dh, -rh, sh, sl);
        sl = __fadd_rn(sl, __fsub_rn(dl, rl));
        ph = __fadd_rn(sh, sl);
        pl = __fsub_rn(sl, __fsub_rn(ph, sh));
    }
    const float r = __frcp_rn(ph);
    float e = __fmaf_rn(-ph, r, 1.f);  // exact: 1 - ph * RN(1/ph)
    e = __fmaf_rn(-pl, r, e);
    rh = r;
    rl = __fmul_rn(e, r);
    return __fadd_rn(rh, rl);
}

// The line part of a residual, (prev - cur) [if has_l] + (nxt - cur) [if has_r],
// as hi + lo with hi + lo equal to it up to one rounding of the low part:
// (prev + nxt) exactly by TwoSum, then minus k cur (k = 1 or 2 links, exact
// scaling) by a second TwoSum -- two error-free sums where the differences
// taken one by one need three.
__device__ __forceinline__ void lap_exact(float prev, float cur, float nxt, bool has_l, bool has_r, float &hi,
                                          float &lo) {
    float sh, sl, th, tl;
    two_sum(has_l ? prev : 0.f, has_r ? nxt : 0.f, sh, sl);
    two_sum(sh, -((has_l && has_r) ? 2.f * cur : (has_l || has_r ? cur : 0.f)), th, tl);
    hi = th;
    lo = __fadd_rn(tl, sl);
}

// Residual of one node's line equation at the current iterate, divided by gw
// (volts), with gs = g / gw:
//   r' = hl (prev - cur) + hr (nxt - cur) + gs src,  hl, hr in {0, 1},
//   src = (o - vin) - cur on a wordline (o = bitline node, cur = u - vin),
//   src = (o + vin) - cur on a bitline (o = wordline deviation, cur = d);
// unknowns are deviations from the ideal state, so every difference is
// between nearby values.
// Solving T' d = r' with T' = T / gw gives the same correction without a
// multiply by gw per node; the line kernels store gs and the multipliers
// gw / pivot.  RES 0 FP32, 1 FP64, 2 float-float, 3 float-float line
// differences with an FP32 cell term.
template <bool WORD, int RES>
__device__ __forceinline__ float line_residual_s(float prev, float cur, float nxt, float gs, float o, float vin,
                                                 bool has_l, bool has_r) {
    if (RES == 1) {
        const double dp = widen_f64(prev), dc = widen_f64(cur), dn = widen_f64(nxt);
        const double src = WORD ? (widen_f64(o) - widen_f64(vin)) - dc : (widen_f64(o) + widen_f64(vin)) - dc;
        const double lap = (has_l ? dp - dc : 0.0) + (has_r ? dn - dc : 0.0);  // exact: widened FP32 inputs
        return __double2float_rn(fma(widen_f64(gs), src, lap));
    } else if (RES == 2) {
        float sh, sl, th, tl, lh;
        two_sum(o, WORD ? -vin : vin, sh, sl);           // o -/+ vin
        two_sum(sh, -cur, th, tl);                        // ... - own
        float lap_lo;
        lap_exact(prev, cur, nxt, has_l, has_r, lh, lap_lo);
        const float src_lo = __fadd_rn(tl, sl);
        const float ph = __fmul_rn(gs, th), pl = __fmaf_rn(gs, th, -ph);
        float rh, rl;
        two_sum(lh, ph, rh, rl);
        const float lo = __fadd_rn(__fadd_rn(rl, __fadd_rn(lap_lo, pl)), __fmul_rn(gs, src_lo));
        return __fadd_rn(rh, lo);
    } else if (RES == 3) {
        // the line differences exactly (their rounding dominates when the wire
        // carries a large gradient), the cell term in FP32: for tiles whose cell
        // term is small enough that its rounding stays far below the tolerance
        float lh, lap_lo;
        lap_exact(prev, cur, nxt, has_l, has_r, lh, lap_lo);
        const float src = WORD ? (o - vin) - cur : (o + vin) - cur;
        return __fadd_rn(lh, __fmaf_rn(gs, src, lap_lo));
    } else {
        const float src = WORD ? (o - vin) - cur : (o + vin) - cur;
        const float lap = (has_l ? prev - cur : 0.f) + (has_r ? nxt - cur : 0.f);
        return fmaf(gs, src, lap);
    }
}

}  // namespace fadesim

namespace fadesim {

// Stop test and relaxation factor of the line iteration, evaluated identically
// by every thread (and every CTA of a cluster) from the same per-iteration
// maxima.  delta = largest correction of the iteration, vm = largest deviation.
//   error estimate  delta * rho / (1 - rho), rho the larger of the last ratio,
//                   the 3-iteration geometric rate and omega - 1, and at least
//                   1/2 once over-relaxed (SOR modes oscillate: a single small
//                   correction can hide an error several times larger);
//   floor           4 ulps of the largest deviation (FP32 resolution);
//   relaxation      block Gauss-Seidel for 3 iterations, then
//                   omega = 2 / (1 + sqrt(1 - rho_GS)) (Young, 2-block
//                   partition), refined at iteration 12 from the observed SOR
//                   rate lambda via mu^2 = (lambda + omega - 1)^2 / (lambda omega^2);
//                   a vector after the first of a tile takes, at iteration 3,
//                   the final omega of the previous one instead (same matrix:
//                   the early rates underestimate rho_GS, the refined omega
//                   does not).
//   precision       (adaptive schedule) the next iteration's residual is made
//                   precise when it is expected to be the last one -- its
//                   predicted estimate delta * rho * rho / (1 - rho) within 4x
//                   of the tolerance --, when the corrections have come within
//                   ~1000 ulps of the largest deviation (where FP32 residual
//                   noise can dominate), or when they stall (no 10% progress in
//                   an iteration).  Before a rate has been observed,
//                   rho is the first observed rate (delta_2 / delta_1) of the
//                   previous vector of the same tile (hint), or unknown: the
//                   rate of the first step, larger than the later ones, is
//                   what the first prediction needs.
// (The per-iteration quotients use the fast division: the estimates need a
// few digits, and every thread evaluates them after every iteration.)
struct LineStop {
    float omega;
    bool adapt;
    int it;
    float h0, h1, h2, h3;  // delta of this and the 3 previous iterations
    float rho;             // rate used by the last update (0: unknown)
    float hint;            // rate carried from the previous vector of the tile (0: none)
    float first;           // delta_2 / delta_1 of this solve (0: not yet)
    float omega_hint;      // final omega of the previous vector of the tile (<= 1: none)

    __device__ __forceinline__ void init(float omega_fixed, float rate_hint = 0.f, float omega_prev = 0.f) {
        adapt = !(omega_fixed > 0.f);
        omega_hint = omega_prev;
        omega = adapt ? 1.f : omega_fixed;
        it = 0;
        h0 = h1 = h2 = h3 = 0.f;
        hint = rate_hint;
        rho = rate_hint;
        first = 0.f;
    }

    // Whether the next iteration should compute its residual precisely.
    // margin: how far above the tolerance a predicted estimate may be and the
    // iteration still be made precise (4 by default).
    __device__ __forceinline__ bool want_precise(float tol, float vm, float margin = 4.f) const {
        if (it == 0 || !(rho > 0.f)) return false;
        const float r = fminf(rho, 0.999f);
        const float next = h0 * r;
        const float est_next = __fdividef(next * r, 1.f - r);
        const float floor_v = 4.f * 1.1920929e-07f * vm;
        return est_next <= margin * fmaxf(tol, floor_v) || h0 <= 1e-4f * vm || (it >= 3 && h0 >= 0.9f * h1);
    }

    // First-step rate of the finished solve, to seed the next vector of the tile.
    __device__ __forceinline__ float final_rate() const { return first > 0.f ? first : hint; }

    // FLOOR: rho taken at least rho_floor (the two-level method); there, with
    // fp32_limit, the floor does not end the iteration: it runs until the
    // corrections stop shrinking (under 15% progress over three iterations)
    // below it, or the estimate meets the tolerance.
    template <bool FLOOR = false>
    __device__ __forceinline__ bool update(float delta, float vm, float tol, float rho_floor = 0.f,
                                           bool fp32_limit = false) {
        ++it;
        const float prev = h0;
        h3 = h2;
        h2 = h1;
        h1 = h0;
        h0 = delta;
        if (it == 1) return delta <= 0.f;
        const float floor_v = 4.f * 1.1920929e-07f * vm;
        const float ratio = prev > 0.f ? __fdividef(delta, prev) : 0.f;
        const float rate3 = (it >= 4 && h3 > 0.f) ? cbrtf(delta / h3) : 0.f;
        rho = fmaxf(fmaxf(ratio, rate3), omega - 1.f);
        if (omega > 1.f) rho = fmaxf(rho, 0.5f);
        if (FLOOR) rho = fmaxf(rho, rho_floor);
        if (it == 2) first = ratio;
        const float est = rho < 0.999f ? __fdividef(delta * rho, 1.f - rho) : INFINITY;
        const bool stalled = delta <= floor_v && ratio >= 0.9f;
        if (adapt) {
            if (it == 3 && omega_hint > 1.f) {
                omega = omega_hint;
            } else if (it == 3 && ratio > 0.05f && ratio < 1.f) {
                omega = fminf(1.95f, 2.f / (1.f + sqrtf(1.f - ratio)));
            } else if (it == 12 && omega > 1.f && rate3 > omega - 1.f + 0.02f && rate3 < 1.f) {
                const float mu2 = (rate3 + omega - 1.f) * (rate3 + omega - 1.f) / (rate3 * omega * omega);
                if (mu2 < 1.f) {
                    const float w2 = 2.f / (1.f + sqrtf(1.f - mu2));
                    if (w2 > omega + 0.01f) omega = fminf(1.95f, w2);
                }
            }
        }
        if (FLOOR && fp32_limit) return est <= tol || (delta <= floor_v && it >= 4 && delta >= 0.85f * h3);
        return est <= fmaxf(tol, floor_v) || stalled;
    }
};

}  // namespace fadesim
