// Shared helpers for the fadesim_gb300 CUDA kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fadesim_gb300.h"

namespace fadesim {

// Device-side accumulators for fadesim_solve_stats (one per call).
struct DevStats {
    unsigned long long solves;
    unsigned long long iters_sum;
    int iters_max;
    int status_or;
    unsigned long long queue_head;  // next work item of the call's queue (persistent kernels claim items)
    unsigned long long warm_rejected;  // solves whose warm start was discarded
};

// Solver controls shared by the converging kernels.
struct SolveCtl {
    float tol_v;          // target max node error (V)
    int max_iters;        // iteration / sweep cap
    int residual_period;  // precise residual every k iterations (<0: never)
    float omega;          // <= 0: adaptive
    int residual_ff;      // precise residual in float-float (FP32 pipe) instead of FP64
    float precise_margin; // adaptive schedule: precise when the predicted estimate is within this factor of tol
    // sinh cells (nonlinear_params = [R_on, R_off, a_on, b_on, a_off, b_off])
    int nl;
    float nl_R_on, nl_inv_dR;        // z = (1/g_lin - R_on) / (R_off - R_on), clamped at 0
    float nl_a_on, nl_a_off;         // a of I = b sinh(a V)
    float nl_r0_on, nl_r0_off;       // 1 / (a b): the state's resistance at V -> 0
    int nl_single_a;                 // a_on == a_off: g(V) = g(0) sinh(a V) / (a V) for every cell
    // additive read noise on every cell current: N(0, (sigma I_cell)^2)
    float noise_sigma;
    unsigned long long noise_seed;
};

// One element of an FP32 or FP64 input array, as FP32.
__device__ __forceinline__ float load_io(const void *p, size_t i, bool f64) {
    return f64 ? (float)static_cast<const double *>(p)[i] : static_cast<const float *>(p)[i];
}

// Input voltage i of a solve in the output type: the FP64 input unrounded when
// both the input and the outputs are FP64 (the solve itself runs on the FP32
// copy; its node deviations change by ~1e-7 of themselves with that rounding,
// while the rounding of the wordline voltage itself, up to 6e-8 V per volt,
// would otherwise reach every node of the row unchanged).
template <typename TIO>
__device__ __forceinline__ TIO vin_exact(const void *p, size_t i, bool f64, float staged) {
    if constexpr (sizeof(TIO) == 8) {
        if (f64) return static_cast<const double *>(p)[i];
    }
    return (TIO)staged;
}

// sinh(t)/t, t >= 0.  Below t = 1 its Maclaurin series sum_k t^(2k) / (2k+1)!
// in Horner form in u = t^2, through t^12 / 13! (the first omitted term,
// t^14 / 15! < 8e-13, is far below FP32 resolution); above, sinhf(t) / t.
// Cell voltages of a read stay well under 1 / a, so the series is the path.
__device__ __forceinline__ float sinhc(float t) {
    if (t < 1.f) {
        const float u = t * t;
        float p = 1.f / 6227020800.f;        // 1 / 13!
        p = fmaf(p, u, 1.f / 39916800.f);    // 1 / 11!
        p = fmaf(p, u, 1.f / 362880.f);      // 1 / 9!
        p = fmaf(p, u, 1.f / 5040.f);        // 1 / 7!
        p = fmaf(p, u, 1.f / 120.f);         // 1 / 5!
        p = fmaf(p, u, 1.f / 6.f);           // 1 / 3!
        return fmaf(p, u, 1.f);
    }
    return sinhf(t) / t;
}

// sinhc as a real call: the line kernels evaluate it once per node of a fully
// unrolled 32-node segment, for two passes and up to three residual forms, and
// inlined copies of the series push the sinh-cell kernels' code past the
// instruction caches (38% of the 512 x 512 kernel's stall samples waited for
// instructions; one shared copy: 41.5k -> 51.3k solves/s).
static __device__ __noinline__ float sinhc_call(float t) { return sinhc(t); }

// Chord conductance I(V)/V of the reference's sinh cell at cell voltage V for
// a cell at position z between the on and off states:
// 1/R(V), R(V) = (1-z) |V| / (b_on sinh(a_on |V|)) + z |V| / (b_off sinh(a_off |V|)),
// i.e. with s = sinh(a x) / (a x) and r0 = 1 / (a b):  R = (1-z) r0_on / s_on + z r0_off / s_off,
// evaluated as s_on s_off / ((1-z) r0_on s_off + z r0_off s_on) -- one division.
__device__ __forceinline__ float nl_geff(float z, float V, const SolveCtl &c) {
    const float x = fabsf(V);
    const float s_on = sinhc_call(c.nl_a_on * x), s_off = sinhc_call(c.nl_a_off * x);
    return __fdividef(s_on * s_off, fmaf((1.f - z) * c.nl_r0_on, s_off, z * c.nl_r0_off * s_on));
}

__device__ __forceinline__ float nl_z(float g, const SolveCtl &c) {
    return g > 0.f ? fmaxf(0.f, (1.f / g - c.nl_R_on) * c.nl_inv_dR) : 0.f;
}

// What the line kernels keep per sinh cell, from its linear conductance g:
// its position z -- or, when both states share a (nl_single_a), its V -> 0
// conductance over gw, 1 / (gw ((1-z) r0_on + z r0_off)): then the chord
// conductance is that times sinh(a|V|) / (a|V|), with no division per use.
__device__ __forceinline__ float nl_cell(float g, const SolveCtl &c, float inv_gw) {
    const float z = nl_z(g, c);
    return c.nl_single_a ? inv_gw / fmaf(1.f - z, c.nl_r0_on, z * c.nl_r0_off) : z;
}

// Chord conductance over gw at cell voltage V, from the value nl_cell keeps.
__device__ __forceinline__ float nl_gs(float cell, float V, const SolveCtl &c, float inv_gw) {
    return c.nl_single_a ? cell * sinhc_call(c.nl_a_on * fabsf(V)) : nl_geff(cell, V, c) * inv_gw;
}

// Chord conductance at cell voltage V, from the value nl_cell keeps.
__device__ __forceinline__ float nl_g(float cell, float V, const SolveCtl &c, float gw) {
    return c.nl_single_a ? (cell * gw) * sinhc(c.nl_a_on * fabsf(V)) : nl_geff(cell, V, c);
}

// Second counter of the cycle-to-cycle variation draws (normal_from(seed, cell,
// kVariationStream)); the read noise uses (seed, solve, cell of a tile < 2^18),
// so the two streams never share a counter pair.
constexpr unsigned long long kVariationStream = 0x7661726961ull;

// Standard normal from a counter (splitmix64 hash, Box-Muller): the same value
// for the same (seed, a, b) on every run and every device.
__device__ __forceinline__ float normal_from(unsigned long long seed, unsigned long long a, unsigned long long b) {
    unsigned long long zz = seed + 0x9E3779B97F4A7C15ull * (a * 0x100000001B3ull + b + 1ull);
    zz = (zz ^ (zz >> 30)) * 0xBF58476D1CE4E5B9ull;
    zz = (zz ^ (zz >> 27)) * 0x94D049BB133111EBull;
    zz ^= zz >> 31;
    const float u1 = ((float)(unsigned int)(zz >> 40) + 0.5f) * (1.f / 16777216.f);   // (0, 1)
    const float u2 = (float)(unsigned int)(zz & 0xffffffu) * (1.f / 16777216.f);      // [0, 1)
    return sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void record_solve(DevStats *st, int *iters_out, long long solve_idx, int iters,
                                             int status) {
    if (iters_out) iters_out[solve_idx] = iters;
    if (st) {
        atomicAdd(&st->solves, 1ull);
        atomicAdd(&st->iters_sum, (unsigned long long)iters);
        atomicMax(&st->iters_max, iters);
        atomicOr(&st->status_or, status);
    }
}

template <typename T>
__device__ __forceinline__ float to_f(T v) { return (float)v; }

}  // namespace fadesim
