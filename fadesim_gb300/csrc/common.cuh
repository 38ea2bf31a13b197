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
};

// Solver controls shared by the converging kernels.
struct SolveCtl {
    float tol_v;          // target max node error (V)
    int max_iters;        // iteration / sweep cap
    int residual_period;  // precise residual every k iterations (<0: never)
    float omega;          // <= 0: adaptive
    int residual_ff;      // precise residual in float-float (FP32 pipe) instead of FP64
};

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
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
