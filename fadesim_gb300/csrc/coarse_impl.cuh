// Coarse correction of the two-level block line relaxation (128 x 128 tiles).
//
// With strong cells (1 kOhm on 128-node lines) the line iteration converges
// slowly: the slow error is smooth and nearly equal on the wordline and the
// bitline plane (the cells lock them together).  After every iteration the
// two-level method removes that part on a 16 x 16 coarse grid: with the same
// bilinear interpolation Phi for both planes, P = [Phi; Phi], the correction
// is e = P A_c^-1 P^T r, where A_c = P^T A P holds only the wires (the cell
// terms cancel for u = d) and is solved through the separable factors of
// coarse_tables.h (fadesim_gb300/coarse_tables.py).  r is the residual after
// the bitline pass: at omega 1 the bitline equations hold and the wordline
// residual is g / gw times the bitline correction, so the bitline pass itself
// restricts it (coarse_restrict) and no extra residual pass is needed.
//
// Fine node i of a line (c = 8 nodes per coarse cell) sits at coarse position
// f = (i + 1/2) / 8 - 1/2 between coarse nodes floor(f) and floor(f) + 1
// (weights 1 - t and t, t = f - floor(f)), clamped to the grid at both ends.
// A bitline segment of the 128 layout (32 rows from 32 s) meets the six
// coarse rows 4 s - 1 .. 4 s + 4 (slots 0..5); a warp's eight bitlines
// 8 w .. 8 w + 7 meet coarse columns w - 1, w, w + 1.
#pragma once
#include <cuda_runtime.h>

#include "coarse_tables.h"

namespace fadesim {

constexpr int COARSE_SLOTS = 6;   // coarse rows one 32-row segment meets
constexpr int COARSE_EST = 17;    // row stride of the correction in shared memory (bank spread)
// shared floats of the coarse step: Zr, Zc, Zc^T, lr, lc, the accumulated
// restriction, two products and the correction (stride 17)
constexpr int COARSE_SMEM_FLOATS = 3 * 256 + 2 * 16 + 256 + 2 * 256 + 16 * COARSE_EST;

// Slot (0..5) of the lower coarse row of node k of a segment, and the weight
// t of the upper one (compile-time for unrolled k).
__host__ __device__ constexpr int coarse_lo_slot(int k) { return (k & 7) < 4 ? (k >> 3) : (k >> 3) + 1; }
__host__ __device__ constexpr float coarse_t(int k) {
    return (k & 7) < 4 ? ((float)(k & 7) + 4.5f) * 0.125f : ((float)(k & 7) - 3.5f) * 0.125f;
}

__device__ __forceinline__ int coarse_clamp(int I) { return I < 0 ? 0 : (I > COARSE_N - 1 ? COARSE_N - 1 : I); }

// Load the factor tables into shared memory (Zc also transposed).
__device__ __forceinline__ void coarse_load_tables(float *cs) {
    for (int e = threadIdx.x; e < 256; e += blockDim.x) {
        cs[e] = coarse_table_128[e];                       // Zr[K][a]
        cs[256 + e] = coarse_table_128[256 + e];           // Zc[K][b]
        cs[512 + (e & 15) * 16 + (e >> 4)] = coarse_table_128[256 + e];  // Zc^T[b][K]
    }
    for (int e = threadIdx.x; e < 32; e += blockDim.x) cs[768 + e] = coarse_table_128[512 + e];  // lr, lc
}

// Pointers into the coarse step's shared memory.
struct CoarseSmem {
    float *Zr, *Zc, *ZcT, *lr, *lc, *R, *T1, *T2, *E;
    __device__ __forceinline__ explicit CoarseSmem(float *cs)
        : Zr(cs), Zc(cs + 256), ZcT(cs + 512), lr(cs + 768), lc(cs + 784), R(cs + 800), T1(cs + 1056),
          T2(cs + 1312), E(cs + 1568) {}
};

// Slot a of a segment receives nodes 8 (a - 2) + 4 .. 8 a + 3: it is complete
// after node 8 a + 3 (slots 4 and 5 after the last node).
__host__ __device__ constexpr bool coarse_slot_done_after(int k) { return (k & 7) == 3 && (k >> 3) < 4; }

// Restriction of one coarse row slot of a bitline segment (the sum Sa of its
// nodes' residual contributions, already weighted by the row interpolation)
// onto the coarse grid: the column weights of the lane's bitline, a sum over
// the warp's eight bitlines of the same segment, and shared atomics into R
// (zeroed before the pass).  Every lane of the warp calls it.
__device__ __forceinline__ void coarse_restrict_slot(float Sa, int a, float *R, int line, int s) {
    const int l = line & 7;           // lane's bitline within its coarse half-cells
    const int w = line >> 3;          // coarse column of the warp's bitlines
    const float t = l < 4 ? ((float)l + 4.5f) * 0.125f : ((float)l - 3.5f) * 0.125f;
    // lanes l < 4 feed columns (w - 1, w), lanes l >= 4 (w, w + 1)
    float mid = (l < 4 ? t : 1.f - t) * Sa;
    float side = (l < 4 ? 1.f - t : t) * Sa;
    mid += __shfl_xor_sync(0xffffffffu, mid, 1);
    side += __shfl_xor_sync(0xffffffffu, side, 1);
    mid += __shfl_xor_sync(0xffffffffu, mid, 2);
    side += __shfl_xor_sync(0xffffffffu, side, 2);
    mid += __shfl_xor_sync(0xffffffffu, mid, 4);
    const int I = coarse_clamp(4 * s - 1 + a);
    if (l == 0) {
        atomicAdd(&R[I * 16 + w], mid);
        atomicAdd(&R[I * 16 + coarse_clamp(w - 1)], side);
    } else if (l == 4) {
        atomicAdd(&R[I * 16 + coarse_clamp(w + 1)], side);
    }
}

// E = Zr ((Zr^T R Zc) / (lr_a + lc_b)) Zc^T with all threads of the CTA (two
// per entry, each summing alternate terms); R is cleared for the next
// restriction.  Starts after a barrier that completed R; ends with one.
__device__ __forceinline__ void coarse_solve(const CoarseSmem &c) {
    const int tid = threadIdx.x;
    const int p = tid >> 1, h = tid & 1;  // entry (p >> 4, p & 15), half h
    const int I = p >> 4, J = p & 15;
    const bool act = p < 256;
    float acc = 0.f;
    if (act) {
#pragma unroll
        for (int q = 0; q < 8; ++q) acc = fmaf(c.Zr[(2 * q + h) * 16 + I], c.R[(2 * q + h) * 16 + J], acc);
    }
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    if (act && h == 0) c.T1[p] = acc;
    __syncthreads();
    if (act && h == 0) c.R[p] = 0.f;
    acc = 0.f;
    if (act) {
#pragma unroll
        for (int q = 0; q < 8; ++q) acc = fmaf(c.T1[I * 16 + 2 * q + h], c.Zc[(2 * q + h) * 16 + J], acc);
    }
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    if (act && h == 0) c.T2[p] = acc / (c.lr[I] + c.lc[J]);
    __syncthreads();
    acc = 0.f;
    if (act) {
#pragma unroll
        for (int q = 0; q < 8; ++q) acc = fmaf(c.Zr[I * 16 + 2 * q + h], c.T2[(2 * q + h) * 16 + J], acc);
    }
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    if (act && h == 0) c.T1[p] = acc;
    __syncthreads();
    acc = 0.f;
    if (act) {
#pragma unroll
        for (int q = 0; q < 8; ++q) acc = fmaf(c.T1[I * 16 + 2 * q + h], c.ZcT[(2 * q + h) * 16 + J], acc);
    }
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    if (act && h == 0) c.E[I * COARSE_EST + J] = acc;
    __syncthreads();
}

}  // namespace fadesim
