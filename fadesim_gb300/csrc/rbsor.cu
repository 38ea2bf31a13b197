// Plain red-black point SOR for the crossbar nodal system (sm_103a).
//
// The comparator the accelerated solver is measured against: the reference's
// node-wise SOR update (split_arr_matmul.cu:27-119, crossbarHspice/2dArray.cc:
// 1551-1590) with a red-black colouring instead of the serial order, so that
// every node of one colour relaxes in parallel.  Colour of wordline node
// (i, j) is (i+j)&1 and of bitline node (i, j) is (i+j+1)&1; a node's wire
// neighbours and its partner in the other plane all have the other colour.
//
// One CTA solves one (tile, vector) pair at a time with both deviation planes
// and the conductances in shared memory; every half-sweep each cell updates
// exactly one of its two nodes (branch-free pointer selection).  Thread t owns
// column t % 128 at rows t / 128 + 8k: consecutive lanes walk consecutive
// columns (conflict-free), and no index is divided per cell.  Updates are
// in residual form, v += omega * r / diag, on deviations from the ideal state
// (FP32 throughout).  The stop test runs every CHECK sweeps on the observed
// contraction of the sweep-to-sweep change.
#include <math.h>

#include "kernels.h"

namespace fadesim {

constexpr int RB_THREADS = 1024;
constexpr int RB_CHECK = 8;
constexpr int RB_MAXL = 128;
constexpr int RB_ROWSTEP = RB_THREADS / RB_MAXL;  // rows between a thread's cells

__host__ __device__ inline int rb_ld(int m) { return m + 1; }

size_t rbsor_smem(int n, int m) {
    return (size_t)(3 * n * rb_ld(m) + n + 2 * 2 * (RB_THREADS / 32)) * sizeof(float);
}

template <typename TIO>
__global__ void __launch_bounds__(RB_THREADS, 1) rbsor_kernel(SolveArgs a) {
    extern __shared__ float4 smem4[];
    const int n = a.n, m = a.m, LDP = rb_ld(m);
    float *Gs = reinterpret_cast<float *>(smem4);
    float *U = Gs + n * LDP;
    float *D = U + n * LDP;
    float *vin_s = D + n * LDP;
    float *red = vin_s + n;  // [2][2][32]
    const int tid = threadIdx.x;
    const int ldG = a.numY * m;
    const TIO *inp = static_cast<const TIO *>(a.input);
    const TIO *Gg = static_cast<const TIO *>(a.G);
    TIO *out = static_cast<TIO *>(a.out);
    const float gw = a.gw;
    const float omega = a.ctl.omega;
    const int col = tid % RB_MAXL, row0 = tid / RB_MAXL;  // this thread's column and first row
    long long cached_tile = -1;

    for (long long item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const long long tile = item / a.nchunks;
        const int chunk = (int)(item % a.nchunks);
        const int x = (int)(tile / a.numY), y = (int)(tile % a.numY);
        const int b0 = chunk * a.vchunk, b1 = min(a.B, b0 + a.vchunk);
        if (tile != cached_tile) {
            __syncthreads();
            for (int e = tid; e < n * m; e += RB_THREADS) {
                const int i = e / m, j = e - i * m;
                Gs[i * LDP + j] = (float)Gg[((size_t)x * n + i) * ldG + (size_t)y * m + j];
            }
            cached_tile = tile;
        }
        for (int b = b0; b < b1; ++b) {
            __syncthreads();
            for (int e = tid; e < n * LDP; e += RB_THREADS) {
                U[e] = 0.f;
                D[e] = 0.f;
            }
            if (tid < n) vin_s[tid] = (float)inp[((size_t)b * a.numX + x) * n + tid];
            if (a.init) {
                // warm start: initial deviation planes [2][n][m] of this solve
                const float *w0 = a.init + (((size_t)b * a.numX + x) * a.numY + y) * 2 * n * m;
                for (int e = tid; e < n * m; e += RB_THREADS) {
                    const int i = e / m, j = e - i * m;
                    U[i * LDP + j] = w0[e];
                    D[i * LDP + j] = w0[(size_t)n * m + e];
                }
            }
            __syncthreads();
            float prev_check = 0.f;
            int sweeps = 0, status = 0, par = 0;
            while (true) {
                float dmax = 0.f, vmax = 0.f;
                for (int c = 0; c < 2; ++c) {
                    // thread -> cells (i0 + 8k, j): along its rows the colour of a cell
                    // does not change, so a thread relaxes one plane per half-sweep
                    if (col < m) {
                        const bool isU = ((row0 + col) & 1) == c;
                        float *self = isU ? U : D;
                        const float *oth = isU ? D : U;
                        const int o = isU ? 1 : LDP;  // neighbour stride along the line
                        for (int i = row0; i < n; i += RB_ROWSTEP) {
                            const int q = i * LDP + col;
                            // neighbours along the line: wordline (j-1, j+1), bitline (i-1, i+1)
                            const bool has1 = isU ? true : (i > 0);        // source link / upper link
                            const bool in1 = isU ? (col > 0) : (i > 0);      // neighbour is an unknown
                            const bool has2 = isU ? (col + 1 < m) : true;    // right link / lower link
                            const bool in2 = isU ? (col + 1 < m) : (i + 1 < n);
                            const float v = self[q];
                            const float n1 = in1 ? self[q - o] : 0.f;
                            const float n2 = in2 ? self[q + o] : 0.f;
                            const float g = Gs[q];
                            const float vi = vin_s[i];
                            const float src = isU ? (oth[q] - vi) - v : (oth[q] + vi) - v;
                            const float g1 = has1 ? gw : 0.f, g2 = has2 ? gw : 0.f;
                            const float r = g1 * (n1 - v) + g2 * (n2 - v) + g * src;
                            const float dv = __fdividef(omega * r, g1 + g2 + g);
                            const float nv = v + dv;
                            self[q] = nv;
                            dmax = isfinite(nv) ? fmaxf(dmax, fabsf(dv)) : INFINITY;
                            vmax = fmaxf(vmax, fabsf(nv));
                        }
                    }
                    __syncthreads();
                }
                ++sweeps;
                if (sweeps % RB_CHECK == 0 || sweeps >= a.ctl.max_iters) {
                    dmax = warp_max(dmax);
                    vmax = warp_max(vmax);
                    if ((tid & 31) == 0) {
                        red[(par * 2 + 0) * 32 + (tid >> 5)] = dmax;
                        red[(par * 2 + 1) * 32 + (tid >> 5)] = vmax;
                    }
                    __syncthreads();
                    float delta = 0.f, vm = 0.f;
                    for (int w = 0; w < RB_THREADS / 32; ++w) {
                        delta = fmaxf(delta, red[(par * 2 + 0) * 32 + w]);
                        vm = fmaxf(vm, red[(par * 2 + 1) * 32 + w]);
                    }
                    par ^= 1;
                    if (!isfinite(delta) || !isfinite(vm)) {
                        status = FADESIM_ST_NONFINITE;
                        break;
                    }
                    if (sweeps > RB_CHECK) {
                        const float floor_v = 4.f * 1.1920929e-07f * vm;
                        const float ratio = prev_check > 0.f ? powf(delta / prev_check, 1.f / RB_CHECK) : 0.f;
                        const float rho = fmaxf(ratio, omega - 1.f);
                        const float est = rho < 0.9999f ? delta * rho / (1.f - rho) : INFINITY;
                        const bool stalled = delta <= floor_v && ratio >= 0.999f;
                        if (est <= fmaxf(a.ctl.tol_v, floor_v) || stalled) {
                            status = FADESIM_ST_CONVERGED;
                            break;
                        }
                    }
                    prev_check = delta;
                    if (sweeps >= a.ctl.max_iters) {
                        status = FADESIM_ST_MAXITER;
                        break;
                    }
                }
            }
            if (a.ret_V) {
                for (int e = tid; e < n * m; e += RB_THREADS) {
                    const int i = e / m, j = e - i * m;
                    const int q = i * LDP + j;
                    const TIO uu = (TIO)U[q] + (TIO)vin_s[i];
                    const size_t sol = ((size_t)b * a.numX + x) * a.numY + y;
                    if (a.ret_V == 2) {
                        out[(sol * 2 + 0) * n * m + (size_t)i * m + j] = uu;
                        out[(sol * 2 + 1) * n * m + (size_t)i * m + j] = (TIO)D[q];
                    } else {
                        out[(sol * n + i) * m + j] = uu - (TIO)D[q];
                    }
                }
            } else {
                for (int j = tid; j < m; j += RB_THREADS) {
                    TIO acc = 0;
                    for (int i = 0; i < n; ++i) {
                        const int q = i * LDP + j;
                        acc += (TIO)Gs[q] * (((TIO)U[q] + (TIO)vin_s[i]) - (TIO)D[q]);
                    }
                    out[((size_t)b * a.numX + x) * ldG + (size_t)y * m + j] = acc;
                }
            }
            if (tid == 0) record_solve(a.stats, a.iters_out, ((long long)b * a.numX + x) * a.numY + y, sweeps, status);
        }
    }
}

cudaError_t rbsor_prepare(int dtype) {
    const int bytes = (int)rbsor_smem(RB_MAXL, RB_MAXL);
    return dtype == FADESIM_F64
               ? cudaFuncSetAttribute(rbsor_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)
               : cudaFuncSetAttribute(rbsor_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t launch_rbsor(const SolveArgs &a, int dtype, int grid, cudaStream_t st) {
    const size_t smem = rbsor_smem(a.n, a.m);
    if (dtype == FADESIM_F64) rbsor_kernel<double><<<grid, RB_THREADS, smem, st>>>(a);
    else rbsor_kernel<float><<<grid, RB_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace fadesim
