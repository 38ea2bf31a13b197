// Plain red-black point SOR for tiles larger than 128 x 128 (sm_103a),
// cluster-resident: the comparator of the line relaxation at 256 x 256 (4-CTA
// clusters) and 512 x 512 (16-CTA clusters).
//
// Same node update as rbsor.cu (the reference's SOR step, split_arr_matmul.cu:
// 27-119, crossbarHspice/2dArray.cc:1551-1590, in residual form on deviations
// from the ideal state, red-black colouring: wordline node (i, j) has colour
// (i+j)&1, bitline node (i, j) colour (i+j+1)&1).  Each CTA of a cluster keeps a
// band of RPC consecutive rows of the conductances and of both planes in its
// shared memory; wordline neighbours and the partner node are in the band, and
// the bitline neighbours above the first row and below the last row of a band
// are read from the neighbouring CTAs' shared memory (distributed shared
// memory).  A half-sweep updates one colour and reads only the other, so one
// cluster barrier after every half-sweep orders all reads of a colour after its
// last writes.  Every CHECK sweeps the CTAs publish their largest correction
// and deviation; all CTAs read all of them after the half-sweep's barrier, so
// the stop decision -- and with it the barrier sequence -- is identical in every
// CTA of the cluster.
//
// Thread t owns column t % LDM at local rows t / LDM + (1024 / LDM) k: the row
// step is even and so is RPC, so along its rows a thread's cells keep their
// colour and it relaxes one plane per half-sweep; consecutive lanes walk
// consecutive columns (conflict-free).
//
// Node values are compensated: the FP32 value in shared memory plus an FP32
// low part in global memory (this CTA's slot of the call's scratch, L2-
// resident; the halo rows' low parts in the neighbouring CTAs' slots).  With
// FP32 storage alone the point iteration stalls where most corrections fall
// below half an ulp of the node: on a 256 x 256 four-state tile with 0.2 V
// Bernoulli inputs that is 1.4e-6 V from the nodal solution (a numpy FP32
// emulation of this update, against 1e-8 V in FP64), above the 1e-6 V the
// comparison asks for.  The residual takes every term as high minus high plus
// low minus low, and each update adds the correction to the low part and
// renormalises with an error-free sum (TwoSum), so the iteration converges as
// in ~FP64 at FP32 arithmetic.
#include <cooperative_groups.h>
#include <math.h>

#include "kernels.h"
#include "line_common.cuh"

namespace cg = cooperative_groups;

namespace fadesim {

namespace {

constexpr int RBC_T = 1024;
constexpr int RBC_CHECK = 8;
constexpr int RBC_NW = RBC_T / 32;

template <int LDM>
struct RbcCfg;
template <>
struct RbcCfg<256> {
    static constexpr int C = 4, RPC = 64;
};
template <>
struct RbcCfg<512> {
    static constexpr int C = 16, RPC = 32;
};

template <int LDM>
constexpr size_t rbc_smem_floats() {
    return (size_t)3 * RbcCfg<LDM>::RPC * LDM + RbcCfg<LDM>::RPC + 2 * RBC_NW + 4 + 2 + LDM;
}

template <int LDM, typename TIO>
__global__ void __launch_bounds__(RBC_T, 1) rbsor_cluster_kernel(SolveArgs a) {
    constexpr int C = RbcCfg<LDM>::C, RPC = RbcCfg<LDM>::RPC, STEP = RBC_T / LDM;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    extern __shared__ float4 smem4[];
    float *Gs = reinterpret_cast<float *>(smem4);
    float *U = Gs + RPC * LDM;
    float *D = U + RPC * LDM;
    float *vin_s = D + RPC * LDM;
    float *red = vin_s + RPC;      // [2][RBC_NW]: per-warp maxima of this CTA
    float *cred = red + 2 * RBC_NW;  // [2 parities][2]: this CTA's maxima, read by the cluster
    float *bcast = cred + 4;       // [2]: the cluster's maxima, gathered by warp 0
    float *part = bcast + 2;       // [LDM]: this band's part of every column current
    const int tid = threadIdx.x;
    const int n = a.n, m = a.m, ldG = a.numY * m;
    const int row0 = rank * RPC;
    const int nloc = max(0, min(RPC, n - row0));
    const TIO *inp = static_cast<const TIO *>(a.input);
    const TIO *Gg = static_cast<const TIO *>(a.G);
    TIO *out = static_cast<TIO *>(a.out);
    const float gw = a.gw, omega = a.ctl.omega;
    const int col = tid % LDM, lr0 = tid / LDM;  // this thread's column and first local row
    // the neighbouring bands' bitline planes (halo rows)
    const float *D_above = rank > 0 ? cluster.map_shared_rank(D, rank - 1) : nullptr;
    const float *D_below = rank + 1 < C ? cluster.map_shared_rank(D, rank + 1) : nullptr;
    // low parts of both planes: this CTA's scratch slot [2][RPC][LDM]; the
    // neighbouring bands' in the neighbouring CTAs' slots (a cluster's CTAs are
    // consecutive blocks)
    constexpr size_t SLOT = (size_t)2 * RPC * LDM;
    float *Ul = a.scratch + (size_t)blockIdx.x * SLOT;
    float *Dl = Ul + (size_t)RPC * LDM;
    const float *Dl_above = rank > 0 ? a.scratch + (size_t)(blockIdx.x - 1) * SLOT + (size_t)RPC * LDM : nullptr;
    const float *Dl_below = rank + 1 < C ? a.scratch + (size_t)(blockIdx.x + 1) * SLOT + (size_t)RPC * LDM : nullptr;
    const long long cid = blockIdx.x / C, ncl = gridDim.x / C;
    long long cached_tile = -1;

    for (long long item = cid; item < a.nitems; item += ncl) {
        const long long tile = item / a.nchunks;
        const int chunk = (int)(item % a.nchunks);
        const int x = (int)(tile / a.numY), y = (int)(tile % a.numY);
        const int b0 = chunk * a.vchunk, b1 = min(a.B, b0 + a.vchunk);
        if (tile != cached_tile) {
            __syncthreads();
            for (int e = tid; e < RPC * LDM; e += RBC_T) {
                const int lr = e / LDM, j = e - lr * LDM;
                Gs[e] = (lr < nloc && j < m) ? (float)Gg[((size_t)x * n + row0 + lr) * ldG + (size_t)y * m + j] : 0.f;
            }
            cached_tile = tile;
        }
        for (int b = b0; b < b1; ++b) {
            __syncthreads();
            for (int e = tid; e < RPC * LDM; e += RBC_T) {
                U[e] = 0.f;
                D[e] = 0.f;
                Ul[e] = 0.f;
                Dl[e] = 0.f;
            }
            if (tid < RPC) vin_s[tid] = tid < nloc ? (float)inp[((size_t)b * a.numX + x) * n + row0 + tid] : 0.f;
            cluster.sync();  // every band cleared before any halo is read
            float prev_check = 0.f;
            int sweeps = 0, status = 0, par = 0;
            while (true) {
                float dmax = 0.f, vmax = 0.f;
                const bool check = (sweeps + 1) % RBC_CHECK == 0 || sweeps + 1 >= a.ctl.max_iters;
                for (int c = 0; c < 2; ++c) {
                    if (col < m) {
                        const bool isU = ((row0 + lr0 + col) & 1) == c;
                        float *self = isU ? U : D;
                        float *selfl = isU ? Ul : Dl;
                        const float *oth = isU ? D : U;
                        const float *othl = isU ? Dl : Ul;
#pragma unroll 2
                        for (int lr = lr0; lr < nloc; lr += STEP) {
                            const int gi = row0 + lr;
                            const int q = lr * LDM + col;
                            const float v = self[q], vl = selfl[q];
                            float n1 = 0.f, n1l = 0.f, n2 = 0.f, n2l = 0.f, g1, g2;
                            if (isU) {
                                // wordline: source link at the left end, open at the right end
                                if (col > 0) {
                                    n1 = self[q - 1];
                                    n1l = selfl[q - 1];
                                }
                                if (col + 1 < m) {
                                    n2 = self[q + 1];
                                    n2l = selfl[q + 1];
                                }
                                g1 = gw;
                                g2 = col + 1 < m ? gw : 0.f;
                            } else {
                                // bitline: open at the top, grounded below the last row
                                if (lr > 0) {
                                    n1 = self[q - LDM];
                                    n1l = selfl[q - LDM];
                                } else if (gi > 0) {
                                    n1 = D_above[(RPC - 1) * LDM + col];
                                    n1l = Dl_above[(RPC - 1) * LDM + col];
                                }
                                if (lr + 1 < nloc) {
                                    n2 = self[q + LDM];
                                    n2l = selfl[q + LDM];
                                } else if (gi + 1 < n) {
                                    n2 = D_below[col];
                                    n2l = Dl_below[col];
                                }
                                g1 = gi > 0 ? gw : 0.f;
                                g2 = gw;
                            }
                            const float g = Gs[q];
                            const float vi = vin_s[lr];
                            // every difference as high minus high plus low minus low
                            const float src = ((isU ? (oth[q] - vi) : (oth[q] + vi)) - v) + (othl[q] - vl);
                            const float r = g1 * ((n1 - v) + (n1l - vl)) + g2 * ((n2 - v) + (n2l - vl)) + g * src;
                            const float dv = __fdividef(omega * r, g1 + g2 + g);
                            // (v, vl) + dv, renormalised without loss
                            float nv, nl;
                            two_sum(v, vl + dv, nv, nl);
                            self[q] = nv;
                            selfl[q] = nl;
                            dmax = isfinite(nv) ? fmaxf(dmax, fabsf(dv)) : INFINITY;
                            vmax = fmaxf(vmax, fabsf(nv));
                        }
                    }
                    if (c == 1 && check) {
                        dmax = warp_max(dmax);
                        vmax = warp_max(vmax);
                        if ((tid & 31) == 0) {
                            red[tid >> 5] = dmax;
                            red[RBC_NW + (tid >> 5)] = vmax;
                        }
                        __syncthreads();
                        if (tid < 32) {
                            const float d0 = warp_max(red[tid]);
                            const float v0 = warp_max(red[RBC_NW + tid]);
                            if (tid == 0) {
                                cred[par * 2 + 0] = d0;
                                cred[par * 2 + 1] = v0;
                            }
                        }
                    }
                    cluster.sync();  // this colour final everywhere (and this CTA's maxima published)
                }
                ++sweeps;
                if (check) {
                    // warp 0 gathers the cluster's maxima; every thread then reads them
                    if (tid < 32) {
                        const float *cr = cluster.map_shared_rank(cred, tid < C ? tid : 0);
                        const float d0 = warp_max(tid < C ? cr[par * 2 + 0] : 0.f);
                        const float v0 = warp_max(tid < C ? cr[par * 2 + 1] : 0.f);
                        if (tid == 0) {
                            bcast[0] = d0;
                            bcast[1] = v0;
                        }
                    }
                    __syncthreads();
                    const float delta = bcast[0], vm = bcast[1];
                    par ^= 1;
                    if (!isfinite(delta) || !isfinite(vm)) {
                        status = FADESIM_ST_NONFINITE;
                        break;
                    }
                    if (sweeps > RBC_CHECK) {
                        // as rbsor.cu: the estimate against the tolerance, floored at 4
                        // ulps of the largest deviation, or corrections that stall there.
                        // With compensated nodes the corrections stall only at the
                        // residual's own rounding (~0.1-0.3 ulp of the largest
                        // deviation), ~4e-8 V from the solution at 256 x 256 in a numpy
                        // FP32 emulation, where FP32 nodes alone stall at 1.4e-6 V.
                        const float floor_v = 4.f * 1.1920929e-07f * vm;
                        const float ratio = prev_check > 0.f ? powf(delta / prev_check, 1.f / RBC_CHECK) : 0.f;
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
            const size_t sol = ((size_t)b * a.numX + x) * a.numY + y;
            if (a.ret_V) {
                for (int e = tid; e < nloc * m; e += RBC_T) {
                    const int lr = e / m, j = e - lr * m, i = row0 + lr;
                    const int q = lr * LDM + j;
                    const TIO uu = ((TIO)U[q] + (TIO)Ul[q]) + (TIO)vin_s[lr];
                    const TIO dd = (TIO)D[q] + (TIO)Dl[q];
                    if (a.ret_V == 2) {
                        out[(sol * 2 + 0) * n * m + (size_t)i * m + j] = uu;
                        out[(sol * 2 + 1) * n * m + (size_t)i * m + j] = dd;
                    } else {
                        out[(sol * n + i) * m + j] = uu - dd;
                    }
                }
            } else {
                // this band's part of every column current, summed over the bands in rank order
                for (int j = tid; j < m; j += RBC_T) {
                    float acc = 0.f;
                    for (int lr = 0; lr < nloc; ++lr) {
                        const int q = lr * LDM + j;
                        acc += Gs[q] * (((U[q] + vin_s[lr]) - D[q]) + (Ul[q] - Dl[q]));
                    }
                    part[j] = acc;
                }
                cluster.sync();
                if (rank == 0) {
                    for (int j = tid; j < m; j += RBC_T) {
                        TIO acc = 0;
                        for (int r = 0; r < C; ++r) acc += (TIO)cluster.map_shared_rank(part, r)[j];
                        out[((size_t)b * a.numX + x) * ldG + (size_t)y * m + j] = acc;
                        if (!isfinite((float)acc)) status |= FADESIM_ST_NONFINITE;
                    }
                }
                cluster.sync();  // the partial sums read before the next solve overwrites them
            }
            if (tid == 0 && rank == 0) record_solve(a.stats, a.iters_out, (long long)sol, sweeps, status);
            if (rank == 0 && (status & FADESIM_ST_NONFINITE) && a.stats) atomicOr(&a.stats->status_or, status);
        }
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
}

template <int LDM>
cudaError_t rbc_launch_t(int *clusters, const SolveArgs *a, int dtype, int grid, cudaStream_t st) {
    void (*kern)(SolveArgs) =
        dtype == FADESIM_F64 ? rbsor_cluster_kernel<LDM, double> : rbsor_cluster_kernel<LDM, float>;
    const size_t smem = rbc_smem_floats<LDM>() * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (RbcCfg<LDM>::C > 8) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = RbcCfg<LDM>::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(RBC_T);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (clusters) {
        cfg.gridDim = dim3(RbcCfg<LDM>::C);
        return cudaOccupancyMaxActiveClusters(clusters, kern, &cfg);
    }
    cfg.gridDim = dim3(grid);
    e = cudaLaunchKernelEx(&cfg, kern, *a);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace

int rbsor_cluster_ld(int n, int m) {
    const int L = n > m ? n : m;
    if (L <= 128) return 0;
    if (L <= 256) return 256;
    if (L <= 512) return 512;
    return 0;
}

int rbsor_cluster_size(int ld) { return ld == 256 ? RbcCfg<256>::C : RbcCfg<512>::C; }

size_t rbsor_cluster_scratch_floats_per_cta(int ld) {
    return ld == 256 ? (size_t)2 * RbcCfg<256>::RPC * 256 : (size_t)2 * RbcCfg<512>::RPC * 512;
}

cudaError_t rbsor_cluster_occupancy(int ld, int dtype, int *clusters) {
    if (ld == 256) return rbc_launch_t<256>(clusters, nullptr, dtype, 0, 0);
    if (ld == 512) return rbc_launch_t<512>(clusters, nullptr, dtype, 0, 0);
    return cudaErrorInvalidValue;
}

cudaError_t launch_rbsor_cluster(const SolveArgs &a, int ld, int dtype, int grid, cudaStream_t st) {
    if (ld == 256) return rbc_launch_t<256>(nullptr, &a, dtype, grid, st);
    if (ld == 512) return rbc_launch_t<512>(nullptr, &a, dtype, grid, st);
    return cudaErrorInvalidValue;
}

}  // namespace fadesim
