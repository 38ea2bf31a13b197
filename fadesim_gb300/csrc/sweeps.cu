// The reference's own sweep order, for callers that want its exact iterates
// (a fixed sweep count such as PimTorch's default 600, or its delta break).
//
// One launch is one sweep over every (tile, vector) solve: a CTA per solve,
// first every wordline row relaxed left -> right by one thread each (new left
// neighbour, old right neighbour, old bitline node), then, after a barrier,
// every bitline column bottom -> top (old upper, new lower, new wordline node)
// (split_arr_matmul.cu:27-119).  Updates are in place, which is what the
// reference's ping-pong buffers amount to.  The update expressions keep the
// reference's form and operand order so the compiler treats them alike.  With
// a break threshold the host reads the count of nodes that moved more than it
// after every sweep and stops when it is zero for the whole call, as the
// reference does with its two .item() reductions (:297-306).
#include "kernels.h"

namespace fadesim {

template <typename S>
__global__ void sweep_init_kernel(const S *__restrict__ input, S *__restrict__ U, S *__restrict__ D, int B,
                                  int numX, int numY, int n, int m) {
    const size_t total = (size_t)B * numX * numY * n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t i = (e / m) % n;
        const size_t bx = e / ((size_t)numY * n * m);  // b*numX + x
        U[e] = input[bx * n + i];
        D[e] = 0;
    }
}

template <typename S>
__global__ void sweep_kernel(const S *__restrict__ input, const S *__restrict__ G, S *__restrict__ U,
                             S *__restrict__ D, int numX, int numY, int n, int m, S g_wire, S beta, S thr,
                             unsigned int *moved) {
    const int b = blockIdx.x, x = blockIdx.y, y = blockIdx.z;
    const size_t plane = (((size_t)b * numX + x) * numY + y) * n * m;
    S *u = U + plane;
    S *d = D + plane;
    const size_t ldG = (size_t)numY * m;
    const S *g = G + (size_t)x * n * ldG + (size_t)y * m;  // g[i*ldG + j]
    const S g_load = g_wire;
    unsigned int cnt = 0;
    const int t = threadIdx.x;
    if (t < n) {
        const int row = t;
        S *ur = u + (size_t)row * m;
        const S *dr = d + (size_t)row * m;
        const S *gr = g + (size_t)row * ldG;
        int j = 0;
        S left = input[((size_t)b * numX + x) * n + row];
        S right = ur[j + 1];
        S other = dr[j];
        S sumg = g_wire + g_load + gr[j];
        S old = ur[j];
        S nv = beta * (g_load * left + g_wire * right + gr[j] * other) / sumg + (1 - beta) * old;
        ur[j] = nv;
        cnt += (nv - old > thr || old - nv > thr);
        for (j = 1; j < m - 1; ++j) {
            left = ur[j - 1];
            right = ur[j + 1];
            other = dr[j];
            sumg = g_wire * 2 + gr[j];
            old = ur[j];
            nv = beta * (g_wire * (left + right) + gr[j] * other) / sumg + (1 - beta) * old;
            ur[j] = nv;
            cnt += (nv - old > thr || old - nv > thr);
        }
        sumg = g_wire + gr[j];
        left = ur[j - 1];
        other = dr[j];
        old = ur[j];
        nv = beta * (g_wire * left + gr[j] * other) / sumg + (1 - beta) * old;
        ur[j] = nv;
        cnt += (nv - old > thr || old - nv > thr);
    }
    __syncthreads();
    if (t < m) {
        const int col = t;
        int i = n - 1;
        S up = d[(size_t)(i - 1) * m + col];
        S down = 0;
        S other = u[(size_t)i * m + col];
        S gi = g[(size_t)i * ldG + col];
        S sumg = g_wire + g_load + gi;
        S old = d[(size_t)i * m + col];
        S nv = beta * (g_wire * up + g_load * down + gi * other) / sumg + (1 - beta) * old;
        d[(size_t)i * m + col] = nv;
        cnt += (nv - old > thr || old - nv > thr);
        for (i = n - 2; i > 0; --i) {
            up = d[(size_t)(i - 1) * m + col];
            down = d[(size_t)(i + 1) * m + col];
            other = u[(size_t)i * m + col];
            gi = g[(size_t)i * ldG + col];
            sumg = g_wire * 2 + gi;
            old = d[(size_t)i * m + col];
            nv = beta * (g_wire * (up + down) + gi * other) / sumg + (1 - beta) * old;
            d[(size_t)i * m + col] = nv;
            cnt += (nv - old > thr || old - nv > thr);
        }
        down = d[(size_t)(i + 1) * m + col];
        other = u[(size_t)i * m + col];
        gi = g[(size_t)i * ldG + col];
        sumg = g_wire + gi;
        old = d[(size_t)i * m + col];
        nv = beta * (g_wire * down + gi * other) / sumg + (1 - beta) * old;
        d[(size_t)i * m + col] = nv;
        cnt += (nv - old > thr || old - nv > thr);
    }
    if (moved && cnt) atomicAdd(moved, cnt);
}

template <typename S>
__global__ void sweep_output_kernel(const S *__restrict__ G, const S *__restrict__ U, const S *__restrict__ D,
                                    S *__restrict__ out, int B, int numX, int numY, int n, int m, int ret_V) {
    const size_t ldG = (size_t)numY * m;
    if (ret_V) {
        const size_t total = (size_t)B * numX * numY * n * m;
        const size_t nm = (size_t)n * m;
        for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
             e += (size_t)gridDim.x * blockDim.x) {
            if (ret_V == 2) {
                out[(e / nm) * 2 * nm + e % nm] = U[e];
                out[(e / nm) * 2 * nm + nm + e % nm] = D[e];
            } else {
                out[e] = U[e] - D[e];
            }
        }
        return;
    }
    const size_t total = (size_t)B * numX * numY * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int col = (int)(e % m);
        const size_t bxy = e / m;
        const int y = (int)(bxy % numY);
        const int x = (int)((bxy / numY) % numX);
        const size_t b = bxy / ((size_t)numY * numX);
        const S *u = U + bxy * n * m;
        const S *d = D + bxy * n * m;
        const S *g = G + (size_t)x * n * ldG + (size_t)y * m + col;
        S acc = 0;
        for (int i = 0; i < n; ++i) acc += (u[(size_t)i * m + col] - d[(size_t)i * m + col]) * g[(size_t)i * ldG];
        out[(b * numX + x) * ldG + (size_t)y * m + col] = acc;
    }
}

static int grid_for(size_t total) {
    size_t g = (total + 255) / 256;
    return (int)(g > 8192 ? 8192 : (g < 1 ? 1 : g));
}

cudaError_t launch_sweep_init(const SolveArgs &a, int dtype, void *U, void *D, cudaStream_t st) {
    const size_t total = (size_t)a.B * a.numX * a.numY * a.n * a.m;
    if (dtype == FADESIM_F64)
        sweep_init_kernel<double><<<grid_for(total), 256, 0, st>>>((const double *)a.input, (double *)U, (double *)D,
                                                                   a.B, a.numX, a.numY, a.n, a.m);
    else
        sweep_init_kernel<float><<<grid_for(total), 256, 0, st>>>((const float *)a.input, (float *)U, (float *)D, a.B,
                                                                  a.numX, a.numY, a.n, a.m);
    return cudaGetLastError();
}

cudaError_t launch_sweep(const SolveArgs &a, int dtype, void *U, void *D, double gw, double beta, double thr,
                         unsigned int *moved, cudaStream_t st) {
    const dim3 grid(a.B, a.numX, a.numY);
    const int L = a.n > a.m ? a.n : a.m;
    const int threads = ((L + 31) / 32) * 32;
    if (dtype == FADESIM_F64)
        sweep_kernel<double><<<grid, threads, 0, st>>>((const double *)a.input, (const double *)a.G, (double *)U,
                                                       (double *)D, a.numX, a.numY, a.n, a.m, gw, beta, thr, moved);
    else
        sweep_kernel<float><<<grid, threads, 0, st>>>((const float *)a.input, (const float *)a.G, (float *)U,
                                                      (float *)D, a.numX, a.numY, a.n, a.m, (float)gw, (float)beta,
                                                      (float)thr, moved);
    return cudaGetLastError();
}

cudaError_t launch_sweep_output(const SolveArgs &a, int dtype, const void *U, const void *D, cudaStream_t st) {
    const size_t total = a.ret_V ? (size_t)a.B * a.numX * a.numY * a.n * a.m : (size_t)a.B * a.numX * a.numY * a.m;
    if (dtype == FADESIM_F64)
        sweep_output_kernel<double><<<grid_for(total), 256, 0, st>>>((const double *)a.G, (const double *)U,
                                                                     (const double *)D, (double *)a.out, a.B, a.numX,
                                                                     a.numY, a.n, a.m, a.ret_V);
    else
        sweep_output_kernel<float><<<grid_for(total), 256, 0, st>>>((const float *)a.G, (const float *)U,
                                                                    (const float *)D, (float *)a.out, a.B, a.numX,
                                                                    a.numY, a.n, a.m, a.ret_V);
    return cudaGetLastError();
}

}  // namespace fadesim
