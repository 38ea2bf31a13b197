// The reference extension's other IR-drop models, with their own iterates:
//
// * ir_gs_ou_local / ir_gs_ou: the Gauss-Seidel/SOR sweep of ir_drop_gs with
//   given source and ground load conductances (split_arr_matmul.cu:27-119,
//   690-813), or on every operation unit (OU, an ou_rows x ou_cols sub-array)
//   of the tile at once, each OU reaching the source and ground through the
//   lumped wire that lies outside it: g_wire / (first column + 1) on the
//   wordline side, g_wire / (rows - last row) on the bitline side
//   (:1086-1327).
// * ir2s / ir2s_ou_local / ir2s_ou: the "IR-drop to source" iteration
//   (:336-687, 816-1084): from the previous voltages, each line's remaining
//   cell current is carried back to the source through the wire resistances
//   (Jacobi: both planes from the previous iterate), with a load resistance at
//   the source and ground ends (r_wire * (first column + 1) and r_wire * (rows -
//   last row) per OU in ir2s_ou).  As in the reference the line current sums
//   persist between iterations (what is left after subtracting each cell's
//   current is carried over).
//
// All five share one layout: planes [B, numX, numY, rows, cols] in global
// memory, a tile split into OUs (one OU for the non-OU functions), one block per
// (vector, tile) solve.  The update expressions keep the reference's form and
// operand order.  With a break threshold the host reads the count of nodes
// that moved more than it after every iteration (the reference's two .item()
// reductions, :297-306).
#include "kernels.h"
#include "trace.h"

namespace fadesim {

namespace {

int fail(int code, const char *msg) { return report_error(code, msg); }

struct OuShape {
    int n, m, on, om;        // tile rows, cols; OU rows, cols
    int nox, noy;            // OUs per tile column / row
    int ou_loads;            // 1: lumped loads from the OU's position; 0: the given loads
};

template <typename S>
__global__ void fam_init_kernel(const S *__restrict__ input, S *__restrict__ U, S *__restrict__ D, int B,
                                int numX, int numY, int n, int m) {
    const size_t total = (size_t)B * numX * numY * n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t i = (e / m) % n;
        const size_t bx = e / ((size_t)numY * n * m);  // b*numX + x
        U[e] = input[bx * n + i];
        D[e] = 0;
    }
}

// One Gauss-Seidel/SOR sweep of every OU of every solve, in place (new left and
// lower neighbours, old right and upper neighbours, as the reference's
// ping-pong buffers amount to).  gll / gdl: source / ground load conductance of
// a single-OU tile (ou_loads 0).
template <typename S>
__global__ void fam_gs_sweep_kernel(const S *__restrict__ input, const S *__restrict__ G, S *__restrict__ U,
                                    S *__restrict__ D, int numX, int numY, OuShape o, S g_wire, S gll, S gdl, S beta,
                                    S thr, unsigned int *moved) {
    const int b = blockIdx.x, x = blockIdx.y, y = blockIdx.z;
    const int n = o.n, m = o.m;
    const size_t plane = (((size_t)b * numX + x) * numY + y) * n * m;
    S *u = U + plane;
    S *d = D + plane;
    const size_t ldG = (size_t)numY * m;
    const S *g = G + (size_t)x * n * ldG + (size_t)y * m;  // g[i*ldG + j]
    unsigned int cnt = 0;
    // wordline segments: one thread per (row, OU column)
    for (int w = threadIdx.x; w < n * o.noy; w += blockDim.x) {
        const int row = w / o.noy, s = (w % o.noy) * o.om;
        S *ur = u + (size_t)row * m;
        const S *dr = d + (size_t)row * m;
        const S *gr = g + (size_t)row * ldG;
        const S g_load_left = o.ou_loads ? g_wire / (S)(s + 1) : gll;
        int j = s;
        S left = input[((size_t)b * numX + x) * n + row];
        S right = ur[j + 1];
        S other = dr[j];
        S sumg = g_wire + g_load_left + gr[j];
        S old = ur[j];
        S nv = beta * (g_load_left * left + g_wire * right + gr[j] * other) / sumg + (1 - beta) * old;
        ur[j] = nv;
        cnt += (nv - old > thr || old - nv > thr);
        for (j = s + 1; j < s + o.om - 1; ++j) {
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
    // bitline segments: one thread per (column, OU row), bottom -> top
    for (int w = threadIdx.x; w < m * o.nox; w += blockDim.x) {
        const int col = w / o.nox, s = (w % o.nox) * o.on;
        int i = s + o.on - 1;
        const S g_load_down = o.ou_loads ? g_wire / (S)(n - i) : gdl;
        S up = d[(size_t)(i - 1) * m + col];
        S down = 0;
        S other = u[(size_t)i * m + col];
        S gi = g[(size_t)i * ldG + col];
        S sumg = g_wire + g_load_down + gi;
        S old = d[(size_t)i * m + col];
        S nv = beta * (g_wire * up + g_load_down * down + gi * other) / sumg + (1 - beta) * old;
        d[(size_t)i * m + col] = nv;
        cnt += (nv - old > thr || old - nv > thr);
        for (i = s + o.on - 2; i > s; --i) {
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
    if (moved) {
        for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
        if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(moved, cnt);
    }
}

// One IR2S iteration of every OU of every solve: reads the previous planes
// (Up, Dp), writes the new ones (Un, Dn).  Rsum [B, numX, numY, n, noy] and
// Csum [B, numX, numY, m, nox] are the persistent per-segment current sums.
// rll / rdl: source / ground load resistance of a single-OU tile (ou_loads 0).
template <typename S>
__global__ void fam_ir2s_kernel(const S *__restrict__ input, const S *__restrict__ G, const S *__restrict__ Up,
                                const S *__restrict__ Dp, S *__restrict__ Un, S *__restrict__ Dn, S *__restrict__ Rsum,
                                S *__restrict__ Csum, int numX, int numY, OuShape o, S r_wire, S rll, S rdl, S thr,
                                unsigned int *moved) {
    const int b = blockIdx.x, x = blockIdx.y, y = blockIdx.z;
    const int n = o.n, m = o.m;
    const size_t sol = ((size_t)b * numX + x) * numY + y;
    const size_t plane = sol * n * m;
    const S *up = Up + plane, *dp = Dp + plane;
    S *un = Un + plane, *dn = Dn + plane;
    const size_t ldG = (size_t)numY * m;
    const S *g = G + (size_t)x * n * ldG + (size_t)y * m;
    unsigned int cnt = 0;
    for (int w = threadIdx.x; w < n * o.noy; w += blockDim.x) {
        const int row = w / o.noy, sy = w % o.noy, s = sy * o.om;
        S &acc = Rsum[(sol * n + row) * o.noy + sy];
        const size_t r0 = (size_t)row * m;
        for (int j = s; j < s + o.om; ++j) acc += (up[r0 + j] - dp[r0 + j]) * g[(size_t)row * ldG + j];
        int j = s;
        const S in = input[((size_t)b * numX + x) * n + row];
        S nv = o.ou_loads ? in - acc * (r_wire * (S)(j + 1)) : in - acc * rll;
        un[r0 + j] = nv;
        cnt += (nv - up[r0 + j] > thr || up[r0 + j] - nv > thr);
        acc -= (up[r0 + j] - dp[r0 + j]) * g[(size_t)row * ldG + j];
        for (j = s + 1; j < s + o.om; ++j) {
            nv = un[r0 + j - 1] - acc * r_wire;
            un[r0 + j] = nv;
            cnt += (nv - up[r0 + j] > thr || up[r0 + j] - nv > thr);
            acc -= (up[r0 + j] - dp[r0 + j]) * g[(size_t)row * ldG + j];
        }
    }
    for (int w = threadIdx.x; w < m * o.nox; w += blockDim.x) {
        const int col = w / o.nox, sx = w % o.nox, s = sx * o.on;
        S &acc = Csum[(sol * m + col) * o.nox + sx];
        for (int i = s; i < s + o.on; ++i)
            acc += (up[(size_t)i * m + col] - dp[(size_t)i * m + col]) * g[(size_t)i * ldG + col];
        int i = s + o.on - 1;
        S nv = o.ou_loads ? acc * (r_wire * (S)(n - i)) : acc * rdl;
        dn[(size_t)i * m + col] = nv;
        cnt += (nv - dp[(size_t)i * m + col] > thr || dp[(size_t)i * m + col] - nv > thr);
        acc -= (up[(size_t)i * m + col] - dp[(size_t)i * m + col]) * g[(size_t)i * ldG + col];
        for (i = s + o.on - 2; i >= s; --i) {
            nv = dn[(size_t)(i + 1) * m + col] + acc * r_wire;
            dn[(size_t)i * m + col] = nv;
            cnt += (nv - dp[(size_t)i * m + col] > thr || dp[(size_t)i * m + col] - nv > thr);
            acc -= (up[(size_t)i * m + col] - dp[(size_t)i * m + col]) * g[(size_t)i * ldG + col];
        }
    }
    if (moved) {
        for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
        if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(moved, cnt);
    }
}

// Bitline currents of every OU row group: out[b, x, ou_x, y*m + col] = sum over
// the OU's rows (ascending) of (u - d) g; one group = a whole column.
template <typename S>
__global__ void fam_current_kernel(const S *__restrict__ U, const S *__restrict__ D, const S *__restrict__ G,
                                   S *__restrict__ out, int B, int numX, int numY, OuShape o) {
    const int n = o.n, m = o.m;
    const size_t total = (size_t)B * numX * o.nox * numY * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int col = (int)(e % m);
        const int y = (int)((e / m) % numY);
        const int sx = (int)((e / ((size_t)m * numY)) % o.nox);
        const size_t bx = e / ((size_t)m * numY * o.nox);  // b*numX + x
        const int x = (int)(bx % numX);
        const size_t plane = (bx * numY + y) * n * m;
        const S *g = G + (size_t)x * n * numY * m + (size_t)y * m + col;
        S acc = 0;
        for (int i = sx * o.on; i < (sx + 1) * o.on; ++i)
            acc += (U[plane + (size_t)i * m + col] - D[plane + (size_t)i * m + col]) * g[(size_t)i * numY * m];
        out[e] = acc;
    }
}

template <typename S>
__global__ void fam_voltage_kernel(const S *__restrict__ U, const S *__restrict__ D, S *__restrict__ out, size_t total) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        out[e] = U[e] - D[e];
}

int fam_grid(size_t total) {
    size_t g = (total + 255) / 256;
    return (int)(g > 16384 ? 16384 : (g < 1 ? 1 : g));
}

// Host driver shared by the five entry points.
template <typename S>
int fam_run(bool ir2s, const void *input_v, const void *G_v, int B, OuShape o, int numX, int numY, int iter_times,
            double wire, double load_l, double load_d, double beta, int enable_break, double thr, int ret_V,
            void *out_v, cudaStream_t st) {
    const S *input = static_cast<const S *>(input_v);
    const S *G = static_cast<const S *>(G_v);
    S *out = static_cast<S *>(out_v);
    const size_t plane_elems = (size_t)B * numX * numY * o.n * o.m;
    const size_t rsum = (size_t)B * numX * numY * o.n * o.noy, csum = (size_t)B * numX * numY * o.m * o.nox;
    const size_t bytes = (ir2s ? 4 : 2) * plane_elems * sizeof(S) + (ir2s ? (rsum + csum) * sizeof(S) : 0) + 256;
    char *buf = nullptr;
    cudaError_t e = lib_malloc_async((void **)&buf, bytes, st);
    if (e != cudaSuccess) return fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    S *U = reinterpret_cast<S *>(buf), *D = U + plane_elems;
    S *U2 = ir2s ? D + plane_elems : nullptr, *D2 = ir2s ? U2 + plane_elems : nullptr;
    S *Rs = ir2s ? D2 + plane_elems : nullptr, *Cs = ir2s ? Rs + rsum : nullptr;
    unsigned int *moved = reinterpret_cast<unsigned int *>(buf + bytes - 256);
    int rc = FADESIM_OK;
    fam_init_kernel<S><<<fam_grid(plane_elems), 256, 0, st>>>(input, U, D, B, numX, numY, o.n, o.m);
    e = cudaGetLastError();
    if (e == cudaSuccess && ir2s) {
        e = cudaMemcpyAsync(U2, U, 2 * plane_elems * sizeof(S), cudaMemcpyDeviceToDevice, st);  // U2, D2 <- U, D
        if (e == cudaSuccess) e = cudaMemsetAsync(Rs, 0, (rsum + csum) * sizeof(S), st);
    }
    if (e != cudaSuccess) rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    const dim3 grid(B, numX, numY);
    const int threads = (int)min(1024, ((max(o.n * o.noy, o.m * o.nox) + 31) / 32) * 32);
    for (int it = 0; rc == FADESIM_OK && it < iter_times && B > 0; ++it) {
        unsigned int *mv = enable_break ? moved : nullptr;
        if (mv && (e = cudaMemsetAsync(mv, 0, sizeof(unsigned int), st)) != cudaSuccess) {
            rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
            break;
        }
        if (ir2s) {
            fam_ir2s_kernel<S><<<grid, threads, 0, st>>>(input, G, U, D, U2, D2, Rs, Cs, numX, numY, o, (S)wire,
                                                          (S)load_l, (S)load_d, (S)thr, mv);
            S *t = U;
            U = U2;
            U2 = t;
            t = D;
            D = D2;
            D2 = t;
        } else {
            fam_gs_sweep_kernel<S><<<grid, threads, 0, st>>>(input, G, U, D, numX, numY, o, (S)wire, (S)load_l,
                                                              (S)load_d, (S)beta, (S)thr, mv);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) {
            rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
            break;
        }
        if (mv) {
            unsigned int h = 0;
            e = cudaMemcpyAsync(&h, mv, sizeof(h), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
                break;
            }
            if (h == 0) break;
        }
    }
    if (rc == FADESIM_OK) {
        if (ret_V)
            fam_voltage_kernel<S><<<fam_grid(plane_elems), 256, 0, st>>>(U, D, out, plane_elems);
        else
            fam_current_kernel<S><<<fam_grid((size_t)B * numX * o.nox * numY * o.m), 256, 0, st>>>(U, D, G, out, B,
                                                                                                 numX, numY, o);
        if ((e = cudaGetLastError()) != cudaSuccess) rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    }
    cudaFreeAsync(buf, st);
    return rc;
}

int fam_check(int dtype, const void *input, const void *G, void *out, int B, int n, int m, int on, int om, int numX,
              int numY, int iter_times, double wire) {
    if (dtype != FADESIM_F32 && dtype != FADESIM_F64) return fail(FADESIM_E_ARG, "dtype must be f32 or f64");
    if (n < 2) return fail(FADESIM_E_ARG, "row_size should be >=2");
    if (m < 2) return fail(FADESIM_E_ARG, "col_size should be >=2");
    if (on < 2 || om < 2 || n % on || m % om)
        return fail(FADESIM_E_ARG, "ou size must divide the array size and be at least 2 x 2");
    if (B < 0 || numX < 1 || numY < 1 || iter_times < 0) return fail(FADESIM_E_ARG, "bad batch, tile or iteration count");
    if (!(wire > 0)) return fail(FADESIM_E_ARG, "wire resistance / conductance must be positive");
    if (B > 0 && (!input || !G || !out)) return fail(FADESIM_E_ARG, "null pointer");
    if (numY > 65535 || numX > 65535) return fail(FADESIM_E_ARG, "numX and numY must be < 65536");
    return FADESIM_OK;
}

int fam_dispatch(int dtype, bool ir2s, const void *input, const void *G, int B, OuShape o, int numX, int numY,
                 int iter_times, double wire, double load_l, double load_d, double beta, int enable_break, double thr,
                 int ret_V, void *out, void *stream) {
    if (B == 0) return FADESIM_OK;
    TraceRange trace(ir2s ? "fadesim_ir2s_family" : "fadesim_ir_gs_ou_family");
    cudaStream_t st = (cudaStream_t)stream;
    return dtype == FADESIM_F64
               ? fam_run<double>(ir2s, input, G, B, o, numX, numY, iter_times, wire, load_l, load_d, beta, enable_break,
                                 thr, ret_V, out, st)
               : fam_run<float>(ir2s, input, G, B, o, numX, numY, iter_times, wire, load_l, load_d, beta, enable_break,
                                thr, ret_V, out, st);
}

}  // namespace

}  // namespace fadesim

using namespace fadesim;

extern "C" int fadesim_ir_gs_ou_local(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                      int col_size, int numX, int numY, int iter_times, double g_wire,
                                      double g_load_left, double g_load_down, double beta, int enable_break,
                                      double break_threshould, void *out, void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, row_size, col_size, numX, numY,
                       iter_times, g_wire);
    if (rc) return rc;
    if (!(g_load_left > 0) || !(g_load_down > 0)) return fail(FADESIM_E_ARG, "load conductances must be positive");
    OuShape o{row_size, col_size, row_size, col_size, 1, 1, 0};
    return fam_dispatch(dtype, false, input, G, batch_size, o, numX, numY, iter_times, g_wire, g_load_left,
                        g_load_down, beta, enable_break, break_threshould, 0, out, stream);
}

extern "C" int fadesim_ir_gs_ou(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                int col_size, int ou_row_size, int ou_col_size, int numX, int numY, int iter_times,
                                double g_wire, double beta, int enable_break, double break_threshould, void *out,
                                void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY,
                       iter_times, g_wire);
    if (rc) return rc;
    OuShape o{row_size, col_size, ou_row_size, ou_col_size, row_size / ou_row_size, col_size / ou_col_size, 1};
    return fam_dispatch(dtype, false, input, G, batch_size, o, numX, numY, iter_times, g_wire, g_wire, g_wire, beta,
                        enable_break, break_threshould, 0, out, stream);
}

extern "C" int fadesim_ir2s(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                            int numX, int numY, int iter_times, double r_wire, int enable_break,
                            double break_threshould, int ret_V, void *out, void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, row_size, col_size, numX, numY,
                       iter_times, r_wire);
    if (rc) return rc;
    OuShape o{row_size, col_size, row_size, col_size, 1, 1, 0};
    return fam_dispatch(dtype, true, input, G, batch_size, o, numX, numY, iter_times, r_wire, r_wire, r_wire, 1.0,
                        enable_break, break_threshould, ret_V ? 1 : 0, out, stream);
}

extern "C" int fadesim_ir2s_ou_local(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                     int col_size, int numX, int numY, int iter_times, double r_wire,
                                     double r_load_left, double r_load_down, int enable_break,
                                     double break_threshould, void *out, void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, row_size, col_size, numX, numY,
                       iter_times, r_wire);
    if (rc) return rc;
    if (!(r_load_left >= 0) || !(r_load_down >= 0)) return fail(FADESIM_E_ARG, "load resistances must be >= 0");
    OuShape o{row_size, col_size, row_size, col_size, 1, 1, 0};
    return fam_dispatch(dtype, true, input, G, batch_size, o, numX, numY, iter_times, r_wire, r_load_left,
                        r_load_down, 1.0, enable_break, break_threshould, 0, out, stream);
}

extern "C" int fadesim_ir2s_ou(int dtype, const void *input, const void *G, int batch_size, int row_size,
                               int col_size, int ou_row_size, int ou_col_size, int numX, int numY, int iter_times,
                               double r_wire, int enable_break, double break_threshould, void *out, void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY,
                       iter_times, r_wire);
    if (rc) return rc;
    OuShape o{row_size, col_size, ou_row_size, ou_col_size, row_size / ou_row_size, col_size / ou_col_size, 1};
    return fam_dispatch(dtype, true, input, G, batch_size, o, numX, numY, iter_times, r_wire, r_wire, r_wire, 1.0,
                        enable_break, break_threshould, 0, out, stream);
}
