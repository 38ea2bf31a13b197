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
//
// Sinh cells (nonlinear_cell_enable, :455-475, 603-622, 727-746, 996-1016,
// 1241-1260): before every iteration each solve's conductances are recomputed
// cell by cell, in the I/O type, from u - d of the iterate before the newest
// one (what the reference's ping-pong buffers hold when it recomputes them;
// iterations 0 and 1 both see the initial planes), |V| < 1e-5 set to +-1e-5
// (deal_v, :142-166), R(V) = (1-z) |V| / (b_on sinh(a_on |V|)) + z |V| /
// (b_off sinh(a_off |V|)) with z = (1/g - R_on) / (R_off - R_on) from the linear
// conductance, negative z set to 0 (:176-196).  The conductances then live in
// one plane per solve, and the currents use the last of them (get_current).
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
                                    S thr, unsigned int *moved, int gsol) {
    const int b = blockIdx.x, x = blockIdx.y, y = blockIdx.z;
    const int n = o.n, m = o.m;
    const size_t plane = (((size_t)b * numX + x) * numY + y) * n * m;
    S *u = U + plane;
    S *d = D + plane;
    // g[i*ldG + j]: the tile's map, or this solve's own plane (sinh cells)
    const size_t ldG = gsol ? (size_t)m : (size_t)numY * m;
    const S *g = gsol ? G + plane : G + (size_t)x * n * ldG + (size_t)y * m;
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
                                unsigned int *moved, int gsol) {
    const int b = blockIdx.x, x = blockIdx.y, y = blockIdx.z;
    const int n = o.n, m = o.m;
    const size_t sol = ((size_t)b * numX + x) * numY + y;
    const size_t plane = sol * n * m;
    const S *up = Up + plane, *dp = Dp + plane;
    S *un = Un + plane, *dn = Dn + plane;
    const size_t ldG = gsol ? (size_t)m : (size_t)numY * m;
    const S *g = gsol ? G + plane : G + (size_t)x * n * ldG + (size_t)y * m;
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
                                   S *__restrict__ out, int B, int numX, int numY, OuShape o, int gsol) {
    const int n = o.n, m = o.m;
    const size_t total = (size_t)B * numX * o.nox * numY * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int col = (int)(e % m);
        const int y = (int)((e / m) % numY);
        const int sx = (int)((e / ((size_t)m * numY)) % o.nox);
        const size_t bx = e / ((size_t)m * numY * o.nox);  // b*numX + x
        const int x = (int)(bx % numX);
        const size_t plane = (bx * numY + y) * n * m;
        const size_t ldG = gsol ? (size_t)m : (size_t)numY * m;
        const S *g = gsol ? G + plane + col : G + (size_t)x * n * numY * m + (size_t)y * m + col;
        S acc = 0;
        for (int i = sx * o.on; i < (sx + 1) * o.on; ++i)
            acc += (U[plane + (size_t)i * m + col] - D[plane + (size_t)i * m + col]) * g[(size_t)i * ldG];
        out[e] = acc;
    }
}

// Sinh-cell parameters in the I/O type.
template <typename S>
struct FamNl {
    S R_on, dR, a_on, b_on, a_off, b_off;
};

// z = (1/g - R_on) / (R_off - R_on), negative z set to 0, per cell of the maps
// [numX, n, numY*m] (get_nonlinear_ratio_z, :176-182).
template <typename S>
__global__ void fam_nl_z_kernel(const S *__restrict__ G, S *__restrict__ z, size_t total, FamNl<S> p) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const S r = (S)1 / G[e];
        const S v = (r - p.R_on) / p.dR;
        z[e] = v < (S)0 ? (S)0 : v;
    }
}

// Before an iteration: every solve's conductances from the lagged planes
// (deal_v, then 1 / R(V), :142-196), and the lag advanced to the current
// planes.  Gn, U, D, LU, LD are [B, numX, numY, n, m]; z is [numX, n, numY*m].
template <typename S>
__global__ void fam_nl_refresh_kernel(const S *__restrict__ z, const S *__restrict__ U, const S *__restrict__ D,
                                      S *__restrict__ LU, S *__restrict__ LD, S *__restrict__ Gn, int B, int numX,
                                      int numY, int n, int m, FamNl<S> p) {
    const size_t total = (size_t)B * numX * numY * n * m;
    const S eps = (S)1e-5;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int j = (int)(e % m);
        const int i = (int)((e / m) % n);
        const int y = (int)((e / ((size_t)m * n)) % numY);
        const int x = (int)((e / ((size_t)m * n * numY)) % numX);
        S V = LU[e] - LD[e];
        if (V < eps && V > -eps) V = V > (S)0 ? eps : -eps;
        const S Va = V < (S)0 ? -V : V;
        const S zz = z[((size_t)x * n + i) * numY * m + (size_t)y * m + j];
        const S I_on = p.b_on * sinh(Va * p.a_on);
        const S I_off = p.b_off * sinh(Va * p.a_off);
        Gn[e] = (S)1 / (((S)1 - zz) * Va / I_on + zz * Va / I_off);
        LU[e] = U[e];
        LD[e] = D[e];
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

// Host driver shared by the five entry points.  nl: the sinh-cell parameters
// [R_on, R_off, a_on, b_on, a_off, b_off], or null for linear cells.
template <typename S>
int fam_run(bool ir2s, const void *input_v, const void *G_v, int B, OuShape o, int numX, int numY, int iter_times,
            double wire, double load_l, double load_d, double beta, int enable_break, double thr, int ret_V,
            const double *nl, void *out_v, cudaStream_t st, int *done_out = nullptr) {
    const S *input = static_cast<const S *>(input_v);
    const S *G = static_cast<const S *>(G_v);
    S *out = static_cast<S *>(out_v);
    const size_t plane_elems = (size_t)B * numX * numY * o.n * o.m;
    const size_t map_elems = (size_t)numX * o.n * numY * o.m;
    const size_t rsum = (size_t)B * numX * numY * o.n * o.noy, csum = (size_t)B * numX * numY * o.m * o.nox;
    // planes U, D (+ U2, D2 for IR2S), the IR2S line sums, and for sinh cells
    // the cell positions z, the per-solve conductances and the lagged planes
    const size_t elems = (ir2s ? 4 : 2) * plane_elems + (ir2s ? rsum + csum : 0) +
                         (nl ? map_elems + 3 * plane_elems : 0);
    const size_t bytes = elems * sizeof(S) + 256;
    char *buf = nullptr;
    cudaError_t e = lib_malloc_async((void **)&buf, bytes, st);
    if (e != cudaSuccess) return fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    S *U = reinterpret_cast<S *>(buf), *D = U + plane_elems;
    S *next = D + plane_elems;
    S *U2 = nullptr, *D2 = nullptr, *Rs = nullptr, *Cs = nullptr;
    if (ir2s) {
        U2 = next;
        D2 = U2 + plane_elems;
        Rs = D2 + plane_elems;
        Cs = Rs + rsum;
        next = Cs + csum;
    }
    S *Z = nullptr, *Gn = nullptr, *LU = nullptr, *LD = nullptr;
    FamNl<S> p{};
    if (nl) {
        Z = next;
        Gn = Z + map_elems;
        LU = Gn + plane_elems;
        LD = LU + plane_elems;
        p = FamNl<S>{(S)nl[0], (S)(nl[1] - nl[0]), (S)nl[2], (S)nl[3], (S)nl[4], (S)nl[5]};
    }
    unsigned int *moved = reinterpret_cast<unsigned int *>(buf + bytes - 256);
    int rc = FADESIM_OK;
    fam_init_kernel<S><<<fam_grid(plane_elems), 256, 0, st>>>(input, U, D, B, numX, numY, o.n, o.m);
    e = cudaGetLastError();
    if (e == cudaSuccess && ir2s) {
        e = cudaMemcpyAsync(U2, U, 2 * plane_elems * sizeof(S), cudaMemcpyDeviceToDevice, st);  // U2, D2 <- U, D
        if (e == cudaSuccess) e = cudaMemsetAsync(Rs, 0, (rsum + csum) * sizeof(S), st);
    }
    if (e == cudaSuccess && nl) {
        e = cudaMemcpyAsync(LU, U, plane_elems * sizeof(S), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(LD, D, plane_elems * sizeof(S), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) {
            fam_nl_z_kernel<S><<<fam_grid(map_elems), 256, 0, st>>>(G, Z, map_elems, p);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    const S *Gi = nl ? Gn : G;  // what the iterations read
    const int gsol = nl ? 1 : 0;
    int done = 0;
    const dim3 grid(B, numX, numY);
    const int threads = (int)min(1024, ((max(o.n * o.noy, o.m * o.nox) + 31) / 32) * 32);
    for (int it = 0; rc == FADESIM_OK && it < iter_times && B > 0; ++it) {
        unsigned int *mv = enable_break ? moved : nullptr;
        if (mv && (e = cudaMemsetAsync(mv, 0, sizeof(unsigned int), st)) != cudaSuccess) {
            rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
            break;
        }
        if (nl) {
            fam_nl_refresh_kernel<S><<<fam_grid(plane_elems), 256, 0, st>>>(Z, U, D, LU, LD, Gn, B, numX, numY, o.n,
                                                                             o.m, p);
            if ((e = cudaGetLastError()) != cudaSuccess) {
                rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
                break;
            }
        }
        if (ir2s) {
            fam_ir2s_kernel<S><<<grid, threads, 0, st>>>(input, Gi, U, D, U2, D2, Rs, Cs, numX, numY, o, (S)wire,
                                                          (S)load_l, (S)load_d, (S)thr, mv, gsol);
            S *t = U;
            U = U2;
            U2 = t;
            t = D;
            D = D2;
            D2 = t;
        } else {
            fam_gs_sweep_kernel<S><<<grid, threads, 0, st>>>(input, Gi, U, D, numX, numY, o, (S)wire, (S)load_l,
                                                              (S)load_d, (S)beta, (S)thr, mv, gsol);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) {
            rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
            break;
        }
        ++done;
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
        // the currents use the last conductances the iterations used (the linear
        // map when no iteration ran)
        const bool last_nl = nl && done > 0;
        if (ret_V)
            fam_voltage_kernel<S><<<fam_grid(plane_elems), 256, 0, st>>>(U, D, out, plane_elems);
        else
            fam_current_kernel<S><<<fam_grid((size_t)B * numX * o.nox * numY * o.m), 256, 0, st>>>(
                U, D, last_nl ? Gn : G, out, B, numX, numY, o, last_nl ? 1 : 0);
        if ((e = cudaGetLastError()) != cudaSuccess) rc = fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    }
    cudaFreeAsync(buf, st);
    if (done_out) *done_out = done;
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

// Sinh-cell parameters of a family call: null for linear cells, an argument
// error (code in *rc) for an unusable set.  Checks as fadesim_ir_drop_gs_ex.
const double *fam_nl(int enable, const double *params, int n_params, int *rc) {
    *rc = FADESIM_OK;
    if (!enable) return nullptr;
    if (!params || n_params < 6) {
        *rc = fail(FADESIM_E_ARG, "nonlinear_params must hold [R_on, R_off, a_on, b_on, a_off, b_off]");
        return nullptr;
    }
    const double *q = params;
    if (!(q[1] > q[0]) || !(q[0] > 0) || !(q[2] > 0) || !(q[3] > 0) || !(q[4] > 0) || !(q[5] > 0)) {
        *rc = fail(FADESIM_E_ARG, "nonlinear_params need R_off > R_on > 0 and positive a, b");
        return nullptr;
    }
    return params;
}

int fam_dispatch(int dtype, bool ir2s, const void *input, const void *G, int B, OuShape o, int numX, int numY,
                 int iter_times, double wire, double load_l, double load_d, double beta, int enable_break, double thr,
                 int ret_V, const double *nl, void *out, void *stream) {
    if (B == 0) return FADESIM_OK;
    TraceRange trace(ir2s ? "fadesim_ir2s_family" : "fadesim_ir_gs_ou_family");
    cudaStream_t st = (cudaStream_t)stream;
    return dtype == FADESIM_F64
               ? fam_run<double>(ir2s, input, G, B, o, numX, numY, iter_times, wire, load_l, load_d, beta, enable_break,
                                 thr, ret_V, nl, out, st)
               : fam_run<float>(ir2s, input, G, B, o, numX, numY, iter_times, wire, load_l, load_d, beta, enable_break,
                                thr, ret_V, nl, out, st);
}

}  // namespace

// ir_drop_gs's own sweep order with sinh cells (split_arr_matmul.cu:204-333
// with nonlinear_cell_enable): the family's sweep with both loads g_wire, which
// is that sweep (:275, 290) -- same update order, same lagged conductances.
int family_gs_nonlinear(int dtype, const void *input, const void *G, int B, int n, int m, int numX, int numY,
                        int iter_times, double g_wire, double beta, int enable_break, double thr, const double *nl,
                        int ret_V, void *out, int *done, cudaStream_t st) {
    int rc = fam_check(dtype, input, G, out, B, n, m, n, m, numX, numY, iter_times, g_wire);
    if (rc) return rc;
    OuShape o{n, m, n, m, 1, 1, 0};
    *done = 0;
    if (B == 0) return FADESIM_OK;
    TraceRange trace("fadesim_ir_drop_gs_sweeps_nonlinear");
    return dtype == FADESIM_F64
               ? fam_run<double>(false, input, G, B, o, numX, numY, iter_times, g_wire, g_wire, g_wire, beta,
                                 enable_break, thr, ret_V, nl, out, st, done)
               : fam_run<float>(false, input, G, B, o, numX, numY, iter_times, g_wire, g_wire, g_wire, beta,
                                enable_break, thr, ret_V, nl, out, st, done);
}

}  // namespace fadesim

using namespace fadesim;

extern "C" int fadesim_ir_gs_ou_local(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                      int col_size, int numX, int numY, int iter_times, double g_wire,
                                      double g_load_left, double g_load_down, double beta, int enable_break,
                                      double break_threshould, int nonlinear_cell_enable,
                                      const double *nonlinear_params, int n_nonlinear_params, void *out,
                                      void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, row_size, col_size, numX, numY,
                       iter_times, g_wire);
    if (rc) return rc;
    if (!(g_load_left > 0) || !(g_load_down > 0)) return fail(FADESIM_E_ARG, "load conductances must be positive");
    const double *nl = fam_nl(nonlinear_cell_enable, nonlinear_params, n_nonlinear_params, &rc);
    if (rc) return rc;
    OuShape o{row_size, col_size, row_size, col_size, 1, 1, 0};
    return fam_dispatch(dtype, false, input, G, batch_size, o, numX, numY, iter_times, g_wire, g_load_left,
                        g_load_down, beta, enable_break, break_threshould, 0, nl, out, stream);
}

extern "C" int fadesim_ir_gs_ou(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                int col_size, int ou_row_size, int ou_col_size, int numX, int numY, int iter_times,
                                double g_wire, double beta, int enable_break, double break_threshould,
                                int nonlinear_cell_enable, const double *nonlinear_params, int n_nonlinear_params,
                                void *out, void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY,
                       iter_times, g_wire);
    if (rc) return rc;
    const double *nl = fam_nl(nonlinear_cell_enable, nonlinear_params, n_nonlinear_params, &rc);
    if (rc) return rc;
    OuShape o{row_size, col_size, ou_row_size, ou_col_size, row_size / ou_row_size, col_size / ou_col_size, 1};
    return fam_dispatch(dtype, false, input, G, batch_size, o, numX, numY, iter_times, g_wire, g_wire, g_wire, beta,
                        enable_break, break_threshould, 0, nl, out, stream);
}

extern "C" int fadesim_ir2s(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                            int numX, int numY, int iter_times, double r_wire, int enable_break,
                            double break_threshould, int nonlinear_cell_enable, const double *nonlinear_params,
                            int n_nonlinear_params, int ret_V, void *out, void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, row_size, col_size, numX, numY,
                       iter_times, r_wire);
    if (rc) return rc;
    const double *nl = fam_nl(nonlinear_cell_enable, nonlinear_params, n_nonlinear_params, &rc);
    if (rc) return rc;
    OuShape o{row_size, col_size, row_size, col_size, 1, 1, 0};
    return fam_dispatch(dtype, true, input, G, batch_size, o, numX, numY, iter_times, r_wire, r_wire, r_wire, 1.0,
                        enable_break, break_threshould, ret_V ? 1 : 0, nl, out, stream);
}

extern "C" int fadesim_ir2s_ou_local(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                     int col_size, int numX, int numY, int iter_times, double r_wire,
                                     double r_load_left, double r_load_down, int enable_break,
                                     double break_threshould, int nonlinear_cell_enable,
                                     const double *nonlinear_params, int n_nonlinear_params, void *out,
                                     void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, row_size, col_size, numX, numY,
                       iter_times, r_wire);
    if (rc) return rc;
    if (!(r_load_left >= 0) || !(r_load_down >= 0)) return fail(FADESIM_E_ARG, "load resistances must be >= 0");
    const double *nl = fam_nl(nonlinear_cell_enable, nonlinear_params, n_nonlinear_params, &rc);
    if (rc) return rc;
    OuShape o{row_size, col_size, row_size, col_size, 1, 1, 0};
    return fam_dispatch(dtype, true, input, G, batch_size, o, numX, numY, iter_times, r_wire, r_load_left,
                        r_load_down, 1.0, enable_break, break_threshould, 0, nl, out, stream);
}

extern "C" int fadesim_ir2s_ou(int dtype, const void *input, const void *G, int batch_size, int row_size,
                               int col_size, int ou_row_size, int ou_col_size, int numX, int numY, int iter_times,
                               double r_wire, int enable_break, double break_threshould, int nonlinear_cell_enable,
                               const double *nonlinear_params, int n_nonlinear_params, void *out, void *stream) {
    int rc = fam_check(dtype, input, G, out, batch_size, row_size, col_size, ou_row_size, ou_col_size, numX, numY,
                       iter_times, r_wire);
    if (rc) return rc;
    const double *nl = fam_nl(nonlinear_cell_enable, nonlinear_params, n_nonlinear_params, &rc);
    if (rc) return rc;
    OuShape o{row_size, col_size, ou_row_size, ou_col_size, row_size / ou_row_size, col_size / ou_col_size, 1};
    return fam_dispatch(dtype, true, input, G, batch_size, o, numX, numY, iter_times, r_wire, r_wire, r_wire, 1.0,
                        enable_break, break_threshould, 0, nl, out, stream);
}
