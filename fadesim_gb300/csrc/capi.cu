// C ABI of the solver (include/fadesim_gb300.h): argument checks, method
// choice, scratch and launches.  Scratch is stream-ordered (from the library's
// memory pool, freed with cudaFreeAsync, on the caller's stream), so a call
// never synchronises unless the caller asks for stats or the reference's
// delta break.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <mutex>
#include <string>

#include "kernels.h"
#include "trace.h"

using namespace fadesim;

static thread_local std::string g_err;

static int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CUDA_TRY(x)                                                                            \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess) return fail(FADESIM_E_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace fadesim {
int report_error(int code, const char *msg) { return fail(code, msg); }

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[MAX_DEVICES] = {};

cudaError_t lib_pool(cudaMemPool_t *pool) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        e = cudaMemPoolCreate(&g_pools[dev], &props);
        if (e != cudaSuccess) {
            g_pools[dev] = nullptr;
            return e;
        }
        // keep what the pool has mapped between calls (fadesim_release_memory trims it)
        unsigned long long keep = ~0ull;
        e = cudaMemPoolSetAttribute(g_pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(g_pools[dev]);  // nothing was allocated from it yet
            g_pools[dev] = nullptr;
            return e;
        }
    }
    *pool = g_pools[dev];
    return cudaSuccess;
}
}  // namespace

cudaError_t lib_malloc_async(void **p, size_t bytes, cudaStream_t st) {
    cudaMemPool_t pool;
    cudaError_t e = lib_pool(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, st);
}
}  // namespace fadesim

extern "C" int fadesim_release_memory(void) {
    std::lock_guard<std::mutex> lock(fadesim::g_pool_mutex);
    for (int d = 0; d < fadesim::MAX_DEVICES; ++d) {
        if (!fadesim::g_pools[d]) continue;
        const cudaError_t e = cudaMemPoolTrimTo(fadesim::g_pools[d], 0);
        if (e != cudaSuccess) return fail(FADESIM_E_CUDA, std::string("cudaMemPoolTrimTo: ") + cudaGetErrorString(e));
    }
    return FADESIM_OK;
}

extern "C" const char *fadesim_last_error(void) { return g_err.c_str(); }
extern "C" const char *fadesim_version(void) { return "fadesim_gb300 0.1 (sm_103a)"; }

namespace {

struct Scratch {
    void *p = nullptr;
    cudaStream_t st = nullptr;
    ~Scratch() {
        if (p) cudaFreeAsync(p, st);
    }
};

// Margin of the adaptive precision schedule (FADESIM_PRECISE_MARGIN, default
// 4): an iteration is made precise when its predicted error estimate is
// within this factor of the tolerance.
float precise_margin() {
    static const float v = [] {
        const char *e = getenv("FADESIM_PRECISE_MARGIN");
        const float f = e ? (float)atof(e) : 4.f;
        return f > 0.f ? f : 4.f;
    }();
    return v;
}

int device_sms() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

// Work split: whole tiles per item when there are enough tiles, else vectors
// of one tile spread over several items.
void plan_items(SolveArgs &a, int grid, int vectors_per_cta) {
    const long long tiles = (long long)a.numX * a.numY;
    int vchunk;
    if (vectors_per_cta > 0) {
        vchunk = vectors_per_cta;
    } else {
        long long want_items = 2LL * grid;
        long long chunks = (want_items + tiles - 1) / tiles;
        if (chunks < 1) chunks = 1;
        if (chunks > a.B) chunks = a.B;
        vchunk = (int)((a.B + chunks - 1) / chunks);
    }
    if (vchunk < 1) vchunk = 1;
    if (vchunk > a.B) vchunk = a.B;
    a.vchunk = vchunk;
    a.nchunks = (a.B + vchunk - 1) / vchunk;
    a.nitems = tiles * a.nchunks;
}

// Set by the host-buffer entry around each group's call: the group's device
// counters (zeroed by the caller), so that no group reads its counters back
// and the pipeline never waits on the host.
thread_local DevStats *g_group_stats = nullptr;

int finish_stats(DevStats *dst, fadesim_solve_stats *stats, cudaStream_t st) {
    if (!stats) return FADESIM_OK;
    DevStats h;
    CUDA_TRY(cudaMemcpyAsync(&h, dst, sizeof(h), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    stats->solves = (int64_t)h.solves;
    stats->iters_sum = (int64_t)h.iters_sum;
    stats->iters_max = h.iters_max;
    stats->status_or = h.status_or;
    stats->warm_rejected = (int64_t)h.warm_rejected;
    return FADESIM_OK;
}

int run_converging(int method, int dtype, SolveArgs a, const fadesim_solve_opts *opts, fadesim_solve_stats *stats,
                   cudaStream_t st) {
    const int L = a.n > a.m ? a.n : a.m;
    a.ctl.tol_v = (opts && opts->tol_v > 0) ? (float)opts->tol_v : 1e-8f;
    a.ctl.residual_period = opts ? opts->residual_period : 0;  // 0: adaptive schedule
    a.ctl.residual_ff = (opts && opts->residual_kind == 1) ? 0 : 1;
    a.ctl.precise_margin = precise_margin();
    a.fp32_limit = (opts && opts->fp32_limit) ? 1 : 0;
    const int sms = device_sms();
    int grid = 0, ld = 0;
    size_t scratch_floats = 0;
    int cld = 0;
    if (method == FADESIM_METHOD_LINE) {
        ld = line_relax_ld(a.n, a.m);
        cld = ld ? 0 : cluster_relax_ld(a.n, a.m);
        if (!ld && !cld) return fail(FADESIM_E_UNSUPPORTED, "line relaxation in this build handles rows, cols <= 512");
        const int want = opts ? opts->kernel_ld : 0;  // a forced layout (the autotuner's shape axis)
        if (want) {
            if (want != 32 && want != 64 && want != 128 && want != 256 && want != 512)
                return fail(FADESIM_E_ARG, "kernel_ld must be 0, 32, 64, 128, 256 or 512");
            if (L > want) return fail(FADESIM_E_ARG, "kernel_ld is smaller than the tile");
            ld = want <= 128 ? want : 0;
            cld = want > 128 ? want : 0;
        }
        a.ctl.max_iters = (opts && opts->max_iters > 0) ? opts->max_iters : 400;
        a.ctl.omega = (opts && opts->omega > 0) ? (float)opts->omega : 0.f;
        if (ld) {
            CUDA_TRY(line_relax_prepare(ld, dtype));
            int per_sm = 0;
            CUDA_TRY(line_relax_occupancy(ld, dtype, &per_sm));
            if (per_sm < 1) return fail(FADESIM_E_CUDA, "line relaxation kernel does not fit on this device");
            grid = per_sm * sms;
            plan_items(a, grid, opts ? opts->vectors_per_cta : 0);
            if ((long long)grid > a.nitems) grid = (int)a.nitems;
            scratch_floats = line_relax_scratch_floats_per_cta(ld) * grid;
        } else {
            const int csize = cluster_relax_size(cld);
            int clusters = 0;
            CUDA_TRY(cluster_relax_occupancy(cld, dtype, &clusters));
            if (clusters < 1)
                return fail(FADESIM_E_UNSUPPORTED, "this device cannot co-schedule the cluster the tile size needs");
            plan_items(a, clusters, opts ? opts->vectors_per_cta : 0);
            if ((long long)clusters > a.nitems) clusters = (int)a.nitems;
            grid = clusters * csize;
            scratch_floats = cluster_relax_scratch_floats_per_cta(cld) * grid;
        }
    } else {
        if (L > 512) return fail(FADESIM_E_UNSUPPORTED, "red-black SOR in this build handles rows, cols <= 512");
        a.ctl.max_iters = (opts && opts->max_iters > 0) ? opts->max_iters : 20000;
        a.ctl.omega = (opts && opts->omega > 0) ? (float)opts->omega
                                                : (float)(2.0 / (1.0 + sin(M_PI / (2.0 * L + 1.0))));
        cld = rbsor_cluster_ld(a.n, a.m);
        const int want = opts ? opts->kernel_ld : 0;  // a forced layout: 128 single-CTA, 256 / 512 clusters
        if (want) {
            if (want != 128 && want != 256 && want != 512)
                return fail(FADESIM_E_ARG, "kernel_ld must be 0, 128, 256 or 512 for red-black SOR");
            if (L > want) return fail(FADESIM_E_ARG, "kernel_ld is smaller than the tile");
            cld = want > 128 ? want : 0;
        }
        if (a.init && cld)
            return fail(FADESIM_E_UNSUPPORTED, "red-black SOR starts from given planes on tiles up to 128 x 128");
        if (!cld) {
            CUDA_TRY(rbsor_prepare(dtype));
            grid = sms;
            plan_items(a, grid, opts ? opts->vectors_per_cta : 0);
            if ((long long)grid > a.nitems) grid = (int)a.nitems;
        } else {
            int clusters = 0;
            CUDA_TRY(rbsor_cluster_occupancy(cld, dtype, &clusters));
            if (clusters < 1)
                return fail(FADESIM_E_UNSUPPORTED, "this device cannot co-schedule the cluster the tile size needs");
            plan_items(a, clusters, opts ? opts->vectors_per_cta : 0);
            if ((long long)clusters > a.nitems) clusters = (int)a.nitems;
            grid = clusters * rbsor_cluster_size(cld);
            scratch_floats = rbsor_cluster_scratch_floats_per_cta(cld) * grid;
        }
    }
    Scratch scr;
    scr.st = st;
    const size_t bytes = scratch_floats * sizeof(float) + sizeof(DevStats) + 256;
    CUDA_TRY(lib_malloc_async(&scr.p, bytes, st));
    DevStats *dst = g_group_stats ? g_group_stats : reinterpret_cast<DevStats *>(scr.p);
    a.stats = dst;
    a.scratch = reinterpret_cast<float *>(reinterpret_cast<char *>(scr.p) + 256);
    if (!g_group_stats) CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(DevStats), st));
    if (method == FADESIM_METHOD_LINE && ld) {
        CUDA_TRY(launch_line_relax(a, ld, dtype, grid, st));
    } else if (method == FADESIM_METHOD_LINE) {
        CUDA_TRY(launch_cluster_relax(a, cld, dtype, grid, st));
    } else if (cld) {
        CUDA_TRY(launch_rbsor_cluster(a, cld, dtype, grid, st));
    } else {
        CUDA_TRY(launch_rbsor(a, dtype, grid, st));
    }
    return g_group_stats ? FADESIM_OK : finish_stats(dst, stats, st);
}

int run_sweeps(int dtype, SolveArgs a, int iter_times, double gw, double beta, int enable_break, double thr,
               fadesim_solve_stats *stats, int *iters_out, cudaStream_t st) {
    if (a.n > 1024 || a.m > 1024) return fail(FADESIM_E_ARG, "row_size and col_size must be <= 1024");
    const size_t es = dtype == FADESIM_F64 ? 8 : 4;
    const size_t plane = (size_t)a.B * a.numX * a.numY * a.n * a.m * es;
    Scratch scr;
    scr.st = st;
    CUDA_TRY(lib_malloc_async(&scr.p, 2 * plane + 256, st));
    unsigned int *moved = reinterpret_cast<unsigned int *>(scr.p);
    void *U = reinterpret_cast<char *>(scr.p) + 256;
    void *D = reinterpret_cast<char *>(U) + plane;
    CUDA_TRY(launch_sweep_init(a, dtype, U, D, st));
    int done = 0;
    for (int it = 0; it < iter_times; ++it) {
        if (enable_break) CUDA_TRY(cudaMemsetAsync(moved, 0, sizeof(unsigned int), st));
        CUDA_TRY(launch_sweep(a, dtype, U, D, gw, beta, thr, enable_break ? moved : nullptr, st));
        ++done;
        if (enable_break) {
            unsigned int h = 0;
            CUDA_TRY(cudaMemcpyAsync(&h, moved, sizeof(h), cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            if (h == 0) break;
        }
    }
    CUDA_TRY(launch_sweep_output(a, dtype, U, D, st));
    if (iters_out) {
        // every solve ran the same number of sweeps
        const size_t nsol = (size_t)a.B * a.numX * a.numY;
        std::string tmp(nsol * sizeof(int), '\0');
        int *h = reinterpret_cast<int *>(&tmp[0]);
        for (size_t k = 0; k < nsol; ++k) h[k] = done;
        CUDA_TRY(cudaMemcpyAsync(iters_out, h, nsol * sizeof(int), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (stats) {
        stats->solves = (int64_t)a.B * a.numX * a.numY;
        stats->iters_sum = stats->solves * done;
        stats->iters_max = done;
        stats->status_or = (enable_break && done < iter_times) ? FADESIM_ST_CONVERGED : FADESIM_ST_MAXITER;
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    return FADESIM_OK;
}

}  // namespace

namespace fadesim {
void set_group_stats(DevStats *d) { g_group_stats = d; }
}  // namespace fadesim

static thread_local const float *g_warm_init = nullptr;

extern "C" int fadesim_ir_drop_gs_ex(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                     int col_size, int numX, int numY, int iter_times, double g_wire, double beta,
                                     int enable_break, double break_threshould, int nonlinear_cell_enable,
                                     const double *nonlinear_params, int n_nonlinear_params, int ret_V, void *out,
                                     const fadesim_solve_opts *opts, fadesim_solve_stats *stats,
                                     int *per_solve_iters, void *stream) {
    TraceRange trace("fadesim_ir_drop_gs_ex");
    g_err.clear();
    if (dtype != FADESIM_F32 && dtype != FADESIM_F64) return fail(FADESIM_E_ARG, "dtype must be f32 or f64");
    if (batch_size == 0 && row_size >= 2 && col_size >= 2) {
        if (stats) *stats = fadesim_solve_stats{0, 0, 0, 0, 0};
        return FADESIM_OK;  // nothing to solve; empty tensors may carry null pointers
    }
    if (!input || !G || !out) return fail(FADESIM_E_ARG, "input, G and out must be device pointers");
    if (row_size < 2) return fail(FADESIM_E_ARG, "row_size should be >=2");
    if (col_size < 2) return fail(FADESIM_E_ARG, "col_size should be >=2");
    if (batch_size < 0 || numX < 1 || numY < 1) return fail(FADESIM_E_ARG, "batch_size >= 0, numX >= 1, numY >= 1");
    if (!(g_wire > 0) || !isfinite(g_wire)) return fail(FADESIM_E_ARG, "g_wire must be positive and finite");
    if (nonlinear_cell_enable) {
        if (!nonlinear_params || n_nonlinear_params < 6)
            return fail(FADESIM_E_ARG, "nonlinear_params must hold [R_on, R_off, a_on, b_on, a_off, b_off]");
        const double *q = nonlinear_params;
        if (!(q[1] > q[0]) || !(q[2] > 0) || !(q[3] > 0) || !(q[4] > 0) || !(q[5] > 0))
            return fail(FADESIM_E_ARG, "nonlinear_params need R_off > R_on and positive a, b");
    }
    if (stats) *stats = fadesim_solve_stats{0, 0, 0, 0, 0};
    if (batch_size == 0) return FADESIM_OK;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    SolveArgs a{};
    a.input = input;
    a.G = G;
    a.out = out;
    a.B = batch_size;
    a.n = row_size;
    a.m = col_size;
    a.numX = numX;
    a.numY = numY;
    a.gw = (float)g_wire;
    a.ret_V = ret_V == 2 ? 2 : (ret_V ? 1 : 0);
    a.iters_out = per_solve_iters;
    a.init = g_warm_init;
    a.f64 = dtype == FADESIM_F64 ? 1 : 0;
    if (a.init && ret_V == 1) return fail(FADESIM_E_UNSUPPORTED, "warm starts return currents or both planes");
    if (nonlinear_cell_enable) {
        const double *q = nonlinear_params;
        a.ctl.nl = 1;
        a.ctl.nl_R_on = (float)q[0];
        a.ctl.nl_inv_dR = (float)(1.0 / (q[1] - q[0]));
        a.ctl.nl_a_on = (float)q[2];
        a.ctl.nl_a_off = (float)q[4];
        a.ctl.nl_r0_on = (float)(1.0 / (q[2] * q[3]));
        a.ctl.nl_r0_off = (float)(1.0 / (q[4] * q[5]));
        a.ctl.nl_single_a = q[2] == q[4] ? 1 : 0;
    }
    if (opts && opts->read_noise_sigma > 0) {
        a.ctl.noise_sigma = (float)opts->read_noise_sigma;
        a.ctl.noise_seed = opts->noise_seed;
    }
    int method = opts ? opts->method : FADESIM_METHOD_AUTO;
    if (method == FADESIM_METHOD_LINE_COARSE) {
        // the line method; its kernel takes the coarse correction on the tiles it suits
        a.two_level = 1;
        method = FADESIM_METHOD_LINE;
    }
    if (method == FADESIM_METHOD_AUTO)
        method = (line_relax_ld(row_size, col_size) || cluster_relax_ld(row_size, col_size)) ? FADESIM_METHOD_LINE
                                                                                           : FADESIM_METHOD_SWEEPS;
    if (nonlinear_cell_enable && method == FADESIM_METHOD_SWEEPS) {
        // the reference's own sweeps with per-sweep re-linearised cells
        if (iter_times < 0) return fail(FADESIM_E_ARG, "iter_times must be >= 0");
        if (ret_V == 2) return fail(FADESIM_E_UNSUPPORTED, "ret_V = 2 is not available for the sweep method");
        if (row_size > 1024 || col_size > 1024) return fail(FADESIM_E_ARG, "row_size and col_size must be <= 1024");
        if (a.ctl.noise_sigma > 0) return fail(FADESIM_E_UNSUPPORTED, "read noise applies to the line method's currents");
        int done = 0;
        const int rc = family_gs_nonlinear(dtype, input, G, batch_size, row_size, col_size, numX, numY, iter_times,
                                           g_wire, beta, enable_break, break_threshould, nonlinear_params,
                                           ret_V ? 1 : 0, out, &done, st);
        if (rc != FADESIM_OK) return rc;
        if (per_solve_iters) {
            const size_t nsol = (size_t)batch_size * numX * numY;
            std::string tmp(nsol * sizeof(int), '\0');
            int *h = reinterpret_cast<int *>(&tmp[0]);
            for (size_t k = 0; k < nsol; ++k) h[k] = done;
            CUDA_TRY(cudaMemcpyAsync(per_solve_iters, h, nsol * sizeof(int), cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaStreamSynchronize(st));
        }
        if (stats) {
            stats->solves = (int64_t)batch_size * numX * numY;
            stats->iters_sum = stats->solves * done;
            stats->iters_max = done;
            stats->status_or = (enable_break && done < iter_times) ? FADESIM_ST_CONVERGED : FADESIM_ST_MAXITER;
            CUDA_TRY(cudaStreamSynchronize(st));
        }
        return FADESIM_OK;
    }
    if (nonlinear_cell_enable && method != FADESIM_METHOD_LINE)
        return fail(FADESIM_E_UNSUPPORTED, "nonlinear cells are solved by the line method or the sweep order");
    if (a.ctl.noise_sigma > 0 && (method != FADESIM_METHOD_LINE || ret_V))
        return fail(FADESIM_E_UNSUPPORTED, "read noise applies to the line method's currents");
    switch (method) {
        case FADESIM_METHOD_LINE:
        case FADESIM_METHOD_RBSOR:
            return run_converging(method, dtype, a, opts, stats, st);
        case FADESIM_METHOD_SWEEPS:
            if (iter_times < 0) return fail(FADESIM_E_ARG, "iter_times must be >= 0");
            return run_sweeps(dtype, a, iter_times, g_wire, beta, enable_break, break_threshould, stats,
                              per_solve_iters, st);
    }
    return fail(FADESIM_E_ARG, "unknown method");
}

extern "C" int fadesim_ir_drop_gs_f32(const float *input, const float *G, int batch_size, int row_size, int col_size,
                                      int numX, int numY, int iter_times, double g_wire, double beta,
                                      int enable_break, double break_threshould, int nonlinear_cell_enable,
                                      const double *nonlinear_params, int n_nonlinear_params, int ret_V, float *out,
                                      void *stream) {
    return fadesim_ir_drop_gs_ex(FADESIM_F32, input, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire,
                                 beta, enable_break, break_threshould, nonlinear_cell_enable, nonlinear_params,
                                 n_nonlinear_params, ret_V, out, nullptr, nullptr, nullptr, stream);
}

extern "C" int fadesim_ir_drop_gs_f64(const double *input, const double *G, int batch_size, int row_size,
                                      int col_size, int numX, int numY, int iter_times, double g_wire, double beta,
                                      int enable_break, double break_threshould, int nonlinear_cell_enable,
                                      const double *nonlinear_params, int n_nonlinear_params, int ret_V, double *out,
                                      void *stream) {
    return fadesim_ir_drop_gs_ex(FADESIM_F64, input, G, batch_size, row_size, col_size, numX, numY, iter_times, g_wire,
                                 beta, enable_break, break_threshould, nonlinear_cell_enable, nonlinear_params,
                                 n_nonlinear_params, ret_V, out, nullptr, nullptr, nullptr, stream);
}

extern "C" int fadesim_ir_drop_gs_warm(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                       int col_size, int numX, int numY, double g_wire, const float *init,
                                       int nonlinear_cell_enable, const double *nonlinear_params,
                                       int n_nonlinear_params, void *out, const fadesim_solve_opts *opts,
                                       fadesim_solve_stats *stats, int *per_solve_iters, void *stream) {
    if (!init) return fail(FADESIM_E_ARG, "init planes required");
    fadesim_solve_opts o = opts ? *opts : fadesim_solve_opts{};
    if (o.method == FADESIM_METHOD_AUTO) o.method = FADESIM_METHOD_LINE;
    if (o.method != FADESIM_METHOD_LINE && o.method != FADESIM_METHOD_LINE_COARSE && o.method != FADESIM_METHOD_RBSOR)
        return fail(FADESIM_E_UNSUPPORTED, "warm starts apply to the line and red-black SOR methods");
    g_warm_init = init;
    const int rc = fadesim_ir_drop_gs_ex(dtype, input, G, batch_size, row_size, col_size, numX, numY, 0, g_wire, 1.0,
                                         0, 0.0, nonlinear_cell_enable, nonlinear_params, n_nonlinear_params, 0, out,
                                         &o, stats, per_solve_iters, stream);
    g_warm_init = nullptr;
    return rc;
}
