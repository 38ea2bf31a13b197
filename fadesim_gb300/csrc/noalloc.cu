// fadesim_ir_drop_gs_noalloc_f32: the line-relaxation solve without any
// device allocation, for callers that cannot call cudaMalloc.
//
// Who needs it: code that runs where allocation is not allowed or not
// possible -- inside a CUDA graph being captured by someone else, inside a
// host callback or a real-time loop with a no-allocation rule, or a host
// program with a fixed device-memory budget that must not grow after start-up.
// Those callers pass inputs and outputs they already own; the solver's scratch
// (per-CTA line pivots and the call's counters) then lives in one file-scope
// device array, fixed at FADESIM_NOALLOC_SCRATCH_BYTES, which every GPU that
// loads this library holds until the process exits.
//
// Rules of use:
// * The first call on each device looks up the array's device address with
//   cudaGetSymbolAddress (that device current); make that first call before
//   any stream capture.  The address is kept for the process: do not use this
//   entry across a cudaDeviceReset (the module, and the array with it, may be
//   reloaded elsewhere).
// * The solve stops at tol 1e-8 V (estimated max node error) or after 400 line
//   iterations; fadesim_noalloc_last_status reads the finished call's counters
//   (solves, iterations, status bits) back from the array without allocating.
// * All calls share the array and it keeps the last call's contents: calls
//   that overlap on the GPU (other streams, other host threads) race on it.
//   The counters are cleared at the start of every call; the pivots are
//   rewritten before use.
// * Tiles up to 128 x 128 only (the shared-memory-resident line kernel); the
//   grid is capped by how many CTA pivot slots fit in the array.
#include <math.h>

#include <mutex>
#include <string>

#include "kernels.h"

#define FADESIM_NOALLOC_SCRATCH_BYTES (24u << 20)

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[FADESIM_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {};
thread_local std::string g_noalloc_err;

int noalloc_fail(int code, const std::string &m) {
    g_noalloc_err = m;
    return code;
}

// Device address of the static scratch on the current device (set up once).
cudaError_t scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" const char *fadesim_noalloc_last_error(void) { return g_noalloc_err.c_str(); }

extern "C" size_t fadesim_noalloc_scratch_bytes(void) { return FADESIM_NOALLOC_SCRATCH_BYTES; }

extern "C" int fadesim_ir_drop_gs_noalloc_f32(const float *input, const float *G, int batch_size, int row_size,
                                              int col_size, int numX, int numY, double g_wire, float *out,
                                              void *stream) {
    using namespace fadesim;
    g_noalloc_err.clear();
    if (row_size < 2 || col_size < 2 || row_size > 128 || col_size > 128)
        return noalloc_fail(FADESIM_E_ARG,
                            "fadesim_ir_drop_gs_noalloc_f32: row_size and col_size must be in 2..128 "
                            "(its fixed scratch serves the 128x128 shared-memory line solver)");
    if (batch_size < 0 || numX < 1 || numY < 1)
        return noalloc_fail(FADESIM_E_ARG, "fadesim_ir_drop_gs_noalloc_f32: batch_size >= 0, numX >= 1, numY >= 1");
    if (!(g_wire > 0) || !isfinite(g_wire))
        return noalloc_fail(FADESIM_E_ARG, "fadesim_ir_drop_gs_noalloc_f32: g_wire must be positive and finite");
    if (batch_size == 0) return FADESIM_OK;
    if (!input || !G || !out) return noalloc_fail(FADESIM_E_ARG, "fadesim_ir_drop_gs_noalloc_f32: null pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

    const int ld = line_relax_ld(row_size, col_size);
    const size_t per_cta = line_relax_scratch_floats_per_cta(ld) * sizeof(float);
    const size_t stats_bytes = 256;
    const long long max_ctas = (long long)((FADESIM_NOALLOC_SCRATCH_BYTES - stats_bytes) / per_cta);
    if (max_ctas < 1) return noalloc_fail(FADESIM_E_ARG, "fadesim_ir_drop_gs_noalloc_f32: tile too large for the scratch");

    void *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess)
        return noalloc_fail(FADESIM_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    if ((e = line_relax_prepare(ld, FADESIM_F32)) != cudaSuccess)
        return noalloc_fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    int per_sm = 0, dev = 0, sms = 0;
    if ((e = line_relax_occupancy(ld, FADESIM_F32, &per_sm)) != cudaSuccess)
        return noalloc_fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    if (per_sm < 1)
        return noalloc_fail(FADESIM_E_CUDA, "fadesim_ir_drop_gs_noalloc_f32: line relaxation kernel does not fit on "
                                            "this device");
    if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return noalloc_fail(FADESIM_E_CUDA, std::string("device query: ") + cudaGetErrorString(e));
    if (sms < 1) return noalloc_fail(FADESIM_E_CUDA, "fadesim_ir_drop_gs_noalloc_f32: device reports no SMs");

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
    a.ret_V = 0;
    a.f64 = 0;
    a.ctl.tol_v = 1e-8f;
    a.ctl.max_iters = 400;
    a.ctl.residual_period = 0;  // adaptive, as the default of the allocating entry
    a.ctl.omega = 0.f;
    a.ctl.residual_ff = 1;
    a.ctl.precise_margin = 4.f;
    long long grid = (long long)per_sm * sms;
    if (grid > max_ctas) grid = max_ctas;
    // whole tiles per work item when tiles are plentiful, else split vectors
    const long long tiles = (long long)numX * numY;
    long long chunks = (2 * grid + tiles - 1) / tiles;
    if (chunks < 1) chunks = 1;
    if (chunks > batch_size) chunks = batch_size;
    a.vchunk = (int)((batch_size + chunks - 1) / chunks);
    a.nchunks = (batch_size + a.vchunk - 1) / a.vchunk;
    a.nitems = tiles * a.nchunks;
    if (grid > a.nitems) grid = a.nitems;
    a.stats = reinterpret_cast<DevStats *>(base);
    a.scratch = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(base) + stats_bytes);
    a.iters_out = nullptr;
    if ((e = cudaMemsetAsync(a.stats, 0, sizeof(DevStats), st)) != cudaSuccess)
        return noalloc_fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    if ((e = launch_line_relax(a, ld, FADESIM_F32, (int)grid, st)) != cudaSuccess)
        return noalloc_fail(FADESIM_E_CUDA, cudaGetErrorString(e));
    return FADESIM_OK;
}

extern "C" int fadesim_noalloc_last_status(fadesim_solve_stats *stats, void *stream) {
    using namespace fadesim;
    g_noalloc_err.clear();
    if (!stats) return noalloc_fail(FADESIM_E_ARG, "fadesim_noalloc_last_status: stats must not be NULL");
    *stats = fadesim_solve_stats{0, 0, 0, 0, 0};
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    DevStats h{};
    cudaError_t e = cudaMemcpyFromSymbolAsync(&h, g_noalloc_scratch, sizeof(DevStats), 0, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return noalloc_fail(FADESIM_E_CUDA, std::string("fadesim_noalloc_last_status: ") + cudaGetErrorString(e));
    stats->solves = (int64_t)h.solves;
    stats->iters_sum = (int64_t)h.iters_sum;
    stats->iters_max = h.iters_max;
    stats->status_or = h.status_or;
    stats->warm_rejected = (int64_t)h.warm_rejected;
    return FADESIM_OK;
}
