// Host-buffer entry of the solver: the caller's inputs and outputs stay in host
// memory and the library moves them, pipelined over groups of tiles so that the
// copies of one group overlap the solve of another.
//
// The reference's ir_drop_gs (split_arr_matmul.cu:204-333) takes device
// tensors and leaves the transfers to its callers, which move data with
// .to(device) before the call and .cpu() after it
// (splitArrayArithmetic.py:1082, 1124), so copy and solve serialise.  Tiles
// are independent, so the numX axis splits into groups; group g runs on slot
// stream g % NSLOT as
//   H2D(G_g, input_g) -> solve(g) -> D2H(out_g)
// with its own device buffers, and the slot streams run concurrently: while one
// group solves, the next one's inputs come in and the previous one's currents
// go out, on the two copy engines.  input [B, numX, rows] and out [B, numX, ...]
// are strided by numX in host memory; a group's slice is one pitched copy.
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "trace.h"

namespace {

constexpr int NSLOT = 3;
constexpr int MAX_DEVICES = 64;

// The slot streams of each device, created on first use and kept for the
// process (calls from several host threads share them: their work then
// queues behind each other, each call with its own buffers).
std::mutex g_stream_mutex;
cudaStream_t g_streams[MAX_DEVICES][NSLOT] = {};

cudaError_t slot_streams(cudaStream_t *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_stream_mutex);
    for (int s = 0; s < NSLOT; ++s) {
        if (!g_streams[dev][s]) {
            e = cudaStreamCreateWithFlags(&g_streams[dev][s], cudaStreamNonBlocking);
            if (e != cudaSuccess) {
                g_streams[dev][s] = nullptr;
                return e;
            }
        }
        out[s] = g_streams[dev][s];
    }
    return cudaSuccess;
}

// This call's slot buffers: freed (stream-ordered, back to the library's
// pool) once the slots' work is done, on every return path.
struct SlotSet {
    cudaStream_t st[NSLOT] = {};
    void *buf[NSLOT] = {};
    int n = 0;
    ~SlotSet() {
        for (int s = 0; s < n; ++s) {
            cudaStreamSynchronize(st[s]);
            if (buf[s]) cudaFreeAsync(buf[s], st[s]);
        }
        for (int s = 0; s < n; ++s) cudaStreamSynchronize(st[s]);
    }
};

// The group counters of one call, returned to the library's pool on every
// return path (after the caller's stream has passed them).
struct GroupStats {
    fadesim::DevStats *d = nullptr;
    cudaStream_t st = nullptr;
    ~GroupStats() {
        if (d) cudaFreeAsync(d, st);
    }
};

int fail_cuda(const char *what, cudaError_t e) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    return fadesim::report_error(FADESIM_E_CUDA, msg.c_str());
}

}  // namespace

extern "C" int fadesim_ir_drop_gs_host(int dtype, const void *input, const void *G, int batch_size, int row_size,
                                       int col_size, int numX, int numY, int iter_times, double g_wire, double beta,
                                       int enable_break, double break_threshould, int nonlinear_cell_enable,
                                       const double *nonlinear_params, int n_nonlinear_params, int ret_V, void *out,
                                       const fadesim_solve_opts *opts, fadesim_solve_stats *stats, int group_x,
                                       void *stream) {
    fadesim::TraceRange trace("fadesim_ir_drop_gs_host");
    if (dtype != FADESIM_F32 && dtype != FADESIM_F64)
        return fadesim::report_error(FADESIM_E_ARG, "dtype must be FADESIM_F32 or FADESIM_F64");
    if (batch_size < 0 || numX < 0 || numY < 0 || row_size < 2 || col_size < 2)
        return fadesim::report_error(FADESIM_E_ARG, "row_size and col_size must be >= 2, counts >= 0");
    if (ret_V < 0 || ret_V > 2) return fadesim::report_error(FADESIM_E_ARG, "ret_V must be 0, 1 or 2");
    if (stats) memset(stats, 0, sizeof(*stats));
    if (batch_size == 0 || numX == 0 || numY == 0) return FADESIM_OK;
    if (!input || !G || !out) return fadesim::report_error(FADESIM_E_ARG, "null host buffer");

    const size_t es = dtype == FADESIM_F64 ? 8 : 4;
    const size_t n = (size_t)row_size, m = (size_t)col_size;
    // elements per x of each array
    const size_t g_x = n * (size_t)numY * m;
    const size_t in_x = n;
    const size_t out_x = ret_V == 2 ? (size_t)numY * 2 * n * m : ret_V == 1 ? (size_t)numY * n * m : (size_t)numY * m;

    // groups of numX: automatic -- about 8 groups in whole multiples of the SM
    // count of tiles, with a first and a last group of one SM count each, so
    // that the copy-in before the first solve and the copy-out after the last
    // one (the only copies nothing overlaps) are short -- or group_x each
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    std::vector<int> gx0;  // first x of every group, then numX
    if (group_x <= 0) {
        const long long tiles = (long long)numX * numY;
        long long per = (tiles + 7) / 8;
        per = ((per + sms - 1) / sms) * sms;
        group_x = (int)((per + numY - 1) / numY);
        const int edge = (sms + numY - 1) / numY;  // x values of one SM count of tiles
        if (group_x > numX) group_x = numX;
        if (numX > 2 * edge + group_x) {
            gx0.push_back(0);
            for (int x = edge; x < numX - edge; x += group_x) gx0.push_back(x);
            gx0.push_back(numX - edge);
        }
    }
    if (group_x > numX) group_x = numX;
    if (gx0.empty())
        for (int x = 0; x < numX; x += group_x) gx0.push_back(x);
    const int ngroups = (int)gx0.size();
    gx0.push_back(numX);

    const size_t gbytes = (size_t)group_x * g_x * es;
    const size_t ibytes = (size_t)batch_size * group_x * in_x * es;
    const size_t obytes = (size_t)batch_size * group_x * out_x * es;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };

    cudaStream_t caller = (cudaStream_t)stream;
    // every group's device counters, zeroed on the caller's stream before the
    // slots start and read back once at the end (converging methods; the sweep
    // order reports through the per-group host stats)
    GroupStats gstats;
    gstats.st = caller;
    if (stats) {
        cudaError_t ea = fadesim::lib_malloc_async(reinterpret_cast<void **>(&gstats.d),
                                                   (size_t)ngroups * sizeof(fadesim::DevStats), caller);
        if (ea == cudaSuccess)
            ea = cudaMemsetAsync(gstats.d, 0, (size_t)ngroups * sizeof(fadesim::DevStats), caller);
        if (ea != cudaSuccess) return fail_cuda("group counters", ea);
    }
    cudaEvent_t start;
    cudaError_t e = cudaEventCreateWithFlags(&start, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail_cuda("cudaEventCreateWithFlags", e);
    e = cudaEventRecord(start, caller);
    SlotSet slots;
    const int nslot = ngroups < NSLOT ? ngroups : NSLOT;
    cudaStream_t streams[NSLOT];
    if (e == cudaSuccess) e = slot_streams(streams);
    for (int s = 0; s < nslot && e == cudaSuccess; ++s) {
        slots.st[s] = streams[s];
        slots.n = s + 1;
        e = cudaStreamWaitEvent(slots.st[s], start, 0);
        if (e == cudaSuccess)
            e = fadesim::lib_malloc_async(&slots.buf[s], al(gbytes) + al(ibytes) + al(obytes), slots.st[s]);
    }
    cudaEventDestroy(start);
    if (e != cudaSuccess) return fail_cuda("slot setup", e);

    const char *hG = static_cast<const char *>(G);
    const char *hin = static_cast<const char *>(input);
    char *hout = static_cast<char *>(out);
    for (int g = 0; g < ngroups; ++g) {
        const int s = g % nslot;
        cudaStream_t st = slots.st[s];
        const int x0 = gx0[g];
        const int gx = gx0[g + 1] - x0;  // <= group_x
        char *dG = static_cast<char *>(slots.buf[s]);
        char *din = dG + al(gbytes);
        char *dout = din + al(ibytes);
        e = cudaMemcpyAsync(dG, hG + (size_t)x0 * g_x * es, (size_t)gx * g_x * es, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return fail_cuda("cudaMemcpyAsync (G)", e);
        // input rows of batch b for x0..x0+gx: one row of a pitched copy
        e = cudaMemcpy2DAsync(din, (size_t)gx * in_x * es, hin + (size_t)x0 * in_x * es, (size_t)numX * in_x * es,
                              (size_t)gx * in_x * es, (size_t)batch_size, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return fail_cuda("cudaMemcpy2DAsync (input)", e);
        fadesim_solve_stats gs{0, 0, 0, 0, 0};
        fadesim::set_group_stats(stats ? gstats.d + g : nullptr);
        const int rc = fadesim_ir_drop_gs_ex(dtype, din, dG, batch_size, row_size, col_size, gx, numY, iter_times,
                                             g_wire, beta, enable_break, break_threshould, nonlinear_cell_enable,
                                             nonlinear_params, n_nonlinear_params, ret_V, dout, opts,
                                             stats ? &gs : nullptr, nullptr, st);
        fadesim::set_group_stats(nullptr);
        if (rc != FADESIM_OK) return rc;
        if (stats) {
            stats->solves += gs.solves;
            stats->iters_sum += gs.iters_sum;
            if (gs.iters_max > stats->iters_max) stats->iters_max = gs.iters_max;
            stats->status_or |= gs.status_or;
            stats->warm_rejected += gs.warm_rejected;
        }
        e = cudaMemcpy2DAsync(hout + (size_t)x0 * out_x * es, (size_t)numX * out_x * es, dout,
                              (size_t)gx * out_x * es, (size_t)gx * out_x * es, (size_t)batch_size,
                              cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return fail_cuda("cudaMemcpy2DAsync (out)", e);
    }
    for (int s = 0; s < nslot; ++s) {
        e = cudaStreamSynchronize(slots.st[s]);
        if (e != cudaSuccess) return fail_cuda("cudaStreamSynchronize", e);
    }
    if (stats) {
        // the converging groups' counters (all zero for the sweep order)
        std::vector<fadesim::DevStats> h((size_t)ngroups);
        e = cudaMemcpy(h.data(), gstats.d, (size_t)ngroups * sizeof(fadesim::DevStats), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail_cuda("cudaMemcpy (group counters)", e);
        for (const fadesim::DevStats &d : h) {
            stats->solves += (int64_t)d.solves;
            stats->iters_sum += (int64_t)d.iters_sum;
            if (d.iters_max > stats->iters_max) stats->iters_max = d.iters_max;
            stats->status_or |= d.status_or;
            stats->warm_rejected += (int64_t)d.warm_rejected;
        }
    }
    return FADESIM_OK;
}
