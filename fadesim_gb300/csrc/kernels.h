// Host-side launch interface of the solver kernels (internal to the library).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace fadesim {

// Arguments common to the per-(tile, vector) solve kernels.  Layouts are the
// reference extension's (split_arr_matmul.cu:200-203,238,310-332).
struct SolveArgs {
    const void *input;  // [B, numX, n]
    const void *G;      // [numX, n, numY*m]
    void *out;          // [B, numX, numY*m] or, with ret_V, [B, numX, numY, n, m]
    int B, n, m, numX, numY;
    float gw;           // wire conductance 1/r_wire
    int ret_V;
    int vchunk;         // vectors per work item
    int nchunks;        // work items per tile
    long long nitems;   // tiles * nchunks
    SolveCtl ctl;
    float *scratch;     // per-CTA scratch (kernel specific)
    int *iters_out;     // optional [B, numX, numY]
    DevStats *stats;    // optional
    const float *init;  // optional warm start: deviation planes [B, numX, numY, 2, n, m] (u - vin, d)
    int f64;            // input, G and out are FP64 (else FP32); the solve itself is FP32
    int two_level;      // the two-level line relaxation (coarse correction) on full 128 x 128 tiles
                        // with linear cells whose cells couple the planes strongly
    int fp32_limit;     // two-level kernel: iterate past the FP32 floor until the corrections stall
};

// Record msg as the message of fadesim_last_error() and return code.
int report_error(int code, const char *msg);

// Stream-ordered device allocation from the library's own memory pool on the
// current device (created on first use, keeping freed memory for reuse, so
// repeated calls do not map and unmap device memory); free with cudaFreeAsync.
cudaError_t lib_malloc_async(void **p, size_t bytes, cudaStream_t st);

// Block line relaxation, planes resident in shared memory (n, m <= 128).
// Returns the LD (32/64/128) used, or 0 if the shape does not fit.
int line_relax_ld(int n, int m);
size_t line_relax_smem(int ld);
int line_relax_threads(int ld);
size_t line_relax_scratch_floats_per_cta(int ld);
cudaError_t line_relax_prepare(int ld, int dtype);
cudaError_t line_relax_occupancy(int ld, int dtype, int *ctas_per_sm);
cudaError_t launch_line_relax(const SolveArgs &a, int ld, int dtype, int grid, cudaStream_t st);

// Block line relaxation for 128 < rows, cols <= 512 on thread-block clusters
// (4 CTAs up to 256, 16 CTAs up to 512).  Returns 256/512, or 0 if the shape
// is not handled.
int cluster_relax_ld(int n, int m);
int cluster_relax_size(int ld);
size_t cluster_relax_scratch_floats_per_cta(int ld);
cudaError_t cluster_relax_occupancy(int ld, int dtype, int *clusters);
cudaError_t launch_cluster_relax(const SolveArgs &a, int ld, int dtype, int grid, cudaStream_t st);

// Plain red-black point SOR, planes resident in shared memory (n, m <= 128).
size_t rbsor_smem(int n, int m);
cudaError_t rbsor_prepare(int dtype);
cudaError_t launch_rbsor(const SolveArgs &a, int dtype, int grid, cudaStream_t st);

// Plain red-black point SOR for 128 < rows, cols <= 512 on thread-block clusters
// (4 CTAs up to 256, 16 CTAs up to 512), bands of rows per CTA, halo rows read
// through distributed shared memory.  Returns 256/512, or 0 if not handled.
int rbsor_cluster_ld(int n, int m);
int rbsor_cluster_size(int ld);
size_t rbsor_cluster_scratch_floats_per_cta(int ld);  // the low parts of both planes of one band
cudaError_t rbsor_cluster_occupancy(int ld, int dtype, int *clusters);
cudaError_t launch_rbsor_cluster(const SolveArgs &a, int ld, int dtype, int grid, cudaStream_t st);

// The reference's sweep order (split_arr_matmul.cu:27-119), one sweep per launch.
cudaError_t launch_sweep(const SolveArgs &a, int dtype, void *U, void *D, double gw, double beta,
                         double thr, unsigned int *moved, cudaStream_t st);
cudaError_t launch_sweep_init(const SolveArgs &a, int dtype, void *U, void *D, cudaStream_t st);
cudaError_t launch_sweep_output(const SolveArgs &a, int dtype, const void *U, const void *D, cudaStream_t st);

// The same sweep order with sinh cells (nl = [R_on, R_off, a_on, b_on, a_off, b_off]),
// conductances recomputed before every sweep from the iterate before the newest
// (irfamily.cu); *done = sweeps run.  Returns FADESIM_OK or a FADESIM_E_* code.
int family_gs_nonlinear(int dtype, const void *input, const void *G, int B, int n, int m, int numX, int numY,
                        int iter_times, double g_wire, double beta, int enable_break, double thr, const double *nl,
                        int ret_V, void *out, int *done, cudaStream_t st);

// Tensor-core 3x3 convolution of the warm-start network (warmnet_tc.cu): TMA
// loads, tcgen05.mma into TMEM.  conv3x3_tc_supported: Cin a multiple of 32,
// Cout a multiple of 16 up to 128, W a power of two from 16 to 128, H a
// multiple of 8, 16-byte aligned buffers.  err: device flag set when a bounded wait
// expires (conv_tc_error_flag: the library's own, per device).
bool conv3x3_tc_supported(const void *X, const void *Wt, const void *Y, int H, int W, int Cin, int Cout);
cudaError_t conv3x3_fwd_tc(const void *X, const void *Wt, const float *bias, const void *skip, void *Y, int N, int H,
                           int W, int Cin, int Cout, int flags, int *err, cudaStream_t st);
int *conv_tc_error_flag();
// The host-buffer entry's per-group device counters for the next converging
// solve on this thread (nullptr: the solve keeps and reads back its own).
void set_group_stats(DevStats *d);
// Tensor-core weight gradient dW[Cout][9][Cin] += (FP32 atomics): Cin and Cout
// multiples of 32, Cout <= 128, W a power of two from 16 to 128, H a multiple
// of 8, 16-byte aligned activations.
bool conv3x3_wgrad_tc_supported(const void *dY, const void *X, int H, int W, int Cin, int Cout);
cudaError_t conv3x3_wgrad_tc(const void *dY, const void *X, float *dW, int N, int H, int W, int Cin, int Cout,
                             int *err, cudaStream_t st);

}  // namespace fadesim
