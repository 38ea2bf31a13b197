/*
 * fadesim_gb300: C ABI of the GB300 (sm_103a) crossbar IR-drop solver.
 *
 * All pointers passed to the solve entry points are DEVICE pointers (CUDA
 * global memory on the current device) unless the comment says otherwise.
 * Every call is asynchronous on the given CUDA stream (NULL = legacy default
 * stream) and returns 0 on success or a negative FADESIM_E* code;
 * fadesim_last_error() then gives a message.  Argument checks mirror the
 * reference's TORCH_CHECKs (split_arr_matmul.cu:21-24,222-225).
 *
 * Layouts follow the reference extension (split_arr_matmul.cu:200-203,238):
 *   input  [batch, numX, rows]              wordline drive voltages
 *   G      [numX, rows, numY*cols]          cell conductances
 *   out    [batch, numX, numY*cols]         bitline currents, or, with ret_V,
 *          [batch, numX, numY, rows, cols]  cell voltages u - d
 */
#ifndef FADESIM_GB300_H
#define FADESIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FADESIM_OK 0
#define FADESIM_E_ARG (-1)       /* bad argument (size, pointer, option) */
#define FADESIM_E_CUDA (-2)      /* a CUDA call failed */
#define FADESIM_E_UNSUPPORTED (-3) /* valid request this build does not implement */

/* dtype codes */
#define FADESIM_F32 0
#define FADESIM_F64 1

/* solver methods */
#define FADESIM_METHOD_AUTO 0      /* line relaxation up to 512 x 512, else the sweep order */
#define FADESIM_METHOD_LINE 1      /* block line relaxation, residual form, to tolerance (<= 512 x 512;
                                      > 128 on 4- or 16-CTA clusters) */
#define FADESIM_METHOD_RBSOR 2     /* plain red-black point SOR, residual form, to tolerance (<= 512 x 512;
                                      > 128 on 4- or 16-CTA clusters) */
#define FADESIM_METHOD_SWEEPS 3    /* the reference's sweep order for exactly iter_times sweeps */
#define FADESIM_METHOD_LINE_COARSE 4  /* the line relaxation with a coarse-grid correction after every
                                         iteration (two-level) on full 128 x 128 tiles of linear cells
                                         whose cells couple the planes strongly (sum of g / g_wire over
                                         the tile >= 3, e.g. 1 kOhm - 1 MOhm cells): 3x fewer iterations
                                         there; every other tile as FADESIM_METHOD_LINE */

/* per-solve status bits (fadesim_solve_stats.status_or, per_solve_status) */
#define FADESIM_ST_CONVERGED 1
#define FADESIM_ST_MAXITER 2
#define FADESIM_ST_NONFINITE 4
#define FADESIM_ST_WARM_REJECTED 8  /* the warm start was discarded and the solve restarted from zero */

typedef struct fadesim_solve_opts {
    int method;            /* FADESIM_METHOD_* */
    double tol_v;          /* target max node error in volts (converging methods); <=0: 1e-8 */
    int max_iters;         /* cap on line iterations / point sweeps; <=0: method default */
    int residual_period;   /* precise residual every k line iterations, and always for the final
                              convergence test; 0 (default): adaptive -- FP32 residuals while the
                              corrections are far above the FP32 residual noise, precise on the
                              iteration expected to be the last; <0: FP32 residuals only */
    double omega;          /* relaxation factor; <=0: adaptive (line) or autotuned table (rbsor) */
    int vectors_per_cta;   /* input vectors one CTA solves per work item; <=0: automatic */
    int residual_kind;     /* precise residual arithmetic: 0 = float-float (default: error-free FP32
                              transforms, FP64-class accuracy on the FP32 pipe), 1 = native FP64 */
    double read_noise_sigma;        /* > 0: each cell current gets N(0, (sigma * I_cell)^2) in the returned
                                       bitline currents (line method); not a reference feature */
    unsigned long long noise_seed;  /* counter-based: same seed, same noise */
    int kernel_ld;         /* kernel layout, 0 = by tile size; else the line (or red-black) kernel of that
                              size: 32 / 64 / 128 one tile per CTA, 256 / 512 one tile per 4- / 16-CTA
                              cluster (>= rows and cols; red-black SOR: 128, 256, 512) */
    int fp32_limit;        /* 1: below the FP32 resolution floor (4 ulps of the largest deviation) keep
                              iterating until the corrections stop shrinking, not just until the error
                              estimate reaches the floor (small nodes, e.g. the bitline ends that carry
                              a unit response's currents, keep converging there).  Honoured by
                              FADESIM_METHOD_LINE_COARSE on full 128 x 128 tiles of linear cells. */
} fadesim_solve_opts;

typedef struct fadesim_solve_stats {
    int64_t solves;        /* (tile, vector) solves run */
    int64_t iters_sum;     /* sum over solves of iterations (line) or sweeps (rbsor, sweeps) */
    int iters_max;
    int status_or;         /* OR of per-solve status bits */
    int64_t warm_rejected; /* solves whose warm start was discarded (FADESIM_ST_WARM_REJECTED) */
} fadesim_solve_stats;

/* Drop-in for the reference's ir_drop_gs (split_arr_matmul.cu:204-220, bound
 * by PYBIND11_MODULE at :1429-1437 and called from
 * pimtorch/.../nn/splitArrayArithmetic.py:488-511).  Same arguments, same
 * meaning, same output.  The default method solves each (tile, vector) pair to
 * tol_v = 1e-8 V against the converged nodal solution; iter_times, beta,
 * enable_break and break_threshould keep their reference meaning only under
 * FADESIM_METHOD_SWEEPS (see fadesim_ir_drop_gs_ex).  nonlinear_params holds
 * [R_on, R_off, a_on, b_on, a_off, b_off] (commonConst.py:207) and is read only
 * when nonlinear_cell_enable != 0. */
int fadesim_ir_drop_gs_f32(const float *input, const float *G, int batch_size, int row_size, int col_size,
                           int numX, int numY, int iter_times, double g_wire, double beta, int enable_break,
                           double break_threshould, int nonlinear_cell_enable, const double *nonlinear_params,
                           int n_nonlinear_params, int ret_V, float *out, void *stream);

int fadesim_ir_drop_gs_f64(const double *input, const double *G, int batch_size, int row_size, int col_size,
                           int numX, int numY, int iter_times, double g_wire, double beta, int enable_break,
                           double break_threshould, int nonlinear_cell_enable, const double *nonlinear_params,
                           int n_nonlinear_params, int ret_V, double *out, void *stream);

/* Extended form of the same boundary (the optional entry the reference's
 * interface leaves room for next to ir_drop_gs): explicit method and
 * tolerance, ret_V = 2 for both node planes [batch, numX, numY, 2, rows, cols]
 * (wordline u then bitline d), optional stats (HOST pointer, filled after a stream sync when not
 * NULL) and optional per-solve iteration counts (DEVICE int32
 * [batch, numX, numY]).  dtype is FADESIM_F32 or FADESIM_F64 and types input,
 * G and out. */
int fadesim_ir_drop_gs_ex(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                          int numX, int numY, int iter_times, double g_wire, double beta, int enable_break,
                          double break_threshould, int nonlinear_cell_enable, const double *nonlinear_params,
                          int n_nonlinear_params, int ret_V, void *out, const fadesim_solve_opts *opts,
                          fadesim_solve_stats *stats, int *per_solve_iters, void *stream);

/* fadesim_ir_drop_gs_ex on HOST buffers: input, G and out are host memory (page-locked for the
 * copies to overlap), laid out as for fadesim_ir_drop_gs_ex.  The library copies them in and out
 * itself, pipelined over groups of group_x values of numX (0: about eight groups of whole
 * multiples of the SM count of tiles) on three internal streams ordered after `stream`, so one
 * group's copies overlap another's solve.  Returns when out holds the result.  Replaces the
 * transfers the reference's callers make around ir_drop_gs, which takes device tensors
 * (splitArrayArithmetic.py:485-511): .to(device) before and .cpu() after
 * (splitArrayArithmetic.py:1082, 1124), serialised with the solve.  stats (host, may be NULL)
 * sums the groups' statistics; asking for them makes every group wait for its own solve before
 * the next group is queued. */
int fadesim_ir_drop_gs_host(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                            int numX, int numY, int iter_times, double g_wire, double beta, int enable_break,
                            double break_threshould, int nonlinear_cell_enable, const double *nonlinear_params,
                            int n_nonlinear_params, int ret_V, void *out, const fadesim_solve_opts *opts,
                            fadesim_solve_stats *stats, int group_x, void *stream);

/* Return the device memory the library keeps for reuse (its stream-ordered scratch and staging
 * buffers come from a per-device pool that keeps freed memory mapped between calls) to the
 * system.  Call when no solve is in flight.  FADESIM_OK or FADESIM_E_CUDA. */
int fadesim_release_memory(void);

/* ---- the reference extension's other exports (split_arr_matmul.cu:1429-1437),
 * reproducing their iterates: same arguments and meaning, dtype (FADESIM_F32 /
 * FADESIM_F64) typing input, G and out.  nonlinear_cell_enable != 0 selects the
 * reference's sinh cells, nonlinear_params = [R_on, R_off, a_on, b_on, a_off, b_off]
 * (commonConst.py:207): before every iteration each solve's conductances are
 * recomputed from u - d of the iterate before the newest, |V| < 1e-5 clamped to
 * +-1e-5, as the reference's host loops do (:455-475, 603-622, 727-746, 996-1016,
 * 1241-1260).  ou_* functions split every rows x cols tile into ou_row_size x
 * ou_col_size operation units solved at once, each through the lumped wire
 * outside it, and return currents per OU row group
 * [batch, numX * rows / ou_row_size, numY * cols]; the others return
 * [batch, numX, numY * cols] (ir2s with ret_V: cell voltages
 * [batch, numX, numY, rows, cols]). ---- */

/* ir2s (split_arr_matmul.cu:419-545): IR-drop-to-source iteration, r_wire the wire and load resistance. */
int fadesim_ir2s(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size, int numX,
                 int numY, int iter_times, double r_wire, int enable_break, double break_threshould,
                 int nonlinear_cell_enable, const double *nonlinear_params, int n_nonlinear_params, int ret_V,
                 void *out, void *stream);
/* ir2s_ou_local (:565-680): ir2s with source and ground load resistances. */
int fadesim_ir2s_ou_local(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                          int numX, int numY, int iter_times, double r_wire, double r_load_left, double r_load_down,
                          int enable_break, double break_threshould, int nonlinear_cell_enable,
                          const double *nonlinear_params, int n_nonlinear_params, void *out, void *stream);
/* ir2s_ou (:953-1084): ir2s on every OU at once. */
int fadesim_ir2s_ou(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                    int ou_row_size, int ou_col_size, int numX, int numY, int iter_times, double r_wire,
                    int enable_break, double break_threshould, int nonlinear_cell_enable,
                    const double *nonlinear_params, int n_nonlinear_params, void *out, void *stream);
/* ir_gs_ou_local (:690-813): the ir_drop_gs sweep with source and ground load conductances. */
int fadesim_ir_gs_ou_local(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                           int numX, int numY, int iter_times, double g_wire, double g_load_left, double g_load_down,
                           double beta, int enable_break, double break_threshould, int nonlinear_cell_enable,
                           const double *nonlinear_params, int n_nonlinear_params, void *out, void *stream);
/* ir_gs_ou (:1197-1310): the sweep on every OU at once. */
int fadesim_ir_gs_ou(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                     int ou_row_size, int ou_col_size, int numX, int numY, int iter_times, double g_wire, double beta,
                     int enable_break, double break_threshould, int nonlinear_cell_enable,
                     const double *nonlinear_params, int n_nonlinear_params, void *out, void *stream);

/* ---- integer stages around the solve (bit-exact with the reference's float32
 * arithmetic given the same currents).  Device pointers, async on stream. ---- */

/* q = round-half-even(x / 2^s) as int32; s from the host as the reference computes it
 * (fixedPoint/nn/fixedPointArithmetic.py:76-96, quantization_tensor). */
int fadesim_quantize_f32(const float *x, long long n, int s, int32_t *q, void *stream);

/* Input voltages for nbits input-bit cycles, stacked on the batch:
 * v[bit*B + b, x, r] = ((xq[b, x*rows + r] >> bit*dac_bits) & (2^dac_bits - 1)) * inputV, zero-padded
 * to numX*rows (splitArrayArithmetic.py:1199-1201 bit slicing, :714-749 padding and voltage). */
int fadesim_slice_inputs_f32(const int32_t *xq, int B, int insize, int rows, int numX, int nbits, int dac_bits,
                             float inputV, float *v, void *stream);

/* Conductance map of one weight slice of one PN array: G[x, r, y*cols + c] = slice * dG + Gmin, slice =
 * ((negative ? max(-w, 0) : max(w, 0)) >> shift) & (2^cell_bits - 1), padded cells at state 0
 * (splitArrayArithmetic.py:1191-1195,1212-1215 PN split and slicing, :753-757 mapping). */
int fadesim_map_conductance_f32(const int32_t *wq, int insize, int outsize, int rows, int cols, int numX, int numY,
                                int shift, int cell_bits, int negative, float dG, float Gmin, float *G, void *stream);

/* ADC codes round(I / adcUseI * levels) summed over row tiles, cropped, scaled, pos - neg, and
 * shift-added over input bits i and slices j in the reference's order, the top input bit subtracted
 * when complement != 0 (splitArrayArithmetic.py:835-836, 961-978, 1224-1227).  I is
 * [nslices][2][nbits][B][numX][ldI]; out is [B, outsize]; s12 = s1 + s2. */
int fadesim_adc_shift_add_f32(const float *I, int nbits, int nslices, int B, int numX, int ldI, int outsize,
                              float adcUseI, float levels, float scale, int s12, int dac_bits, int cell_bits,
                              int input_bits, int complement, float *out, void *stream);

/* Input voltages of a convolution (or, as the 1x1 case N = batch, C = in_features, H = W = 1, of a
 * linear layer) straight from the NCHW int32 quantised image, the unfold done by addressing
 * (torch.nn.functional.unfold as Conv2d_sp calls it, fixedPoint/nn/modules/conv_split.py:106-107):
 * matrix row p = (n, oh, ow), column k = (ch, ki, kj), then a column of ones_q when has_ones (a
 * bias mapped into the array, conv_split.py:113-115), then zeros to numX*rows.
 * v[bit*M + p, x, r] = level * inputV with M = N*OH*OW and level = (q >> bit*dac_bits) & mask, or
 * -((|q| >> bit*dac_bits) & mask) for a negative q when neg_pulse != 0 (negative-pulse input mode,
 * splitArrayArithmetic.py:1183-1187,1202-1203). */
int fadesim_slice_inputs_im2col_f32(const int32_t *xq, int N, int C, int H, int W, int kh, int kw, int sh, int sw,
                                    int ph, int pw, int dh, int dw, int has_ones, int ones_q, int rows, int numX,
                                    int nbits, int dac_bits, int neg_pulse, float inputV, float *v, void *stream);

/* Conductance map of one weight slice of a Ref-column array (phyArrMode.Ref): G [numX, rows,
 * numY*(cols+2)]; data cells hold ((min(w + plus, maximum)) >> shift) & (2^cell_bits - 1), padded cells
 * state 0, and each column block ends with a state-0 and a state-1 reference column on every row
 * (splitArrayArithmetic.py:758-771, 1229-1242). */
int fadesim_map_conductance_ref_f32(const int32_t *wq, int insize, int outsize, int rows, int cols, int numX,
                                    int numY, int shift, int cell_bits, int plus, int maximum, float dG, float Gmin,
                                    float *G, void *stream);

/* fadesim_adc_shift_add_f32 for both array modes, with the float32 bias and the output layout of
 * the layer.  ref_cols == 0: PN, I as above.  ref_cols == cols: Ref, I [nslices][nbits][B][numX][ldI]
 * with ldI = numY*(cols+2); per row tile the state-0 column's code is subtracted from each column's
 * and, for slice 0, rint(plus * (code_one - code_zero)) too (splitArrayArithmetic.py:980-996).
 * bias (may be NULL) is added after the shift-add (linear_split.py:73-76, conv_split.py:123-126);
 * L > 0 writes [B/L, outsize, L] (a convolution's NCHW output, L = OH*OW), else [B, outsize]. */
int fadesim_adc_shift_add_ex_f32(const float *I, int ref_cols, int nbits, int nslices, int B, int numX, int ldI,
                                 int outsize, float adcUseI, float levels, float scale, int s12, int dac_bits,
                                 int cell_bits, int input_bits, int complement, float plus, const float *bias, int L,
                                 float *out, void *stream);

/* Cycle-to-cycle conductance variation of a map of n cells: out[k] = G[k] / divisor[k], one
 * correctly rounded FP32 division, where divisor holds exp(sigma * N(0,1)) drawn by the caller (the
 * reference draws them from its CPU generator, conductance_variation.py:6-13, and divides on the
 * map's device); with divisor == NULL the divisor is exp(sigma * z_k), z_k a standard normal from a
 * counter hash of (seed, offset + k), the same on every run and device (R becomes R * exp(sigma z),
 * a lognormal spread, without a host round trip).  out may alias G.  sigma >= 0. */
int fadesim_vary_conductance_f32(const float *G, const float *divisor, long long n, double sigma,
                                 unsigned long long seed, unsigned long long offset, float *out, void *stream);

/* Allocation-free variant of the line solve (FP32, bitline currents only).
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- code running inside someone else's stream capture, host
 * callbacks or real-time loops that forbid allocation, programs with a fixed
 * device-memory budget.  Inputs and outputs as fadesim_ir_drop_gs_f32 (method
 * FADESIM_METHOD_LINE, tol 1e-8 V, at most 400 line iterations).  Its scratch
 * is one static device array of fadesim_noalloc_scratch_bytes() bytes (24 MiB)
 * that every GPU loading the library holds until exit.  The first call on a
 * device sets up that array's address and should come before any stream
 * capture; the address is kept, so do not use this entry across a
 * cudaDeviceReset.  All calls share the array: calls that overlap on the GPU
 * race.  Tiles larger than 128 x 128 are rejected with FADESIM_E_ARG;
 * fadesim_noalloc_last_error() gives the message.  It calls no cudaMalloc,
 * cudaFree or allocating library routine. */
int fadesim_ir_drop_gs_noalloc_f32(const float *input, const float *G, int batch_size, int row_size, int col_size,
                                   int numX, int numY, double g_wire, float *out, void *stream);
size_t fadesim_noalloc_scratch_bytes(void);
const char *fadesim_noalloc_last_error(void);
/* The counters of the last fadesim_ir_drop_gs_noalloc_f32 call that finished on this device (solves,
 * iterations, OR of the FADESIM_ST_* bits: FADESIM_ST_MAXITER or FADESIM_ST_NONFINITE mark a failed
 * solve), copied from the static array to the HOST struct *stats after the copy, queued on `stream`
 * behind that call, has completed (this synchronises `stream`).  Allocates nothing. */
int fadesim_noalloc_last_status(fadesim_solve_stats *stats, void *stream);

/* fadesim_ir_drop_gs_ex started from given node planes (a learned warm start): init is a DEVICE
 * FP32 array [batch, numX, numY, 2, rows, cols] of wordline deviations u - vin and bitline voltages
 * d.  The line method (every tile size up to 512 x 512, linear or sinh cells -- nonlinear_* as in
 * fadesim_ir_drop_gs_ex) iterates from them to the same tolerance; a prediction whose first
 * correction is as large as the solution is discarded (FADESIM_ST_WARM_REJECTED) and the solve
 * restarts from the ideal state.  opts->method FADESIM_METHOD_RBSOR starts the plain red-black SOR
 * from the planes instead (tiles up to 128 x 128, linear cells: the comparator the learned start
 * is measured against). */
int fadesim_ir_drop_gs_warm(int dtype, const void *input, const void *G, int batch_size, int row_size, int col_size,
                            int numX, int numY, double g_wire, const float *init, int nonlinear_cell_enable,
                            const double *nonlinear_params, int n_nonlinear_params, void *out,
                            const fadesim_solve_opts *opts, fadesim_solve_stats *stats, int *per_solve_iters,
                            void *stream);

/* ---- kernels of the learned warm-start network (no reference counterpart; the
 * reference's learned-solver precedent is its SCN/fcm training path, which
 * this path does not drop in for).  Device pointers, async on stream, return
 * FADESIM_OK, FADESIM_E_ARG or FADESIM_E_CUDA.  Activations are NHWC bf16 with
 * channels a multiple of 16; weights [Cout][3][3][Cin] bf16 with Cout a
 * multiple of 8 and at most 128; "same" zero padding. ---- */

/* Y = act(conv3x3(X, W) + bias) (+ skip): flags 1 = ReLU, 2 = add skip after
 * the activation, 4 = store FP32 instead of bf16, 8 = use the mma.sync kernel even where the
 * tensor-core kernel applies.  The tensor-core kernel (TMA loads, tcgen05.mma into tensor memory)
 * runs when Cin is a multiple of 32, Cout a multiple of 16, Wd a power of two from 16 to 128, H a
 * multiple of 8 and the buffers 16-byte aligned; other shapes run on mma.sync. */
int fadesim_conv3x3_fwd_bf16(const void *X, const void *W, const float *bias, const void *skip, void *Y, int N,
                             int H, int Wd, int Cin, int Cout, int flags, void *stream);
/* The tensor-core convolutions' error flag on the current device (0: none; 1-3: a bounded wait of
 * a launch expired -- a stage never freed / filled, the accumulator never completed), read after
 * the work queued on `stream` has finished, and cleared.  Negative: FADESIM_E_CUDA. */
int fadesim_conv_tc_status(void *stream);
/* Which parts of an H x Wd, Cin -> Cout convolution run on the tensor-core kernels (16-byte
 * aligned buffers): bit 0 fadesim_conv3x3_fwd_bf16 (flag 8 clear), bit 1
 * fadesim_conv3x3_wgrad_bf16 (Cin and Cout multiples of 32 as well). */
int fadesim_conv_tc_shape(int H, int Wd, int Cin, int Cout);
/* dW[Cout][3][3][Cin] += sum over pixels of dY x X (FP32 accumulation with atomics: zero dW first).
 * On the tensor cores (tcgen05, MN-major operands straight from the NHWC activations) when Cin and
 * Cout are multiples of 32, Cout <= 128, Wd a power of two from 16 to 128 and H a multiple of 8;
 * mma.sync otherwise. */
int fadesim_conv3x3_wgrad_bf16(const void *dY, const void *X, float *dW, int N, int H, int Wd, int Cin, int Cout,
                               void *stream);
/* Wf[ci][8 - tap][co] = W[co][tap][ci], ci padded to Cin_pad8: the weights of the input-gradient convolution. */
int fadesim_weight_flip_bf16(const void *W, void *Wf, int Cin, int Cout, int Cin_pad8, void *stream);
/* db[c] += sum over P pixels of dY[p, c]. */
int fadesim_bias_grad_bf16(const void *dY, float *db, long long P, int C, void *stream);
/* 2x2 average pool (upsample = 0) or nearest 2x upsample (upsample = 1), or their gradients
 * (backward = 1).  H, W are the full-resolution side's size for the pool and the low-resolution
 * side's for the upsample, in both directions. */
int fadesim_pool_bf16(const void *X, void *Y, int N, int H, int W, int C, int backward, int upsample, void *stream);
/* dZ = dY where Yact > 0, else 0. */
int fadesim_relu_bwd_bf16(const void *dY, const void *Yact, void *dZ, long long n, void *stream);
/* C = A + B (bf16). */
int fadesim_add_bf16(const void *A, const void *B, void *C, long long n, void *stream);
/* Mean squared error of the first Cv of Cp FP32 prediction channels [P, Cp] against target [P, Cv]:
 * loss (FP32, accumulated: zero it first) and the bf16 gradient dpred [P, Cp] (0 past Cv). */
int fadesim_mse_f32(const float *pred, const float *target, void *dpred, float *loss, long long P, int Cp, int Cv,
                    void *stream);
/* One Adam step (bias-corrected, step >= 1) on FP32 master weights w with moments m, v; refreshes the
 * bf16 copy wb. */
int fadesim_adam_f32(float *w, void *wb, const float *g, float *m, float *v, long long n, float lr, float b1,
                     float b2, float eps, int step, void *stream);

/* ---- measurement helper (no reference counterpart) ---- */

/* Shared-memory read bandwidth probe: `blocks` CTAs of 1024 threads each read iters (a multiple
 * of 8) 16-byte shared-memory words per thread, conflict-free, and add one sum per CTA to
 * sink[blockIdx] (DEVICE, blocks floats).  Bytes read = blocks * 1024 * iters * 16; timed by the
 * caller, it gives the measured shared-memory peak the line kernels' roofline is quoted against. */
int fadesim_smem_read_probe(float *sink, int blocks, int iters, void *stream);

/* Message for the last failing call on this thread. */
const char *fadesim_last_error(void);

/* Library version string. */
const char *fadesim_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FADESIM_GB300_H */
