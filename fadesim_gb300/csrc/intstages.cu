// Integer stages of PimTorch's bit-sliced crossbar matmul (sm_103a), bit-exact
// with the reference's float32 arithmetic given the same bitline currents.
//
// Reference: pimtorch/pimfixedpoint/fixedPoint/nn/splitArrayArithmetic.py
//   splitArr_matmul_nn :1161-1260 (quantise, PN split or Ref offset, bit/slice
//          loops, negative pulses, shift-add)
//   matmul :705-771 (padding, input voltages, conductance map, reference
//          columns), :835-836 (ADC), :961-996 (sum over row tiles, crop, scale,
//          pos - neg or reference-column subtraction)
// fixedPoint/nn/fixedPointArithmetic.py:76-96 (quantisation) and
// fixedPoint/nn/modules/conv_split.py:106-134 (Conv2d_sp: unfold, matmul, fold).
//
// Every float operation is a separately rounded IEEE float32 op in the
// reference's order (__fmul_rn / __fadd_rn / __fdiv_rn keep the compiler from
// fusing them); scalar operands arrive already rounded to float32, as torch
// rounds a Python scalar combined with a float32 tensor.
#include <math.h>
#include <stdint.h>

#include "kernels.h"

namespace {

__global__ void quantize_kernel(const float *__restrict__ x, long long n, float res, int32_t *__restrict__ q) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        q[e] = (int32_t)rintf(__fdiv_rn(x[e], res));  // round half to even, as torch.round
}

// v[(bit*B + b), x, r] = ((xq[b, x*rows + r] >> (bit0 + bit*dac)) & mask) * inputV, zero past insize
__global__ void slice_inputs_kernel(const int32_t *__restrict__ xq, int B, int insize, int rows, int numX, int nbits,
                                    int dac_bits, float inputV, float *__restrict__ v) {
    const long long total = (long long)nbits * B * numX * rows;
    const int mask = (1 << dac_bits) - 1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % rows);
        const int x = (int)((e / rows) % numX);
        const long long bb = e / ((long long)rows * numX);  // bit*B + b
        const int b = (int)(bb % B);
        const int bit = (int)(bb / B);
        const int c = x * rows + r;
        float out = 0.f;
        if (c < insize) {
            const int level = (xq[(long long)b * insize + c] >> (bit * dac_bits)) & mask;
            out = __fmul_rn((float)level, inputV);
        }
        v[e] = out;
    }
}

// Input voltages straight from an NCHW int32 image, the unfold done by
// addressing: matrix row p = (n, oh, ow) of N*OH*OW, matrix column
// k = (ch, ki, kj) of C*kh*kw (torch unfold's order), then an optional column of
// ones (a bias mapped into the array), then zero padding to numX*rows.
//   v[(bit*M + p), x, r] = level(q(p, x*rows + r), bit) * inputV
// level = (q >> bit*dac) & mask, or -((|q| >> bit*dac) & mask) for a negative q
// under negative-pulse inputs (splitArrayArithmetic.py:1199-1203).  A linear
// layer is the 1x1 case: N = batch, C = in_features, H = W = 1.
struct Im2col {
    int N, C, H, W, kh, kw, sh, sw, ph, pw, dh, dw, OH, OW;
};

__global__ void slice_im2col_kernel(const int32_t *__restrict__ xq, Im2col g, int has_ones, int ones_q, int rows,
                                    int numX, int nbits, int dac_bits, int neg_pulse, float inputV,
                                    float *__restrict__ v) {
    const long long L = (long long)g.OH * g.OW;
    const long long M = (long long)g.N * L;
    const int Kc = g.C * g.kh * g.kw;
    const long long total = (long long)nbits * M * numX * rows;
    const int mask = (1 << dac_bits) - 1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % rows);
        const int x = (int)((e / rows) % numX);
        const long long bp = e / ((long long)rows * numX);  // bit*M + p
        const long long p = bp % M;
        const int bit = (int)(bp / M);
        const int k = x * rows + r;
        int q = 0;
        if (k < Kc) {
            const int ch = k / (g.kh * g.kw), t = k % (g.kh * g.kw);
            const int ki = t / g.kw, kj = t % g.kw;
            const long long n = p / L;
            const int l = (int)(p % L);
            const int h = (l / g.OW) * g.sh - g.ph + ki * g.dh;
            const int w = (l % g.OW) * g.sw - g.pw + kj * g.dw;
            if (h >= 0 && h < g.H && w >= 0 && w < g.W) q = xq[((n * g.C + ch) * g.H + h) * g.W + w];
        } else if (k == Kc && has_ones) {
            q = ones_q;
        }
        const int sh = bit * dac_bits;
        const int level = (neg_pulse && q < 0) ? -(((-q) >> sh) & mask) : ((q >> sh) & mask);
        v[e] = __fmul_rn((float)level, inputV);
    }
}

// G[x, r, y*cols + c] = slice * dG + Gmin for the PN magnitude of w[x*rows + r, y*cols + c]
__global__ void map_conductance_kernel(const int32_t *__restrict__ wq, int insize, int outsize, int rows, int cols,
                                       int numX, int numY, int shift, int cell_bits, int negative, float dG,
                                       float Gmin, float *__restrict__ G) {
    const long long total = (long long)numX * rows * numY * cols;
    const int mask = (1 << cell_bits) - 1;
    const int ldo = numY * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int oc = (int)(e % ldo);        // y*cols + c
        const long long ir = e / ldo;         // x*rows + r
        int level = 0;
        if (ir < insize && oc < outsize) {
            const int w = wq[ir * outsize + oc];
            const int mag = negative ? (w < 0 ? -w : 0) : (w > 0 ? w : 0);
            level = (mag >> shift) & mask;
        }
        G[e] = __fadd_rn(__fmul_rn((float)level, dG), Gmin);
    }
}

// Ref-column map: each column block of cols data columns gets two reference
// columns, state 0 then state 1, on every row including padded ones
// (splitArrayArithmetic.py:758-771); data cells hold slice `shift` of
// min(w + plus, maximum) (:1236-1242), padded cells state 0.
//   G [numX, rows, numY*(cols+2)]
__global__ void map_conductance_ref_kernel(const int32_t *__restrict__ wq, int insize, int outsize, int rows,
                                           int cols, int numX, int numY, int shift, int cell_bits, int plus,
                                           int maximum, float dG, float Gmin, float *__restrict__ G) {
    const int cb = cols + 2;
    const int ldo = numY * cb;
    const long long total = (long long)numX * rows * ldo;
    const int mask = (1 << cell_bits) - 1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int oc = (int)(e % ldo);
        const long long ir = e / ldo;
        const int y = oc / cb, c = oc % cb;
        int level = 0;
        if (c == cols + 1) {
            level = 1;
        } else if (c < cols) {
            const int o = y * cols + c;
            if (ir < insize && o < outsize) {
                int w = wq[ir * outsize + o] + plus;
                w = w > maximum ? maximum : w;
                level = (w >> shift) & mask;
            }
        }
        G[e] = __fadd_rn(__fmul_rn((float)level, dG), Gmin);
    }
}

__device__ __forceinline__ float adc_code(float i, float adcUseI, float levels) {
    return rintf(__fmul_rn(__fdiv_rn(i, adcUseI), levels));  // no clamp, as the reference
}

// One output element per thread: the reference's loops over input bits i and
// weight slices j, in order, with ADC codes summed over row tiles.
//   PN  (ref_cols == 0): I[j][pn][i][b][x][ldI] (pn 0 = positive array),
//        d = sum_x code_pos * scale - sum_x code_neg * scale
//   Ref (ref_cols == cols): I[j][i][b][x][ldI], ldI = numY*(cols+2),
//        d = sum_x (code - code_zero - [j == 0] rint((code_one - code_zero) * plus)) * scale
// as the solves for one (slice, array) pair produce them with the input bits
// stacked on the batch.  Then acc +/-= d * 2^(i*dac + j*cell + s12), the top
// input bit subtracted for complement-code inputs; bias (float32, may be NULL)
// added last; out row-major [B, outsize], or [B/L, outsize, L] when L > 0 (a
// convolution's NCHW output with L = OH*OW positions per image).
__global__ void adc_shift_add_kernel(const float *__restrict__ I, int ref_cols, int nbits, int nslices, int B,
                                     int numX, int ldI, int outsize, float adcUseI, float levels, float scale, int s12,
                                     int dac_bits, int cell_bits, int input_bits, int complement, float plus,
                                     const float *__restrict__ bias, int L, float *__restrict__ out) {
    const long long total = (long long)B * outsize;
    const long long vec = (long long)numX * ldI;  // one input vector's currents
    const int narr = ref_cols ? 1 : 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int o = (int)(e % outsize);
        const long long b = e / outsize;
        int col = o, zcol = 0;
        if (ref_cols) {
            col = (o / ref_cols) * (ref_cols + 2) + o % ref_cols;
            zcol = (o / ref_cols) * (ref_cols + 2) + ref_cols;
        }
        float acc = 0.f;
        for (int i = 0; i < nbits; ++i) {
            for (int j = 0; j < nslices; ++j) {
                float d;
                if (!ref_cols) {
                    const float *Ip = I + (((long long)(j * narr + 0) * nbits + i) * B + b) * vec + col;
                    const float *In = I + (((long long)(j * narr + 1) * nbits + i) * B + b) * vec + col;
                    float cp = 0.f, cn = 0.f;  // integer-valued: sums are exact
                    for (int x = 0; x < numX; ++x) {
                        cp = __fadd_rn(cp, adc_code(Ip[(long long)x * ldI], adcUseI, levels));
                        cn = __fadd_rn(cn, adc_code(In[(long long)x * ldI], adcUseI, levels));
                    }
                    d = __fsub_rn(__fmul_rn(cp, scale), __fmul_rn(cn, scale));
                } else {
                    const float *Ir = I + (((long long)j * nbits + i) * B + b) * vec;
                    float cs = 0.f;
                    for (int x = 0; x < numX; ++x) {
                        const float *row = Ir + (long long)x * ldI;
                        const float cz = adc_code(row[zcol], adcUseI, levels);
                        float t = __fsub_rn(adc_code(row[col], adcUseI, levels), cz);
                        if (j == 0)
                            t = __fsub_rn(t, rintf(__fmul_rn(__fsub_rn(adc_code(row[zcol + 1], adcUseI, levels), cz),
                                                             plus)));
                        cs = __fadd_rn(cs, t);
                    }
                    d = __fmul_rn(cs, scale);
                }
                const int k = i * dac_bits + j * cell_bits + s12;
                const float t = __fmul_rn(d, ldexpf(1.f, k));  // power of two: exact
                acc = (i * dac_bits != input_bits - 1 || !complement) ? __fadd_rn(acc, t) : __fsub_rn(acc, t);
            }
        }
        if (bias) acc = __fadd_rn(acc, bias[o]);
        if (L > 0)
            out[((b / L) * outsize + o) * L + b % L] = acc;
        else
            out[e] = acc;
    }
}

// Cycle-to-cycle variation of a conductance map: out = G / f with f the
// host-drawn divisor (the reference's exp(sigma N(0,1)) from its CPU generator,
// conductance_variation.py:6-13; one correctly rounded division, as torch's),
// or, without divisors, f = exp(sigma z) with z standard normal from a counter
// hash of (seed, offset + k): the same numbers on every run and device, drawn
// where the map lives (R becomes R exp(sigma z), the lognormal spread).
__global__ void vary_conductance_kernel(const float *__restrict__ G, const float *__restrict__ div, long long n,
                                        float sigma, unsigned long long seed, unsigned long long offset,
                                        float *__restrict__ out) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float f = div ? div[e]
                            : expf(sigma * fadesim::normal_from(seed, offset + (unsigned long long)e,
                                                                fadesim::kVariationStream));
        out[e] = __fdiv_rn(G[e], f);
    }
}

int grid_for(long long total) {
    long long g = (total + 255) / 256;
    return (int)(g > 16384 ? 16384 : (g < 1 ? 1 : g));
}

}  // namespace

extern "C" int fadesim_vary_conductance_f32(const float *G, const float *divisor, long long n, double sigma,
                                            unsigned long long seed, unsigned long long offset, float *out,
                                            void *stream) {
    if (!G || !out || n < 0 || !isfinite(sigma) || sigma < 0) return FADESIM_E_ARG;
    if (n == 0) return FADESIM_OK;
    vary_conductance_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(G, divisor, n, (float)sigma, seed, offset,
                                                                          out);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_quantize_f32(const float *x, long long n, int s, int32_t *q, void *stream) {
    if (!x || !q || n < 0) return FADESIM_E_ARG;
    if (n == 0) return FADESIM_OK;
    quantize_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x, n, ldexpf(1.f, s), q);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_slice_inputs_f32(const int32_t *xq, int B, int insize, int rows, int numX, int nbits,
                                        int dac_bits, float inputV, float *v, void *stream) {
    if (!xq || !v || B < 0 || rows < 1 || numX * rows < insize || nbits < 1 || dac_bits < 1) return FADESIM_E_ARG;
    const long long total = (long long)nbits * B * numX * rows;
    if (total == 0) return FADESIM_OK;
    slice_inputs_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(xq, B, insize, rows, numX, nbits, dac_bits,
                                                                          inputV, v);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_map_conductance_f32(const int32_t *wq, int insize, int outsize, int rows, int cols, int numX,
                                           int numY, int shift, int cell_bits, int negative, float dG, float Gmin,
                                           float *G, void *stream) {
    if (!wq || !G || numX * rows < insize || numY * cols < outsize || cell_bits < 1) return FADESIM_E_ARG;
    const long long total = (long long)numX * rows * numY * cols;
    map_conductance_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(wq, insize, outsize, rows, cols, numX,
                                                                             numY, shift, cell_bits, negative, dG,
                                                                             Gmin, G);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_slice_inputs_im2col_f32(const int32_t *xq, int N, int C, int H, int W, int kh, int kw, int sh,
                                               int sw, int ph, int pw, int dh, int dw, int has_ones, int ones_q,
                                               int rows, int numX, int nbits, int dac_bits, int neg_pulse,
                                               float inputV, float *v, void *stream) {
    if (!xq || !v || N < 0 || C < 1 || H < 1 || W < 1 || kh < 1 || kw < 1 || sh < 1 || sw < 1 || ph < 0 || pw < 0 ||
        dh < 1 || dw < 1 || rows < 1 || numX < 1 || nbits < 1 || dac_bits < 1 || dac_bits > 30)
        return FADESIM_E_ARG;
    Im2col g{N, C, H, W, kh, kw, sh, sw, ph, pw, dh, dw, 0, 0};
    g.OH = (H + 2 * ph - dh * (kh - 1) - 1) / sh + 1;
    g.OW = (W + 2 * pw - dw * (kw - 1) - 1) / sw + 1;
    if (H + 2 * ph - dh * (kh - 1) - 1 < 0 || W + 2 * pw - dw * (kw - 1) - 1 < 0) return FADESIM_E_ARG;
    if ((long long)numX * rows < (long long)C * kh * kw + (has_ones ? 1 : 0)) return FADESIM_E_ARG;
    const long long total = (long long)nbits * N * g.OH * g.OW * numX * rows;
    if (total == 0) return FADESIM_OK;
    slice_im2col_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(xq, g, has_ones, ones_q, rows, numX, nbits,
                                                                          dac_bits, neg_pulse, inputV, v);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_map_conductance_ref_f32(const int32_t *wq, int insize, int outsize, int rows, int cols,
                                               int numX, int numY, int shift, int cell_bits, int plus, int maximum,
                                               float dG, float Gmin, float *G, void *stream) {
    if (!wq || !G || cols < 1 || rows < 1 || (long long)numX * rows < insize || (long long)numY * cols < outsize ||
        cell_bits < 1 || shift < 0)
        return FADESIM_E_ARG;
    const long long total = (long long)numX * rows * numY * (cols + 2);
    if (total == 0) return FADESIM_OK;
    map_conductance_ref_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(
        wq, insize, outsize, rows, cols, numX, numY, shift, cell_bits, plus, maximum, dG, Gmin, G);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_adc_shift_add_ex_f32(const float *I, int ref_cols, int nbits, int nslices, int B, int numX,
                                            int ldI, int outsize, float adcUseI, float levels, float scale, int s12,
                                            int dac_bits, int cell_bits, int input_bits, int complement, float plus,
                                            const float *bias, int L, float *out, void *stream) {
    if (!I || !out || nbits < 1 || nslices < 1 || B < 0 || numX < 1 || ref_cols < 0 || L < 0) return FADESIM_E_ARG;
    if (ref_cols ? (ldI % (ref_cols + 2) != 0 || (long long)(ldI / (ref_cols + 2)) * ref_cols < outsize)
                 : outsize > ldI)
        return FADESIM_E_ARG;
    if (L > 0 && B % L != 0) return FADESIM_E_ARG;
    const long long total = (long long)B * outsize;
    if (total == 0) return FADESIM_OK;
    adc_shift_add_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(
        I, ref_cols, nbits, nslices, B, numX, ldI, outsize, adcUseI, levels, scale, s12, dac_bits, cell_bits,
        input_bits, complement, plus, bias, L, out);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_adc_shift_add_f32(const float *I, int nbits, int nslices, int B, int numX, int ldI, int outsize,
                                         float adcUseI, float levels, float scale, int s12, int dac_bits,
                                         int cell_bits, int input_bits, int complement, float *out, void *stream) {
    if (!I || !out || outsize > ldI || nbits < 1 || nslices < 1) return FADESIM_E_ARG;
    const long long total = (long long)B * outsize;
    if (total == 0) return FADESIM_OK;
    adc_shift_add_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(I, 0, nbits, nslices, B, numX, ldI,
                                                                           outsize, adcUseI, levels, scale, s12,
                                                                           dac_bits, cell_bits, input_bits, complement,
                                                                           0.f, nullptr, 0, out);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}
