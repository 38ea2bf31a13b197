// Integer stages of PimTorch's bit-sliced crossbar matmul (sm_103a), bit-exact
// with the reference's float32 arithmetic given the same bitline currents.
//
// Reference: pimtorch/pimfixedpoint/fixedPoint/nn/splitArrayArithmetic.py
//   splitArr_matmul_nn :1161-1228 (quantise, PN split, bit/slice loops, shift-add)
//   matmul :705-757 (padding, input voltages, conductance map), :835-836 (ADC),
//          :961-978 (sum over row tiles, crop, scale, pos - neg)
// and fixedPoint/nn/fixedPointArithmetic.py:76-96 (quantisation).
//
// Every float operation is a separately rounded IEEE float32 op in the
// reference's order (__fmul_rn / __fadd_rn / __fdiv_rn keep the compiler from
// fusing them); scalar operands arrive already rounded to float32, as torch
// rounds a Python scalar combined with a float32 tensor.
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

// One output element per thread: the reference's loops over input bits i and
// weight slices j, in order, with ADC codes summed over row tiles.
//   I[j][pn][i][b][x][o] currents (pn 0 = positive array), as the solves for one
//   (slice, array) pair produce them with the input bits stacked on the batch.
__global__ void adc_shift_add_kernel(const float *__restrict__ I, int nbits, int nslices, int B, int numX, int ldI,
                                     int outsize, float adcUseI, float levels, float scale, int s12, int dac_bits,
                                     int cell_bits, int input_bits, int complement, float *__restrict__ out) {
    const long long total = (long long)B * outsize;
    const long long vec = (long long)numX * ldI;  // one input vector's currents
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int o = (int)(e % outsize);
        const long long b = e / outsize;
        float acc = 0.f;
        for (int i = 0; i < nbits; ++i) {
            for (int j = 0; j < nslices; ++j) {
                const float *Ip = I + (((long long)(j * 2 + 0) * nbits + i) * B + b) * vec + o;
                const float *In = I + (((long long)(j * 2 + 1) * nbits + i) * B + b) * vec + o;
                float cp = 0.f, cn = 0.f;  // integer-valued: sums are exact
                for (int x = 0; x < numX; ++x) {
                    cp = __fadd_rn(cp, rintf(__fmul_rn(__fdiv_rn(Ip[(long long)x * ldI], adcUseI), levels)));
                    cn = __fadd_rn(cn, rintf(__fmul_rn(__fdiv_rn(In[(long long)x * ldI], adcUseI), levels)));
                }
                const float d = __fsub_rn(__fmul_rn(cp, scale), __fmul_rn(cn, scale));
                const int k = i * dac_bits + j * cell_bits + s12;
                const float t = __fmul_rn(d, ldexpf(1.f, k));  // power of two: exact
                acc = (i * dac_bits != input_bits - 1 || !complement) ? __fadd_rn(acc, t) : __fsub_rn(acc, t);
            }
        }
        out[e] = acc;
    }
}

int grid_for(long long total) {
    long long g = (total + 255) / 256;
    return (int)(g > 16384 ? 16384 : (g < 1 ? 1 : g));
}

}  // namespace

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

extern "C" int fadesim_adc_shift_add_f32(const float *I, int nbits, int nslices, int B, int numX, int ldI, int outsize,
                                         float adcUseI, float levels, float scale, int s12, int dac_bits,
                                         int cell_bits, int input_bits, int complement, float *out, void *stream) {
    if (!I || !out || outsize > ldI || nbits < 1 || nslices < 1) return FADESIM_E_ARG;
    const long long total = (long long)B * outsize;
    if (total == 0) return FADESIM_OK;
    adc_shift_add_kernel<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(I, nbits, nslices, B, numX, ldI, outsize,
                                                                           adcUseI, levels, scale, s12, dac_bits,
                                                                           cell_bits, input_bits, complement, out);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}
