// Kernels of the learned warm-start network (sm_103a): BF16 3x3 convolutions
// on the tensor cores with FP32 accumulation, their input and weight
// gradients, pooling, upsampling, activation, loss and the Adam update.
//
// Layouts: activations NHWC bf16, channels a multiple of 16 (zero padded);
// weights [Cout][3][3][Cin] bf16 with Cout a multiple of 8; "same" zero
// padding.  The convolution is an implicit GEMM, M = pixels, N = Cout,
// K = 9 * Cin.  Where the shape allows (the warm-start network's layers) it
// runs on the tcgen05 / TMA kernel of warmnet_tc.cu; elsewhere, and on request
// (flags 8), on the kernel here, issued as mma.sync.m16n8k16 (bf16 x bf16 ->
// f32).  The input
// gradient is the forward kernel run on dY with the weights transposed and
// flipped (W'[ci][8 - tap][co] = W[co][tap][ci]); the weight gradient is a GEMM
// over pixels split across CTAs and reduced with FP32 atomics.
#include <cuda_bf16.h>
#include <stdint.h>

#include "kernels.h"

namespace {

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

constexpr int CF_M = 64;    // pixels per CTA (4 warps x 16)
constexpr int CF_K = 16;    // channels per K step
constexpr int CF_PAD = 8;   // shared-memory row padding (bf16 elements)

// Y[p, co] = act(sum_{tap, ci} X[p + tap, ci] W[co, tap, ci] + bias[co]) (+ skip[p, co])
// flags: 1 = ReLU, 2 = add skip after the activation, 4 = store FP32 (else bf16)
template <int NT>  // NT = Cout / 8 n-tiles (Cout <= 8 * NT)
__global__ void __launch_bounds__(128) conv3x3_fwd_kernel(const __nv_bfloat16 *__restrict__ X,
                                                          const __nv_bfloat16 *__restrict__ Wt,
                                                          const float *__restrict__ bias,
                                                          const __nv_bfloat16 *__restrict__ skip, void *__restrict__ Y,
                                                          int N, int H, int W, int Cin, int Cout, int flags) {
    __shared__ __align__(16) __nv_bfloat16 As[CF_M][CF_K + CF_PAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[NT * 8][CF_K + CF_PAD];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t4 = lane & 3;
    const long long P = (long long)N * H * W;
    const long long p0 = (long long)blockIdx.x * CF_M;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        for (int c0 = 0; c0 < Cin; c0 += CF_K) {
            // A: 64 pixels x 16 channels, 8 bf16 (16 B) per thread
            {
                const int r = tid >> 1, half = (tid & 1) * 8;
                const long long p = p0 + r;
                uint4 v = make_uint4(0, 0, 0, 0);
                if (p < P) {
                    const int w = (int)(p % W), h = (int)((p / W) % H);
                    const long long nimg = p / ((long long)H * W);
                    const int hh = h + dy, ww = w + dx;
                    if (hh >= 0 && hh < H && ww >= 0 && ww < W)
                        v = *reinterpret_cast<const uint4 *>(X + ((nimg * H + hh) * W + ww) * Cin + c0 + half);
                }
                *reinterpret_cast<uint4 *>(&As[r][half]) = v;
            }
            // B: Cout x 16 (k contiguous per output channel)
            for (int e = tid; e < NT * 8 * 2; e += 128) {
                const int co = e >> 1, half = (e & 1) * 8;
                uint4 v = make_uint4(0, 0, 0, 0);
                if (co < Cout) v = *reinterpret_cast<const uint4 *>(Wt + ((long long)co * 9 + tap) * Cin + c0 + half);
                *reinterpret_cast<uint4 *>(&Bs[co][half]) = v;
            }
            __syncthreads();
            uint32_t a[4];
            const int rb = warp * 16;
            a[0] = ld32(&As[rb + g][2 * t4]);
            a[1] = ld32(&As[rb + g + 8][2 * t4]);
            a[2] = ld32(&As[rb + g][2 * t4 + 8]);
            a[3] = ld32(&As[rb + g + 8][2 * t4 + 8]);
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const uint32_t b0 = ld32(&Bs[j * 8 + g][2 * t4]);
                const uint32_t b1 = ld32(&Bs[j * 8 + g][2 * t4 + 8]);
                mma_bf16(acc[j], a, b0, b1);
            }
            __syncthreads();
        }
    }
    // epilogue
#pragma unroll
    for (int j = 0; j < NT; ++j) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const long long p = p0 + warp * 16 + g + (e >> 1) * 8;
            const int co = j * 8 + 2 * t4 + (e & 1);
            if (p >= P || co >= Cout) continue;
            float v = acc[j][e] + (bias ? bias[co] : 0.f);
            if (flags & 1) v = fmaxf(v, 0.f);
            if (flags & 2) v += __bfloat162float(skip[p * Cout + co]);
            if (flags & 4) reinterpret_cast<float *>(Y)[p * Cout + co] = v;
            else reinterpret_cast<__nv_bfloat16 *>(Y)[p * Cout + co] = __float2bfloat16_rn(v);
        }
    }
}

// dW[co][tap][ci] += sum_p dY[p, co] X[p + tap, ci] over this CTA's pixel chunk.
// CTA: all Cout (<= 128) x 32 K-columns (one tap, 32 input channels).
constexpr int WG_P = 16;
__global__ void __launch_bounds__(128) conv3x3_wgrad_kernel(const __nv_bfloat16 *__restrict__ dY,
                                                            const __nv_bfloat16 *__restrict__ X,
                                                            float *__restrict__ dW, int N, int H, int W, int Cin,
                                                            int Cout, long long chunk) {
    __shared__ __align__(16) __nv_bfloat16 As[128][WG_P + CF_PAD];  // [co][pixel]
    __shared__ __align__(16) __nv_bfloat16 Bs[32][WG_P + CF_PAD];   // [ci][pixel]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t4 = lane & 3;
    const int tap = blockIdx.y / ((Cin + 31) / 32);
    const int ci0 = (blockIdx.y % ((Cin + 31) / 32)) * 32;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const long long P = (long long)N * H * W;
    const long long pa = (long long)blockIdx.x * chunk;
    const long long pb = min(P, pa + chunk);
    const int MT = (Cout + 15) / 16;  // m-tiles, <= 8; warp w takes tiles w and w + 4
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
    for (long long p0 = pa; p0 < pb; p0 += WG_P) {
        // A = dY^T: As[co][pp]
        for (int e = tid; e < 128 * WG_P; e += 128) {
            const int co = e / WG_P, pp = e % WG_P;
            const long long p = p0 + pp;
            As[co][pp] = (co < Cout && p < pb) ? dY[p * Cout + co] : __float2bfloat16_rn(0.f);
        }
        // B = shifted X: Bs[ci][pp]
        for (int e = tid; e < 32 * WG_P; e += 128) {
            const int ci = e / WG_P, pp = e % WG_P;
            const long long p = p0 + pp;
            __nv_bfloat16 v = __float2bfloat16_rn(0.f);
            if (p < pb && ci0 + ci < Cin) {
                const int w = (int)(p % W), h = (int)((p / W) % H);
                const long long nimg = p / ((long long)H * W);
                const int hh = h + dy, ww = w + dx;
                if (hh >= 0 && hh < H && ww >= 0 && ww < W) v = X[((nimg * H + hh) * W + ww) * Cin + ci0 + ci];
            }
            Bs[ci][pp] = v;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int mt = warp + 4 * i;
            if (mt < MT) {
                uint32_t a[4];
                a[0] = ld32(&As[mt * 16 + g][2 * t4]);
                a[1] = ld32(&As[mt * 16 + g + 8][2 * t4]);
                a[2] = ld32(&As[mt * 16 + g][2 * t4 + 8]);
                a[3] = ld32(&As[mt * 16 + g + 8][2 * t4 + 8]);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t b0 = ld32(&Bs[j * 8 + g][2 * t4]);
                    const uint32_t b1 = ld32(&Bs[j * 8 + g][2 * t4 + 8]);
                    mma_bf16(acc[i][j], a, b0, b1);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int mt = warp + 4 * i;
        if (mt >= MT) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int co = mt * 16 + g + (e >> 1) * 8;
                const int ci = ci0 + j * 8 + 2 * t4 + (e & 1);
                if (co < Cout && ci < Cin) atomicAdd(&dW[((long long)co * 9 + tap) * Cin + ci], acc[i][j][e]);
            }
    }
}

// W'[ci][8 - tap][co] = W[co][tap][ci] (transposed, flipped) for the input gradient
__global__ void weight_flip_kernel(const __nv_bfloat16 *__restrict__ Wt, __nv_bfloat16 *__restrict__ Wf, int Cin,
                                   int Cout, int Cin_pad8) {
    const long long total = (long long)Cin_pad8 * 9 * Cout;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int co = (int)(e % Cout);
        const int tap = (int)((e / Cout) % 9);
        const int ci = (int)(e / ((long long)Cout * 9));
        Wf[e] = ci < Cin ? Wt[((long long)co * 9 + (8 - tap)) * Cin + ci] : __float2bfloat16_rn(0.f);
    }
}

__global__ void bias_grad_kernel(const __nv_bfloat16 *__restrict__ dY, float *__restrict__ db, long long P, int C) {
    // one CTA per channel chunk of 32; threads stride over pixels
    const int c = blockIdx.y * 32 + (threadIdx.x & 31);
    float s = 0.f;
    if (c < C)
        for (long long p = blockIdx.x * 8 + (threadIdx.x >> 5); p < P; p += (long long)gridDim.x * 8)
            s += __bfloat162float(dY[p * C + c]);
    if (c < C) atomicAdd(&db[c], s);
}

__global__ void avgpool2_kernel(const __nv_bfloat16 *__restrict__ X, __nv_bfloat16 *__restrict__ Y, int N, int H,
                                int W, int C, int backward) {
    // forward: Y[n, h/2, w/2, c] = mean of the 2x2 block; backward: X is dY (H/2 x W/2), Y is dX (H x W)
    const int Ho = H / 2, Wo = W / 2;
    const long long total = backward ? (long long)N * H * W * C : (long long)N * Ho * Wo * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        if (!backward) {
            const long long q = e / C;
            const int wo = (int)(q % Wo), ho = (int)((q / Wo) % Ho);
            const long long n = q / ((long long)Wo * Ho);
            const __nv_bfloat16 *b = X + ((n * H + 2 * ho) * W + 2 * wo) * C + c;
            const float s = __bfloat162float(b[0]) + __bfloat162float(b[C]) + __bfloat162float(b[(long long)W * C]) +
                            __bfloat162float(b[(long long)W * C + C]);
            Y[e] = __float2bfloat16_rn(0.25f * s);
        } else {
            const long long q = e / C;
            const int w = (int)(q % W), h = (int)((q / W) % H);
            const long long n = q / ((long long)W * H);
            Y[e] = __float2bfloat16_rn(0.25f * __bfloat162float(X[((n * Ho + h / 2) * Wo + w / 2) * C + c]));
        }
    }
}

__global__ void upsample2_kernel(const __nv_bfloat16 *__restrict__ X, __nv_bfloat16 *__restrict__ Y, int N, int H,
                                 int W, int C, int backward) {
    // forward: Y (2H x 2W) nearest from X (H x W); backward: X is dY (2H x 2W), Y is dX (H x W) = 2x2 block sums
    const long long total = backward ? (long long)N * H * W * C : (long long)N * 4 * H * W * C;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const long long q = e / C;
        if (!backward) {
            const int w2 = (int)(q % (2 * W)), h2 = (int)((q / (2 * W)) % (2 * H));
            const long long n = q / (4LL * W * H);
            Y[e] = X[((n * H + h2 / 2) * W + w2 / 2) * C + c];
        } else {
            const int w = (int)(q % W), h = (int)((q / W) % H);
            const long long n = q / ((long long)W * H);
            const long long W2 = 2LL * W;
            const __nv_bfloat16 *b = X + ((n * 2 * H + 2 * h) * W2 + 2 * w) * C + c;
            Y[e] = __float2bfloat16_rn(__bfloat162float(b[0]) + __bfloat162float(b[C]) +
                                       __bfloat162float(b[W2 * C]) + __bfloat162float(b[W2 * C + C]));
        }
    }
}

// dZ = dY * (Y > 0) (ReLU backward from the activation's output), optionally + extra
__global__ void relu_bwd_kernel(const __nv_bfloat16 *__restrict__ dY, const __nv_bfloat16 *__restrict__ Yact,
                                __nv_bfloat16 *__restrict__ dZ, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        dZ[e] = __bfloat162float(Yact[e]) > 0.f ? dY[e] : __float2bfloat16_rn(0.f);
}

__global__ void add_bf16_kernel(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B,
                                __nv_bfloat16 *__restrict__ C, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        C[e] = __float2bfloat16_rn(__bfloat162float(A[e]) + __bfloat162float(B[e]));
}

// loss = mean (pred - target)^2 over valid channels; dpred (bf16) = 2 (pred - target) / count
__global__ void mse_kernel(const float *__restrict__ pred, const float *__restrict__ target,
                           __nv_bfloat16 *__restrict__ dpred, float *__restrict__ loss, long long P, int Cp, int Cv) {
    float s = 0.f;
    const float inv = 1.f / (float)(P * Cv);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < P * Cp; e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e % Cp);
        float gval = 0.f;
        if (c < Cv) {
            const float d = pred[e] - target[(e / Cp) * Cv + c];
            s += d * d;
            gval = 2.f * d * inv;
        }
        dpred[e] = __float2bfloat16_rn(gval);
    }
    s = s * inv;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

// Adam (FP32 master weights), refresh the bf16 copy
__global__ void adam_kernel(float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, const float *__restrict__ gr,
                            float *__restrict__ m, float *__restrict__ v, long long n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float gg = gr[e];
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        const float nw = w[e] - lr * (mm * c1) / (sqrtf(vv * c2) + eps);
        w[e] = nw;
        if (wb) wb[e] = __float2bfloat16_rn(nw);
    }
}

int gridn(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g > 65535 ? 65535 : (g < 1 ? 1 : g));
}

}  // namespace

extern "C" int fadesim_conv3x3_fwd_bf16(const void *X, const void *W, const float *bias, const void *skip, void *Y,
                                        int N, int H, int Wd, int Cin, int Cout, int flags, void *stream) {
    if (!X || !W || !Y || Cin % 16 || Cout % 8 || Cout > 128 || Cout < 8 || ((flags & 2) && !skip)) return FADESIM_E_ARG;
    if (!(flags & 8) && fadesim::conv3x3_tc_supported(X, W, Y, H, Wd, Cin, Cout)) {
        // the tensor-core (tcgen05 / TMA) kernel for the network's shapes
        const cudaError_t e = fadesim::conv3x3_fwd_tc(X, W, bias, skip, Y, N, H, Wd, Cin, Cout, flags & 7,
                                                      fadesim::conv_tc_error_flag(), (cudaStream_t)stream);
        return e == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
    }
    const long long P = (long long)N * H * Wd;
    const dim3 grid((unsigned)((P + CF_M - 1) / CF_M));
    const __nv_bfloat16 *x = (const __nv_bfloat16 *)X, *w = (const __nv_bfloat16 *)W, *sk = (const __nv_bfloat16 *)skip;
    cudaStream_t st = (cudaStream_t)stream;
    switch (Cout / 8) {
#define CASE(k) case k: conv3x3_fwd_kernel<k><<<grid, 128, 0, st>>>(x, w, bias, sk, Y, N, H, Wd, Cin, Cout, flags); break;
        CASE(1) CASE(2) CASE(3) CASE(4) CASE(5) CASE(6) CASE(7) CASE(8) CASE(9) CASE(10) CASE(11) CASE(12) CASE(13)
        CASE(14) CASE(15) CASE(16)
#undef CASE
        default: return FADESIM_E_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_conv3x3_wgrad_bf16(const void *dY, const void *X, float *dW, int N, int H, int Wd, int Cin,
                                          int Cout, void *stream) {
    if (!dY || !X || !dW || Cout > 128 || Cin < 1) return FADESIM_E_ARG;
    if (fadesim::conv3x3_wgrad_tc_supported(dY, X, H, Wd, Cin, Cout)) {
        const cudaError_t e = fadesim::conv3x3_wgrad_tc(dY, X, dW, N, H, Wd, Cin, Cout, fadesim::conv_tc_error_flag(),
                                                        (cudaStream_t)stream);
        return e == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
    }
    const long long P = (long long)N * H * Wd;
    long long chunk = 1024;
    long long nchunks = (P + chunk - 1) / chunk;
    if (nchunks > 4096) {
        nchunks = 4096;
        chunk = ((P + nchunks - 1) / nchunks + WG_P - 1) / WG_P * WG_P;
        nchunks = (P + chunk - 1) / chunk;
    }
    const dim3 grid((unsigned)nchunks, (unsigned)(9 * ((Cin + 31) / 32)));
    conv3x3_wgrad_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)dY, (const __nv_bfloat16 *)X,
                                                                  dW, N, H, Wd, Cin, Cout, chunk);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_weight_flip_bf16(const void *W, void *Wf, int Cin, int Cout, int Cin_pad8, void *stream) {
    const long long n = (long long)Cin_pad8 * 9 * Cout;
    weight_flip_kernel<<<gridn(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)W, (__nv_bfloat16 *)Wf, Cin,
                                                                   Cout, Cin_pad8);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_bias_grad_bf16(const void *dY, float *db, long long P, int C, void *stream) {
    const dim3 grid(256, (unsigned)((C + 31) / 32));
    bias_grad_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)dY, db, P, C);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_pool_bf16(const void *X, void *Y, int N, int H, int W, int C, int backward, int upsample,
                                 void *stream) {
    const long long n = (long long)N * H * W * C * (upsample && !backward ? 4 : 1);
    if (upsample)
        upsample2_kernel<<<gridn(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)X, (__nv_bfloat16 *)Y, N,
                                                                     H, W, C, backward);
    else
        avgpool2_kernel<<<gridn(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)X, (__nv_bfloat16 *)Y, N, H,
                                                                    W, C, backward);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_relu_bwd_bf16(const void *dY, const void *Yact, void *dZ, long long n, void *stream) {
    relu_bwd_kernel<<<gridn(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)dY,
                                                                (const __nv_bfloat16 *)Yact, (__nv_bfloat16 *)dZ, n);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_add_bf16(const void *A, const void *B, void *C, long long n, void *stream) {
    add_bf16_kernel<<<gridn(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B,
                                                                (__nv_bfloat16 *)C, n);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_mse_f32(const float *pred, const float *target, void *dpred, float *loss, long long P, int Cp,
                               int Cv, void *stream) {
    mse_kernel<<<gridn(P * Cp), 256, 0, (cudaStream_t)stream>>>(pred, target, (__nv_bfloat16 *)dpred, loss, P, Cp, Cv);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}

extern "C" int fadesim_adam_f32(float *w, void *wb, const float *g, float *m, float *v, long long n, float lr,
                                float b1, float b2, float eps, int step, void *stream) {
    const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
    adam_kernel<<<gridn(n), 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16 *)wb, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}
