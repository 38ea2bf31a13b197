// Shared-memory read bandwidth probe (sm_103a): the measured denominator of the
// line kernels' shared-memory roofline.
//
// Every CTA of 1024 threads fills 32 KB of shared memory, then each thread
// reads 16-byte words, consecutive threads at consecutive addresses (a warp's
// LDS.128 covers 512 contiguous bytes: four conflict-free wavefronts), at a
// stride that walks the whole buffer, into eight independent sums;
// one sum per CTA goes to global memory so nothing is optimised away.  Bytes
// read = blocks x 1024 x iters x 16; two CTAs fit an SM.
#include "kernels.h"

namespace {

constexpr int kThreads = 1024;
constexpr int kWords = 2048;  // float4 words: 32 KB

__global__ void __launch_bounds__(kThreads, 2) smem_read_kernel(float *__restrict__ sink, int iters) {
    __shared__ float4 buf[kWords];
    const int tid = threadIdx.x;
    for (int w = tid; w < kWords; w += kThreads)
        buf[w] = make_float4((float)w, (float)(w + 1), (float)(w + 2), (float)(w + 3));
    __syncthreads();
    float acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = 0.f;
    int base = tid;
    for (int it = 0; it < iters; it += 8) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            // eight distinct addresses per step (k * kWords / 8 apart): no two
            // loads of one step may coincide, or the compiler merges them
            const float4 v = buf[(base + k * (kWords / 8)) & (kWords - 1)];
            acc[k] += (v.x + v.y) + (v.z + v.w);
        }
        base = (base + 32) & (kWords - 1);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += acc[k];
    s = fadesim::warp_max(s);
    if ((tid & 31) == 0) atomicAdd(&sink[blockIdx.x], s);
}

}  // namespace

extern "C" int fadesim_smem_read_probe(float *sink, int blocks, int iters, void *stream) {
    if (!sink || blocks < 1 || iters < 8 || iters % 8 != 0) return FADESIM_E_ARG;
    smem_read_kernel<<<blocks, kThreads, 0, (cudaStream_t)stream>>>(sink, iters);
    return cudaGetLastError() == cudaSuccess ? FADESIM_OK : FADESIM_E_CUDA;
}
