// Dispatch of the block line relaxation kernels (line_impl.cuh) by tile size;
// each size's kernels are compiled in their own translation unit.
#include "line_impl.cuh"

namespace fadesim {

cudaError_t line_relax_prepare_32();
cudaError_t line_relax_prepare_64();
cudaError_t line_relax_prepare_128();
cudaError_t line_relax_occupancy_32(int *n);
cudaError_t line_relax_occupancy_64(int *n);
cudaError_t line_relax_occupancy_128(int *n);
cudaError_t launch_line_relax_32(const SolveArgs &a, int grid, cudaStream_t st);
cudaError_t launch_line_relax_64(const SolveArgs &a, int grid, cudaStream_t st);
cudaError_t launch_line_relax_128(const SolveArgs &a, int grid, cudaStream_t st);

int line_relax_ld(int n, int m) {
    const int L = n > m ? n : m;
    if (L <= 32) return 32;
    if (L <= 64) return 64;
    if (L <= 128) return 128;
    return 0;
}

static int nwarps(int ld) { return ld == 128 ? LineCfg<128>::NW : (ld == 64 ? LineCfg<64>::NW : LineCfg<32>::NW); }
int line_relax_threads(int ld) { return nwarps(ld) * 32; }
size_t line_relax_smem(int ld) { return line_relax_smem_ld(ld, nwarps(ld)); }
// chain multipliers of both passes (2 x SEG x T = 2 x LD x LD floats), segment products (2 x T) and, on
// the 32 and 64 layouts, the wordline unit response of linear cells (SEG x T)
size_t line_relax_scratch_floats_per_cta(int ld) {
    return (size_t)(ld < 128 ? 3 : 2) * ld * ld + 2 * (size_t)nwarps(ld) * 32;
}

// The I/O type is carried by the launch arguments (SolveArgs::f64); dtype is
// accepted for symmetry with the other solvers.
cudaError_t line_relax_prepare(int ld, int) {
    switch (ld) {
        case 32: return line_relax_prepare_32();
        case 64: return line_relax_prepare_64();
        case 128: return line_relax_prepare_128();
    }
    return cudaErrorInvalidValue;
}

cudaError_t line_relax_occupancy(int ld, int, int *ctas) {
    switch (ld) {
        case 32: return line_relax_occupancy_32(ctas);
        case 64: return line_relax_occupancy_64(ctas);
        case 128: return line_relax_occupancy_128(ctas);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_line_relax(const SolveArgs &a, int ld, int, int grid, cudaStream_t st) {
    switch (ld) {
        case 32: return launch_line_relax_32(a, grid, st);
        case 64: return launch_line_relax_64(a, grid, st);
        case 128: return launch_line_relax_128(a, grid, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace fadesim
