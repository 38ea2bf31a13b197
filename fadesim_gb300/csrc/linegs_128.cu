// Block line relaxation kernels for tiles up to 128 x 128 (line_impl.cuh).
#include "line_impl.cuh"

namespace fadesim {

cudaError_t line_relax_prepare_128() { return line_relax_prepare_t<128>(); }
cudaError_t line_relax_occupancy_128(int *n) { return line_relax_occupancy_t<128>(n); }
cudaError_t launch_line_relax_128(const SolveArgs &a, int grid, cudaStream_t st) {
    return launch_line_relax_t<128>(a, grid, st);
}

}  // namespace fadesim
