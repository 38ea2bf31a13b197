// Block line relaxation kernels for tiles up to 64 x 64 (line_impl.cuh).
#include "line_impl.cuh"

namespace fadesim {

cudaError_t line_relax_prepare_64() { return line_relax_prepare_t<64>(); }
cudaError_t line_relax_occupancy_64(int *n) { return line_relax_occupancy_t<64>(n); }
cudaError_t launch_line_relax_64(const SolveArgs &a, int grid, cudaStream_t st) {
    return launch_line_relax_t<64>(a, grid, st);
}

}  // namespace fadesim
