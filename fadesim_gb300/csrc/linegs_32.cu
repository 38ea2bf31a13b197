// Block line relaxation kernels for tiles up to 32 x 32 (line_impl.cuh).
#include "line_impl.cuh"

namespace fadesim {

cudaError_t line_relax_prepare_32() { return line_relax_prepare_t<32>(); }
cudaError_t line_relax_occupancy_32(int *n) { return line_relax_occupancy_t<32>(n); }
cudaError_t launch_line_relax_32(const SolveArgs &a, int grid, cudaStream_t st) {
    return launch_line_relax_t<32>(a, grid, st);
}

}  // namespace fadesim
