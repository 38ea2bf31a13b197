// The two-level block line relaxation on full 128 x 128 tiles with linear
// cells (line_impl.cuh, coarse_impl.cuh): its own translation unit.
#include "line_impl.cuh"

namespace fadesim {

cudaError_t line_relax_prepare_128_coarse() {
    return cudaFuncSetAttribute(line_relax_kernel<128, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)line_relax_smem_two(128, LineCfg<128>::NW));
}

cudaError_t launch_line_relax_128_coarse(const SolveArgs &a, int grid, cudaStream_t st) {
    line_relax_kernel<128, false, true, true>
        <<<grid, LineCfg<128>::T, line_relax_smem_two(128, LineCfg<128>::NW), st>>>(a);
    return cudaGetLastError();
}

}  // namespace fadesim
