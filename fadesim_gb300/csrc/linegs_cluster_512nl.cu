// Cluster-resident line relaxation kernels for tiles up to 512 x 512, sinh cells
// (cluster_impl.cuh); one translation unit per size and cell law, compiled in parallel.
#include "cluster_impl.cuh"

namespace fadesim {

cudaError_t cl_launch_cfg_512_nl(int *clusters, const SolveArgs *a, int grid, cudaStream_t st) {
    return cl_launch_cfg_t<512, true>(clusters, a, grid, st);
}

}  // namespace fadesim
