// Dispatch of the cluster-resident line relaxation kernels (cluster_impl.cuh)
// by tile size; each size is compiled in its own translation unit.
#include "cluster_impl.cuh"

namespace fadesim {

cudaError_t cl_launch_cfg_256(int *clusters, const SolveArgs *a, int grid, cudaStream_t st);
cudaError_t cl_launch_cfg_512(int *clusters, const SolveArgs *a, int grid, cudaStream_t st);
cudaError_t cl_launch_cfg_256_nl(int *clusters, const SolveArgs *a, int grid, cudaStream_t st);
cudaError_t cl_launch_cfg_512_nl(int *clusters, const SolveArgs *a, int grid, cudaStream_t st);

int cluster_relax_ld(int n, int m) {
    const int L = n > m ? n : m;
    if (L <= 128) return 0;
    if (L <= 256) return 256;
    if (L <= 512) return 512;
    return 0;
}

int cluster_relax_size(int ld) { return ld == 256 ? CCfg<256>::C : CCfg<512>::C; }

size_t cluster_relax_scratch_floats_per_cta(int) { return (size_t)3 * CL_SEG * CL_T + 2 * CL_T; }

// The I/O type travels in the launch arguments (SolveArgs::f64).
cudaError_t cluster_relax_occupancy(int ld, int, int *clusters) {
    if (ld == 256) return cl_launch_cfg_256(clusters, nullptr, 0, 0);
    if (ld == 512) return cl_launch_cfg_512(clusters, nullptr, 0, 0);
    return cudaErrorInvalidValue;
}

cudaError_t launch_cluster_relax(const SolveArgs &a, int ld, int, int grid, cudaStream_t st) {
    if (ld == 256)
        return a.ctl.nl ? cl_launch_cfg_256_nl(nullptr, &a, grid, st) : cl_launch_cfg_256(nullptr, &a, grid, st);
    if (ld == 512)
        return a.ctl.nl ? cl_launch_cfg_512_nl(nullptr, &a, grid, st) : cl_launch_cfg_512(nullptr, &a, grid, st);
    return cudaErrorInvalidValue;
}

}  // namespace fadesim
