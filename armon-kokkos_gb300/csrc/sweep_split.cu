// sweep_split.cu -- the two halves of a split axis pass (sweep_split.cuh) for both storage types.
// Built with --fmad=false and IEEE division / square root, like the fused pass.
#include "launch.h"
#include "sweep_split.cuh"

namespace armon {
namespace {

template <class T, int S, int P, bool L>
cudaError_t launch_split_one(const SweepArgs<T>& a, int grid, int block, cudaStream_t st)
{
    sweep_faces_kernel<T, S, L><<<grid, block, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sweep_cells_kernel<T, S, P, L><<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_split_t(const SweepArgs<T>& a, int scheme, int proj, bool last, int grid, int block, cudaStream_t st)
{
#define ARMON_S(S, P) return last ? launch_split_one<T, S, P, true>(a, grid, block, st) : launch_split_one<T, S, P, false>(a, grid, block, st)
    if (scheme == 1) {
        if (proj == 2) ARMON_S(1, 2);
        ARMON_S(1, 1);
    }
    if (proj == 2) ARMON_S(0, 2);
    ARMON_S(0, 1);
#undef ARMON_S
}

}  // namespace

cudaError_t launch_sweep_split(const SweepArgs<double>& a, int scheme, int proj, bool last, int grid, int block,
                               cudaStream_t st)
{
    return launch_split_t<double>(a, scheme, proj, last, grid, block, st);
}

cudaError_t launch_sweep_split(const SweepArgs<float>& a, int scheme, int proj, bool last, int grid, int block,
                               cudaStream_t st)
{
    return launch_split_t<float>(a, scheme, proj, last, grid, block, st);
}

}  // namespace armon
