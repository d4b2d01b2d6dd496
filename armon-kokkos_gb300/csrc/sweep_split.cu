// sweep_split.cu -- the two halves of a split axis pass (sweep_split.cuh) for both storage types.
// Built with --fmad=false and IEEE division / square root, like the fused pass.
#include "launch.h"
#include "sweep_split.cuh"

namespace armon {
namespace {

template <class T, int S, int P, bool L>
cudaError_t launch_split_one(const SweepArgs<T>& a, int grid, int block, cudaStream_t st)
{
    sweep_faces_kernel<T, S, P, L><<<grid, block, 0, st>>>(a);
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

template <class T, int S, int P, bool L>
cudaError_t launch_batch_split_one(const SweepArgs<T>* doms, const int* offsets, int ndom, int grid, int pass,
                                   BatchOrder faces, BatchOrder cells, int block, cudaStream_t st)
{
    sweep_batch_faces_kernel<T, S, P, L><<<grid, block, 0, st>>>(doms, offsets, ndom, pass, faces);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    sweep_batch_cells_kernel<T, S, P, L><<<grid, block, 0, st>>>(doms, offsets, ndom, pass, cells);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_batch_split_t(const SweepArgs<T>* doms, const int* offsets, int ndom, int grid, int pass,
                                 BatchOrder faces, BatchOrder cells, int scheme, int proj, bool last, int block,
                                 cudaStream_t st)
{
#define ARMON_S(S, P)                                                                                              \
    return last ? launch_batch_split_one<T, S, P, true>(doms, offsets, ndom, grid, pass, faces, cells, block, st)  \
                : launch_batch_split_one<T, S, P, false>(doms, offsets, ndom, grid, pass, faces, cells, block, st)
    if (scheme == 1) {
        if (proj == 2) ARMON_S(1, 2);
        ARMON_S(1, 1);
    }
    if (proj == 2) ARMON_S(0, 2);
    ARMON_S(0, 1);
#undef ARMON_S
}

template <class T>
int batch_split_blocks_per_sm_t(int scheme, int proj, int block)
{
    int n = 0;
    cudaError_t e;
    if (scheme == 1)
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_cells_kernel<T, 1, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_cells_kernel<T, 1, 1, true>, block, 0);
    else
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_cells_kernel<T, 0, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_cells_kernel<T, 0, 1, true>, block, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

template <class T>
int split_blocks_per_sm_t(int scheme, int proj, int block)
{
    int n = 0;
    cudaError_t e;
    if (scheme == 1)
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_cells_kernel<T, 1, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_cells_kernel<T, 1, 1, true>, block, 0);
    else
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_cells_kernel<T, 0, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_cells_kernel<T, 0, 1, true>, block, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

}  // namespace

int sweep_split_blocks_per_sm(bool fp32, int scheme, int proj, int block)
{
    return fp32 ? split_blocks_per_sm_t<float>(scheme, proj, block) : split_blocks_per_sm_t<double>(scheme, proj, block);
}

cudaError_t launch_sweep_batch_split(const SweepArgs<double>* doms, const int* offsets, int ndom, int total_blocks,
                                     int pass, BatchOrder faces, BatchOrder cells, int scheme, int proj, bool last,
                                     int block, cudaStream_t st)
{
    return launch_batch_split_t<double>(doms, offsets, ndom, total_blocks, pass, faces, cells, scheme, proj, last, block,
                                        st);
}

cudaError_t launch_sweep_batch_split(const SweepArgs<float>* doms, const int* offsets, int ndom, int total_blocks,
                                     int pass, BatchOrder faces, BatchOrder cells, int scheme, int proj, bool last,
                                     int block, cudaStream_t st)
{
    return launch_batch_split_t<float>(doms, offsets, ndom, total_blocks, pass, faces, cells, scheme, proj, last, block,
                                       st);
}

int sweep_batch_split_blocks_per_sm(bool fp32, int scheme, int proj, int block)
{
    return fp32 ? batch_split_blocks_per_sm_t<float>(scheme, proj, block)
                : batch_split_blocks_per_sm_t<double>(scheme, proj, block);
}

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
