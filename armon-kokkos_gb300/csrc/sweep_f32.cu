// sweep_f32.cu -- instantiation of the solver kernels for float storage and arithmetic.
// Built without FMA contraction, like the FP64 units: every operation rounds on its own, so the
// single-domain and the batched kernels (separately compiled) give the same bits, and a domain's
// result does not depend on what it shares a launch with.  The FP32 variant is compared with the
// FP64 oracle by tolerance (dt and the conservation sums stay FP64).
#include "solver_kernels.cuh"

namespace armon {

cudaError_t launch_sweep(const SweepArgs<float>& a, int scheme, int proj, bool last, int grid, int block,
                         cudaStream_t st)
{
    return launch_sweep_t<float>(a, scheme, proj, last, grid, block, st);
}

cudaError_t launch_sweep_batch(const SweepArgs<float>* doms, const int* offsets, int ndom, int total_blocks, int pass,
                               BatchOrder ord, int scheme, int proj, bool last, int block, cudaStream_t st)
{
    return launch_sweep_batch_t<float>(doms, offsets, ndom, total_blocks, pass, ord, scheme, proj, last, block, st);
}

int sweep_blocks_per_sm_f32(int scheme, int proj, int block)
{
    return sweep_blocks_per_sm_t<float>(scheme, proj, block);
}

int sweep_batch_blocks_per_sm_f32(int scheme, int proj, int block)
{
    return sweep_batch_blocks_per_sm_t<float>(scheme, proj, block);
}

cudaError_t launch_init_f32(const InitArgs& a, int64_t ncells, const InitPtrs& p, cudaStream_t st)
{
    int64_t blocks = (ncells + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    init_kernel<float><<<(int)blocks, 256, 0, st>>>(a, ncells, p);
    return cudaGetLastError();
}

cudaError_t launch_init_sod_f32(const SodInit& a, int64_t ncells, void* rho, void* umat, void* vmat, void* Emat,
                                cudaStream_t st)
{
    int64_t blocks = (ncells + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    init_sod_kernel<float><<<(int)blocks, 256, 0, st>>>(a, ncells, (float*)rho, (float*)umat, (float*)vmat, (float*)Emat);
    return cudaGetLastError();
}

cudaError_t launch_begin_f32(const BeginArgs& a, int grid, cudaStream_t st)
{
    begin_kernel<float><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_conservation_f32(const ConsArgs& a, int grid, cudaStream_t st)
{
    conservation_partial_kernel<float><<<grid, 256, 0, st>>>(a);
    conservation_final_kernel<<<1, 32, 0, st>>>(a.partials, grid, a.out);
    return cudaGetLastError();
}

}  // namespace armon
