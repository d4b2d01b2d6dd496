// sweep_f64.cu -- instantiation of the solver kernels for double storage and arithmetic.
// Built with --fmad=false and IEEE division / square root: bit-exact with the reference's
// strict FP64 build.
#include "solver_kernels.cuh"

namespace armon {

cudaError_t launch_sweep(const SweepArgs<double>& a, int scheme, int proj, bool last, int grid, int block,
                         cudaStream_t st)
{
    return launch_sweep_t<double>(a, scheme, proj, last, grid, block, st);
}

cudaError_t launch_sweep_batch(const SweepArgs<double>* doms, const int* offsets, int ndom, int total_blocks, int pass,
                               BatchOrder ord, int scheme, int proj, bool last, int block, cudaStream_t st)
{
    return launch_sweep_batch_t<double>(doms, offsets, ndom, total_blocks, pass, ord, scheme, proj, last, block, st);
}

int sweep_blocks_per_sm_f64(int scheme, int proj, int block)
{
    return sweep_blocks_per_sm_t<double>(scheme, proj, block);
}

int sweep_batch_blocks_per_sm_f64(int scheme, int proj, int block)
{
    return sweep_batch_blocks_per_sm_t<double>(scheme, proj, block);
}

cudaError_t launch_init_f64(const InitArgs& a, int64_t ncells, const InitPtrs& p, cudaStream_t st)
{
    int64_t blocks = (ncells + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    init_kernel<double><<<(int)blocks, 256, 0, st>>>(a, ncells, p);
    return cudaGetLastError();
}

cudaError_t launch_init_sod_f64(const SodInit& a, int64_t ncells, void* rho, void* umat, void* vmat, void* Emat,
                                cudaStream_t st)
{
    int64_t blocks = (ncells + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    init_sod_kernel<double><<<(int)blocks, 256, 0, st>>>(a, ncells, (double*)rho, (double*)umat, (double*)vmat, (double*)Emat);
    return cudaGetLastError();
}

cudaError_t launch_begin_f64(const BeginArgs& a, int grid, cudaStream_t st)
{
    begin_kernel<double><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_conservation_f64(const ConsArgs& a, int grid, cudaStream_t st)
{
    conservation_partial_kernel<double><<<grid, 256, 0, st>>>(a);
    conservation_final_kernel<<<1, 32, 0, st>>>(a.partials, grid, a.out);
    return cudaGetLastError();
}

}  // namespace armon
