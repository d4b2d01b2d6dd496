// launch.h -- host-side launchers of the solver kernels, one overload per storage type.
// sweep_f64.cu and sweep_f32.cu (both built with --fmad=false) define them; solver.cu and
// batch.cu drive them.
#pragma once

#include <cuda_runtime.h>

#include "init.cuh"
#include "sweep.cuh"

namespace armon {

// Fused axis pass (sweep.cuh).
cudaError_t launch_sweep(const SweepArgs<double>& a, int scheme, int proj, bool last, int grid, int block,
                         cudaStream_t st);
cudaError_t launch_sweep(const SweepArgs<float>& a, int scheme, int proj, bool last, int grid, int block,
                         cudaStream_t st);

// Split axis pass (sweep_split.cuh): the face half, then the cell half, on the same grid; a.faces
// must hold 3 * a.face_stride values.
cudaError_t launch_sweep_split(const SweepArgs<double>& a, int scheme, int proj, bool last, int grid, int block,
                               cudaStream_t st);
cudaError_t launch_sweep_split(const SweepArgs<float>& a, int scheme, int proj, bool last, int grid, int block,
                               cudaStream_t st);

// Split axis pass over many domains: the face half with order `faces`, then the cell half with
// order `cells`; each domain's arguments carry its face buffer.
cudaError_t launch_sweep_batch_split(const SweepArgs<double>* doms, const int* offsets, int ndom, int total_blocks,
                                     int pass, BatchOrder faces, BatchOrder cells, int scheme, int proj, bool last,
                                     int block, cudaStream_t st);
cudaError_t launch_sweep_batch_split(const SweepArgs<float>* doms, const int* offsets, int ndom, int total_blocks,
                                     int pass, BatchOrder faces, BatchOrder cells, int scheme, int proj, bool last,
                                     int block, cudaStream_t st);
// Blocks of the split batch pass's cell half resident on one SM.
int sweep_batch_split_blocks_per_sm(bool fp32, int scheme, int proj, int block);
// Blocks of the split pass's cell half (sweep_cells_kernel, last pass of a cycle) resident on one SM.
int sweep_split_blocks_per_sm(bool fp32, int scheme, int proj, int block);

// Fused axis pass over many domains (sweep_batch_kernel): doms / offsets are device arrays.
cudaError_t launch_sweep_batch(const SweepArgs<double>* doms, const int* offsets, int ndom, int total_blocks, int pass,
                               BatchOrder ord, int scheme, int proj, bool last, int block, cudaStream_t st);
cudaError_t launch_sweep_batch(const SweepArgs<float>* doms, const int* offsets, int ndom, int total_blocks, int pass,
                               BatchOrder ord, int scheme, int proj, bool last, int block, cudaStream_t st);

// Blocks of the batch kernel (last pass of a cycle) resident on one SM.
int sweep_blocks_per_sm_f64(int scheme, int proj, int block);
int sweep_blocks_per_sm_f32(int scheme, int proj, int block);
inline int sweep_blocks_per_sm(bool fp32, int scheme, int proj, int block)
{
    return fp32 ? sweep_blocks_per_sm_f32(scheme, proj, block) : sweep_blocks_per_sm_f64(scheme, proj, block);
}
int sweep_batch_blocks_per_sm_f64(int scheme, int proj, int block);
int sweep_batch_blocks_per_sm_f32(int scheme, int proj, int block);
inline int sweep_batch_blocks_per_sm(bool fp32, int scheme, int proj, int block)
{
    return fp32 ? sweep_batch_blocks_per_sm_f32(scheme, proj, block) : sweep_batch_blocks_per_sm_f64(scheme, proj, block);
}

// init_test over all nb_cells cells (src/kernels/init_test.cpp:51-104).
struct InitPtrs {
    void *x, *y, *rho, *Emat, *umat, *vmat, *mask, *pmat, *cmat, *gmat, *ustar, *pstar;
};
cudaError_t launch_init_f64(const InitArgs& a, int64_t ncells, const InitPtrs& p, cudaStream_t st);
cudaError_t launch_init_f32(const InitArgs& a, int64_t ncells, const InitPtrs& p, cudaStream_t st);
inline cudaError_t launch_init(const InitArgs& a, int64_t ncells, const InitPtrs& p, bool fp32, cudaStream_t st)
{
    return fp32 ? launch_init_f32(a, ncells, p, st) : launch_init_f64(a, ncells, p, st);
}

// The Sod-interface state (init.cuh: SodInit) over all ncells cells.
cudaError_t launch_init_sod_f64(const SodInit& a, int64_t ncells, void* rho, void* umat, void* vmat, void* Emat,
                                cudaStream_t st);
cudaError_t launch_init_sod_f32(const SodInit& a, int64_t ncells, void* rho, void* umat, void* vmat, void* Emat,
                                cudaStream_t st);
inline cudaError_t launch_init_sod(const SodInit& a, int64_t ncells, void* rho, void* umat, void* vmat, void* Emat,
                                   bool fp32, cudaStream_t st)
{
    return fp32 ? launch_init_sod_f32(a, ncells, rho, umat, vmat, Emat, st)
                : launch_init_sod_f64(a, ncells, rho, umat, vmat, Emat, st);
}

// EOS of the real cells + dt_CFL of that state + reset of the loop state (the start of time_loop,
// src/armon_2D.cpp:327-346).
struct BeginArgs {
    int32_t nx, ny;
    int64_t origin, row_length;
    double gamma;
    void *rho, *umat, *vmat, *Emat, *pmat, *cmat, *gmat;
    StepState* state;
    StepConfig cfg;
    double* partials;
    int32_t buf_base;
    int32_t eos_only;   // 1: only p, c, g of the real cells from rho, umat, vmat, Emat (no dt, no state)
};
cudaError_t launch_begin_f64(const BeginArgs& a, int grid, cudaStream_t st);
cudaError_t launch_begin_f32(const BeginArgs& a, int grid, cudaStream_t st);
inline cudaError_t launch_begin(const BeginArgs& a, bool fp32, int grid, cudaStream_t st)
{
    return fp32 ? launch_begin_f32(a, grid, st) : launch_begin_f64(a, grid, st);
}

// Sums of rho*ds and rho*ds*E over the real cells in FP64, in a fixed order (two kernels).
struct ConsArgs {
    int32_t nx, ny;
    int64_t origin, row_length;
    double ds;
    const void *rho, *Emat;
    double* partials;   // 2 per block of the first kernel
    double* out;        // 2 values
};
cudaError_t launch_conservation_f64(const ConsArgs& a, int grid, cudaStream_t st);
cudaError_t launch_conservation_f32(const ConsArgs& a, int grid, cudaStream_t st);
inline cudaError_t launch_conservation(const ConsArgs& a, bool fp32, int grid, cudaStream_t st)
{
    return fp32 ? launch_conservation_f32(a, grid, st) : launch_conservation_f64(a, grid, st);
}

}  // namespace armon
