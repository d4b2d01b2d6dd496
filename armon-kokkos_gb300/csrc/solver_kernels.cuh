// solver_kernels.cuh -- the kernels around the fused sweep (init, start of the time loop,
// conservation sums) and the typed launchers.  Included once per storage type by
// sweep_f64.cu / sweep_f32.cu with ARMON_T defined.
#pragma once

#include "launch.h"

namespace armon {

template <class T>
__global__ void init_kernel(InitArgs a, int64_t ncells, InitPtrs p)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncells; i += (int64_t)gridDim.x * blockDim.x)
        init_cell<T>(a, i, (T*)p.x, (T*)p.y, (T*)p.rho, (T*)p.Emat, (T*)p.umat, (T*)p.vmat, (T*)p.mask,
                     (T*)p.pmat, (T*)p.cmat, (T*)p.gmat, (T*)p.ustar, (T*)p.pstar);
}

template <class T>
__global__ void init_sod_kernel(SodInit a, int64_t ncells, T* rho, T* umat, T* vmat, T* Emat)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncells; i += (int64_t)gridDim.x * blockDim.x)
        init_sod_cell<T>(a, i, rho, umat, vmat, Emat);
}

// Shared tail of the dt reductions: block max of (ax, ay), partial per block, and the last block
// to finish returns true with the grid maxima in (*gx, *gy) (thread 0 only).
__device__ inline bool grid_dt_maxima(DtAcc acc, double* partials, uint32_t* counter, double* gx, double* gy)
{
    __shared__ double red[2][32];
    __shared__ int last;
    for (int o = 16; o > 0; o >>= 1)
        acc.merge(__shfl_xor_sync(0xffffffffu, acc.ax, o), __shfl_xor_sync(0xffffffffu, acc.ay, o));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) { red[0][warp] = acc.ax; red[1][warp] = acc.ay; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ax = red[0][0], ay = red[1][0];
        for (int w = 1; w < nw; w++) { ax = kmax(ax, red[0][w]); ay = kmax(ay, red[1][w]); }
        partials[2 * blockIdx.x] = ax;
        partials[2 * blockIdx.x + 1] = ay;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    DtAcc tot;
    tot.init();
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
        tot.merge(__ldcg(&partials[2 * b]), __ldcg(&partials[2 * b + 1]));
    for (int o = 16; o > 0; o >>= 1)
        tot.merge(__shfl_xor_sync(0xffffffffu, tot.ax, o), __shfl_xor_sync(0xffffffffu, tot.ay, o));
    __syncthreads();
    if (lane == 0) { red[0][warp] = tot.ax; red[1][warp] = tot.ay; }
    __syncthreads();
    if (threadIdx.x != 0) return false;
    double ax = red[0][0], ay = red[1][0];
    for (int w = 1; w < nw; w++) { ax = kmax(ax, red[0][w]); ay = kmax(ay, red[1][w]); }
    *gx = ax;
    *gy = ay;
    return true;
}

template <class T>
__global__ void begin_kernel(BeginArgs a)
{
    // update_EOS on the real cells (src/armon_2D.cpp:85-101, src/kernels/fluid_eos.cpp:9-23) and
    // the dt_CFL of that state for cycle 0 (eos_only: the EOS alone).  The same IEEE operations in
    // the same order as the axis pass's EOS (u^2 + v^2 and v^2 + u^2 are the same sum), so the values
    // are the same bits.
    DtAcc acc;
    acc.init();
    const int64_t nreal = (int64_t)a.nx * a.ny;
    const T gamma = T(a.gamma);
    T* rho = (T*)a.rho; T* umat = (T*)a.umat; T* vmat = (T*)a.vmat; T* E = (T*)a.Emat;
    T* pmat = (T*)a.pmat; T* cmat = (T*)a.cmat; T* gmat = (T*)a.gmat;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nreal; k += (int64_t)gridDim.x * blockDim.x) {
        int64_t j = k / a.nx, i = k - j * a.nx;
        int64_t idx = a.origin + j * a.row_length + i;
        T e = E[idx] - T(0.5) * (umat[idx] * umat[idx] + vmat[idx] * vmat[idx]);
        T p = (gamma - 1) * rho[idx] * e;
        T c = sqrt(gamma * p / rho[idx]);
        pmat[idx] = p;
        cmat[idx] = c;
        gmat[idx] = (1 + gamma) / 2;
        acc.add(umat[idx], vmat[idx], c);
    }
    if (a.eos_only) return;
    acc.finish();
    double gx, gy;
    if (grid_dt_maxima(acc, a.partials, &a.state->counter, &gx, &gy)) {
        StepState s{};
        s.time = 0;
        s.current_dt = 0;
        s.next_dt = 0;
        s.raw_dt = dt_from_maxima(gx, gy, a.cfg.dt_dx, a.cfg.dt_dy);
        s.cycle = 0;
        s.status = STATUS_RUNNING;
        s.counter = 0;
        s.buf_base = a.buf_base;
        *a.state = s;
    }
}

template <class T>
__global__ void conservation_partial_kernel(ConsArgs a)
{
    // src/kernels/reductions.cpp:27-49 over the real cells: cell_mass = rho * mask * ds with
    // mask == 1, cell_energy = cell_mass * E.  Fixed assignment of cells to threads and a fixed
    // reduction tree, so the sums are reproducible for a given grid size.
    __shared__ double sm[2][256];
    const int64_t nreal = (int64_t)a.nx * a.ny;
    const T* rho = (const T*)a.rho;
    const T* E = (const T*)a.Emat;
    double m = 0, e = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nreal; k += (int64_t)gridDim.x * blockDim.x) {
        int64_t j = k / a.nx, i = k - j * a.nx;
        int64_t idx = a.origin + j * a.row_length + i;
        double cm = double(rho[idx]) * 1.0 * a.ds;
        m += cm;
        e += cm * double(E[idx]);
    }
    sm[0][threadIdx.x] = m;
    sm[1][threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sm[0][threadIdx.x] += sm[0][threadIdx.x + w];
            sm[1][threadIdx.x] += sm[1][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.partials[2 * blockIdx.x] = sm[0][0];
        a.partials[2 * blockIdx.x + 1] = sm[1][0];
    }
}

static __global__ void conservation_final_kernel(const double* partials, int n, double* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double m = 0, e = 0;
        for (int b = 0; b < n; b++) { m += partials[2 * b]; e += partials[2 * b + 1]; }
        out[0] = m;
        out[1] = e;
    }
}

template <class T, int S, int P, bool L>
static cudaError_t launch_one(const SweepArgs<T>& a, int grid, int block, cudaStream_t st)
{
    sweep_kernel<T, S, P, L><<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

template <class T>
static cudaError_t launch_sweep_t(const SweepArgs<T>& a, int scheme, int proj, bool last, int grid, int block,
                                  cudaStream_t st)
{
    if (scheme == 1) {
        if (proj == 2) return last ? launch_one<T, 1, 2, true>(a, grid, block, st) : launch_one<T, 1, 2, false>(a, grid, block, st);
        return last ? launch_one<T, 1, 1, true>(a, grid, block, st) : launch_one<T, 1, 1, false>(a, grid, block, st);
    }
    if (proj == 2) return last ? launch_one<T, 0, 2, true>(a, grid, block, st) : launch_one<T, 0, 2, false>(a, grid, block, st);
    return last ? launch_one<T, 0, 1, true>(a, grid, block, st) : launch_one<T, 0, 1, false>(a, grid, block, st);
}

template <class T, int S, int P, bool L>
static cudaError_t launch_batch_one(const SweepArgs<T>* doms, const int* offsets, int ndom, int grid, int pass,
                                    BatchOrder ord, int block, cudaStream_t st)
{
    sweep_batch_kernel<T, S, P, L><<<grid, block, 0, st>>>(doms, offsets, ndom, pass, ord);
    return cudaGetLastError();
}

template <class T>
static cudaError_t launch_sweep_batch_t(const SweepArgs<T>* doms, const int* offsets, int ndom, int grid, int pass,
                                        BatchOrder ord, int scheme, int proj, bool last, int block, cudaStream_t st)
{
#define ARMON_B(S, P)                                                                                  \
    return last ? launch_batch_one<T, S, P, true>(doms, offsets, ndom, grid, pass, ord, block, st)     \
                : launch_batch_one<T, S, P, false>(doms, offsets, ndom, grid, pass, ord, block, st)
    if (scheme == 1) {
        if (proj == 2) ARMON_B(1, 2);
        ARMON_B(1, 1);
    }
    if (proj == 2) ARMON_B(0, 2);
    ARMON_B(0, 1);
#undef ARMON_B
}

// Blocks of the (heavier) last-pass single-domain kernel that fit on one SM.
template <class T>
static int sweep_blocks_per_sm_t(int scheme, int proj, int block)
{
    int n = 0;
    cudaError_t e;
    if (scheme == 1)
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_kernel<T, 1, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_kernel<T, 1, 1, true>, block, 0);
    else
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_kernel<T, 0, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_kernel<T, 0, 1, true>, block, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

// Blocks of the (heavier) last-pass batch kernel that fit on one SM.
template <class T>
static int sweep_batch_blocks_per_sm_t(int scheme, int proj, int block)
{
    int n = 0;
    cudaError_t e;
    if (scheme == 1)
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_kernel<T, 1, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_kernel<T, 1, 1, true>, block, 0);
    else
        e = proj == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_kernel<T, 0, 2, true>, block, 0)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_batch_kernel<T, 0, 1, true>, block, 0);
    return (e == cudaSuccess && n > 0) ? n : 1;
}

}  // namespace armon
