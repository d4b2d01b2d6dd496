// order.cuh -- longest-first dispatch of the units of a fused pass (solver.cu, batch.cu).
//
// Each block of a pass records the SM cycles its unit took; once per cycle order_units_kernel turns
// those costs into the order in which the next cycle's blocks take the units, most expensive first,
// so that the cheap units fill the tail of the launch.  Which block takes which unit never changes a
// result: the units are independent and the dt partials are reduced by maximum.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace armon {

constexpr int kOrderClasses = 64;
constexpr int kMaxOrderArrays = 6;

struct UnitCounts {
    int n[kMaxOrderArrays];   // units of cost / order array k (block k of the kernel)
};

// A counting sort of array blockIdx.x's units into kOrderClasses classes of cost / (max + 1), the
// most expensive class first; the order within a class is left to the shared-memory atomics.
static __global__ void __launch_bounds__(1024) order_units_kernel(const uint32_t* __restrict__ cost, uint32_t* __restrict__ order,
                                                           int cap, UnitCounts counts)
{
    const int n = counts.n[blockIdx.x];
    cost += (size_t)blockIdx.x * cap;
    order += (size_t)blockIdx.x * cap;
    __shared__ unsigned start[kOrderClasses];
    __shared__ unsigned wmax[32];
    __shared__ unsigned top;
    unsigned m = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, cost[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    for (int c = threadIdx.x; c < kOrderClasses; c += blockDim.x) start[c] = 0;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned v = threadIdx.x < (blockDim.x >> 5) ? wmax[threadIdx.x] : 0u;
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) top = v;
    }
    __syncthreads();
    const uint64_t scale = (uint64_t)top + 1;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        atomicAdd(&start[kOrderClasses - 1 - (int)((uint64_t)cost[i] * kOrderClasses / scale)], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned sum = 0;
        for (int c = 0; c < kOrderClasses; c++) { const unsigned h = start[c]; start[c] = sum; sum += h; }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = kOrderClasses - 1 - (int)((uint64_t)cost[i] * kOrderClasses / scale);
        order[atomicAdd(&start[c], 1u)] = (uint32_t)i;
    }
}

// order[k][i] = i and cost[k][i] = 0 for `arrays` arrays of cap entries
static __global__ void reset_order_kernel(uint32_t* __restrict__ order, uint32_t* __restrict__ cost, int cap, int arrays)
{
    const int total = cap * arrays;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        order[i] = (uint32_t)(i % cap);
        cost[i] = 0;
    }
}

}  // namespace armon
