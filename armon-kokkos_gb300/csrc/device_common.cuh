// device_common.cuh -- types and device helpers shared by the fused sweep and the stage kernels.
//
// Everything here keeps the reference's floating-point semantics exactly: the translation units
// that include it are compiled with --fmad=false (no contraction) and IEEE division and square
// root, and min / max are the std::min / std::max ternaries that Kokkos::min / Kokkos::max use
// (they differ from fmin / fmax on NaN and signed zeros).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "softfp.cuh"

namespace armon {

template <class T> __host__ __device__ __forceinline__ T kmin(T a, T b) { return (b < a) ? b : a; }
template <class T> __host__ __device__ __forceinline__ T kmax(T a, T b) { return (a < b) ? b : a; }

// Constants of one solve, read by every pass (src/parameters.h:34-108 subset).
struct StepConfig {
    double cfl, Dt, max_time;
    double dt_dx, dt_dy;            // domain_size[0] / nx and domain_size[1] / ny, as dt_CFL uses
    int32_t cst_dt, dt_on_even_cycles, max_cycles, splitting;
};

// Device-resident loop state.  Only the last pass of a cycle (or the init kernel) writes it, so
// every pass of a cycle sees the same values.  raw_dt is dt_CFL of the current state
// (src/kernels/reductions.cpp:8-24), computed in the epilogue of the pass that produced it.
struct StepState {
    double time, current_dt, next_dt, raw_dt;
    int32_t cycle, status;
    uint32_t counter;               // block-completion counter of the dt reduction
    int32_t buf_base;               // state buffer set = (cycle * passes + pass + buf_base) % 2
};

enum : int32_t { STATUS_RUNNING = 0, STATUS_INVALID_DT = 1 };

// The dt logic of time_step / local_time_step (src/armon_2D.cpp:212-252), evaluated by every
// pass of a cycle from the committed state.
struct CycleDt {
    double current, next;
    bool run, invalid;
};

__host__ __device__ inline bool is_finite_d(double x) { return x - x == 0.0; }

__host__ __device__ inline CycleDt cycle_time_step(const StepState& st, const StepConfig& cfg)
{
    CycleDt r;
    r.run = st.status == STATUS_RUNNING && st.time < cfg.max_time && st.cycle < cfg.max_cycles;
    r.invalid = false;
    double cur = st.next_dt, nxt;
    if (cfg.cst_dt) {
        nxt = cfg.Dt;
    } else if (!cfg.dt_on_even_cycles || (st.cycle % 2 == 0) || cur == 0) {
        double dt = st.raw_dt, local;
        if (!is_finite_d(dt) || dt <= 0)
            local = dt;
        else if (cur == 0)
            local = cfg.cfl * dt;
        else {
            double a = cfg.cfl * dt, b = 1.05 * cur;
            local = (b < a) ? b : a;   // std::min
        }
        if (!is_finite_d(local) || local <= 0) r.invalid = true;
        nxt = local;
    } else {
        nxt = cur;
    }
    if (st.cycle == 0) cur = nxt;
    r.current = cur;
    r.next = nxt;
    return r;
}

// Params::split_axes (src/parameters.cpp:212-255) for pass k of `cycle`.
__host__ __device__ inline void split_axis(int32_t splitting, int32_t cycle, int k, int* axis, double* factor)
{
    int a1 = (cycle % 2 == 0) ? 1 : 0;   // Y on even cycles, X on odd
    int a2 = 1 - a1;
    *factor = 1.0;
    switch (splitting) {
    case 0: *axis = k == 0 ? 0 : 1; break;                                   // Sequential
    case 1: *axis = k == 0 ? a1 : a2; break;                                 // SequentialSym
    case 2: *axis = k == 1 ? a2 : a1; *factor = k == 1 ? 1.0 : 0.5; break;   // Strang
    case 3: *axis = 0; break;                                                // X_only
    default: *axis = 1; break;                                               // Y_only
    }
}

__host__ __device__ inline int passes_per_cycle(int32_t splitting)
{
    return splitting == 2 ? 3 : (splitting >= 3 ? 1 : 2);
}

// The reduction of dt_CFL over the real cells, kept as the two maxima it depends on:
// min_i RN(dx / a_i) == RN(dx / max_i a_i) for a_i >= 0 because correctly rounded division is
// monotone, so the per-cell divisions of the reference collapse into one.  A cell whose x term is
// NaN is skipped whole, and a NaN y term alone is skipped, exactly as the reference's
// Kokkos::min chain (kmin(acc, kmin(dx/ax, dy/ay)), identity DBL_MAX) treats them.
struct DtAcc {
    double ax, ay;
    uint32_t fx, fy;        // the FP32 variant's maxima, as float bit patterns (finish() folds them in)
    __device__ __forceinline__ void init() { ax = 0.0; ay = 0.0; fx = 0; fy = 0; }
    __device__ __forceinline__ void add(double u, double v, double c)
    {
        // kmax of non-negative values: for sign-clear, non-NaN doubles the IEEE order is the
        // unsigned order of the bit patterns, so the compares run on the integer pipes
        const uint64_t inf = 0x7FF0000000000000ull;
        uint64_t mx, my;
        const uint64_t ub = sfp::bits(u), vb = sfp::bits(v), cb = sfp::bits(c);
        if ((ub & inf) != inf && (vb & inf) != inf && (cb & inf) != inf && (int64_t)cb >= 0) {
            // finite u, v and c >= +0: max(|u + c|, |u - c|) == RN(|u| + c), since one of the two
            // is exactly that sum and rounding is monotone (the other's magnitude is smaller)
            mx = sfp::bits(sfp::absval(u) + c);
            my = sfp::bits(sfp::absval(v) + c);
        } else {
            const uint64_t a1 = sfp::bits(sfp::absval(u + c));
            const uint64_t a2 = sfp::bits(sfp::absval(u - c));
            const uint64_t b1 = sfp::bits(sfp::absval(v + c));
            const uint64_t b2 = sfp::bits(sfp::absval(v - c));
            // kmax(a1, a2) = (a1 < a2) ? a2 : a1, where a NaN a1 is kept and a NaN a2 is not taken
            mx = (a1 <= inf && a2 <= inf && a1 < a2) ? a2 : a1;
            my = (b1 <= inf && b2 <= inf && b1 < b2) ? b2 : b1;
        }
        if (mx <= inf) {
            const uint64_t cur = sfp::bits(ax);
            if (cur < mx) ax = __longlong_as_double((long long)mx);
            if (my <= inf) {
                const uint64_t cy = sfp::bits(ay);
                if (cy < my) ay = __longlong_as_double((long long)my);
            }
        }
    }
    __device__ __forceinline__ void merge(double ox, double oy) { ax = kmax(ax, ox); ay = kmax(ay, oy); }
    // The same for FP32 fields: the per-cell speeds in FP32 and their maxima as float bit patterns
    // (the unsigned order of non-negative floats; FP64 arithmetic per cell would put the FP32
    // variant on GB300's 1/64-rate FP64 pipe); float -> double is exact and monotone, so folding the
    // maxima into FP64 once gives what a per-cell FP64 maximum gives.  dt and the step logic are FP64.
    __device__ __forceinline__ void add(float u, float v, float c)
    {
        const float mx = kmax(fabsf(u + c), fabsf(u - c));
        const float my = kmax(fabsf(v + c), fabsf(v - c));
        if (mx == mx) {
            fx = max(fx, __float_as_uint(mx));
            if (my == my) fy = max(fy, __float_as_uint(my));
        }
    }
    __device__ __forceinline__ void finish()
    {
        ax = kmax(ax, double(__uint_as_float(fx)));
        ay = kmax(ay, double(__uint_as_float(fy)));
    }
};

__host__ __device__ inline double dt_from_maxima(double ax, double ay, double dx, double dy)
{
    double qx = dx / ax, qy = dy / ay;
    double v = kmin(qx, qy);
    const double dbl_max = 1.7976931348623157e308;
    return kmin(dbl_max, v);
}

}  // namespace armon
