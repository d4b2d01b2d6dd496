// init.cuh -- test-case initial state (src/kernels/init_test.cpp:12-104,
// src/kernels/test_cases.h:36-121), shared by the init_test entry point and the solver.
#pragma once

#include <cmath>

#include "device_common.cuh"

namespace armon {

// TestParams of src/kernels/test_cases.h:16-21, computed on the host as the reference does.
struct TestParams {
    double high_rho, low_rho, high_E, low_E, high_u, low_u, high_v, low_v;
};

inline TestParams make_test_params(int test, double test_option)
{
    TestParams tp{};
    switch (test) {
    case 3:  // Bizarrium, src/kernels/init_test.cpp:25-35
        tp.high_rho = 1.42857142857e+4; tp.low_rho = 10000.;
        tp.high_E = 4.48657821135e+6;   tp.low_E = 31250;
        tp.high_u = 0.; tp.low_u = 250.; tp.high_v = 0.; tp.low_v = 0.;
        break;
    case 4:  // Sedov, src/kernels/init_test.cpp:38-48 (Kokkos::pow(r, 2) == r * r)
        tp.high_rho = 1.; tp.low_rho = 1.;
        tp.high_E = 0.851072 / (M_PI * (test_option * test_option));
        tp.low_E = 2.5e-14;
        break;
    default:  // Sod, Sod_y, Sod_circ, src/kernels/init_test.cpp:12-22
        tp.high_rho = 1.; tp.low_rho = 0.125;
        tp.high_E = 2.5;  tp.low_E = 2.0;
        break;
    }
    return tp;
}

// region_high of each test case (src/kernels/test_cases.h:50-121).  For Sod_circ a positive
// test_option replaces the squared radius 0.09 (an extension; the reference passes 0 there).
__host__ __device__ inline bool region_high(int test, double x, double y, double test_option)
{
    switch (test) {
    case 1: return y <= 0.5;
    case 2: {
        double r2 = test_option > 0 ? test_option : 0.09;
        return ((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)) <= r2;
    }
    case 4: return (x * x + y * y) <= test_option * test_option;
    default: return x <= 0.5;
    }
}

struct InitArgs {
    int64_t row_length, nb_ghosts, nx, ny, pos_x, pos_y, g_nx, g_ny;
    double sx, sy, ox, oy, test_option;
    int32_t test, debug_indexes;
    TestParams tp;
};

// Body of init_test for cell i (src/kernels/init_test.cpp:62-103), with T the storage type.
template <class T>
__device__ __forceinline__ void init_cell(const InitArgs& a, int64_t i, T* x, T* y, T* rho, T* Emat, T* umat,
                                          T* vmat, T* mask, T* pmat, T* cmat, T* gmat, T* ustar, T* pstar)
{
    int64_t ix = (i % a.row_length) - a.nb_ghosts;
    int64_t iy = (i / a.row_length) - a.nb_ghosts;
    int64_t g_ix = ix + a.pos_x;
    int64_t g_iy = iy + a.pos_y;
    // Coordinates and the region test in FP64 for every storage type, so that an FP32 solve
    // starts from the FP64 initial state rounded to FP32.
    double xi = double(g_ix) / double(a.nx) * a.sx + a.ox;
    double yi = double(g_iy) / double(a.ny) * a.sy + a.oy;
    if (x) x[i] = T(xi);
    if (y) y[i] = T(yi);
    double x_mid = xi + a.sx / double(2 * a.g_nx);
    double y_mid = yi + a.sy / double(2 * a.g_ny);
    if (a.debug_indexes) {
        rho[i] = T(i + 1); Emat[i] = T(i + 1); umat[i] = T(i + 1); vmat[i] = T(i + 1);
    } else if (region_high(a.test, x_mid, y_mid, a.test_option)) {
        rho[i] = T(a.tp.high_rho); Emat[i] = T(a.tp.high_E); umat[i] = T(a.tp.high_u); vmat[i] = T(a.tp.high_v);
    } else {
        rho[i] = T(a.tp.low_rho); Emat[i] = T(a.tp.low_E); umat[i] = T(a.tp.low_u); vmat[i] = T(a.tp.low_v);
    }
    if (mask) mask[i] = T(0 <= ix && ix < a.nx && 0 <= iy && iy < a.ny);
    pmat[i] = 0;
    cmat[i] = 1;
    gmat[i] = 0;
    if (ustar) ustar[i] = 0;
    if (pstar) pstar[i] = 0;
}

// A Sod-type interface state over all cells (armon_sod_interface of include/armon_gb300.h): cell
// centres as init_cell computes them, then the planar or circular test, in FP64 for every storage
// type; u = v = 0.  E_high / E_low are p / ((1.4 - 1) rho) of each state.
struct SodInit {
    int64_t row_length, nb_ghosts, nx, ny;
    double sx, sy, ox, oy;
    int32_t shape, pad;
    double cx, cy, nxv, nyv, offset, r2;
    double rho_high, E_high, rho_low, E_low;
};

template <class T>
__device__ __forceinline__ void init_sod_cell(const SodInit& a, int64_t i, T* rho, T* umat, T* vmat, T* Emat)
{
    const int64_t ix = (i % a.row_length) - a.nb_ghosts;
    const int64_t iy = (i / a.row_length) - a.nb_ghosts;
    const double x = double(ix) / double(a.nx) * a.sx + a.ox + a.sx / double(2 * a.nx);
    const double y = double(iy) / double(a.ny) * a.sy + a.oy + a.sy / double(2 * a.ny);
    const double dx = x - a.cx, dy = y - a.cy;
    const bool high = a.shape == 0 ? dx * a.nxv + dy * a.nyv <= a.offset : dx * dx + dy * dy <= a.r2;
    rho[i] = T(high ? a.rho_high : a.rho_low);
    Emat[i] = T(high ? a.E_high : a.E_low);
    umat[i] = T(0);
    vmat[i] = T(0);
}

}  // namespace armon
