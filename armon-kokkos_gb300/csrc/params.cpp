// params.cpp -- the reference's Params logic (src/parameters.cpp) for the C ABI, plus error
// plumbing shared by the library.
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "armon_gb300.h"
#include "host_common.h"

namespace armon {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

}  // namespace armon

extern "C" {

const char* armon_last_error(void) { return armon::g_last_error.c_str(); }

int armon_params_sizeof(void) { return (int)sizeof(armon_params); }

int armon_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

// Member initialisers of src/parameters.h:36-97.
void armon_params_defaults(armon_params* p)
{
    std::memset(p, 0, sizeof(*p));
    p->test = ARMON_SOD;
    p->scheme = ARMON_GAD;
    p->riemann = 0;
    p->projection = ARMON_EULER;
    p->limiter = ARMON_MINMOD;
    p->current_axis = ARMON_AXIS_X;
    p->axis_splitting = ARMON_SEQUENTIAL;
    p->nb_ghosts = 3;
    p->nx = 10;
    p->ny = 10;
    p->stencil_width = -1;
    p->domain_origin[0] = NAN;
    p->domain_origin[1] = NAN;
    p->max_cycles = 100;
    p->output_precision = 9;
    p->verbose = 2;
    p->comparison_tolerance = 1e-13;
}

// src/parameters.cpp:11-18
int armon_min_ghosts(const armon_params* p)
{
    int m = 1;
    m += p->scheme == ARMON_GAD;
    m += p->projection == ARMON_EULER_2ND;
    m += (p->projection == ARMON_EULER_2ND) && (p->scheme == ARMON_GAD);
    return m;
}

// TestCase defaults, src/kernels/test_cases.h:41-121
static double default_cfl(int t) { return t == ARMON_BIZARRIUM ? 0.6 : (t == ARMON_SEDOV ? 0.7 : 0.95); }
static double default_max_time(int t) { return t == ARMON_BIZARRIUM ? 80e-6 : (t == ARMON_SEDOV ? 1.0 : 0.20); }

// Params::init = set_default_values + init_indexing + update_axis, src/parameters.cpp:21-67, 195-210
void armon_params_init(armon_params* p)
{
    if (p->cfl == 0) p->cfl = default_cfl(p->test);
    if (p->max_time == 0) p->max_time = default_max_time(p->test);
    if (p->domain_size[0] <= 0 || p->domain_size[1] <= 0) {
        p->domain_size[0] = p->test == ARMON_SEDOV ? 2 : 1;
        p->domain_size[1] = p->test == ARMON_SEDOV ? 2 : 1;
    }
    if (std::isnan(p->domain_origin[0]) || std::isnan(p->domain_origin[1])) {
        p->domain_origin[0] = p->test == ARMON_SEDOV ? -1 : 0;
        p->domain_origin[1] = p->test == ARMON_SEDOV ? -1 : 0;
    }
    if (p->stencil_width == -1) p->stencil_width = armon_min_ghosts(p);

    p->row_length = p->nb_ghosts * 2 + p->nx;
    p->col_length = p->nb_ghosts * 2 + p->ny;
    p->nb_cells = p->row_length * p->col_length;
    p->ideb = p->row_length * p->nb_ghosts + p->nb_ghosts;
    p->ifin = p->row_length * (p->ny - 1 + p->nb_ghosts) + p->nb_ghosts + p->nx - 1;
    p->index_start = p->ideb;
    p->idx_row = p->row_length;
    p->idx_col = 1;

    if (p->current_axis == ARMON_AXIS_X) {
        p->s = 1;
        p->dx = p->domain_size[0] / double(p->nx);
    } else {
        p->s = p->row_length;
        p->dx = p->domain_size[1] / double(p->ny);
    }
}

// Params::check, src/parameters.cpp:70-109 (the warnings do not change the outcome)
int armon_params_check(const armon_params* p)
{
    if (p->projection == ARMON_PROJ_NONE) return 0;
    if (p->nx <= 0 || p->ny <= 0) return 0;
    if (p->cst_dt && p->Dt == 0.) return 0;
    if (p->stencil_width > p->nb_ghosts) return 0;
    if (p->test < 0 || p->test > 4 || p->scheme < 0 || p->scheme > 1 || p->limiter < 0 || p->limiter > 2 ||
        p->projection < 0 || p->projection > 2 || p->axis_splitting < 0 || p->axis_splitting > 4)
        return 0;
    return 1;
}

void armon_boundary_factors(int test, int side, double* uf, double* vf)
{
    const bool lr = side == ARMON_LEFT || side == ARMON_RIGHT;
    double fu = 1, fv = 1;   // BC_FreeFlow
    switch (test) {
    case ARMON_SOD:       if (lr) fu = -1; break;               // Dirichlet_X on the x walls
    case ARMON_SOD_Y:     if (!lr) fv = -1; break;              // Dirichlet_Y on the y walls
    case ARMON_SOD_CIRC:  if (lr) fu = -1; else fv = -1; break;
    case ARMON_BIZARRIUM: if (side == ARMON_LEFT) fu = -1; else if (side != ARMON_RIGHT) fv = -1; break;
    default: break;                                              // Sedov
    }
    *uf = fu;
    *vf = fv;
}

double armon_test_option(const armon_params* p, double dx, double dy)
{
    if (p->test == ARMON_SEDOV && p->test_option == 0)
        return std::hypot(dx, dy) / 1.41421356237309504880;   // TestSedov::test_option
    return p->test_option;
}

}  // extern "C"
