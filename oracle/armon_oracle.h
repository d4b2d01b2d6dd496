/*
 * armon_oracle.h -- CPU restatement of the Armon-Kokkos 2-D Lagrange-remap time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the tests, the smoke check and the
 * CPU-baseline leg of bench.py call it to check (or time, as the reference's CPU path) the
 * product.  The product library never includes, links or loads anything in this directory.
 *
 * Each function restates one function of the reference (Keluaa/Armon-Kokkos), with the same
 * iteration sets and the same floating-point expression order, so that a strict IEEE build
 * (-O2 -fno-fast-math -ffp-contract=off) gives the reference's strict-build results bit for
 * bit.  Citations are file:line inside the reference project.
 *
 * The parameter block `o_params` has the same memory layout as `armon_params` of the product
 * (include/armon_gb300.h); a CPU test checks the two layouts field by field.
 */
#ifndef ARMON_ORACLE_H
#define ARMON_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/kernels/indexing.h:28-33 */
typedef struct { int64_t start, end; } o_range;
/* src/kernels/indexing.h:39-45 */
typedef struct { int64_t start, step; } o_inner1d;
/* src/kernels/indexing.h:60-73 */
typedef struct {
    int64_t main_range_start, main_range_step, row_range_start;
    uint64_t row_range_length;
} o_inner2d;

/* src/kernels/indexing.h:93-116 (col_end/row_end inclusive) */
typedef struct {
    int64_t col_start, col_step, col_end;
    int64_t row_start, row_step, row_end;
} o_domain;

/* src/parameters.h:17-31, src/kernels/test_cases.h:8-14, src/kernels/limiters.h:8-12 */
enum { O_SOD = 0, O_SOD_Y = 1, O_SOD_CIRC = 2, O_BIZARRIUM = 3, O_SEDOV = 4 };
enum { O_GODUNOV = 0, O_GAD = 1 };
enum { O_PROJ_NONE = 0, O_EULER = 1, O_EULER_2ND = 2 };
enum { O_LIM_NONE = 0, O_MINMOD = 1, O_SUPERBEE = 2 };
enum { O_SEQUENTIAL = 0, O_SEQUENTIAL_SYM = 1, O_STRANG = 2, O_X_ONLY = 3, O_Y_ONLY = 4 };
enum { O_AXIS_X = 0, O_AXIS_Y = 1 };
enum { O_LEFT = 0, O_RIGHT = 1, O_TOP = 2, O_BOTTOM = 3 };

/* Field list of src/parameters.h:34-108, as a C block.  `test_option` is an extension:
 * for Sod_circ it is the squared radius of the high-pressure disc (0 = the reference's 0.09),
 * for Sedov the blast radius (0 = derived from dx, dy as the reference does). */
typedef struct {
    int32_t test, scheme, riemann, projection, limiter, current_axis, axis_splitting;
    int32_t nb_ghosts, nx, ny, stencil_width;
    int32_t cst_dt, dt_on_even_cycles;
    int32_t row_length, col_length, nb_cells, ideb, ifin, index_start, idx_row, idx_col, s;
    int32_t cycle, max_cycles;
    int32_t write_output, write_ghosts, write_throughput, output_precision, verbose, compare;
    double dx, cfl, Dt;
    double domain_size[2], domain_origin[2];
    double cycle_dt, current_cycle_dt, next_cycle_dt, time;
    double max_time, comparison_tolerance, test_option;
} o_params;

/* The 16 arrays of src/data.h:15-43, in the order of DataHolder::vars_array plus the mask. */
typedef struct {
    double *x, *y, *rho, *umat, *vmat, *Emat, *pmat, *cmat, *gmat, *ustar, *pstar;
    double *work_array_1, *work_array_2, *work_array_3, *work_array_4;
    double *domain_mask;
} o_data;

/* ---- kernels: src/kernels/kernels.h:10-86 ---- */
void o_perfect_gas_EOS(o_range r, o_inner2d ir, double gamma,
                       const double* rho, const double* Emat, const double* umat, const double* vmat,
                       double* pmat, double* cmat, double* gmat);
void o_acoustic(o_range r, o_inner2d ir, int64_t s, double* ustar, double* pstar,
                const double* rho, const double* u, const double* pmat, const double* cmat);
void o_acoustic_GAD(o_range r, o_inner2d ir, int64_t s, double dt, double dx,
                    double* ustar, double* pstar,
                    const double* rho, const double* u, const double* pmat, const double* cmat,
                    int limiter);
void o_cell_update(o_range r, o_inner2d ir, int64_t s, double dx, double dt,
                   const double* ustar, const double* pstar, double* rho, double* u, double* Emat);
void o_euler_projection(o_range r, o_inner2d ir, int64_t s, double dx, double dt,
                        const double* ustar, double* rho, double* umat, double* vmat, double* Emat,
                        const double* a_rho, const double* a_urho, const double* a_vrho, const double* a_Erho);
void o_advection_first_order(o_range r, o_inner2d ir, int64_t s, double dt,
                             const double* ustar, const double* rho, const double* umat,
                             const double* vmat, const double* Emat,
                             double* a_rho, double* a_urho, double* a_vrho, double* a_Erho);
void o_advection_second_order(o_range r, o_inner2d ir, int64_t s, double dx, double dt,
                              const double* ustar, const double* rho, const double* umat,
                              const double* vmat, const double* Emat,
                              double* a_rho, double* a_urho, double* a_vrho, double* a_Erho);
void o_boundary_conditions(o_range r, o_inner1d ir, int64_t stencil_width, int64_t disp,
                           double u_factor, double v_factor,
                           double* rho, double* umat, double* vmat, double* pmat,
                           double* cmat, double* gmat, double* Emat);
void o_read_border_array(o_range r, o_inner2d ir, int64_t side_length, int64_t nghost,
                         const double* rho, const double* umat, const double* vmat, const double* pmat,
                         const double* cmat, const double* gmat, const double* Emat, double* value_array);
void o_write_border_array(o_range r, o_inner2d ir, int64_t side_length, int64_t nghost,
                          double* rho, double* umat, double* vmat, double* pmat,
                          double* cmat, double* gmat, double* Emat, const double* value_array);
void o_init_test(o_range r, o_inner2d ir, int64_t row_length, int64_t nb_ghosts,
                 int64_t nx, int64_t ny, double sx, double sy, double ox, double oy,
                 int64_t pos_x, int64_t pos_y, int64_t g_nx, int64_t g_ny,
                 double* x, double* y, double* rho, double* Emat, double* umat, double* vmat,
                 double* domain_mask, double* pmat, double* cmat, double* gmat,
                 double* ustar, double* pstar, int test, int debug_indexes, double test_option);
double o_dt_CFL(o_range r, o_inner1d ir, double dx, double dy,
                const double* umat, const double* vmat, const double* cmat, const double* domain_mask);
void o_conservation_vars(o_range r, o_inner1d ir, double dx,
                         const double* rho, const double* Emat, const double* domain_mask,
                         double* total_mass, double* total_energy);

/* ---- domains: src/ranges.cpp, src/kernels/indexing.cpp ---- */
o_domain o_real_domain(const o_params* p);
o_domain o_domain_fluxes(const o_params* p);
o_domain o_domain_cell_update(const o_params* p);
o_domain o_domain_advection(const o_params* p);
o_domain o_complete_domain(const o_params* p);
o_domain o_boundary_conditions_domain(const o_params* p, int side, int32_t* disp);
uint64_t o_domain_length(o_domain d);
uint64_t o_domain_row_length(o_domain d);
uint64_t o_domain_col_length(o_domain d);
int64_t o_domain_begin(o_domain d);
int64_t o_domain_end(o_domain d);
void o_domain_iter1D(o_domain d, o_range* r, o_inner1d* ir);
void o_domain_direct_iter1D(o_domain d, o_range* r, o_inner1d* ir);
void o_domain_iter2D(o_domain d, o_range* r, o_inner2d* ir);
int64_t o_scale_index_2d(o_inner2d ir, uint64_t i);

/* ---- params: src/parameters.cpp ---- */
int o_min_ghosts(const o_params* p);
void o_params_defaults(o_params* p);   /* the member initialisers of src/parameters.h:36-97 */
void o_params_init(o_params* p);       /* Params::init, src/parameters.cpp:21-34 */
int o_params_check(const o_params* p); /* Params::check, src/parameters.cpp:70-109 */
void o_update_axis(o_params* p, int axis);
/* Params::split_axes (src/parameters.cpp:212-255): writes up to 3 (axis, factor) pairs. */
int o_split_axes(const o_params* p, int32_t* axes, double* factors);
void o_boundary_factors(int test, int side, double* u_factor, double* v_factor);
double o_default_cfl(int test);
double o_default_max_time(int test);

/* ---- driver: src/armon_2D.cpp ---- */
void o_init_test_p(const o_params* p, o_data* d, int debug_indexes);
void o_update_EOS(const o_params* p, o_data* d);
void o_boundary_conditions_p(const o_params* p, o_data* d);
void o_numerical_fluxes(const o_params* p, o_data* d);
void o_cell_update_p(const o_params* p, o_data* d);
void o_projection_remap(const o_params* p, o_data* d);
double o_local_time_step(const o_params* p, o_data* d, double prev_dt);
/* returns 0, or 1 when the reference would stop on an invalid dt (src/armon_2D.cpp:238-242) */
int o_time_step(o_params* p, o_data* d);
void o_conservation_vars_p(const o_params* p, o_data* d, double* mass, double* energy);
/* one solver_cycle (src/armon_2D.cpp:304-324) without the step checkpoints; 0 or 1 as above */
int o_solver_cycle(o_params* p, o_data* d);
/* time_loop (src/armon_2D.cpp:327-386) without printing or step checkpoints.
 * Returns the loop time in seconds; *status = 1 on an invalid dt. */
double o_time_loop(o_params* p, o_data* d, int* status);

int o_params_sizeof(void);
int o_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
