/*
 * armon_oracle.c -- CPU restatement of the Armon-Kokkos 2-D Lagrange-remap time step.
 *
 * TEST INFRASTRUCTURE ONLY (see armon_oracle.h).  Two builds are made from this one file:
 *   liboracle.so       strict IEEE (-O2 -fno-fast-math -ffp-contract=off): the parity checker;
 *   liboracle_fast.so  the reference's Release flags (-O3 -funroll-loops -ffast-math): the
 *                      timed CPU baseline.
 * Loops are OpenMP `parallel for schedule(static)` over the same flat index ranges the
 * reference's Kokkos RangePolicy walks (src/kernels/parallel_kernels.h:45-65, default build).
 * Every kernel body keeps the reference's expression order; comments cite file:line.
 */
#include "armon_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OMP_FOR _Pragma("omp parallel for schedule(static)")

/* Kokkos::min / Kokkos::max have std::min / std::max semantics: (b < a) ? b : a and
 * (a < b) ? b : a.  The ternaries are kept so that NaN and signed-zero cases match. */
static inline double kmin(double a, double b) { return (b < a) ? b : a; }
static inline double kmax(double a, double b) { return (a < b) ? b : a; }

/* src/kernels/indexing.h:60-73 */
int64_t o_scale_index_2d(o_inner2d ir, uint64_t i)
{
    int64_t ix = (int64_t)(i / ir.row_range_length);
    int64_t iy = (int64_t)(i % ir.row_range_length);
    int64_t j = ir.main_range_start + ix * ir.main_range_step;
    return ir.row_range_start + iy + j;
}

/* src/kernels/indexing.h:39-45 */
static inline int64_t scale1d(o_inner1d ir, uint64_t i) { return (int64_t)i * ir.step + ir.start; }

/* ------------------------------------------------------------------------------------------ */
/* Kernels                                                                                     */
/* ------------------------------------------------------------------------------------------ */

/* src/kernels/fluid_eos.cpp:9-23.  Kokkos::pow(x, 2) is x*x (the compiler folds pow(x, 2.0)). */
void o_perfect_gas_EOS(o_range r, o_inner2d ir, double gamma,
                       const double* rho, const double* Emat, const double* umat, const double* vmat,
                       double* pmat, double* cmat, double* gmat)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        double e = Emat[i] - 0.5 * (umat[i] * umat[i] + vmat[i] * vmat[i]);
        pmat[i] = (gamma - 1) * rho[i] * e;
        cmat[i] = sqrt(gamma * pmat[i] / rho[i]);
        gmat[i] = (1 + gamma) / 2;
    }
}

/* src/kernels/fluid_eos.cpp:26-62 (host only: its pow(., 3), pow(., 4) go through libm) */
void o_bizarrium_EOS(o_range r, o_inner2d ir,
                     const double* rho, const double* umat, const double* vmat, const double* Emat,
                     double* pmat, double* cmat, double* gmat)
{
    const double rho0 = 1e4, K0 = 1e11, Cv0 = 1e3, T0 = 300, eps0 = 0;
    const double G0 = 1.5, s = 1.5, q = -42080895. / 14941154., rr = 727668333. / 149411540.;
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        double x = rho[i] / rho0 - 1;
        double g = G0 * (1 - rho0 / rho[i]);
        double f0 = (1 + (s / 3 - 2) * x + q * (x * x) + rr * (x * x * x)) / (1 - s * x);
        double f1 = (s / 3 - 2 + 2 * q * x + 3 * rr * (x * x) + s * f0) / (1 - s * x);
        double f2 = (2 * q + 6 * rr * x + 2 * s * f1) / (1 - s * x);
        double f3 = (6 * rr + 3 * s * f2) / (1 - s * x);
        double eps_k0 = eps0 - Cv0 * T0 * (1 + g) + 0.5 * (K0 / rho0) * (x * x) * f0;
        double pk0 = -Cv0 * T0 * G0 * rho0 + (0.5 * K0 * x * (1 + x) * (1 + x) * (2 * f0 + x * f1));
        double pk0prime = -0.5 * K0 * pow(1 + x, 3.0)
                * rho0 * (2 * (1 + 3 * x) * f0 + 2 * x * (2 + 3 * x) * f1 + (x * x) * (1 + x) * f2);
        double pk0second = 0.5 * K0 * pow(1 + x, 4.0) * (rho0 * rho0)
                * (12 * (1 + 2 * x) * f0 + 6 * (1 + 6 * x + 6 * (x * x)) * f1 + 6 * x * (1 + x) * (1 + 2 * x) * f2
                   + (x * (1 + x)) * (x * (1 + x)) * f3);
        double e = Emat[i] - 0.5 * (umat[i] * umat[i] + vmat[i] * vmat[i]);
        pmat[i] = pk0 + G0 * rho0 * (e - eps_k0);
        cmat[i] = sqrt(G0 * rho0 * (pmat[i] - pk0) - pk0prime) / rho[i];
        gmat[i] = 0.5 / (pow(rho[i], 3.0) * (cmat[i] * cmat[i]))
                * (pk0second + (G0 * rho0) * (G0 * rho0) * (pmat[i] - pk0));
    }
}

/* src/kernels/acoustic.cpp:10-19 */
static inline void godunov(double rho_i, double rho_im, double c_i, double c_im,
                           double u_i, double u_im, double p_i, double p_im,
                           double* ustar_i, double* pstar_i)
{
    double rc_l = rho_im * c_im;
    double rc_r = rho_i * c_i;
    *ustar_i = (rc_l * u_im + rc_r * u_i + (p_im - p_i)) / (rc_l + rc_r);
    *pstar_i = (rc_r * p_im + rc_l * p_i + rc_l * rc_r * (u_im - u_i)) / (rc_l + rc_r);
}

/* src/kernels/acoustic.cpp:22-37 */
void o_acoustic(o_range r, o_inner2d ir, int64_t s, double* ustar, double* pstar,
                const double* rho, const double* u, const double* pmat, const double* cmat)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        double us, ps;
        godunov(rho[i], rho[i - s], cmat[i], cmat[i - s], u[i], u[i - s], pmat[i], pmat[i - s], &us, &ps);
        ustar[i] = us;
        pstar[i] = ps;
    }
}

/* src/kernels/limiters.h:15-34 */
static inline double limiter(int L, double r)
{
    switch (L) {
    case O_MINMOD:   return kmax(0.0, kmin(1.0, r));
    case O_SUPERBEE: return kmax(kmax(0.0, kmin(1.0, 2 * r)), kmin(2.0, r));
    default:         return 1.0;
    }
}

/* src/kernels/acoustic.cpp:40-88 */
void o_acoustic_GAD(o_range r, o_inner2d ir, int64_t s, double dt, double dx,
                    double* ustar, double* pstar,
                    const double* rho, const double* u, const double* pmat, const double* cmat,
                    int L)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        double ustar_im, pstar_im, ustar_i, pstar_i, ustar_ip, pstar_ip;
        godunov(rho[i - s], rho[i - 2 * s], cmat[i - s], cmat[i - 2 * s],
                u[i - s], u[i - 2 * s], pmat[i - s], pmat[i - 2 * s], &ustar_im, &pstar_im);
        godunov(rho[i], rho[i - s], cmat[i], cmat[i - s],
                u[i], u[i - s], pmat[i], pmat[i - s], &ustar_i, &pstar_i);
        godunov(rho[i + s], rho[i], cmat[i + s], cmat[i],
                u[i + s], u[i], pmat[i + s], pmat[i], &ustar_ip, &pstar_ip);

        double r_um = (ustar_ip - u[i]) / (ustar_i - u[i - s] + 1e-6);
        double r_pm = (pstar_ip - pmat[i]) / (pstar_i - pmat[i - s] + 1e-6);
        double r_up = (u[i - s] - ustar_im) / (u[i] - ustar_i + 1e-6);
        double r_pp = (pmat[i - s] - pstar_im) / (pmat[i] - pstar_i + 1e-6);

        r_um = limiter(L, r_um);
        r_pm = limiter(L, r_pm);
        r_up = limiter(L, r_up);
        r_pp = limiter(L, r_pp);

        double dm_l = rho[i - s] * dx;
        double dm_r = rho[i] * dx;
        double Dm = (dm_l + dm_r) / 2;

        double rc_l = rho[i - s] * cmat[i - s];
        double rc_r = rho[i] * cmat[i];
        double theta = 0.5 * (1 - (rc_l + rc_r) / 2 * (dt / Dm));

        ustar[i] = ustar_i + theta * (r_up * (u[i] - ustar_i) - r_um * (ustar_i - u[i - s]));
        pstar[i] = pstar_i + theta * (r_pp * (pmat[i] - pstar_i) - r_pm * (pstar_i - pmat[i - s]));
    }
}

/* src/kernels/euler_projection.cpp:9-22 */
void o_cell_update(o_range r, o_inner2d ir, int64_t s, double dx, double dt,
                   const double* ustar, const double* pstar, double* rho, double* u, double* Emat)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        double dm = rho[i] * dx;
        rho[i] = dm / (dx + dt * (ustar[i + s] - ustar[i]));
        u[i] += dt / dm * (pstar[i] - pstar[i + s]);
        Emat[i] += dt / dm * (pstar[i] * ustar[i] - pstar[i + s] * ustar[i + s]);
    }
}

/* src/kernels/euler_projection.cpp:25-48 */
void o_euler_projection(o_range r, o_inner2d ir, int64_t s, double dx, double dt,
                        const double* ustar, double* rho, double* umat, double* vmat, double* Emat,
                        const double* a_rho, const double* a_urho, const double* a_vrho, const double* a_Erho)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        double dX = dx + dt * (ustar[i + s] - ustar[i]);
        double tmp_rho  = (dX * rho[i]           - (a_rho[i + s]  - a_rho[i]))  / dx;
        double tmp_urho = (dX * rho[i] * umat[i] - (a_urho[i + s] - a_urho[i])) / dx;
        double tmp_vrho = (dX * rho[i] * vmat[i] - (a_vrho[i + s] - a_vrho[i])) / dx;
        double tmp_Erho = (dX * rho[i] * Emat[i] - (a_Erho[i + s] - a_Erho[i])) / dx;
        rho[i]  = tmp_rho;
        umat[i] = tmp_urho / tmp_rho;
        vmat[i] = tmp_vrho / tmp_rho;
        Emat[i] = tmp_Erho / tmp_rho;
    }
}

/* src/kernels/euler_projection.cpp:51-70 */
void o_advection_first_order(o_range r, o_inner2d ir, int64_t s, double dt,
                             const double* ustar, const double* rho, const double* umat,
                             const double* vmat, const double* Emat,
                             double* a_rho, double* a_urho, double* a_vrho, double* a_Erho)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        double disp = dt * ustar[i];
        int64_t is = i;
        i -= (int64_t)(disp > 0) * s;
        a_rho[is]  = disp * (rho[i]);
        a_urho[is] = disp * (rho[i] * umat[i]);
        a_vrho[is] = disp * (rho[i] * vmat[i]);
        a_Erho[is] = disp * (rho[i] * Emat[i]);
    }
}

/* src/kernels/euler_projection.cpp:73-79 */
static inline double slope_minmod(double u_im, double u_i, double u_ip, double r_m, double r_p)
{
    double D_u_p = r_p * (u_ip - u_i);
    double D_u_m = r_m * (u_i - u_im);
    double sg = copysign(1.0, D_u_p);
    return sg * kmax(0.0, kmin(sg * D_u_p, sg * D_u_m));
}

/* src/kernels/euler_projection.cpp:82-120 */
void o_advection_second_order(o_range r, o_inner2d ir, int64_t s, double dx, double dt,
                              const double* ustar, const double* rho, const double* umat,
                              const double* vmat, const double* Emat,
                              double* a_rho, double* a_urho, double* a_vrho, double* a_Erho)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        int64_t is = i;
        double disp = dt * ustar[i];
        double Dx;
        if (disp > 0) {
            Dx = -(dx - dt * ustar[i - s]);
            i = i - s;
        } else {
            Dx = dx + dt * ustar[i + s];
        }

        double Dx_lm = dx + dt * (ustar[i] - ustar[i - s]);
        double Dx_l  = dx + dt * (ustar[i + s] - ustar[i]);
        double Dx_lp = dx + dt * (ustar[i + 2 * s] - ustar[i + s]);

        double r_m = (2 * Dx_l) / (Dx_l + Dx_lm);
        double r_p = (2 * Dx_l) / (Dx_l + Dx_lp);

        double slope_r  = slope_minmod(rho[i - s], rho[i], rho[i + s], r_m, r_p);
        double slope_ur = slope_minmod(rho[i - s] * umat[i - s], rho[i] * umat[i], rho[i + s] * umat[i + s], r_m, r_p);
        double slope_vr = slope_minmod(rho[i - s] * vmat[i - s], rho[i] * vmat[i], rho[i + s] * vmat[i + s], r_m, r_p);
        double slope_Er = slope_minmod(rho[i - s] * Emat[i - s], rho[i] * Emat[i], rho[i + s] * Emat[i + s], r_m, r_p);

        double length_factor = Dx / (2 * Dx_l);
        a_rho[is]  = disp * (rho[i]           - slope_r  * length_factor);
        a_urho[is] = disp * (rho[i] * umat[i] - slope_ur * length_factor);
        a_vrho[is] = disp * (rho[i] * vmat[i] - slope_vr * length_factor);
        a_Erho[is] = disp * (rho[i] * Emat[i] - slope_Er * length_factor);
    }
}

/* src/kernels/halo_exchange.cpp:9-36 */
void o_boundary_conditions(o_range r, o_inner1d ir, int64_t stencil_width, int64_t disp,
                           double u_factor, double v_factor,
                           double* rho, double* umat, double* vmat, double* pmat,
                           double* cmat, double* gmat, double* Emat)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = scale1d(ir, (uint64_t)k);
        int64_t ip = i + disp;
        for (int64_t w = 0; w < stencil_width; w++) {
            rho[i]  = rho[ip];
            umat[i] = umat[ip] * u_factor;
            vmat[i] = vmat[ip] * v_factor;
            pmat[i] = pmat[ip];
            cmat[i] = cmat[ip];
            gmat[i] = gmat[ip];
            Emat[i] = Emat[ip];
            i  -= disp;
            ip += disp;
        }
    }
}

/* src/kernels/halo_exchange.cpp:39-64 */
void o_read_border_array(o_range r, o_inner2d ir, int64_t side_length, int64_t nghost,
                         const double* rho, const double* umat, const double* vmat, const double* pmat,
                         const double* cmat, const double* gmat, const double* Emat, double* value_array)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t idx = o_scale_index_2d(ir, (uint64_t)k);
        int64_t itr = k;
        int64_t i = itr / nghost;
        int64_t i_g = itr % nghost;
        int64_t i_arr = (i_g * side_length + i) * 7;
        value_array[i_arr + 0] = rho[idx];
        value_array[i_arr + 1] = umat[idx];
        value_array[i_arr + 2] = vmat[idx];
        value_array[i_arr + 3] = pmat[idx];
        value_array[i_arr + 4] = cmat[idx];
        value_array[i_arr + 5] = gmat[idx];
        value_array[i_arr + 6] = Emat[idx];
    }
}

/* src/kernels/halo_exchange.cpp:67-92 */
void o_write_border_array(o_range r, o_inner2d ir, int64_t side_length, int64_t nghost,
                          double* rho, double* umat, double* vmat, double* pmat,
                          double* cmat, double* gmat, double* Emat, const double* value_array)
{
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t idx = o_scale_index_2d(ir, (uint64_t)k);
        int64_t itr = k;
        int64_t i = itr / nghost;
        int64_t i_g = itr % nghost;
        int64_t i_arr = (i_g * side_length + i) * 7;
        rho[idx]  = value_array[i_arr + 0];
        umat[idx] = value_array[i_arr + 1];
        vmat[idx] = value_array[i_arr + 2];
        pmat[idx] = value_array[i_arr + 3];
        cmat[idx] = value_array[i_arr + 4];
        gmat[idx] = value_array[i_arr + 5];
        Emat[idx] = value_array[i_arr + 6];
    }
}

/* TestParams of src/kernels/init_test.cpp:12-48 */
typedef struct { double high_rho, low_rho, high_E, low_E, high_u, low_u, high_v, low_v; } test_params;

static test_params make_test_params(int test, double test_option)
{
    test_params tp = {0};
    switch (test) {
    case O_BIZARRIUM:
        tp.high_rho = 1.42857142857e+4; tp.low_rho = 10000.;
        tp.high_E = 4.48657821135e+6;   tp.low_E = 31250;
        tp.high_u = 0.; tp.low_u = 250.; tp.high_v = 0.; tp.low_v = 0.;
        break;
    case O_SEDOV:
        tp.high_rho = 1.; tp.low_rho = 1.;
        tp.high_E = 0.851072 / (M_PI * (test_option * test_option));
        tp.low_E = 2.5e-14;
        break;
    default: /* Sod, Sod_y, Sod_circ */
        tp.high_rho = 1.; tp.low_rho = 0.125;
        tp.high_E = 2.5;  tp.low_E = 2.0;
        break;
    }
    return tp;
}

/* region_high of each test case, src/kernels/test_cases.h:50-121 */
static inline int region_high(int test, double x, double y, double test_option)
{
    switch (test) {
    case O_SOD_Y:    return y <= 0.5;
    case O_SOD_CIRC: {
        double r2 = test_option > 0 ? test_option : 0.09;
        return ((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5)) <= r2;
    }
    case O_SEDOV:    return (x * x + y * y) <= test_option * test_option;
    default:         return x <= 0.5;   /* Sod, Bizarrium */
    }
}

/* src/kernels/init_test.cpp:51-104 */
void o_init_test(o_range r, o_inner2d ir, int64_t row_length, int64_t nb_ghosts,
                 int64_t nx, int64_t ny, double sx, double sy, double ox, double oy,
                 int64_t pos_x, int64_t pos_y, int64_t g_nx, int64_t g_ny,
                 double* x, double* y, double* rho, double* Emat, double* umat, double* vmat,
                 double* domain_mask, double* pmat, double* cmat, double* gmat,
                 double* ustar, double* pstar, int test, int debug_indexes, double test_option)
{
    test_params tp = make_test_params(test, test_option);
    OMP_FOR
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = o_scale_index_2d(ir, (uint64_t)k);
        int64_t ix = (i % row_length) - nb_ghosts;
        int64_t iy = (i / row_length) - nb_ghosts;
        int64_t g_ix = ix + pos_x;
        int64_t g_iy = iy + pos_y;

        x[i] = (double)g_ix / (double)nx * sx + ox;
        y[i] = (double)g_iy / (double)ny * sy + oy;

        double x_mid = x[i] + sx / (double)(2 * g_nx);
        double y_mid = y[i] + sy / (double)(2 * g_ny);

        if (debug_indexes) {
            rho[i] = (double)(i + 1);
            Emat[i] = (double)(i + 1);
            umat[i] = (double)(i + 1);
            vmat[i] = (double)(i + 1);
        } else if (region_high(test, x_mid, y_mid, test_option)) {
            rho[i] = tp.high_rho; Emat[i] = tp.high_E; umat[i] = tp.high_u; vmat[i] = tp.high_v;
        } else {
            rho[i] = tp.low_rho;  Emat[i] = tp.low_E;  umat[i] = tp.low_u;  vmat[i] = tp.low_v;
        }

        domain_mask[i] = (0 <= ix && ix < nx && 0 <= iy && iy < ny);
        pmat[i] = 0;
        cmat[i] = 1;
        gmat[i] = 0;
        ustar[i] = 0;
        pstar[i] = 0;
    }
}

/* src/kernels/reductions.cpp:8-24.  Kokkos::Min starts every partial at
 * reduction_identity<double>::min() == DBL_MAX and joins with (src < dest) ? src : dest. */
double o_dt_CFL(o_range r, o_inner1d ir, double dx, double dy,
                const double* umat, const double* vmat, const double* cmat, const double* domain_mask)
{
    double result = DBL_MAX;
#pragma omp parallel
    {
        double dt_loop = DBL_MAX;
#pragma omp for schedule(static)
        for (int64_t k = r.start; k < r.end; k++) {
            int64_t i = scale1d(ir, (uint64_t)k);
            double max_cx = kmax(fabs(umat[i] + cmat[i]), fabs(umat[i] - cmat[i])) * domain_mask[i];
            double max_cy = kmax(fabs(vmat[i] + cmat[i]), fabs(vmat[i] - cmat[i])) * domain_mask[i];
            dt_loop = kmin(dt_loop, kmin(dx / max_cx, dy / max_cy));
        }
#pragma omp critical
        { if (dt_loop < result) result = dt_loop; }
    }
    return result;
}

/* src/kernels/reductions.cpp:27-49.  Summed serially here so that the oracle is deterministic. */
void o_conservation_vars(o_range r, o_inner1d ir, double dx,
                         const double* rho, const double* Emat, const double* domain_mask,
                         double* total_mass, double* total_energy)
{
    double ds = dx * dx;
    double m = 0, e = 0;
    for (int64_t k = r.start; k < r.end; k++) {
        int64_t i = scale1d(ir, (uint64_t)k);
        double cell_mass = rho[i] * domain_mask[i] * ds;
        double cell_energy = cell_mass * Emat[i];
        m += cell_mass;
        e += cell_energy;
    }
    *total_mass = m;
    *total_energy = e;
}

/* ------------------------------------------------------------------------------------------ */
/* Domains: src/kernels/indexing.cpp:5-111, src/ranges.cpp:5-106                               */
/* ------------------------------------------------------------------------------------------ */

static uint64_t range_length(int64_t start, int64_t step, int64_t stop)
{
    if ((start != stop) && ((step > 0) != (stop > start))) return 0;
    int64_t diff = stop - start;
    return (uint64_t)(diff / step + 1);
}

static int64_t range_last(int64_t start, int64_t step, int64_t stop)
{
    if (stop == start) return stop;
    int64_t remainder = (stop - start) % step;
    return stop - remainder;
}

uint64_t o_domain_col_length(o_domain d) { return range_length(d.col_start, d.col_step, d.col_end); }
uint64_t o_domain_row_length(o_domain d) { return range_length(d.row_start, d.row_step, d.row_end); }
uint64_t o_domain_length(o_domain d) { return o_domain_col_length(d) * o_domain_row_length(d); }
int64_t o_domain_begin(o_domain d) { return d.col_start + d.row_start; }
int64_t o_domain_end(o_domain d)
{
    return range_last(d.col_start, d.col_step, d.col_end) + range_last(d.row_start, d.row_step, d.row_end);
}

void o_domain_direct_iter1D(o_domain d, o_range* r, o_inner1d* ir)
{
    r->start = 0; r->end = (int64_t)o_domain_length(d);
    ir->start = o_domain_begin(d); ir->step = d.row_step;
}

void o_domain_iter1D(o_domain d, o_range* r, o_inner1d* ir)
{
    r->start = 0; r->end = o_domain_end(d) - o_domain_begin(d) + 1;
    ir->start = o_domain_begin(d); ir->step = d.row_step;
}

void o_domain_iter2D(o_domain d, o_range* r, o_inner2d* ir)
{
    r->start = 0; r->end = (int64_t)o_domain_length(d);
    ir->main_range_start = d.col_start; ir->main_range_step = d.col_step;
    ir->row_range_start = d.row_start; ir->row_range_length = o_domain_row_length(d);
}

static void inflate_dir(o_domain* d, int axis, int64_t n)
{
    if (axis == O_AXIS_X) { d->row_start -= d->row_step * n; d->row_end += d->row_step * n; }
    else                  { d->col_start -= d->col_step * n; d->col_end += d->col_step * n; }
}

static void expand_dir(o_domain* d, int axis, int64_t n)
{
    if (axis == O_AXIS_X) d->row_end += d->row_step * n;
    else                  d->col_end += d->col_step * n;
}

/* src/ranges.h:44-47 */
static inline int64_t index_1D(const o_params* p, int64_t i, int64_t j)
{
    return p->index_start + j * p->idx_row + i * p->idx_col;
}

o_domain o_real_domain(const o_params* p)
{
    o_domain d = { index_1D(p, 0, 0), p->row_length, index_1D(p, 0, p->ny - 1), 0, 1, p->nx - 1 };
    return d;
}

o_domain o_domain_fluxes(const o_params* p)
{
    o_domain d = o_real_domain(p);
    int64_t extra = 1 + (p->projection == O_EULER_2ND);
    inflate_dir(&d, p->current_axis, extra);
    expand_dir(&d, p->current_axis, 1);
    return d;
}

o_domain o_domain_cell_update(const o_params* p)
{
    o_domain d = o_real_domain(p);
    int64_t extra = 1 + (p->projection == O_EULER_2ND);
    inflate_dir(&d, p->current_axis, extra);
    return d;
}

o_domain o_domain_advection(const o_params* p)
{
    o_domain d = o_real_domain(p);
    expand_dir(&d, p->current_axis, 1);
    return d;
}

o_domain o_complete_domain(const o_params* p)
{
    o_domain d = o_real_domain(p);
    inflate_dir(&d, O_AXIS_X, p->nb_ghosts);
    inflate_dir(&d, O_AXIS_Y, p->nb_ghosts);
    return d;
}

o_domain o_boundary_conditions_domain(const o_params* p, int side, int32_t* disp)
{
    int64_t i_start = 0, stride = 1, loop_range = 0;
    switch (side) {
    case O_LEFT:   stride = p->row_length; i_start = index_1D(p, -1, 0);    loop_range = p->ny; *disp = 1;  break;
    case O_RIGHT:  stride = p->row_length; i_start = index_1D(p, p->nx, 0); loop_range = p->ny; *disp = -1; break;
    case O_TOP:    stride = 1; i_start = index_1D(p, 0, p->ny); loop_range = p->nx; *disp = -p->row_length; break;
    default:       stride = 1; i_start = index_1D(p, 0, -1);    loop_range = p->nx; *disp = p->row_length;  break;
    }
    o_domain d = { 0, 1, 0, i_start, stride, i_start + loop_range * stride - stride };
    return d;
}

/* ------------------------------------------------------------------------------------------ */
/* Params: src/parameters.{h,cpp}, src/kernels/test_cases.h                                    */
/* ------------------------------------------------------------------------------------------ */

int o_params_sizeof(void) { return (int)sizeof(o_params); }

int o_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void o_params_defaults(o_params* p)
{
    o_params z = {0};
    *p = z;
    p->test = O_SOD; p->scheme = O_GAD; p->riemann = 0; p->projection = O_EULER;
    p->limiter = O_MINMOD; p->current_axis = O_AXIS_X; p->axis_splitting = O_SEQUENTIAL;
    p->nb_ghosts = 3; p->nx = 10; p->ny = 10; p->stencil_width = -1;
    p->domain_origin[0] = NAN; p->domain_origin[1] = NAN;
    p->max_cycles = 100; p->output_precision = 9; p->verbose = 2;
    p->comparison_tolerance = 1e-13;
}

/* src/parameters.cpp:11-18 */
int o_min_ghosts(const o_params* p)
{
    int m = 1;
    m += p->scheme == O_GAD;
    m += p->projection == O_EULER_2ND;
    m += (p->projection == O_EULER_2ND) && (p->scheme == O_GAD);
    return m;
}

/* src/kernels/test_cases.h:41-121 */
double o_default_cfl(int test)
{
    switch (test) { case O_BIZARRIUM: return 0.6; case O_SEDOV: return 0.7; default: return 0.95; }
}

double o_default_max_time(int test)
{
    switch (test) { case O_BIZARRIUM: return 80e-6; case O_SEDOV: return 1.0; default: return 0.20; }
}

/* BC_* factors of src/kernels/test_cases.h:36-38 per test and side */
void o_boundary_factors(int test, int side, double* uf, double* vf)
{
    int lr = (side == O_LEFT || side == O_RIGHT);
    double fu = 1, fv = 1;                        /* BC_FreeFlow */
    switch (test) {
    case O_SOD:       if (lr) fu = -1; break;                 /* Dirichlet_X on x walls */
    case O_SOD_Y:     if (!lr) fv = -1; break;                /* Dirichlet_Y on y walls */
    case O_SOD_CIRC:  if (lr) fu = -1; else fv = -1; break;
    case O_BIZARRIUM: if (side == O_LEFT) fu = -1; else if (side != O_RIGHT) fv = -1; break;
    default: break;                                          /* Sedov: free flow */
    }
    *uf = fu; *vf = fv;
}

/* src/parameters.cpp:195-210 */
void o_update_axis(o_params* p, int axis)
{
    p->current_axis = axis;
    if (axis == O_AXIS_X) { p->s = 1;             p->dx = p->domain_size[0] / (double)p->nx; }
    else                  { p->s = p->row_length; p->dx = p->domain_size[1] / (double)p->ny; }
}

/* src/parameters.cpp:21-67 */
void o_params_init(o_params* p)
{
    if (p->cfl == 0) p->cfl = o_default_cfl(p->test);
    if (p->max_time == 0) p->max_time = o_default_max_time(p->test);
    if (p->domain_size[0] <= 0 || p->domain_size[1] <= 0) {
        p->domain_size[0] = p->test == O_SEDOV ? 2 : 1;
        p->domain_size[1] = p->test == O_SEDOV ? 2 : 1;
    }
    if (isnan(p->domain_origin[0]) || isnan(p->domain_origin[1])) {
        p->domain_origin[0] = p->test == O_SEDOV ? -1 : 0;
        p->domain_origin[1] = p->test == O_SEDOV ? -1 : 0;
    }
    if (p->stencil_width == -1) p->stencil_width = o_min_ghosts(p);

    p->row_length = p->nb_ghosts * 2 + p->nx;
    p->col_length = p->nb_ghosts * 2 + p->ny;
    p->nb_cells = p->row_length * p->col_length;
    p->ideb = p->row_length * p->nb_ghosts + p->nb_ghosts;
    p->ifin = p->row_length * (p->ny - 1 + p->nb_ghosts) + p->nb_ghosts + p->nx - 1;
    p->index_start = p->ideb;
    p->idx_row = p->row_length;
    p->idx_col = 1;

    o_update_axis(p, p->current_axis);
}

/* src/parameters.cpp:70-109 (errors only; the warnings do not change the outcome) */
int o_params_check(const o_params* p)
{
    if (p->projection == O_PROJ_NONE) return 0;
    if (p->nx <= 0 || p->ny <= 0) return 0;
    if (p->cst_dt && p->Dt == 0.) return 0;
    if (p->stencil_width > p->nb_ghosts) return 0;
    return 1;
}

/* src/parameters.cpp:212-255 */
int o_split_axes(const o_params* p, int32_t* axes, double* factors)
{
    int a1 = (p->cycle % 2 == 0) ? O_AXIS_Y : O_AXIS_X;
    int a2 = (p->cycle % 2 == 0) ? O_AXIS_X : O_AXIS_Y;
    switch (p->axis_splitting) {
    case O_SEQUENTIAL:     axes[0] = O_AXIS_X; factors[0] = 1.0; axes[1] = O_AXIS_Y; factors[1] = 1.0; return 2;
    case O_SEQUENTIAL_SYM: axes[0] = a1; factors[0] = 1.0; axes[1] = a2; factors[1] = 1.0; return 2;
    case O_STRANG:         axes[0] = a1; factors[0] = 0.5; axes[1] = a2; factors[1] = 1.0;
                           axes[2] = a1; factors[2] = 0.5; return 3;
    case O_X_ONLY:         axes[0] = O_AXIS_X; factors[0] = 1.0; return 1;
    case O_Y_ONLY:         axes[0] = O_AXIS_Y; factors[0] = 1.0; return 1;
    default:               return 0;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Driver: src/armon_2D.cpp                                                                    */
/* ------------------------------------------------------------------------------------------ */

static const double* axis_velocity(const o_params* p, const o_data* d)
{
    return p->current_axis == O_AXIS_X ? d->umat : d->vmat;
}

/* src/armon_2D.cpp:112-127 (test_option: TestCase::test_option, src/kernels/test_cases.h:31,105-107) */
void o_init_test_p(const o_params* p, o_data* d, int debug_indexes)
{
    o_range r; o_inner2d ir;
    o_domain_iter2D(o_complete_domain(p), &r, &ir);
    double dx = p->domain_size[0] / (double)p->nx;
    double dy = p->domain_size[1] / (double)p->ny;
    double test_option = p->test_option;
    if (p->test == O_SEDOV && test_option == 0) test_option = hypot(dx, dy) / M_SQRT2;
    o_init_test(r, ir, p->row_length, p->nb_ghosts, p->nx, p->ny,
                p->domain_size[0], p->domain_size[1], p->domain_origin[0], p->domain_origin[1],
                0, 0, p->nx, p->ny,
                d->x, d->y, d->rho, d->Emat, d->umat, d->vmat, d->domain_mask,
                d->pmat, d->cmat, d->gmat, d->ustar, d->pstar, p->test, debug_indexes, test_option);
}

/* src/armon_2D.cpp:85-101 */
void o_update_EOS(const o_params* p, o_data* d)
{
    o_range r; o_inner2d ir;
    o_domain_iter2D(o_real_domain(p), &r, &ir);
    if (p->test == O_BIZARRIUM)
        o_bizarrium_EOS(r, ir, d->rho, d->umat, d->vmat, d->Emat, d->pmat, d->cmat, d->gmat);
    else
        o_perfect_gas_EOS(r, ir, 1.4, d->rho, d->Emat, d->umat, d->vmat, d->pmat, d->cmat, d->gmat);
}

/* src/armon_2D.cpp:130-151 */
void o_boundary_conditions_p(const o_params* p, o_data* d)
{
    int sides[2];
    if (p->current_axis == O_AXIS_X) { sides[0] = O_LEFT; sides[1] = O_RIGHT; }
    else                             { sides[0] = O_TOP;  sides[1] = O_BOTTOM; }
    for (int k = 0; k < 2; k++) {
        int32_t disp;
        o_domain dr = o_boundary_conditions_domain(p, sides[k], &disp);
        double uf, vf;
        o_boundary_factors(p->test, sides[k], &uf, &vf);
        o_range r; o_inner1d ir;
        o_domain_direct_iter1D(dr, &r, &ir);
        o_boundary_conditions(r, ir, p->stencil_width, disp, uf, vf,
                              d->rho, d->umat, d->vmat, d->pmat, d->cmat, d->gmat, d->Emat);
    }
}

/* src/armon_2D.cpp:70-82 */
void o_numerical_fluxes(const o_params* p, o_data* d)
{
    o_range r; o_inner2d ir;
    o_domain_iter2D(o_domain_fluxes(p), &r, &ir);
    const double* u = axis_velocity(p, d);
    if (p->scheme == O_GODUNOV)
        o_acoustic(r, ir, p->s, d->ustar, d->pstar, d->rho, u, d->pmat, d->cmat);
    else
        o_acoustic_GAD(r, ir, p->s, p->cycle_dt, p->dx, d->ustar, d->pstar, d->rho, u, d->pmat, d->cmat,
                       p->limiter);
}

/* src/armon_2D.cpp:104-109 */
void o_cell_update_p(const o_params* p, o_data* d)
{
    o_range r; o_inner2d ir;
    o_domain_iter2D(o_domain_cell_update(p), &r, &ir);
    double* u = p->current_axis == O_AXIS_X ? d->umat : d->vmat;
    o_cell_update(r, ir, p->s, p->dx, p->cycle_dt, d->ustar, d->pstar, d->rho, u, d->Emat);
}

/* src/armon_2D.cpp:154-209 */
void o_projection_remap(const o_params* p, o_data* d)
{
    if (p->projection == O_PROJ_NONE) return;
    o_range r; o_inner2d ir;
    o_domain_iter2D(o_domain_advection(p), &r, &ir);
    if (p->projection == O_EULER)
        o_advection_first_order(r, ir, p->s, p->cycle_dt, d->ustar, d->rho, d->umat, d->vmat, d->Emat,
                                d->work_array_1, d->work_array_2, d->work_array_3, d->work_array_4);
    else
        o_advection_second_order(r, ir, p->s, p->dx, p->cycle_dt, d->ustar, d->rho, d->umat, d->vmat,
                                 d->Emat, d->work_array_1, d->work_array_2, d->work_array_3, d->work_array_4);
    o_domain_iter2D(o_real_domain(p), &r, &ir);
    o_euler_projection(r, ir, p->s, p->dx, p->cycle_dt, d->ustar, d->rho, d->umat, d->vmat, d->Emat,
                       d->work_array_1, d->work_array_2, d->work_array_3, d->work_array_4);
}

/* src/armon_2D.cpp:212-226 */
double o_local_time_step(const o_params* p, o_data* d, double prev_dt)
{
    double dx = p->domain_size[0] / (double)p->nx;
    double dy = p->domain_size[1] / (double)p->ny;
    o_range r; o_inner1d ir;
    o_domain_iter1D(o_real_domain(p), &r, &ir);
    double dt = o_dt_CFL(r, ir, dx, dy, d->umat, d->vmat, d->cmat, d->domain_mask);
    if (!isfinite(dt) || dt <= 0)
        return dt;
    else if (prev_dt == 0)
        return p->cfl * dt;
    else {
        double a = p->cfl * dt, b = 1.05 * prev_dt;
        return (b < a) ? b : a;   /* std::min */
    }
}

/* src/armon_2D.cpp:229-252 */
int o_time_step(o_params* p, o_data* d)
{
    p->current_cycle_dt = p->next_cycle_dt;
    if (p->cst_dt) {
        p->next_cycle_dt = p->Dt;
    } else if (!p->dt_on_even_cycles || (p->cycle % 2 == 0) || p->current_cycle_dt == 0) {
        double local_dt = o_local_time_step(p, d, p->current_cycle_dt);
        if (!isfinite(local_dt) || local_dt <= 0) return 1;
        p->next_cycle_dt = local_dt;
    } else {
        p->next_cycle_dt = p->current_cycle_dt;
    }
    if (p->cycle == 0) p->current_cycle_dt = p->next_cycle_dt;
    return 0;
}

/* src/armon_2D.cpp:287-298 */
void o_conservation_vars_p(const o_params* p, o_data* d, double* mass, double* energy)
{
    o_range r; o_inner1d ir;
    o_domain_iter1D(o_real_domain(p), &r, &ir);
    o_conservation_vars(r, ir, p->dx, d->rho, d->Emat, d->domain_mask, mass, energy);
}

/* src/armon_2D.cpp:304-324 */
int o_solver_cycle(o_params* p, o_data* d)
{
    if (o_time_step(p, d)) return 1;
    int32_t axes[3]; double factors[3];
    int n = o_split_axes(p, axes, factors);
    for (int k = 0; k < n; k++) {
        o_update_axis(p, axes[k]);
        p->cycle_dt = p->current_cycle_dt * factors[k];
        o_update_EOS(p, d);
        o_boundary_conditions_p(p, d);
        o_numerical_fluxes(p, d);
        o_cell_update_p(p, d);
        o_projection_remap(p, d);
    }
    return 0;
}

/* src/armon_2D.cpp:327-386 */
double o_time_loop(o_params* p, o_data* d, int* status)
{
    p->cycle = 0;
    p->time = 0.;
    p->current_cycle_dt = 0.;
    p->next_cycle_dt = 0.;
    *status = 0;

#ifdef _OPENMP
    double t0 = omp_get_wtime();
#endif
    o_update_axis(p, O_AXIS_X);
    o_update_EOS(p, d);

    while (p->time < p->max_time && p->cycle < p->max_cycles) {
        if (o_solver_cycle(p, d)) { *status = 1; break; }
        p->time += p->current_cycle_dt;
        p->cycle++;
    }
#ifdef _OPENMP
    return omp_get_wtime() - t0;
#else
    return 0.0;
#endif
}
