/*
 * ref_driver.cpp -- runs the reference's own armon_2D step API (compiled from its unchanged
 * sources against oracle/kokkos_shim) and writes the solver state in a binary file.
 * TEST INFRASTRUCTURE ONLY: the golden-fixture script (tests/golden/make_golden.py) uses it to
 * pin the oracle to the reference.
 *
 * Usage: ref_driver out.bin key=value ...
 *   keys: test scheme projection limiter splitting nghost nx ny stencil cfl dt cst_dt
 *         dt_on_even_cycles max_cycles max_time size_x size_y origin_x origin_y test_option
 *         stage_dump_cycles (>0: also dump after every stage of the first N cycles)
 *
 * File layout (little endian): repeated records of
 *   char tag[32]; int32 cycle, axis, nb_cells, status; float64 current_dt, next_dt, time, cycle_dt;
 *   float64 arrays[16][nb_cells]  (x y rho umat vmat Emat pmat cmat gmat ustar pstar
 *                                   work_array_1..4 domain_mask)
 *
 * test_option: the reference's Sod_circ ignores it; a Sod_circ radius other than 0.3 is
 * therefore not available from the reference and is only exercised through the oracle.
 */
#include "armon_2D.h"
#include "parameters.h"
#include "ranges.h"
#include "kernels.h"

#include <cstdio>
#include <cstring>
#include <string>

static FILE* g_out = nullptr;

static void dump(const Params& p, const Data& d, const char* tag, int status)
{
    char t[32] = {0};
    std::strncpy(t, tag, 31);
    std::fwrite(t, 1, 32, g_out);
    int32_t ints[4] = {p.cycle, (int32_t)p.current_axis, p.nb_cells, status};
    std::fwrite(ints, sizeof(int32_t), 4, g_out);
    double dbl[4] = {p.current_cycle_dt, p.next_cycle_dt, p.time, p.cycle_dt};
    std::fwrite(dbl, sizeof(double), 4, g_out);
    const view* arrays[16] = {&d.x, &d.y, &d.rho, &d.umat, &d.vmat, &d.Emat, &d.pmat, &d.cmat, &d.gmat,
                              &d.ustar, &d.pstar, &d.work_array_1, &d.work_array_2, &d.work_array_3,
                              &d.work_array_4, &d.domain_mask};
    for (auto* a : arrays) std::fwrite(a->data(), sizeof(double), (size_t)p.nb_cells, g_out);
}

template <class E> static bool parse_enum(const std::string& v, const char* const* names, int n, E& out)
{
    for (int k = 0; k < n; k++) if (v == names[k]) { out = (E)k; return true; }
    return false;
}

int main(int argc, char** argv)
{
    if (argc < 2) { std::fprintf(stderr, "usage: ref_driver out.bin key=value...\n"); return 2; }
    Params p;
    int stage_dump_cycles = 0;
    static const char* tests[] = {"Sod", "Sod_y", "Sod_circ", "Bizarrium", "Sedov"};
    static const char* schemes[] = {"Godunov", "GAD"};
    static const char* projs[] = {"none", "euler", "euler_2nd"};
    static const char* lims[] = {"None", "Minmod", "Superbee"};
    static const char* splits[] = {"Sequential", "SequentialSym", "Strang", "X_only", "Y_only"};
    for (int a = 2; a < argc; a++) {
        std::string kv = argv[a];
        auto eq = kv.find('=');
        if (eq == std::string::npos) { std::fprintf(stderr, "bad arg %s\n", argv[a]); return 2; }
        std::string k = kv.substr(0, eq), v = kv.substr(eq + 1);
        bool ok = true;
        if (k == "test") ok = parse_enum(v, tests, 5, p.test);
        else if (k == "scheme") ok = parse_enum(v, schemes, 2, p.scheme);
        else if (k == "projection") ok = parse_enum(v, projs, 3, p.projection);
        else if (k == "limiter") ok = parse_enum(v, lims, 3, p.limiter);
        else if (k == "splitting") ok = parse_enum(v, splits, 5, p.axis_splitting);
        else if (k == "nghost") p.nb_ghosts = std::stoi(v);
        else if (k == "nx") p.nx = std::stoi(v);
        else if (k == "ny") p.ny = std::stoi(v);
        else if (k == "stencil") p.stencil_width = std::stoi(v);
        else if (k == "cfl") p.cfl = std::stod(v);
        else if (k == "dt") p.Dt = std::stod(v);
        else if (k == "cst_dt") p.cst_dt = std::stoi(v) != 0;
        else if (k == "dt_on_even_cycles") p.dt_on_even_cycles = std::stoi(v) != 0;
        else if (k == "max_cycles") p.max_cycles = std::stoi(v);
        else if (k == "max_time") p.max_time = std::stod(v);
        else if (k == "size_x") p.domain_size[0] = std::stod(v);
        else if (k == "size_y") p.domain_size[1] = std::stod(v);
        else if (k == "origin_x") p.domain_origin[0] = std::stod(v);
        else if (k == "origin_y") p.domain_origin[1] = std::stod(v);
        else if (k == "stage_dump_cycles") stage_dump_cycles = std::stoi(v);
        else ok = false;
        if (!ok) { std::fprintf(stderr, "bad arg %s\n", argv[a]); return 2; }
    }
    p.verbose = 5;
    p.init();
    if (!p.check()) { std::fprintf(stderr, "invalid parameters\n"); return 3; }

    g_out = std::fopen(argv[1], "wb");
    if (!g_out) return 4;

    Data d(p.nb_cells, "Armon_");
    init_test(p, d);
    {
        /* the test option the reference's init_test used (src/armon_2D.cpp:116-118) */
        flt_t dx = p.domain_size[0] / flt_t(p.nx), dy = p.domain_size[1] / flt_t(p.ny);
        std::fprintf(stdout, "test_option=%a\n", (double)p.test_case->test_option(dx, dy));
    }
    dump(p, d, "init_test", 0);

    int status = 0;
    if (stage_dump_cycles > 0) {
        /* The same sequence as time_loop / solver_cycle (src/armon_2D.cpp:304-386), calling the
         * reference's own stage functions, with a dump after each stage. */
        p.cycle = 0; p.time = 0; p.current_cycle_dt = 0; p.next_cycle_dt = 0;
        p.update_axis(Axis::X);
        update_EOS(p, d);
        dump(p, d, "EOS_init", 0);
        while (p.time < p.max_time && p.cycle < p.max_cycles && p.cycle < stage_dump_cycles) {
            time_step(p, d);
            dump(p, d, "time_step", 0);
            for (auto [axis, dt_factor] : p.split_axes()) {
                p.update_axis(axis);
                p.cycle_dt = p.current_cycle_dt * dt_factor;
                update_EOS(p, d);          dump(p, d, "EOS", 0);
                boundary_conditions(p, d); dump(p, d, "boundary_conditions", 0);
                numerical_fluxes(p, d);    dump(p, d, "numerical_fluxes", 0);
                cell_update(p, d);         dump(p, d, "cell_update", 0);
                projection_remap(p, d);    dump(p, d, "projection_remap", 0);
            }
            p.time += p.current_cycle_dt;
            p.cycle++;
        }
    } else {
        HostData hd{0};
        time_loop(p, d, hd);
        auto [mass, energy] = conservation_vars(p, d);
        std::fprintf(stdout, "cycles=%d dt=%.17g time=%.17g mass=%.17g energy=%.17g\n",
                     p.cycle, p.next_cycle_dt, p.time, mass, energy);
    }
    dump(p, d, "final", status);
    std::fclose(g_out);
    return 0;
}
