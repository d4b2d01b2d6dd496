// main_2D.cpp -- the command line of the reference (src/main_2D.cpp) on the GB300 library:
// the same flags, parsed into Params, then armon(params).
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "armon_2D.h"

static const char USAGE[] = R"(
 == Armon (GB300) ==
CFD 2D solver using the conservative Euler equations in the lagrangian description, followed by an
Euler remap.  Runs on one NVIDIA GB300 GPU.

Options:
    -h or --help            Prints this message and exit
    -t <test>               Test case: 'Sod', 'Sod_y', 'Sod_circ', 'Bizarrium' or 'Sedov'
    -s <scheme>             Numeric scheme: 'Godunov' (first order) or 'GAD' (second order)
    --limiter <limiter>     Limiter for the second order scheme: 'None', 'Minmod' (default), 'Superbee'
    --cells Nx,Ny           Number of cells in the 2D mesh
    --nghost N              Number of ghost cells around the 2D domain
    --stencil N             Width of the stencil in cells. Defaults to the minimum number of ghost cells.
    --cycle N               Maximum number of iterations
    --riemann <solver>      Riemann solver: 'acoustic' only
    --projection <scheme>   Projection scheme: 'euler' (1st order) or 'euler_2nd' (2nd order)
    --time T                Maximum simulation time (in seconds)
    --cfl C                 CFL number
    --dt T                  Initial time step (in seconds)
    --cst-dt 0-1            Constant time step mode
    --write-output 0-1      If the variables should be written to the output file
    --write-ghosts 0-1      Include the ghost cells in the output file
    --output <file>         The output file name/path
    --precision D           Number of digits of precision printed to the output file for each value.
    --write-throughput 0-1  Enable writing the cell throughput to a separate file (in Mega cells/sec)
    --splitting <method>    Axis splitting method: 'Sequential' (XYXY...), 'SequentialSym' (XYYXXYY...),
                            'Strang' (XYX with dt/2 for X, then YXY with dt/2 for Y, repeat)
    --compare 0-1           Compare each step of the solver with some reference data.
    --comparison-tolerance T  Relative tolerance of --compare
    --test-option X         Sod_circ: squared radius of the disc (default 0.09); Sedov: blast radius
    --verbose 0-3           Verbosity (0: high, 3: low)
)";

template <class E>
static bool pick(const char* v, const char* const* names, int n, E& out)
{
    for (int k = 0; k < n; k++)
        if (std::strcmp(v, names[k]) == 0) { out = (E)k; return true; }
    return false;
}

bool parse_arguments(Params& p, int argc, char** argv)
{
    static const char* tests[] = {"Sod", "Sod_y", "Sod_circ", "Bizarrium", "Sedov"};
    static const char* schemes[] = {"Godunov", "GAD"};
    static const char* limiters[] = {"None", "Minmod", "Superbee"};
    static const char* projections[] = {"none", "euler", "euler_2nd"};
    static const char* splittings[] = {"Sequential", "SequentialSym", "Strang", "X_only", "Y_only"};
    errno = 0;
    for (int i = 1; i < argc; i++) {
        const char* a = argv[i];
        const char* v = i + 1 < argc ? argv[i + 1] : nullptr;
        if (std::strcmp(a, "-h") == 0 || std::strcmp(a, "--help") == 0) { puts(USAGE); std::exit(0); }
        if (!v) { fprintf(stderr, "Missing value for option: %s\n", a); return false; }
        bool ok = true;
        if (!std::strcmp(a, "-t")) { ok = pick(v, tests, 5, p.test); if (!ok) printf("Unknown test: %s\n", v); }
        else if (!std::strcmp(a, "-s")) { ok = pick(v, schemes, 2, p.scheme); if (!ok) printf("Wrong scheme: %s\n", v); }
        else if (!std::strcmp(a, "--limiter")) { ok = pick(v, limiters, 3, p.limiter); if (!ok) printf("Wrong limiter: %s\n", v); }
        else if (!std::strcmp(a, "--cells")) {
            char* comma = nullptr;
            p.nx = (int)std::strtol(v, &comma, 10);
            p.ny = (comma && *comma == ',') ? (int)std::strtol(comma + 1, nullptr, 10) : p.nx;
        }
        else if (!std::strcmp(a, "--nghost")) p.nb_ghosts = (int)std::strtol(v, nullptr, 10);
        else if (!std::strcmp(a, "--stencil")) p.stencil_width = (int)std::strtol(v, nullptr, 10);
        else if (!std::strcmp(a, "--cycle")) p.max_cycles = (int)std::strtol(v, nullptr, 10);
        else if (!std::strcmp(a, "--verbose")) p.verbose = (int)std::strtol(v, nullptr, 10);
        else if (!std::strcmp(a, "--riemann")) { ok = !std::strcmp(v, "acoustic"); if (!ok) printf("Wrong Riemann solver: %s\n", v); }
        else if (!std::strcmp(a, "--time")) p.max_time = std::strtod(v, nullptr);
        else if (!std::strcmp(a, "--cfl")) p.cfl = std::strtod(v, nullptr);
        else if (!std::strcmp(a, "--dt")) p.Dt = std::strtod(v, nullptr);
        else if (!std::strcmp(a, "--write-output")) p.write_output = std::strtol(v, nullptr, 2);
        else if (!std::strcmp(a, "--write-ghosts")) p.write_ghosts = std::strtol(v, nullptr, 2);
        else if (!std::strcmp(a, "--precision")) p.output_precision = (int)std::strtol(v, nullptr, 10);
        else if (!std::strcmp(a, "--projection")) { ok = pick(v, projections, 3, p.projection); if (!ok) printf("Wrong projection scheme: %s\n", v); }
        else if (!std::strcmp(a, "--cst-dt")) p.cst_dt = std::strtol(v, nullptr, 2);
        else if (!std::strcmp(a, "--output")) p.output_file = v;
        else if (!std::strcmp(a, "--write-throughput")) p.write_throughput = std::strtol(v, nullptr, 2);
        else if (!std::strcmp(a, "--splitting")) { ok = pick(v, splittings, 5, p.axis_splitting); if (!ok) printf("Wrong axis splitting method: %s\n", v); }
        else if (!std::strcmp(a, "--compare")) p.compare = std::strtol(v, nullptr, 2);
        else if (!std::strcmp(a, "--comparison-tolerance")) p.comparison_tolerance = std::strtod(v, nullptr);
        else if (!std::strcmp(a, "--test-option")) p.test_option_value = std::strtod(v, nullptr);
        else { fprintf(stderr, "Wrong option: %s\n", a); return false; }
        if (!ok) return false;
        i++;
    }
    if (errno != 0) {
        fprintf(stderr, "Parsing error occurred: %s\n", std::strerror(errno));
        return false;
    }
    return true;
}

int main(int argc, char* argv[])
{
    Params params;
    if (!parse_arguments(params, argc, argv)) return 1;
    params.init();
    if (!params.check()) return 1;
    if (params.verbose < 3) params.print();
    return armon(params) ? 0 : 1;
}
