// armon_2D.cpp -- the reference's C++ step API (src/armon_2D.cpp, src/parameters.cpp,
// src/ranges.cpp, src/kernels/indexing.cpp, src/io.cpp, src/data.h) on the GB300 kernels.
//
// The stage functions call the per-stage CUDA entry points of include/armon_kernels.h with the
// reference's iteration domains; time_loop drives the fused solver of include/armon_gb300.h on the
// Data arrays (or, with `compare`, the stage functions with the reference's step checkpoints).
#include "armon_2D.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <stdexcept>

#include <cuda_runtime.h>

namespace {

void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        std::fprintf(stderr, "CUDA error in %s: %s\n", what, cudaGetErrorString(e));
        std::exit(1);
    }
}

bool is_finite(flt_t x) { return std::isfinite(x); }

const char* const kNames[16] = {"x", "y", "rho", "umat", "vmat", "Emat", "pmat", "cmat", "gmat", "ustar", "pstar",
                                "work_array_1", "work_array_2", "work_array_3", "work_array_4", "domain_mask"};

}  // namespace

// ---------------------------------------------------------------------------------------------
// Params (src/parameters.cpp)
// ---------------------------------------------------------------------------------------------

armon_params Params::to_c() const
{
    armon_params c;
    armon_params_defaults(&c);
    c.test = (int32_t)test; c.scheme = (int32_t)scheme; c.riemann = (int32_t)riemann;
    c.projection = (int32_t)projection; c.limiter = (int32_t)limiter; c.current_axis = (int32_t)current_axis;
    c.axis_splitting = (int32_t)axis_splitting;
    c.nb_ghosts = nb_ghosts; c.nx = nx; c.ny = ny; c.stencil_width = stencil_width;
    c.cst_dt = cst_dt; c.dt_on_even_cycles = dt_on_even_cycles;
    c.row_length = row_length; c.col_length = col_length; c.nb_cells = nb_cells; c.ideb = ideb; c.ifin = ifin;
    c.index_start = index_start; c.idx_row = idx_row; c.idx_col = idx_col; c.s = s;
    c.cycle = cycle; c.max_cycles = max_cycles;
    c.write_output = write_output; c.write_ghosts = write_ghosts; c.write_throughput = write_throughput;
    c.output_precision = output_precision; c.verbose = verbose; c.compare = compare;
    c.dx = dx; c.cfl = cfl; c.Dt = Dt;
    c.domain_size[0] = domain_size[0]; c.domain_size[1] = domain_size[1];
    c.domain_origin[0] = domain_origin[0]; c.domain_origin[1] = domain_origin[1];
    c.cycle_dt = cycle_dt; c.current_cycle_dt = current_cycle_dt; c.next_cycle_dt = next_cycle_dt; c.time = time;
    c.max_time = max_time; c.comparison_tolerance = comparison_tolerance; c.test_option = test_option_value;
    return c;
}

void Params::from_c(const armon_params& c)
{
    test = (Test)c.test; scheme = (Scheme)c.scheme; riemann = (Riemann)c.riemann;
    projection = (Projection)c.projection; limiter = (Limiter)c.limiter; current_axis = (Axis)c.current_axis;
    axis_splitting = (AxisSplitting)c.axis_splitting;
    nb_ghosts = c.nb_ghosts; nx = c.nx; ny = c.ny; stencil_width = c.stencil_width;
    cst_dt = c.cst_dt; dt_on_even_cycles = c.dt_on_even_cycles;
    row_length = c.row_length; col_length = c.col_length; nb_cells = c.nb_cells; ideb = c.ideb; ifin = c.ifin;
    index_start = c.index_start; idx_row = c.idx_row; idx_col = c.idx_col; s = c.s;
    cycle = c.cycle; max_cycles = c.max_cycles;
    write_output = c.write_output; write_ghosts = c.write_ghosts; write_throughput = c.write_throughput;
    output_precision = c.output_precision; verbose = c.verbose; compare = c.compare;
    dx = c.dx; cfl = c.cfl; Dt = c.Dt;
    domain_size = {c.domain_size[0], c.domain_size[1]};
    domain_origin = {c.domain_origin[0], c.domain_origin[1]};
    cycle_dt = c.cycle_dt; current_cycle_dt = c.current_cycle_dt; next_cycle_dt = c.next_cycle_dt; time = c.time;
    max_time = c.max_time; comparison_tolerance = c.comparison_tolerance; test_option_value = c.test_option;
}

int Params::min_ghosts() const
{
    armon_params c = to_c();
    return armon_min_ghosts(&c);
}

void Params::set_default_values()
{
    // the defaulting half of Params::init (src/parameters.cpp:37-49)
    armon_params c = to_c();
    armon_params_init(&c);
    cfl = c.cfl;
    max_time = c.max_time;
    domain_size = {c.domain_size[0], c.domain_size[1]};
    domain_origin = {c.domain_origin[0], c.domain_origin[1]};
    stencil_width = c.stencil_width;
}

void Params::init_indexing()
{
    // src/parameters.cpp:52-67
    row_length = nb_ghosts * 2 + nx;
    col_length = nb_ghosts * 2 + ny;
    nb_cells = row_length * col_length;
    ideb = row_length * nb_ghosts + nb_ghosts;
    ifin = row_length * (ny - 1 + nb_ghosts) + nb_ghosts + nx - 1;
    index_start = ideb;
    idx_row = row_length;
    idx_col = 1;
}

void Params::init()
{
    set_default_values();
    init_indexing();
    update_axis(current_axis);
}

bool Params::check() const
{
    // src/parameters.cpp:70-109, with its messages
    if (projection == Projection::None) { std::cerr << "ERROR: Lagrangian mode is not supported\n"; return false; }
    if (nx <= 0 || ny <= 0) {
        std::cerr << "ERROR: One of the dimensions of the domain is 0 or negative (nx=" << nx << ", ny=" << ny << ")\n";
        return false;
    }
    if (cst_dt && Dt == 0.) {
        std::cerr << "ERROR: Constant time step is set ('--cst-dt 1') but the initial time step is 0\n";
        return false;
    }
    if (write_output && output_file == nullptr) {
        std::cerr << "ERROR: Write output is on but no output file was given\n";
        return false;
    }
    int mg = min_ghosts();
    if (nb_ghosts < mg)
        std::cerr << "WARNING: There is not enough ghost cells for the given parameters. Expected at least " << mg
                  << ", got " << nb_ghosts << "\n";
    if (stencil_width < mg)
        std::cerr << "WARNING: The stencil width given does not cover the estimated width. Expected at least " << mg
                  << ", got " << stencil_width << "\n";
    if (stencil_width > nb_ghosts) {
        std::cerr << "ERROR: The stencil width cannot be bigger than the number of ghost cells: " << stencil_width
                  << " > " << nb_ghosts << "\n";
        return false;
    }
    return true;
}

void Params::print() const
{
    static const char* tests[] = {"Sod X", "Sod Y", "Cylindrical Sod", "Bizarrium", "Sedov"};
    static const char* lims[] = {"no limiter", "Minmod limiter", "Superbee limiter"};
    static const char* projs[] = {"None", "Euler 1st order", "Euler 2nd order "};
    static const char* splits[] = {"Sequential (X,Y)", "SequentialSym (X,Y,Y,X)", "Strang (½X,Y,½X,½Y,X,½Y)",
                                   "X only", "Y only"};
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, dev);
    printf("Parameters:\n");
    printf(" - gpu:        %s (%d SMs), fused solver\n", prop.name, prop.multiProcessorCount);
    printf(" - ieee bits:  %lu\n", 8 * sizeof(flt_t));
    printf("\n");
    printf(" - test:       %s\n", tests[(int)test]);
    printf(" - riemann:    %s\n", "acoustic");
    printf(" - scheme:     %s, %s\n", scheme == Scheme::Godunov ? "Godunov" : "GAD", lims[(int)limiter]);
    printf(" - domain:     %dx%d (%d ghosts)\n", nx, ny, nb_ghosts);
    printf(" - domain size: %gx%g, origin: (%g, %g)\n", domain_size[0], domain_size[1], domain_origin[0],
           domain_origin[1]);
    printf(" - nb cells:   %g (%g total)\n", double(nx) * ny, double(nb_cells));
    printf(" - CFL:        %g\n", cfl);
    printf(" - Dt init:    %g\n", Dt);
    printf(" - cst dt:     %d\n", cst_dt);
    printf(" - stencil width: %d\n", stencil_width);
    printf(" - projection: %s\n", projs[(int)projection]);
    printf(" - splitting:  %s\n", splits[(int)axis_splitting]);
    printf(" - max time:   %g\n", max_time);
    printf(" - max cycles: %d\n", max_cycles);
    if (write_output) printf(" - output:     '%s'\n", output_file); else printf(" - no output\n");
    if (compare) printf(" - comparison: true, tol: %g\n", comparison_tolerance);
}

void Params::update_axis(Axis axis)
{
    // src/parameters.cpp:195-210
    current_axis = axis;
    if (axis == Axis::X) { s = 1; dx = domain_size[0] / flt_t(nx); }
    else { s = row_length; dx = domain_size[1] / flt_t(ny); }
}

std::vector<std::pair<Axis, flt_t>> Params::split_axes() const
{
    // src/parameters.cpp:212-255
    Axis a1 = (cycle % 2 == 0) ? Axis::Y : Axis::X;
    Axis a2 = (cycle % 2 == 0) ? Axis::X : Axis::Y;
    switch (axis_splitting) {
    case AxisSplitting::Sequential: return {{Axis::X, 1.0}, {Axis::Y, 1.0}};
    case AxisSplitting::SequentialSym: return {{a1, 1.0}, {a2, 1.0}};
    case AxisSplitting::Strang: return {{a1, 0.5}, {a2, 1.0}, {a1, 0.5}};
    case AxisSplitting::X_only: return {{Axis::X, 1.0}};
    case AxisSplitting::Y_only: return {{Axis::Y, 1.0}};
    }
    return {};
}

std::array<flt_t, 2> Params::boundary_condition(Side side) const
{
    double u, v;
    armon_boundary_factors((int)test, (int)side, &u, &v);
    return {u, v};
}

flt_t Params::test_option(flt_t dx_, flt_t dy_) const
{
    armon_params c = to_c();
    return armon_test_option(&c, dx_, dy_);
}

// ---------------------------------------------------------------------------------------------
// Data (src/data.h)
// ---------------------------------------------------------------------------------------------

HostData::HostData(int size)
{
    for (auto* v : vars_array()) v->assign((size_t)size, 0.0);
    domain_mask.assign((size_t)size, 0.0);
}

std::array<std::vector<flt_t>*, 15> HostData::vars_array()
{
    return {&x, &y, &rho, &umat, &vmat, &Emat, &pmat, &cmat, &gmat, &ustar, &pstar,
            &work_array_1, &work_array_2, &work_array_3, &work_array_4};
}

std::array<const std::vector<flt_t>*, 15> HostData::vars_array() const
{
    return {&x, &y, &rho, &umat, &vmat, &Emat, &pmat, &cmat, &gmat, &ustar, &pstar,
            &work_array_1, &work_array_2, &work_array_3, &work_array_4};
}

std::array<std::vector<flt_t>*, 6> HostData::main_vars_array() { return {&x, &y, &rho, &umat, &vmat, &pmat}; }
std::array<const std::vector<flt_t>*, 6> HostData::main_vars_array() const
{
    return {&x, &y, &rho, &umat, &vmat, &pmat};
}

Data::Data(int size, const std::string& label)
{
    owner_ = true;
    auto arrays = all_arrays();
    for (int k = 0; k < 16; k++) {
        labels_[k] = label + kNames[k];
        void* ptr = nullptr;
        cuda_check(cudaMalloc(&ptr, sizeof(flt_t) * (size_t)std::max(size, 1)), "cudaMalloc");
        arrays[k]->data = (flt_t*)ptr;
        arrays[k]->size = size;
        arrays[k]->label = labels_[k].c_str();
    }
}

Data::~Data()
{
    if (!owner_) return;
    for (view* v : all_arrays())
        if (v->data) cudaFree(v->data);
}

Data::Data(Data&& o) noexcept
{
    auto mine = all_arrays();
    auto theirs = o.all_arrays();
    labels_ = std::move(o.labels_);
    for (int k = 0; k < 16; k++) {
        *mine[k] = *theirs[k];
        mine[k]->label = labels_[k].c_str();
        theirs[k]->data = nullptr;
    }
    owner_ = o.owner_;
    o.owner_ = false;
}

std::array<view*, 15> Data::vars_array()
{
    return {&x, &y, &rho, &umat, &vmat, &Emat, &pmat, &cmat, &gmat, &ustar, &pstar,
            &work_array_1, &work_array_2, &work_array_3, &work_array_4};
}

std::array<view*, 16> Data::all_arrays()
{
    return {&x, &y, &rho, &umat, &vmat, &Emat, &pmat, &cmat, &gmat, &ustar, &pstar,
            &work_array_1, &work_array_2, &work_array_3, &work_array_4, &domain_mask};
}

HostData Data::as_mirror() const { return HostData((int)x.size); }

void Data::deep_copy_to_mirror(HostData& mirror) const
{
    Data& self = const_cast<Data&>(*this);
    auto dev = self.all_arrays();
    std::array<std::vector<flt_t>*, 16> host;
    auto hv = mirror.vars_array();
    for (int k = 0; k < 15; k++) host[k] = hv[k];
    host[15] = &mirror.domain_mask;
    for (int k = 0; k < 16; k++) {
        host[k]->resize((size_t)dev[k]->size);
        cuda_check(cudaMemcpy(host[k]->data(), dev[k]->data, sizeof(flt_t) * dev[k]->size, cudaMemcpyDeviceToHost),
                   "deep_copy");
    }
}

void Data::deep_copy_from_mirror(const HostData& mirror)
{
    auto dev = all_arrays();
    std::array<const std::vector<flt_t>*, 16> host;
    auto hv = mirror.vars_array();
    for (int k = 0; k < 15; k++) host[k] = hv[k];
    host[15] = &mirror.domain_mask;
    for (int k = 0; k < 16; k++)
        cuda_check(cudaMemcpy(dev[k]->data, host[k]->data(), sizeof(flt_t) * dev[k]->size, cudaMemcpyHostToDevice),
                   "deep_copy");
}

// ---------------------------------------------------------------------------------------------
// Domains (src/kernels/indexing.cpp:5-111, src/ranges.cpp)
// ---------------------------------------------------------------------------------------------

static unsigned long range_length(long start, long step, long stop)
{
    if ((start != stop) && ((step > 0) != (stop > start))) return 0;
    long diff = stop - start;
    return (unsigned long)(diff / step + 1);
}

static long range_last(long start, long step, long stop)
{
    if (stop == start) return stop;
    return stop - (stop - start) % step;
}

void DomainRange::inflate_dir(Axis axis, long n)
{
    if (axis == Axis::X) { row_start -= row_step * n; row_end += row_step * n; }
    else { col_start -= col_step * n; col_end += col_step * n; }
}

void DomainRange::expand_dir(Axis axis, long n)
{
    if (axis == Axis::X) row_end += row_step * n; else col_end += col_step * n;
}

unsigned long DomainRange::col_length() const { return range_length(col_start, col_step, col_end); }
unsigned long DomainRange::row_length() const { return range_length(row_start, row_step, row_end); }
unsigned long DomainRange::length() const { return col_length() * row_length(); }
long DomainRange::begin() const { return col_start + row_start; }
long DomainRange::end() const { return range_last(col_start, col_step, col_end) + range_last(row_start, row_step, row_end); }

std::tuple<Range, InnerRange1D> DomainRange::directIter1D() const
{
    return {Range{0, (Idx)length()}, InnerRange1D{(Idx)begin(), (Idx)row_step}};
}

std::tuple<Range, InnerRange1D> DomainRange::iter1D() const
{
    return {Range{0, (Idx)(end() - begin() + 1)}, InnerRange1D{(Idx)begin(), (Idx)row_step}};
}

std::tuple<Range, InnerRange2D> DomainRange::iter2D() const
{
    return {Range{0, (Idx)length()}, InnerRange2D{(Idx)col_start, (Idx)col_step, (Idx)row_start, (UIdx)row_length()}};
}

DomainRange real_domain(const Params& p)
{
    return {index_1D(p, 0, 0), p.row_length, index_1D(p, 0, p.ny - 1), 0, 1, p.nx - 1};
}

DomainRange domain_fluxes(const Params& p)
{
    DomainRange dr = real_domain(p);
    long extra = 1 + (p.projection == Projection::Euler_2nd);
    dr.inflate_dir(p.current_axis, extra);
    dr.expand_dir(p.current_axis, 1);
    return dr;
}

DomainRange domain_cell_update(const Params& p)
{
    DomainRange dr = real_domain(p);
    dr.inflate_dir(p.current_axis, 1 + (p.projection == Projection::Euler_2nd));
    return dr;
}

DomainRange domain_advection(const Params& p)
{
    DomainRange dr = real_domain(p);
    dr.expand_dir(p.current_axis, 1);
    return dr;
}

DomainRange complete_domain(const Params& p)
{
    DomainRange dr = real_domain(p);
    dr.inflate_dir(Axis::X, p.nb_ghosts);
    dr.inflate_dir(Axis::Y, p.nb_ghosts);
    return dr;
}

DomainRange boundary_conditions_domain(const Params& p, Side side, int& disp)
{
    int i_start = 0, stride = 1, loop_range = 0;
    switch (side) {
    case Side::Left:   stride = p.row_length; i_start = index_1D(p, -1, 0);   loop_range = p.ny; disp = 1;  break;
    case Side::Right:  stride = p.row_length; i_start = index_1D(p, p.nx, 0); loop_range = p.ny; disp = -1; break;
    case Side::Top:    stride = 1; i_start = index_1D(p, 0, p.ny); loop_range = p.nx; disp = -p.row_length; break;
    case Side::Bottom: stride = 1; i_start = index_1D(p, 0, -1);   loop_range = p.nx; disp = p.row_length;  break;
    }
    return {0, 1, 0, i_start, stride, i_start + loop_range * stride - stride};
}

// ---------------------------------------------------------------------------------------------
// Stage functions (src/armon_2D.cpp:70-298)
// ---------------------------------------------------------------------------------------------

void numerical_fluxes(const Params& p, Data& d)
{
    const view& u = p.current_axis == Axis::X ? d.umat : d.vmat;
    auto [range, inner_range] = domain_fluxes(p).iter2D();
    if (p.scheme == Scheme::Godunov)
        acoustic(&range, &inner_range, p.s, &d.ustar, &d.pstar, &d.rho, &u, &d.pmat, &d.cmat);
    else
        acoustic_GAD(&range, &inner_range, p.s, p.cycle_dt, p.dx, &d.ustar, &d.pstar, &d.rho, &u, &d.pmat, &d.cmat,
                     p.limiter);
}

void update_EOS(const Params& p, Data& d)
{
    auto [range, inner_range] = real_domain(p).iter2D();
    if (p.test == Test::Bizarrium)
        bizarrium_EOS(&range, &inner_range, &d.rho, &d.umat, &d.vmat, &d.Emat, &d.pmat, &d.cmat, &d.gmat);
    else
        perfect_gas_EOS(&range, &inner_range, 1.4, &d.rho, &d.Emat, &d.umat, &d.vmat, &d.pmat, &d.cmat, &d.gmat);
}

void cell_update(const Params& p, Data& d)
{
    auto [range, inner_range] = domain_cell_update(p).iter2D();
    view& u = p.current_axis == Axis::X ? d.umat : d.vmat;
    cell_update(&range, &inner_range, p.s, p.dx, p.cycle_dt, &d.ustar, &d.pstar, &d.rho, &u, &d.Emat);
}

void init_test(const Params& p, Data& d, bool debug_indexes)
{
    auto [range, inner_range] = complete_domain(p).iter2D();
    flt_t dx = p.domain_size[0] / flt_t(p.nx);
    flt_t dy = p.domain_size[1] / flt_t(p.ny);
    flt_t topt = p.test_option(dx, dy);
    init_test(&range, &inner_range, p.row_length, p.nb_ghosts, p.nx, p.ny, p.domain_size[0], p.domain_size[1],
              p.domain_origin[0], p.domain_origin[1], 0, 0, p.nx, p.ny, &d.x, &d.y, &d.rho, &d.Emat, &d.umat,
              &d.vmat, &d.domain_mask, &d.pmat, &d.cmat, &d.gmat, &d.ustar, &d.pstar, p.test, debug_indexes, topt);
}

void boundary_conditions(const Params& p, Data& d, Side side)
{
    int disp;
    DomainRange dr = boundary_conditions_domain(p, side, disp);
    auto f = p.boundary_condition(side);
    auto [range, inner_range] = dr.directIter1D();
    boundary_conditions(&range, &inner_range, p.stencil_width, disp, f[0], f[1], &d.rho, &d.umat, &d.vmat, &d.pmat,
                        &d.cmat, &d.gmat, &d.Emat);
}

void boundary_conditions(const Params& p, Data& d)
{
    if (p.current_axis == Axis::X) { boundary_conditions(p, d, Side::Left); boundary_conditions(p, d, Side::Right); }
    else { boundary_conditions(p, d, Side::Top); boundary_conditions(p, d, Side::Bottom); }
}

void euler_projection(const Params& p, Data& d, const view& ar, const view& au, const view& av, const view& aE)
{
    auto [range, inner_range] = real_domain(p).iter2D();
    euler_projection(&range, &inner_range, p.s, p.dx, p.cycle_dt, &d.ustar, &d.rho, &d.umat, &d.vmat, &d.Emat, &ar,
                     &au, &av, &aE);
}

void advection_first_order(const Params& p, Data& d, view& ar, view& au, view& av, view& aE)
{
    auto [range, inner_range] = domain_advection(p).iter2D();
    advection_first_order(&range, &inner_range, p.s, p.cycle_dt, &d.ustar, &d.rho, &d.umat, &d.vmat, &d.Emat, &ar, &au,
                          &av, &aE);
}

void advection_second_order(const Params& p, Data& d, view& ar, view& au, view& av, view& aE)
{
    auto [range, inner_range] = domain_advection(p).iter2D();
    advection_second_order(&range, &inner_range, p.s, p.dx, p.cycle_dt, &d.ustar, &d.rho, &d.umat, &d.vmat, &d.Emat,
                           &ar, &au, &av, &aE);
}

void projection_remap(const Params& p, Data& d)
{
    if (p.projection == Projection::None) return;
    if (p.projection == Projection::Euler)
        advection_first_order(p, d, d.work_array_1, d.work_array_2, d.work_array_3, d.work_array_4);
    else
        advection_second_order(p, d, d.work_array_1, d.work_array_2, d.work_array_3, d.work_array_4);
    euler_projection(p, d, d.work_array_1, d.work_array_2, d.work_array_3, d.work_array_4);
}

flt_t local_time_step(const Params& p, Data& d, flt_t prev_dt)
{
    flt_t dx = p.domain_size[0] / flt_t(p.nx);
    flt_t dy = p.domain_size[1] / flt_t(p.ny);
    auto [range, inner_range] = real_domain(p).iter1D();
    flt_t dt = dt_CFL(&range, &inner_range, dx, dy, &d.umat, &d.vmat, &d.cmat, &d.domain_mask);
    if (!is_finite(dt) || dt <= 0) return dt;
    if (prev_dt == 0) return p.cfl * dt;
    return std::min(p.cfl * dt, flt_t(1.05) * prev_dt);
}

void time_step(Params& p, Data& d)
{
    p.current_cycle_dt = p.next_cycle_dt;
    if (p.cst_dt) {
        p.next_cycle_dt = p.Dt;
    } else if (!p.dt_on_even_cycles || (p.cycle % 2 == 0) || p.current_cycle_dt == 0) {
        flt_t local_dt = local_time_step(p, d, p.current_cycle_dt);
        if (!is_finite(local_dt) || local_dt <= 0) {
            printf("Invalid dt at cycle %d: %f\n", p.cycle, local_dt);
            std::exit(1);
        }
        p.next_cycle_dt = local_dt;
    } else {
        p.next_cycle_dt = p.current_cycle_dt;
    }
    if (p.cycle == 0) p.current_cycle_dt = p.next_cycle_dt;
}

std::tuple<flt_t, flt_t> conservation_vars(const Params& p, Data& d)
{
    flt_t total_mass = 0, total_energy = 0;
    auto [range, inner_range] = real_domain(p).iter1D();
    conservation_vars(&range, &inner_range, p.dx, &d.rho, &d.Emat, &d.domain_mask, &total_mass, &total_energy);
    return {total_mass, total_energy};
}

// src/armon_2D.cpp:255-284
static bool step_checkpoint(const Params& p, const Data& d, HostData& hd, const char* step_label)
{
    if (!p.compare) return false;
    d.deep_copy_to_mirror(hd);
    char buf[100];
    snprintf(buf, 100, "_%03d_%s", p.cycle, step_label);
    std::string step_file_name = std::string(p.output_file) + buf + "_" + (p.current_axis == Axis::X ? "X" : "Y");
    bool is_different;
    try {
        if (std::strcmp(step_label, "time_step") == 0) is_different = compare_time_step(p, step_file_name);
        else is_different = compare_with_file(p, hd, step_file_name);
    } catch (std::exception& e) {
        std::cerr << "Error while comparing with file '" << step_file_name << "': " << e.what() << std::endl;
        is_different = true;
    }
    if (is_different) {
        std::string diff_file_name = step_file_name + "_diff";
        write_output(p, hd, diff_file_name.c_str());
        printf("Difference file written to %s\n", diff_file_name.c_str());
    }
    return is_different;
}

#define CHECK_STEP(label) if (step_checkpoint(p, d, hd, label)) return true

// src/armon_2D.cpp:304-324, stage by stage
static bool solver_cycle_stages(Params& p, Data& d, HostData& hd)
{
    time_step(p, d);
    CHECK_STEP("time_step");
    for (auto [axis, dt_factor] : p.split_axes()) {
        p.update_axis(axis);
        p.cycle_dt = p.current_cycle_dt * dt_factor;
        update_EOS(p, d);          CHECK_STEP("EOS");
        boundary_conditions(p, d); CHECK_STEP("boundary_conditions");
        numerical_fluxes(p, d);    CHECK_STEP("numerical_fluxes");
        cell_update(p, d);         CHECK_STEP("cell_update");
        projection_remap(p, d);    CHECK_STEP("projection_remap");
    }
    return false;
}

static bool fused_supported(const Params& p)
{
    armon_params c = p.to_c();
    int reach = 2 + (p.scheme == Scheme::GAD) + (p.projection == Projection::Euler_2nd);
    return p.test != Test::Bizarrium && c.nb_ghosts >= reach && p.nx >= p.stencil_width && p.ny >= p.stencil_width;
}

static void print_cycle(const Params& p, flt_t m0, flt_t e0, flt_t m, flt_t e)
{
    flt_t dm = std::abs(m0 - m) / m0 * 100, de = std::abs(e0 - e) / e0 * 100;
    printf("Cycle = %4d, dt = %.18f, t = %.18f, |ΔM| = %#8.6g%%, |ΔE| = %#8.6g%%\n", p.cycle + 1, p.current_cycle_dt,
           p.time, dm, de);
}

std::tuple<double, flt_t, int> time_loop(Params& p, Data& d, HostData& hd)
{
    p.cycle = 0;
    p.time = 0.;
    p.current_cycle_dt = 0.;
    p.next_cycle_dt = 0.;
    auto t0 = std::chrono::steady_clock::now();
    p.update_axis(Axis::X);
    flt_t m0 = 0, e0 = 0;

    if (p.compare || !fused_supported(p)) {
        update_EOS(p, d);
        if (step_checkpoint(p, d, hd, "EOS_init")) goto end_loop;
        if (p.verbose <= 1) std::tie(m0, e0) = conservation_vars(p, d);
        while (p.time < p.max_time && p.cycle < p.max_cycles) {
            if (solver_cycle_stages(p, d, hd)) goto end_loop;
            if (p.verbose <= 1) {
                auto [m, e] = conservation_vars(p, d);
                print_cycle(p, m0, e0, m, e);
            }
            p.time += p.current_cycle_dt;
            p.cycle++;
        }
        cuda_check(cudaDeviceSynchronize(), "last_fence");
    } else {
        armon_params c = p.to_c();
        armon_solver_opts o;
        armon_solver_opts_default(&o);
        auto arrays = d.all_arrays();
        double* ptrs[16];
        for (int k = 0; k < 16; k++) ptrs[k] = arrays[k]->data;
        armon_solver* s = nullptr;
        int rc = armon_solver_create_with_arrays(&c, &o, ptrs, nullptr, &s);
        if (rc == ARMON_OK) rc = armon_solver_begin_loop(s);
        if (rc == ARMON_OK && p.verbose <= 1) {
            std::tie(m0, e0) = conservation_vars(p, d);
            for (;;) {
                armon_params before, st;
                rc = armon_solver_sync_params(s, &before, nullptr);
                if (rc != ARMON_OK || !(before.time < p.max_time && before.cycle < p.max_cycles)) break;
                rc = armon_solver_run(s, 1);
                if (rc != ARMON_OK) break;
                armon_solver_sync_params(s, &st, nullptr);
                // the reference prints after this cycle's passes, before time and cycle advance
                p.cycle = before.cycle;
                p.time = before.time;
                p.current_cycle_dt = st.current_cycle_dt;
                auto sp = p.split_axes();
                p.update_axis(sp.back().first);
                auto [m, e] = conservation_vars(p, d);
                print_cycle(p, m0, e0, m, e);
            }
        } else if (rc == ARMON_OK) {
            rc = armon_solver_run(s, 0);
        }
        armon_params st;
        int32_t status = 0;
        if (s) armon_solver_sync_params(s, &st, &status);
        if (rc == ARMON_ERR_INVALID_DT) {
            printf("Invalid dt at cycle %d: %f\n", st.cycle, st.next_cycle_dt);
            std::exit(1);
        }
        if (rc != ARMON_OK) {
            std::fprintf(stderr, "armon solver error %d: %s\n", rc, armon_last_error());
            std::exit(1);
        }
        armon_solver_destroy(s);
        p.cycle = st.cycle;
        p.time = st.time;
        p.current_cycle_dt = st.current_cycle_dt;
        p.next_cycle_dt = st.next_cycle_dt;
        if (p.cycle > 0) {
            // leave the axis state as the reference's last pass does
            Params q = p;
            q.cycle = p.cycle - 1;
            auto sp = q.split_axes();
            p.update_axis(sp.back().first);
            p.cycle_dt = p.current_cycle_dt * sp.back().second;
        }
    }

end_loop:
    auto t1 = std::chrono::steady_clock::now();
    double loop_time = std::chrono::duration<double>(t1 - t0).count();
    double grind_time = loop_time / (static_cast<double>(p.cycle) * p.nx * p.ny) * 1e6;
    if (p.verbose < 4) {
        printf("\n");
        printf("Time:       %.4g seconds\n", loop_time);
        printf("Grind time: %.4g µs/cell/cycle\n", grind_time);
        printf("Cells/sec:  %.4g Mega cells/sec\n", 1. / grind_time);
        printf("Cycles:     %d\n", p.cycle);
        printf("Final dt:   %.18f\n\n", p.next_cycle_dt);
    }
    return {grind_time, p.next_cycle_dt, p.cycle};
}

bool armon(Params& params)
{
    Data data(params.nb_cells, "Armon_");
    HostData host_data = (params.compare || params.write_output) ? data.as_mirror() : HostData{};
    init_test(params, data);
    if (step_checkpoint(params, data, host_data, "init_test")) return false;
    auto [grind_time, dt, cycles] = time_loop(params, data, host_data);
    (void)dt;
    (void)cycles;
    if (params.write_output) {
        data.deep_copy_to_mirror(host_data);
        write_output(params, host_data);
    }
    if (params.write_throughput) {
        FILE* f = fopen("cell_throughput", "w");
        if (f) {
            fprintf(f, "%f", 1. / grind_time);
            fclose(f);
        }
    }
    return true;
}

// ---------------------------------------------------------------------------------------------
// I/O and comparison (src/io.cpp)
// ---------------------------------------------------------------------------------------------

void write_output(const Params& p, const HostData& d, const char* file_name)
{
    std::fstream file(file_name, std::ios::out);
    int j_deb = p.write_ghosts ? -p.nb_ghosts : 0, j_fin = p.ny + (p.write_ghosts ? p.nb_ghosts : 0);
    int i_deb = p.write_ghosts ? -p.nb_ghosts : 0, i_fin = p.nx + (p.write_ghosts ? p.nb_ghosts : 0);
    const auto vars = d.main_vars_array();
    file << std::scientific;
    file.precision(p.output_precision);
    const int width = p.output_precision + 7;
    for (int j = j_deb; j < j_fin; j++) {
        for (int i = i_deb; i < i_fin; i++) {
            int idx = index_1D(p, i, j);
            auto it = vars.cbegin();
            file << std::setw(width) << (**it)[idx];
            for (it++; it != vars.cend(); it++) file << ", " << std::setw(width) << (**it)[idx];
            file << "\n";
        }
        file << "\n";
    }
    if (p.verbose < 2) std::cout << "Wrote to file: " << file_name << "\n";
}

void write_output(const Params& p, const HostData& d) { write_output(p, d, p.output_file); }

void load_data(const Params& p, HostData& d, std::istream& file)
{
    int j_deb = p.write_ghosts ? -p.nb_ghosts : 0, j_fin = p.ny + (p.write_ghosts ? p.nb_ghosts : 0);
    int i_deb = p.write_ghosts ? -p.nb_ghosts : 0, i_fin = p.nx + (p.write_ghosts ? p.nb_ghosts : 0);
    auto vars = d.main_vars_array();
    for (int j = j_deb; j < j_fin; j++) {
        for (int i = i_deb; i < i_fin; i++) {
            int idx = index_1D(p, i, j);
            auto it = vars.begin();
            file >> (**it)[idx];
            for (it++; it != vars.end(); it++) {
                file.ignore(1, ',');
                file >> (**it)[idx];
            }
        }
    }
}

int compare_with_reference(const Params& params, const HostData& ref_data, const HostData& data)
{
    static const char* names[6] = {"x", "y", "rho", "umat", "vmat", "pmat"};
    auto ref_vars = ref_data.main_vars_array();
    auto vars = data.main_vars_array();
    int i_deb = params.write_ghosts ? -params.nb_ghosts : 0, i_fin = params.nx + (params.write_ghosts ? params.nb_ghosts : 0);
    int j_deb = params.write_ghosts ? -params.nb_ghosts : 0, j_fin = params.ny + (params.write_ghosts ? params.nb_ghosts : 0);
    int total = 0;
    for (int j = j_deb; j < j_fin; j++) {
        int row_deb = index_1D(params, i_deb, j), row_fin = index_1D(params, i_fin, j);
        for (size_t f = 0; f < ref_vars.size(); f++) {
            int row_diff_count = 0, diff_start = row_fin, diff_end = row_deb;
            flt_t max_diff = 0;
            long max_ulp = 0;
            for (int idx = row_deb; idx < row_fin; idx++) {
                flt_t ref_val = (*ref_vars[f])[idx], val = (*vars[f])[idx];
                bool is_eq = is_approx(ref_val, val, params.comparison_tolerance);
                row_diff_count += !is_eq;
                if (!is_eq) {
                    diff_start = std::min(idx, diff_start);
                    diff_end = std::max(idx, diff_end);
                    flt_t diff = std::abs(ref_val - val);
                    if (diff > max_diff) {
                        max_diff = diff;
                        max_ulp = (long)(max_diff / std::abs(ref_val * std::numeric_limits<flt_t>::epsilon()));
                    }
                }
            }
            total += row_diff_count;
            if (row_diff_count > 0) {
                std::streamsize tmp = std::cout.precision();
                std::cout.precision(std::numeric_limits<flt_t>::digits10);
                std::cout << "Row " << std::setw(3) << (j + 1) << " has " << std::setw(3) << row_diff_count
                          << " differences in '" << std::setw(4) << names[f] << "' from " << std::setw(3)
                          << (diff_start - row_deb + 1) << " to " << std::setw(3) << (diff_end - row_deb + 1)
                          << ", max diff: " << max_diff << " (" << max_ulp << " ulp)\n";
                std::cout.precision(tmp);
            }
        }
    }
    return total;
}

bool compare_with_file(const Params& p, const HostData& d, const std::string& ref_file_name)
{
    std::ifstream ref_file(ref_file_name);
    ref_file.exceptions(std::ios::failbit | std::istream::badbit);
    HostData ref_data(p.nb_cells);
    load_data(p, ref_data, ref_file);
    return compare_with_reference(p, ref_data, d) > 0;
}

bool compare_time_step(const Params& p, const std::string& ref_file_name)
{
    std::ifstream ref_file(ref_file_name);
    ref_file.exceptions(std::ios::failbit | std::istream::badbit);
    flt_t ref_dt;
    ref_file >> ref_dt;
    bool is_different = !is_approx(ref_dt, p.current_cycle_dt, p.comparison_tolerance);
    if (is_different) {
        std::streamsize tmp = std::cout.precision();
        std::cout.precision(std::numeric_limits<flt_t>::digits10);
        flt_t diff = ref_dt - p.current_cycle_dt;
        long ulp = (long)(diff / std::numeric_limits<flt_t>::epsilon());
        std::cout << "Time step difference: ref Δt = " << ref_dt << ", Δt = " << p.current_cycle_dt
                  << ", diff = " << diff << " (" << ulp << " ulp)\n";
        std::cout.precision(tmp);
    }
    return is_different;
}
