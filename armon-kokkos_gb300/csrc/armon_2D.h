// armon_2D.h -- the reference's C++ step API for the GB300 library: Params (src/parameters.h),
// DataHolder (src/data.h), the iteration domains (src/ranges.h, src/kernels/indexing.h), the
// per-stage functions and the time loop (src/armon_2D.h:12-41) and the text I/O (src/io.h).
//
// Same names, arguments and meaning as the reference, so a C++ driver written against
// src/armon_2D.h builds against this header.  Differences:
//   - views are armon_view (a device pointer, a length and a label) and Data owns CUDA memory;
//   - Params has no TestCase* member: boundary_condition(side) and test_option(dx, dy) replace
//     test_case->boundaryCondition(side) and test_case->test_option(dx, dy);
//   - time_loop runs the fused GPU solver (one kernel per axis pass, dt kept on the device) unless
//     `compare` is set or the configuration needs the per-stage kernels (Bizarrium, thin domains),
//     in which case it replays the reference's stage sequence with the per-stage GPU kernels.
#pragma once

#include <array>
#include <cmath>
#include <istream>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "armon_gb300.h"
#include "armon_kernels.h"

enum class Scheme { Godunov, GAD };
enum class Riemann { Acoustic };
enum class Projection { None, Euler, Euler_2nd };
enum class AxisSplitting { Sequential, SequentialSym, Strang, X_only, Y_only };
enum class Axis : int { X = 0, Y = 1 };
enum class Side : int { Left, Right, Top, Bottom };

// src/parameters.h:34-108
struct Params {
    Test test = Test::Sod;
    Scheme scheme = Scheme::GAD;
    Riemann riemann = Riemann::Acoustic;
    Projection projection = Projection::Euler;
    Limiter limiter = Limiter::Minmod;
    Axis current_axis = Axis::X;
    AxisSplitting axis_splitting = AxisSplitting::Sequential;

    int nb_ghosts = 3;
    int nx = 10;
    int ny = 10;
    flt_t dx = 0;
    flt_t cfl = 0;
    flt_t Dt = 0;
    int stencil_width = -1;
    bool cst_dt = false;
    bool dt_on_even_cycles = false;
    std::array<flt_t, 2> domain_size = {0, 0};
    std::array<flt_t, 2> domain_origin = {NAN, NAN};

    int row_length = 0;
    int col_length = 0;
    int nb_cells = 0;
    int ideb = 0;
    int ifin = 0;
    int index_start = 0;
    int idx_row = 0;
    int idx_col = 0;
    int s = 0;

    int cycle = 0;
    flt_t cycle_dt = 0.;
    flt_t current_cycle_dt = 0.;
    flt_t next_cycle_dt = 0.;
    flt_t time = 0.;

    int max_cycles = 100;
    flt_t max_time = 0;

    bool write_output = false;
    bool write_ghosts = false;
    bool write_throughput = false;
    int output_precision = 9;
    int verbose = 2;
    const char* output_file = "output_cpp";

    bool compare = false;
    flt_t comparison_tolerance = 1e-13;

    // Extension: the Sod_circ squared radius / the Sedov radius (see armon_params.test_option)
    flt_t test_option_value = 0;

    int min_ghosts() const;
    void init();
    void set_default_values();
    void init_indexing();
    bool check() const;
    void print() const;
    void update_axis(Axis axis);
    std::vector<std::pair<Axis, flt_t>> split_axes() const;

    std::array<flt_t, 2> boundary_condition(Side side) const;
    flt_t test_option(flt_t dx_, flt_t dy_) const;
    armon_params to_c() const;
    void from_c(const armon_params& c);
};

// src/data.h: the 16 arrays on the host
struct HostData {
    std::vector<flt_t> x, y, rho, umat, vmat, Emat, pmat, cmat, gmat, ustar, pstar;
    std::vector<flt_t> work_array_1, work_array_2, work_array_3, work_array_4;
    std::vector<flt_t> domain_mask;

    HostData() = default;
    explicit HostData(int size);
    std::array<std::vector<flt_t>*, 15> vars_array();
    std::array<const std::vector<flt_t>*, 15> vars_array() const;
    std::array<std::vector<flt_t>*, 6> main_vars_array();               // x y rho umat vmat pmat
    std::array<const std::vector<flt_t>*, 6> main_vars_array() const;
};

// src/data.h: the 16 arrays in device memory (labelled "<label><name>")
struct Data {
    view x{}, y{}, rho{}, umat{}, vmat{}, Emat{}, pmat{}, cmat{}, gmat{}, ustar{}, pstar{};
    view work_array_1{}, work_array_2{}, work_array_3{}, work_array_4{};
    mask_view domain_mask{};

    Data() = default;
    explicit Data(int size, const std::string& label = "");
    ~Data();
    Data(const Data&) = delete;
    Data& operator=(const Data&) = delete;
    Data(Data&& o) noexcept;

    HostData as_mirror() const;
    void deep_copy_to_mirror(HostData& mirror) const;
    void deep_copy_from_mirror(const HostData& mirror);
    std::array<view*, 15> vars_array();
    std::array<view*, 16> all_arrays();   // vars_array + domain_mask, the solver's order

private:
    std::array<std::string, 16> labels_;
    bool owner_ = false;
};

// src/kernels/indexing.h:93-116 (col_end and row_end inclusive)
struct DomainRange {
    long col_start, col_step, col_end;
    long row_start, row_step, row_end;

    void inflate_dir(Axis axis, long n);
    void expand_dir(Axis axis, long n);
    unsigned long col_length() const;
    unsigned long row_length() const;
    unsigned long length() const;
    long begin() const;
    long end() const;
    std::tuple<Range, InnerRange1D> directIter1D() const;
    std::tuple<Range, InnerRange1D> iter1D() const;
    std::tuple<Range, InnerRange2D> iter2D() const;
    bool operator==(const DomainRange& o) const
    {
        return col_start == o.col_start && col_step == o.col_step && col_end == o.col_end &&
               row_start == o.row_start && row_step == o.row_step && row_end == o.row_end;
    }
};

// src/ranges.h:12-47
DomainRange real_domain(const Params& p);
DomainRange domain_fluxes(const Params& p);
DomainRange domain_cell_update(const Params& p);
DomainRange domain_advection(const Params& p);
DomainRange complete_domain(const Params& p);
DomainRange boundary_conditions_domain(const Params& p, Side side, int& disp);
inline int index_1D(const Params& p, int i, int j) { return p.index_start + j * p.idx_row + i * p.idx_col; }

// src/armon_2D.h:12-41
void numerical_fluxes(const Params& p, Data& d);
void update_EOS(const Params& p, Data& d);
void cell_update(const Params& p, Data& d);
void init_test(const Params& p, Data& d, bool debug_indexes = false);
void boundary_conditions(const Params& p, Data& d, Side side);
void boundary_conditions(const Params& p, Data& d);
void euler_projection(const Params& p, Data& d, const view& advection_rho, const view& advection_urho,
                      const view& advection_vrho, const view& advection_Erho);
void advection_first_order(const Params& p, Data& d, view& advection_rho, view& advection_urho,
                           view& advection_vrho, view& advection_Erho);
void advection_second_order(const Params& p, Data& d, view& advection_rho, view& advection_urho,
                            view& advection_vrho, view& advection_Erho);
void projection_remap(const Params& p, Data& d);
flt_t local_time_step(const Params& p, Data& d, flt_t prev_dt);
void time_step(Params& p, Data& d);
std::tuple<flt_t, flt_t> conservation_vars(const Params& p, Data& d);
std::tuple<double, flt_t, int> time_loop(Params& p, Data& d, HostData& hd);
bool armon(Params& params);

// src/io.h:10-21
void write_output(const Params& p, const HostData& d, const char* file_name);
void write_output(const Params& p, const HostData& d);
void load_data(const Params& p, HostData& d, std::istream& file);
inline bool is_approx(flt_t a, flt_t b, flt_t tol) { return std::abs(a - b) <= tol * std::max(std::abs(a), std::abs(b)); }
int compare_with_reference(const Params& params, const HostData& ref_data, const HostData& data);
bool compare_with_file(const Params& p, const HostData& d, const std::string& ref_file_name);
bool compare_time_step(const Params& p, const std::string& ref_file_name);
