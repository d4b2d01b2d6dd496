// host_common.h -- host-side helpers shared by the C ABI translation units.
#pragma once

#include <string>

#include "armon_gb300.h"

namespace armon {

void set_error(const std::string& msg);

}  // namespace armon

extern "C" {
// BC_* sign factors of a test case on one side (src/kernels/test_cases.h:36-121).
void armon_boundary_factors(int test, int side, double* u_factor, double* v_factor);
// TestCase::test_option as the driver passes it to init_test (src/armon_2D.cpp:116-118), with
// armon_params.test_option as an override.
double armon_test_option(const armon_params* p, double dx, double dy);
int armon_solver_begin_loop(armon_solver* s);
}
