// host_common.h -- host-side helpers shared by the C ABI translation units.
#pragma once

#include <string>

#include "armon_gb300.h"

namespace armon {

void set_error(const std::string& msg);

}  // namespace armon
