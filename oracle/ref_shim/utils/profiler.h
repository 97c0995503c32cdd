// TEST INFRASTRUCTURE ONLY.  Compile shim for the reference's MPI profiler
// header (utils/profiler.h needs mpi.h): the reference's render/spray.h only
// declares an extern Profiler and relies on the standard headers it pulls in.
#pragma once

#include <cstdint>
#include <limits>
#include <map>
#include <string>
#include <vector>

namespace spray {
class Profiler {};
}  // namespace spray
