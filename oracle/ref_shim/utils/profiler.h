// TEST INFRASTRUCTURE ONLY.  Compile shim for the reference's MPI profiler
// header (utils/profiler.h needs mpi.h): render/spray.h declares an extern
// Profiler and relies on the standard headers it pulls in; utils/
// profiler_util.h wraps its timers in inline helpers the oracle never calls.
#pragma once

#include <cstdint>
#include <limits>
#include <map>
#include <string>
#include <vector>

namespace spray {
class Profiler {
 public:
  void start(int) {}
  void stop(int) {}
  void agg(int, uint64_t) {}
  void reset() {}
  void print(int64_t) {}
};
}  // namespace spray
