// TEST INFRASTRUCTURE ONLY.  Compile shim for glog, which the reference's
// hot-path sources use for assertions and logging: a failed CHECK and
// LOG(FATAL) abort, other log lines are discarded.  Like glog's own header
// it brings in the stream headers the reference's sources rely on.
#pragma once

#include <cstdlib>
#include <iostream>
#include <ostream>
#include <sstream>
#include <string>
#include <vector>

namespace ref_shim {
struct NullLog {
  template <class T>
  NullLog& operator<<(const T&) { return *this; }
};
struct FatalLog {
  bool fatal;
  explicit FatalLog(bool f) : fatal(f) {}
  ~FatalLog() {
    if (fatal) std::abort();
  }
  template <class T>
  FatalLog& operator<<(const T&) { return *this; }
};
}  // namespace ref_shim

#define REF_SHIM_SEV_INFO false
#define REF_SHIM_SEV_WARNING false
#define REF_SHIM_SEV_ERROR false
#define REF_SHIM_SEV_FATAL true
#define LOG(sev) ref_shim::FatalLog(REF_SHIM_SEV_##sev)
#define DLOG(sev) ref_shim::NullLog()
#define VLOG(n) ref_shim::NullLog()
#define CHECK(c) ref_shim::FatalLog(!(c))
#define CHECK_EQ(a, b) CHECK((a) == (b))
#define CHECK_NE(a, b) CHECK((a) != (b))
#define CHECK_LT(a, b) CHECK((a) < (b))
#define CHECK_LE(a, b) CHECK((a) <= (b))
#define CHECK_GT(a, b) CHECK((a) > (b))
#define CHECK_GE(a, b) CHECK((a) >= (b))
#define CHECK_NOTNULL(p) (p)
