// Stand-in for Boost.Log's trivial logger: every record is discarded.
#pragma once
#include <ostream>
namespace gspec_shim {
struct NullLog {
  template <typename T>
  NullLog& operator<<(const T&) { return *this; }
  NullLog& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
}  // namespace gspec_shim
#define BOOST_LOG_TRIVIAL(level) ::gspec_shim::NullLog()
