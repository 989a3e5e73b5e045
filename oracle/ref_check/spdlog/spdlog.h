// Minimal stand-in for <spdlog/spdlog.h>, written for this project.
//
// TEST INFRASTRUCTURE ONLY: lets the reference's apps/cpu_demo/main.cpp
// compile unmodified; every logging call is a no-op (the checkTree driver
// counts only checkTree's own printf output).
#pragma once

// The real header brings in <cstdio> (through fmt); the demo relies on that
// for printf.
#include <cstdio>

namespace spdlog {
namespace level {
enum level_enum { trace, debug, info, warn, err };
}
inline void set_level(level::level_enum) {}
template <class... A>
void info(const char*, const A&...) {}
template <class... A>
void debug(const char*, const A&...) {}
template <class... A>
void error(const char*, const A&...) {}
}  // namespace spdlog
