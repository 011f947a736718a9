// Stand-in for spdlog: the logging calls sit inside `if consteval` and never run.
#pragma once
#include <string>
namespace spdlog {
inline void info(const std::string&) {}
inline void warn(const std::string&) {}
inline void error(const std::string&) {}
inline void critical(const std::string&) {}
inline void debug(const std::string&) {}
inline void trace(const std::string&) {}
}
