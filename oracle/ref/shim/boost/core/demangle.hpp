// Stand-in for boost::core::demangle (type names are only used in log text).
#pragma once
#include <string>
namespace boost { namespace core { inline std::string demangle(const char* n) { return n ? n : ""; } } }
