// Serial stand-in for the TBB range-splitting tags used by DS::Range's splitting constructors.
#pragma once
#include <cstddef>
namespace tbb { namespace detail {
struct split {};
struct proportional_split { std::size_t l = 1, r = 1; std::size_t left() const { return l; } std::size_t right() const { return r; } };
} using detail::split; using detail::proportional_split; }
