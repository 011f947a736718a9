// Serial stand-in for the slice of oneTBB that OpFlow's rangeFor / rangeReduce use.
// Scheduling only: OpFlow's results do not depend on the thread count.
#pragma once
#include <functional>
#include <utility>
#include "../oneapi/tbb/detail/_range_common.h"
namespace tbb {
struct task_arena {
    explicit task_arena(int = 0) {}
    template <class F> auto execute(F&& f) { return f(); }
};
template <class R, class B> void parallel_for(const R& r, const B& body) { body(r); }
template <class R, class V, class B, class J> V parallel_reduce(const R& r, const V& id, const B& body, const J&) { return body(r, id); }
}
namespace tbb {
template <class R, class B> void parallel_reduce(const R& r, B& body) { body(r); }
template <class T> struct blocked_range {
    T b, e;
    blocked_range(T b_, T e_, std::size_t = 1) : b(b_), e(e_) {}
    T begin() const { return b; }
    T end() const { return e; }
};
}
