// Helpers shared by the reference drivers (ref_driver.cpp, ref_solve.cpp): the seeded inputs that the
// oracle and the tests regenerate, and the record writer of the dump format
// ("FIELD <json>\n" + float64 payload).  Test infrastructure only.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

// ---- seeded inputs shared with the oracle and the tests (counter-based splitmix64) ----
static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline double u01(uint64_t seed, uint64_t k) {
    return (double) (mix64(seed + (k + 1) * 0x9E3779B97F4A7C15ull) >> 11) * 0x1.0p-53;
}

static FILE* g_out = nullptr;
static void put(const std::vector<double>& v) { fwrite(v.data(), sizeof(double), v.size(), g_out); }

// Dump the readable range of a field (padded local range clipped to the logical range), x fastest,
// together with the field's ranges.
template <typename F>
static void dump_field(const F& u, const char* name) {
    constexpr int dim = internal::CartesianFieldExprTrait<F>::dim;
    auto rr = u.getLocalReadableRange();
    std::string js = std::format("{{\"name\":\"{}\",\"dim\":{},\"padding\":{}", name, dim, u.padding);
    auto rng = [&](const char* nm, const auto& r) {
        js += std::format(",\"{}\":[", nm);
        for (int d = 0; d < dim; ++d) js += std::format("{}[{},{}]", d ? "," : "", r.start[d], r.end[d]);
        js += "]";
    };
    rng("readable", rr);
    rng("logical", u.logicalRange);
    rng("accessible", u.accessibleRange);
    rng("assignable", u.assignableRange);
    rng("local", u.localRange);
    js += std::format(",\"count\":{}}}", rr.count());
    fprintf(g_out, "FIELD %s\n", js.c_str());
    std::vector<double> v;
    v.reserve(rr.count());
    rangeFor_s(rr, [&](auto&& i) { v.push_back(u.evalAt(i)); });
    put(v);
}

