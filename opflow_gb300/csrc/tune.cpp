// Autotuner cache (tune.h).  Cache file: one line per choice, "<key> <value> <ms>", appended as choices
// are made; loading keeps the last line of each key.
#include "tune.h"
#include "internal.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <unordered_map>

namespace opg {
namespace {

struct TuneCache {
    std::mutex mu;
    std::unordered_map<std::string, int> choice;
    std::string path;  // empty: in memory only
    long long tuned = 0, hits = 0;
    bool env_loaded = false;
};

TuneCache& cache() {
    static TuneCache* c = new TuneCache();  // (never destroyed: used until the process ends)
    return *c;
}

// reads `path` into the map (lock held); a missing file is an empty cache
int load_locked(TuneCache& c, const std::string& path) {
    std::ifstream in(path);
    if (!in) return OPFLOW_OK;
    std::string line;
    int lineno = 0;
    while (std::getline(in, line)) {
        ++lineno;
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ss(line);
        std::string key;
        int value = 0;
        if (!(ss >> key >> value)) return fail(OPFLOW_E_INVALID, "tune cache %s: line %d is not '<key> <value> [ms]'", path.c_str(), lineno);
        c.choice[key] = value;
    }
    return OPFLOW_OK;
}

// OPFLOW_TUNE_CACHE names a cache file for the process unless opflow_tune_set_cache chose one
void env_cache_locked(TuneCache& c) {
    if (c.env_loaded) return;
    c.env_loaded = true;
    const char* e = getenv("OPFLOW_TUNE_CACHE");
    if (e && *e && c.path.empty()) {
        c.path = e;
        load_locked(c, c.path);
    }
}

}  // namespace

bool tune_enabled() {
    const char* e = getenv("OPFLOW_TUNE");
    return !(e && e[0] == '0');
}

unsigned long long tune_hash(const void* p, size_t n, unsigned long long h) {
    const unsigned char* b = (const unsigned char*) p;
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

int tune_cached(const std::string& key, const std::vector<int>& cands) {
    if (cands.empty()) return 0;
    if (!tune_enabled()) return cands[0];
    TuneCache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    env_cache_locked(c);
    auto it = c.choice.find(key);
    if (it != c.choice.end())
        for (int v : cands)
            if (v == it->second) return v;
    return cands[0];
}

int tune_pick(const std::string& key, const std::vector<int>& cands, const std::function<float(int)>& time_ms) {
    if (cands.empty()) return 0;
    if (!tune_enabled() || cands.size() == 1) return cands[0];
    TuneCache& c = cache();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        env_cache_locked(c);
        auto it = c.choice.find(key);
        if (it != c.choice.end())
            for (int v : cands)
                if (v == it->second) {
                    c.hits++;
                    return v;
                }
    }
    // measured outside the lock (other threads keep their cached answers meanwhile)
    int best = cands[0];
    float best_ms = time_ms(cands[0]);
    for (size_t q = 1; q < cands.size(); ++q) {
        const float ms = time_ms(cands[q]);
        // a candidate replaces the default only when it is clearly faster (3 %), so that timing noise
        // does not flip choices between equal configurations
        if (ms >= 0.f && (best_ms < 0.f || ms < best_ms * (best == cands[0] ? 0.97f : 1.0f))) {
            best = cands[q];
            best_ms = ms;
        }
    }
    std::lock_guard<std::mutex> lk(c.mu);
    c.choice[key] = best;
    c.tuned++;
    if (!c.path.empty()) {
        if (FILE* f = std::fopen(c.path.c_str(), "a")) {
            std::fprintf(f, "%s %d %.4f\n", key.c_str(), best, (double) best_ms);
            std::fclose(f);
        }
    }
    return best;
}

}  // namespace opg

using namespace opg;

extern "C" {

int opflow_tune_set_cache(const char* path) {
    TuneCache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    c.env_loaded = true;  // an explicit choice overrides OPFLOW_TUNE_CACHE
    c.path = path ? path : "";
    if (c.path.empty()) return OPFLOW_OK;
    return load_locked(c, c.path);
}

int opflow_tune_lookup(const char* key, int* value) {
    if (!key || !value) return fail(OPFLOW_E_INVALID, "null argument");
    TuneCache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    env_cache_locked(c);
    auto it = c.choice.find(key);
    if (it == c.choice.end()) return fail(OPFLOW_E_INVALID, "no tuned choice for %s", key);
    *value = it->second;
    return OPFLOW_OK;
}

int opflow_tune_stats(long long* tuned, long long* hits, long long* entries) {
    TuneCache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    if (tuned) *tuned = c.tuned;
    if (hits) *hits = c.hits;
    if (entries) *entries = (long long) c.choice.size();
    return OPFLOW_OK;
}

int opflow_tune_clear(void) {
    TuneCache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    c.choice.clear();
    c.tuned = c.hits = 0;
    return OPFLOW_OK;
}

}  // extern "C"
