// Autotuner of launch configurations: among equivalent configurations of a kernel (results are
// identical whichever is chosen) the fastest, measured once on the device and cached per
// (kernel, shape, stencil) key for the process, and in a cache file when one is set.
#pragma once

#include <functional>
#include <string>
#include <vector>

namespace opg {

// Tuning is on unless OPFLOW_TUNE=0 (read at every call).
bool tune_enabled();

// The cached choice for `key`, else the fastest of `cands` by `time_ms` (a run of the candidate on the
// device: its time in ms, or a negative value when it cannot run), which is then cached.  cands[0] is the
// default: returned when tuning is off, and kept when no candidate is measurably faster than it.
int tune_pick(const std::string& key, const std::vector<int>& cands, const std::function<float(int)>& time_ms);

// The cached choice for `key` when it is one of `cands`, else cands[0], without measuring (for callers
// that cannot time a launch, e.g. while a stream is being captured).
int tune_cached(const std::string& key, const std::vector<int>& cands);

// FNV-1a over bytes, for the stencil part of a key
unsigned long long tune_hash(const void* p, size_t n, unsigned long long h = 1469598103934665603ull);

}  // namespace opg
