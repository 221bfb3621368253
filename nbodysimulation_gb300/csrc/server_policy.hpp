// server_policy.hpp -- the host-side decisions of the job server, free of
// CUDA so they build and run anywhere: admission under a slot count and a
// device-memory budget, the length of a round, the snapshot schedule and
// latency percentiles.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace nbgb {

// First-come first-served admission.  The job at the head of the queue is
// admitted as soon as a slot and its bytes are free; later jobs never
// overtake it, so a large job cannot be starved by a stream of small ones.
// A job larger than the whole budget can never run and is refused.
class Admission {
  public:
    Admission(int64_t budget_bytes, int max_jobs) : budget_(budget_bytes), max_jobs_(max_jobs) {}
    bool can_ever_fit(int64_t bytes) const { return bytes <= budget_; }
    bool fits(int64_t bytes) const { return jobs_ < max_jobs_ && in_use_ + bytes <= budget_; }
    void reserve(int64_t bytes) {
        in_use_ += bytes;
        ++jobs_;
        peak_ = std::max(peak_, in_use_);
        peak_jobs_ = std::max(peak_jobs_, jobs_);
    }
    void release(int64_t bytes) {
        in_use_ -= bytes;
        --jobs_;
    }
    int64_t in_use() const { return in_use_; }
    int64_t peak() const { return peak_; }
    int jobs() const { return jobs_; }
    int peak_jobs() const { return peak_jobs_; }
    int64_t budget() const { return budget_; }

  private:
    int64_t budget_;
    int max_jobs_;
    int64_t in_use_ = 0, peak_ = 0;
    int jobs_ = 0, peak_jobs_ = 0;
};

// Steps in the next round: the snapshot period (every job joins at a round
// boundary, so its snapshot points fall on round boundaries), cut short
// when every running job ends earlier.
inline int round_steps(const std::vector<int> &remaining, int snapshot_every) {
    const int period = snapshot_every > 0 ? snapshot_every : 10;
    int most = 0;
    for (int r : remaining) most = std::max(most, r);
    return std::min(period, most);
}

// Steps done after a round of `round` steps, and whether a snapshot is due
// then (a multiple of the period before the last step; the last step's
// state is the result).
inline int steps_after(int done, int total, int round) { return std::min(total, done + round); }
inline bool snapshot_due(int done_after, int total, int snapshot_every) {
    return snapshot_every > 0 && done_after < total && done_after > 0 && done_after % snapshot_every == 0;
}

// Nearest-rank percentile (p in [0, 100]) of the samples; 0 when empty.
inline double percentile(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double rank = std::ceil(p / 100.0 * (double)v.size());
    size_t i = rank < 1.0 ? 0 : (size_t)rank - 1;
    if (i >= v.size()) i = v.size() - 1;
    return v[i];
}

}  // namespace nbgb
