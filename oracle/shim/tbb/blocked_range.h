// A stand-in for oneTBB's blocked_range (the half-open index range the
// reference's parallel loops split), for compiling the reference's render
// path against the oracle's CPU substrate.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstddef>

namespace tbb {
template <typename T>
class blocked_range {
 public:
  blocked_range(T b, T e, std::size_t grain = 1) : b_(b), e_(e), grain_(grain) {}
  T begin() const { return b_; }
  T end() const { return e_; }
  std::size_t grainsize() const { return grain_; }
  bool empty() const { return !(b_ < e_); }

 private:
  T b_, e_;
  std::size_t grain_;
};
}  // namespace tbb
