// A stand-in for oneTBB's blocked_range2d (rows x cols tiles).  TEST
// INFRASTRUCTURE ONLY.
#pragma once
#include <tbb/blocked_range.h>

namespace tbb {
template <typename T>
class blocked_range2d {
 public:
  blocked_range2d(T r0, T r1, std::size_t rg, T c0, T c1, std::size_t cg) : rows_(r0, r1, rg), cols_(c0, c1, cg) {}
  blocked_range2d(T r0, T r1, T c0, T c1) : rows_(r0, r1), cols_(c0, c1) {}
  const blocked_range<T>& rows() const { return rows_; }
  const blocked_range<T>& cols() const { return cols_; }

 private:
  blocked_range<T> rows_, cols_;
};
}  // namespace tbb
