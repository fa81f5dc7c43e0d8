// A stand-in for oneTBB's parallel_for over blocked ranges: splits the range
// into grain-sized pieces (rows for 1-D, 16x16-style tiles for 2-D) and runs
// them on std::thread workers.  Results of the reference's loops do not depend
// on the split (each piece writes its own pixels).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include <tbb/blocked_range.h>
#include <tbb/blocked_range2d.h>
#include <tbb/global_control.h>

namespace tbb {
namespace shim {
inline int threads() {
  const unsigned n = std::thread::hardware_concurrency();
  const int cap = parallelismCap();
  const int t = n ? int(n) : 1;
  return cap > 0 && cap < t ? cap : t;
}
template <typename F>
void runPieces(int n, const F& f) {
  std::atomic<int> next{0};
  auto w = [&]() {
    for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) f(i);
  };
  const int nt = std::min(threads(), std::max(1, n));
  std::vector<std::thread> pool;
  for (int i = 1; i < nt; ++i) pool.emplace_back(w);
  w();
  for (auto& t : pool) t.join();
}
}  // namespace shim

template <typename T, typename F>
void parallel_for(const blocked_range<T>& r, const F& f) {
  if (r.empty()) return;
  const T g = T(std::max<std::size_t>(1, r.grainsize()));
  const int n = int((r.end() - r.begin() + g - 1) / g);
  shim::runPieces(n, [&](int i) {
    const T b = r.begin() + T(i) * g;
    f(blocked_range<T>(b, std::min<T>(r.end(), b + g), r.grainsize()));
  });
}

template <typename T, typename F>
void parallel_for(const blocked_range2d<T>& r, const F& f) {
  if (r.rows().empty() || r.cols().empty()) return;
  const T gr = T(std::max<std::size_t>(1, r.rows().grainsize())), gc = T(std::max<std::size_t>(1, r.cols().grainsize()));
  const int nr = int((r.rows().end() - r.rows().begin() + gr - 1) / gr);
  const int nc = int((r.cols().end() - r.cols().begin() + gc - 1) / gc);
  shim::runPieces(nr * nc, [&](int i) {
    const T rb = r.rows().begin() + T(i / nc) * gr, cb = r.cols().begin() + T(i % nc) * gc;
    f(blocked_range2d<T>(rb, std::min<T>(r.rows().end(), rb + gr), r.rows().grainsize(), cb,
                         std::min<T>(r.cols().end(), cb + gc), r.cols().grainsize()));
  });
}
}  // namespace tbb
