// A stand-in for oneTBB's global_control: while an object with
// max_allowed_parallelism exists, the parallel loops of the stand-in
// parallel_for use at most that many threads.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstddef>

namespace tbb {
namespace shim {
inline int& parallelismCap() {
  static int cap = 0;  // 0 = no cap
  return cap;
}
}  // namespace shim

class global_control {
 public:
  enum parameter { max_allowed_parallelism = 0, thread_stack_size = 1 };
  global_control(parameter p, std::size_t value) : p_(p) {
    if (p_ == max_allowed_parallelism) {
      prev_ = shim::parallelismCap();
      shim::parallelismCap() = int(value);
    }
  }
  ~global_control() {
    if (p_ == max_allowed_parallelism) shim::parallelismCap() = prev_;
  }

 private:
  parameter p_;
  int prev_ = 0;
};
}  // namespace tbb
