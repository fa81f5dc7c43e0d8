// Tiny check harness for the C++ API tests: prints ok/FAIL lines and returns
// the number of failures from report().
#pragma once

#include <cmath>
#include <cstdio>
#include <string>

struct Checks {
  int total = 0, failed = 0;
  void operator()(const std::string& what, bool ok) {
    ++total;
    if (!ok) ++failed;
    std::printf("  %s - %s\n", ok ? "ok  " : "FAIL", what.c_str());
  }
  int report(const char* name) const {
    std::printf("[%s] %d/%d checks passed\n", name, total - failed, total);
    return failed == 0 ? 0 : 1;
  }
};

inline bool near(float a, float b, float eps) { return std::fabs(a - b) <= eps; }
