// main() for test files written against gtest/gtest.h (this repository's
// GoogleTest-compatible subset): runs every registered TEST in registration
// order, reports each one, and returns 1 if any failed.  An exception that
// leaves a test counts as a failure of that test.
#include <cstdio>
#include <exception>

#include "gtest/gtest.h"

int main() {
  auto &cases = ::testing::internal::registry();
  int failed = 0;
  for (auto &c : cases) {
    std::printf("[ RUN      ] %s\n", c.name.c_str());
    std::fflush(stdout);
    ::testing::internal::failures() = 0;
    try {
      c.body();
    } catch (const std::exception &e) {
      std::fprintf(stderr, "uncaught exception: %s\n", e.what());
      ++::testing::internal::failures();
    } catch (...) {
      std::fprintf(stderr, "uncaught exception of unknown type\n");
      ++::testing::internal::failures();
    }
    const bool ok = ::testing::internal::failures() == 0;
    failed += !ok;
    std::printf("[ %s ] %s\n", ok ? "      OK" : " FAILED ", c.name.c_str());
  }
  std::printf("[==========] %zu tests, %d failed\n", cases.size(), failed);
  return failed ? 1 : 0;
}
