// Minimal stand-in for the part of googletest the reference's unit tests use
// (TEST, ASSERT_NEAR, InitGoogleTest, RUN_ALL_TESTS).  Test infrastructure
// only: it lets the reference's own convergence tests run against the
// reference's own sources so their measured values can be recorded as golden
// numbers.  Every ASSERT_NEAR prints one machine-readable line:
//   NEAR <suite>.<name> <value %.17g> <expected %.17g> <tol %.17g> <PASS|FAIL>
#pragma once

#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

namespace testing {
struct TestEntry {
  std::string suite, name;
  std::function<void()> body;
};
inline std::vector<TestEntry>& registry() {
  static std::vector<TestEntry> r;
  return r;
}
inline std::string& current_test() {
  static std::string s;
  return s;
}
inline bool& current_failed() {
  static bool f = false;
  return f;
}
struct Registrar {
  Registrar(const char* s, const char* n, std::function<void()> b) {
    registry().push_back(TestEntry{s, n, std::move(b)});
  }
};
inline void InitGoogleTest(int*, char**) {}
inline void InitGoogleTest() {}
inline int RunAll() {
  int failed = 0;
  for (auto& t : registry()) {
    current_test() = t.suite + "." + t.name;
    current_failed() = false;
    t.body();
    std::printf("TEST %s %s\n", current_test().c_str(), current_failed() ? "FAILED" : "OK");
    failed += current_failed() ? 1 : 0;
  }
  std::printf("SUMMARY %zu tests, %d failed\n", registry().size(), failed);
  return failed ? 1 : 0;
}
}  // namespace testing

#define RUN_ALL_TESTS() ::testing::RunAll()

#define TEST(suite, name)                                                    \
  static void suite##_##name##_body();                                       \
  static ::testing::Registrar suite##_##name##_reg(#suite, #name,            \
                                                   suite##_##name##_body);   \
  static void suite##_##name##_body()

#define ASSERT_NEAR(val, expected, tol)                                      \
  do {                                                                       \
    const double v_ = (val), e_ = (expected), t_ = (tol);                    \
    const bool ok_ = std::fabs(v_ - e_) <= t_;                               \
    std::printf("NEAR %s %.17g %.17g %.17g %s\n",                            \
                ::testing::current_test().c_str(), v_, e_, t_,               \
                ok_ ? "PASS" : "FAIL");                                      \
    if (!ok_) {                                                              \
      ::testing::current_failed() = true;                                    \
      return;                                                                \
    }                                                                        \
  } while (0)
