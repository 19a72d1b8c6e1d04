// gtest.h — the subset of GoogleTest's interface that HEAL's C++ test files
// use (TEST, ASSERT_TRUE / ASSERT_FALSE / ASSERT_EQ, EXPECT_THROW and
// testing::internal::CaptureStderr / GetCapturedStderr), written for this
// repository so that those files compile unmodified without the GoogleTest
// library (HEAL's CMake fetches it from the network).  gtest_main.cpp
// provides main(), which runs every registered test and returns non-zero if
// any failed.
#pragma once

#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <functional>
#include <sstream>
#include <string>
#include <vector>

namespace testing {
namespace internal {

struct Case {
  std::string name;
  std::function<void()> body;
};

inline std::vector<Case> &registry() {
  static std::vector<Case> cases;
  return cases;
}

// failures recorded by the test that is running
inline int &failures() {
  static int n = 0;
  return n;
}

inline bool add_case(const char *suite, const char *name, void (*body)()) {
  registry().push_back({std::string(suite) + "." + name, body});
  return true;
}

inline void fail(const char *file, int line, const std::string &what) {
  std::fprintf(stderr, "%s:%d: Failure\n  %s\n", file, line, what.c_str());
  ++failures();
}

// the text streamed into a failing assertion (`ASSERT_TRUE(x) << "why"`)
struct Message {
  std::ostringstream os;
  template <typename V>
  Message &operator<<(const V &v) {
    os << v;
    return *this;
  }
};

// records the failure when the streamed message is assigned to it
struct Failer {
  const char *file;
  int line;
  const char *what;
  void operator=(const Message &m) const {
    const std::string extra = m.os.str();
    fail(file, line, extra.empty() ? std::string(what) : std::string(what) + "\n  " + extra);
  }
};

// stderr redirected to a temporary file between CaptureStderr and
// GetCapturedStderr
struct Capture {
  int saved = -1;
  std::FILE *file = nullptr;
};
inline Capture &capture() {
  static Capture c;
  return c;
}

inline void CaptureStderr() {
  Capture &c = capture();
  std::fflush(stderr);
  c.file = std::tmpfile();
  if (!c.file) return;
  c.saved = dup(2);
  dup2(fileno(c.file), 2);
}

inline std::string GetCapturedStderr() {
  Capture &c = capture();
  std::string out;
  if (!c.file) return out;
  std::fflush(stderr);
  dup2(c.saved, 2);
  close(c.saved);
  std::rewind(c.file);
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, c.file)) > 0) out.append(buf, got);
  std::fclose(c.file);
  c.file = nullptr;
  c.saved = -1;
  return out;
}

}  // namespace internal
}  // namespace testing

#define HEAL_GTEST_NAME(suite, name) suite##_##name##_Test

#define TEST(suite, name)                                                                                  \
  static void HEAL_GTEST_NAME(suite, name)();                                                             \
  static const bool HEAL_GTEST_NAME(suite, name##_registered) =                                           \
      ::testing::internal::add_case(#suite, #name, &HEAL_GTEST_NAME(suite, name));                          \
  static void HEAL_GTEST_NAME(suite, name)()

// ASSERT_* leave the test on failure, as GoogleTest's do, and take a message
// streamed after them.  `switch (0) case 0: default:` keeps an enclosing
// unbraced if / else from binding to the macro's own else.
#define HEAL_GTEST_ASSERT(cond, text)                                                      \
  switch (0)                                                                               \
  case 0:                                                                                  \
  default:                                                                                 \
    if (cond)                                                                              \
      ;                                                                                    \
    else                                                                                   \
      return ::testing::internal::Failer{__FILE__, __LINE__, text} = ::testing::internal::Message()

#define ASSERT_TRUE(cond) HEAL_GTEST_ASSERT((cond), "expected true: " #cond)
#define ASSERT_FALSE(cond) HEAL_GTEST_ASSERT(!(cond), "expected false: " #cond)
#define ASSERT_EQ(a, b) HEAL_GTEST_ASSERT((a) == (b), "expected equal: " #a " == " #b)

// EXPECT_THROW records a failure and lets the test go on
#define EXPECT_THROW(stmt, exc)                                                            \
  do {                                                                                     \
    bool heal_gtest_caught = false;                                                        \
    try {                                                                                  \
      stmt;                                                                                \
    } catch (const exc &) {                                                                \
      heal_gtest_caught = true;                                                            \
    } catch (...) {                                                                        \
      ::testing::internal::fail(__FILE__, __LINE__, #stmt " threw another type than " #exc); \
      heal_gtest_caught = true;                                                            \
    }                                                                                      \
    if (!heal_gtest_caught)                                                                \
      ::testing::internal::fail(__FILE__, __LINE__, #stmt " did not throw " #exc);         \
  } while (0)
