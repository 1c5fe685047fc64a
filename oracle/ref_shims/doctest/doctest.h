// doctest.h - minimal stand-in for the doctest framework, so that the reference's
// embedded TEST_CASEs (cpp/offset_computer.hpp:259-333, cpp/state_vector.hpp:383-513,
// cpp/hamiltonian.hpp:192-313) compile and run unmodified inside oracle/_ref.
// TEST INFRASTRUCTURE ONLY (the reference vendors doctest; it is not in the tree).
#ifndef QPE_REF_SHIM_DOCTEST_H_
#define QPE_REF_SHIM_DOCTEST_H_

#include <sstream>
#include <string>
#include <vector>

namespace doctest_shim {

struct Case {
  const char* name;
  void (*fn)();
  const char* file;
  int line;
};

inline std::vector<Case>& registry() {
  static std::vector<Case> r;
  return r;
}

struct Stats {
  long checks = 0;
  long failed_checks = 0;
  std::string first_failure;
};

inline Stats& stats() {
  static Stats s;
  return s;
}

struct Abort {};

struct Reg {
  Reg(const char* n, void (*f)(), const char* file, int line) { registry().push_back(Case{n, f, file, line}); }
};

inline void record(bool ok, bool fatal, const char* expr, const char* file, int line) {
  Stats& s = stats();
  ++s.checks;
  if (!ok) {
    ++s.failed_checks;
    if (s.first_failure.empty()) {
      std::ostringstream os;
      os << file << ":" << line << ": " << expr;
      s.first_failure = os.str();
    }
    if (fatal) throw Abort{};
  }
}

}  // namespace doctest_shim

#define DOCTEST_SHIM_CAT_(a, b) a##b
#define DOCTEST_SHIM_CAT(a, b) DOCTEST_SHIM_CAT_(a, b)

#ifdef DOCTEST_CONFIG_DISABLE
#define DOCTEST_SHIM_TC(name, c) [[maybe_unused]] static void DOCTEST_SHIM_CAT(doctest_shim_fn_, c)()
#else
#define DOCTEST_SHIM_TC(name, c)                                                                      \
  static void DOCTEST_SHIM_CAT(doctest_shim_fn_, c)();                                                \
  static ::doctest_shim::Reg DOCTEST_SHIM_CAT(doctest_shim_reg_, c)(name, &DOCTEST_SHIM_CAT(doctest_shim_fn_, c), \
                                                                      __FILE__, __LINE__);            \
  static void DOCTEST_SHIM_CAT(doctest_shim_fn_, c)()
#endif

#define TEST_CASE(name) DOCTEST_SHIM_TC(name, __COUNTER__)
#define REQUIRE_EQ(a, b) ::doctest_shim::record((a) == (b), true, #a " == " #b, __FILE__, __LINE__)
#define REQUIRE_GT(a, b) ::doctest_shim::record((a) > (b), true, #a " > " #b, __FILE__, __LINE__)
#define CHECK(expr) ::doctest_shim::record(static_cast<bool>(expr), false, #expr, __FILE__, __LINE__)
#define REQUIRE(expr) ::doctest_shim::record(static_cast<bool>(expr), true, #expr, __FILE__, __LINE__)
#define CAPTURE(x) ((void)0)

#endif  // QPE_REF_SHIM_DOCTEST_H_
