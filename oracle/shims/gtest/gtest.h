// Oracle build shim (test infrastructure only): a minimal googletest stand-in
// that runs the reference's own known-answer tests (TEST, EXPECT_*/ASSERT_*)
// without googletest installed. Death tests are counted as skipped.
#pragma once
#include <cstdio>
#include <functional>
#include <iomanip>
#include <map>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace testing {
class Test {
public:
    virtual ~Test() = default;
    virtual void SetUp() {}
    virtual void TearDown() {}
};
template <class... T> struct Types {};
namespace shim {
struct Case { std::string name; std::function<void()> fn; };
inline std::vector<Case>& registry() { static std::vector<Case> r; return r; }
inline int& failures() { static int f = 0; return f; }
inline int& skipped() { static int s = 0; return s; }
inline bool& current_failed() { static bool b = false; return b; }
struct Registrar {
    Registrar(const char* suite, const char* name, std::function<void()> fn) {
        registry().push_back({std::string(suite) + "." + name, std::move(fn)});
    }
};
struct AssertAbort {};
template <class A, class B>
inline bool report_eq(const A& a, const B& b, bool want_eq, const char* ea, const char* eb,
                      const char* file, int line) {
    bool eq = (a == b);
    if (eq == want_eq) return true;
    std::ostringstream sa, sb;
    sa << a;
    sb << b;
    std::fprintf(stderr, "%s:%d: expected %s %s %s\n  lhs: %s\n  rhs: %s\n", file, line, ea,
                 want_eq ? "==" : "!=", eb, sa.str().c_str(), sb.str().c_str());
    current_failed() = true;
    ++failures();
    return false;
}
inline bool report_bool(bool v, bool want, const char* e, const char* file, int line) {
    if (v == want) return true;
    std::fprintf(stderr, "%s:%d: expected %s to be %s\n", file, line, e, want ? "true" : "false");
    current_failed() = true;
    ++failures();
    return false;
}
} // namespace shim
inline void InitGoogleTest(int*, char**) {}
} // namespace testing

#define SHIM_TEST_FN(suite, name) shim_test_##suite##_##name
#define TEST(suite, name)                                                                   \
    static void SHIM_TEST_FN(suite, name)();                                                \
    static ::testing::shim::Registrar shim_reg_##suite##_##name(#suite, #name,               \
                                                                SHIM_TEST_FN(suite, name)); \
    static void SHIM_TEST_FN(suite, name)()
#define TEST_F(fixture, name)                                                                        \
    struct shim_fixture_##fixture##_##name : fixture {                                               \
        void TestBody();                                                                             \
    };                                                                                               \
    static ::testing::shim::Registrar shim_reg_##fixture##_##name(#fixture, #name, [] {              \
        shim_fixture_##fixture##_##name t;                                                           \
        t.SetUp();                                                                                   \
        t.TestBody();                                                                                \
        t.TearDown();                                                                                \
    });                                                                                              \
    void shim_fixture_##fixture##_##name::TestBody()
#define EXPECT_EQ(a, b) ::testing::shim::report_eq((a), (b), true, #a, #b, __FILE__, __LINE__)
#define EXPECT_NE(a, b) ::testing::shim::report_eq((a), (b), false, #a, #b, __FILE__, __LINE__)
#define EXPECT_TRUE(a) ::testing::shim::report_bool(static_cast<bool>(a), true, #a, __FILE__, __LINE__)
#define EXPECT_FALSE(a) ::testing::shim::report_bool(static_cast<bool>(a), false, #a, __FILE__, __LINE__)
#define ASSERT_EQ(a, b) do { if (!EXPECT_EQ(a, b)) throw ::testing::shim::AssertAbort{}; } while (0)
#define ASSERT_NE(a, b) do { if (!EXPECT_NE(a, b)) throw ::testing::shim::AssertAbort{}; } while (0)
#define ASSERT_TRUE(a) do { if (!EXPECT_TRUE(a)) throw ::testing::shim::AssertAbort{}; } while (0)
#define ASSERT_FALSE(a) do { if (!EXPECT_FALSE(a)) throw ::testing::shim::AssertAbort{}; } while (0)
#define ASSERT_DEATH(stmt, re) do { ++::testing::shim::skipped(); } while (0)
#define EXPECT_DEATH(stmt, re) do { ++::testing::shim::skipped(); } while (0)
#define RUN_ALL_TESTS() ::testing::shim::run_all()

namespace testing { namespace shim {
inline int run_all() {
    int failedCases = 0;
    for (auto& c : registry()) {
        current_failed() = false;
        try { c.fn(); } catch (const AssertAbort&) {}
        std::printf("[%s] %s\n", current_failed() ? "FAILED" : "    OK", c.name.c_str());
        if (current_failed()) ++failedCases;
    }
    std::printf("%zu cases, %d failed, %d death checks skipped\n", registry().size(), failedCases, skipped());
    return failedCases ? 1 : 0;
}
} }
