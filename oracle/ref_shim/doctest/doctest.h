// ORACLE (test infrastructure only) -- a project-owned subset of doctest's
// API, enough to compile and run the TEST_CASEs that ibis keeps inside its
// own sources: TEST_CASE, CHECK, CHECK_LT, CHECK_GT, doctest::Approx (with
// epsilon() and scale()) and doctest::Context (applyCommandLine, run).
// Approx compares |a - b| < epsilon * (scale + max(|a|, |b|)) with the
// default epsilon 100 * FLT_EPSILON and scale 1, as doctest documents.
// With DOCTEST_CONFIG_DISABLE the test bodies are compiled but not registered.
// IBIS_REF_DOCTEST_VERBOSE in the environment names each test case as it runs.
#ifndef IBIS_REF_SHIM_DOCTEST_H
#define IBIS_REF_SHIM_DOCTEST_H

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <string>
#include <type_traits>
#include <vector>

namespace doctest {

class Approx {
public:
    explicit Approx(double v) : value_(v) {}
    Approx& epsilon(double e) { eps_ = e; return *this; }
    Approx& scale(double s) { scale_ = s; return *this; }
    bool matches(double x) const {
        return std::fabs(x - value_) < eps_ * (scale_ + std::max(std::fabs(x), std::fabs(value_)));
    }
    double value() const { return value_; }

private:
    double value_;
    double eps_ = std::numeric_limits<float>::epsilon() * 100;
    double scale_ = 1.0;
};
template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
bool operator==(T x, const Approx& a) { return a.matches((double)x); }
template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
bool operator==(const Approx& a, T x) { return a.matches((double)x); }
template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
bool operator!=(T x, const Approx& a) { return !a.matches((double)x); }
template <class T, std::enable_if_t<std::is_arithmetic_v<T>, int> = 0>
bool operator!=(const Approx& a, T x) { return !a.matches((double)x); }

namespace detail {
struct TestCase {
    const char* name;
    const char* file;
    int line;
    void (*fn)();
};
inline std::vector<TestCase>& registry() {
    static std::vector<TestCase> r;
    return r;
}
struct Registrar {
    Registrar(const char* name, const char* file, int line, void (*fn)()) { registry().push_back({name, file, line, fn}); }
};
struct State {
    long checks = 0, failed_checks = 0;
    bool current_failed = false;
};
inline State& state() {
    static State s;
    return s;
}
inline void check(bool ok, const char* expr, const char* file, int line) {
    state().checks++;
    if (!ok) {
        state().failed_checks++;
        state().current_failed = true;
        std::fprintf(stderr, "%s:%d: CHECK( %s ) is NOT correct!\n", file, line, expr);
    }
}
}  // namespace detail

class Context {
public:
    Context() = default;
    Context(int argc, char** argv) { applyCommandLine(argc, argv); }
    void applyCommandLine(int argc, char** argv) {
        for (int i = 1; i < argc; i++) {
            const char* a = argv[i];
            if (std::strncmp(a, "-tc=", 4) == 0) filter_ = a + 4;
            else if (std::strncmp(a, "--test-case=", 12) == 0) filter_ = a + 12;
            else if (std::strcmp(a, "--list") == 0 || std::strcmp(a, "-ltc") == 0) list_ = true;
        }
    }
    void setOption(const char*, const char*) {}
    int run() {
        auto& reg = detail::registry();
        std::sort(reg.begin(), reg.end(), [](const detail::TestCase& x, const detail::TestCase& y) {
            const int c = std::strcmp(x.file, y.file);
            return c != 0 ? c < 0 : x.line < y.line;
        });
        long run = 0, failed = 0;
        for (const auto& t : reg) {
            if (!filter_.empty() && std::string(t.name).find(filter_) == std::string::npos) continue;
            if (list_) { std::printf("%s\n", t.name); continue; }
            detail::state().current_failed = false;
            if (verbose_) std::fprintf(stderr, "[doctest subset] %s (%s:%d)\n", t.name, t.file, t.line);
            t.fn();
            run++;
            if (detail::state().current_failed) {
                failed++;
                std::fprintf(stderr, "TEST CASE FAILED: %s (%s:%d)\n", t.name, t.file, t.line);
            }
        }
        if (!list_)
            std::printf("[doctest subset] test cases: %ld | %ld passed | %ld failed; assertions: %ld | %ld failed\n",
                        run, run - failed, failed, detail::state().checks, detail::state().failed_checks);
        return failed ? 1 : 0;
    }

private:
    std::string filter_;
    bool list_ = false;
    bool verbose_ = std::getenv("IBIS_REF_DOCTEST_VERBOSE") != nullptr;
};

}  // namespace doctest

#define DOCTEST_CAT_(a, b) a##b
#define DOCTEST_CAT(a, b) DOCTEST_CAT_(a, b)
#ifdef DOCTEST_CONFIG_DISABLE
#define DOCTEST_TC_(fn, name)          \
    [[maybe_unused]] static void fn(); \
    static void fn()
#else
#define DOCTEST_TC_(fn, name)                                                                 \
    static void fn();                                                                         \
    static ::doctest::detail::Registrar DOCTEST_CAT(fn, _reg)(name, __FILE__, __LINE__, &fn); \
    static void fn()
#endif
#define TEST_CASE(name) DOCTEST_TC_(DOCTEST_CAT(doctest_tc_, __COUNTER__), name)
#define CHECK(...) ::doctest::detail::check(static_cast<bool>(__VA_ARGS__), #__VA_ARGS__, __FILE__, __LINE__)
#define CHECK_LT(a, b) ::doctest::detail::check((a) < (b), #a " < " #b, __FILE__, __LINE__)
#define CHECK_GT(a, b) ::doctest::detail::check((a) > (b), #a " > " #b, __FILE__, __LINE__)
#define CHECK_EQ(a, b) ::doctest::detail::check((a) == (b), #a " == " #b, __FILE__, __LINE__)
#define REQUIRE(...) CHECK(__VA_ARGS__)

#endif
