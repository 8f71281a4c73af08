// ORACLE (test infrastructure only) -- a project-owned subset of spdlog's
// API, enough to compile ibis's own sources unchanged: info / warn / error /
// debug with {}-style placeholders ({}, {:.3}, {:.2e}, {:.1f}, {:>8}), a
// stopwatch, and a global level.  Messages go to stderr; by default only
// errors are shown, IBIS_REF_LOG=info / debug shows more, IBIS_REF_LOG=quiet
// nothing.
#ifndef IBIS_REF_SHIM_SPDLOG_H
#define IBIS_REF_SHIM_SPDLOG_H

#include <cctype>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <utility>

namespace spdlog {

namespace level {
enum level_enum { trace = 0, debug = 1, info = 2, warn = 3, err = 4, critical = 5, off = 6 };
}

class stopwatch {
public:
    stopwatch() : t0_(std::chrono::steady_clock::now()) {}
    std::chrono::duration<double> elapsed() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_);
    }
    void reset() { t0_ = std::chrono::steady_clock::now(); }

private:
    std::chrono::steady_clock::time_point t0_;
};

namespace detail {
inline int& threshold() {
    static int t = [] {
        const char* e = std::getenv("IBIS_REF_LOG");
        if (!e) return (int)level::err;
        if (std::strcmp(e, "quiet") == 0) return (int)level::off;
        if (std::strcmp(e, "debug") == 0) return (int)level::debug;
        if (std::strcmp(e, "info") == 0) return (int)level::info;
        return (int)level::err;
    }();
    return t;
}

template <class T>
void put(std::ostringstream& os, const std::string& spec, const T& v) {
    // spec: [>width][.precision][e|f|g]
    size_t k = 0;
    int width = -1, prec = -1;
    char kind = 0;
    if (k < spec.size() && spec[k] == '>') {
        k++;
        width = std::atoi(spec.c_str() + k);
        while (k < spec.size() && std::isdigit((unsigned char)spec[k])) k++;
    }
    if (k < spec.size() && spec[k] == '.') {
        k++;
        prec = std::atoi(spec.c_str() + k);
        while (k < spec.size() && std::isdigit((unsigned char)spec[k])) k++;
    }
    if (k < spec.size()) kind = spec[k];
    std::ostringstream one;
    if (prec >= 0) one << std::setprecision(prec);
    if (kind == 'e') one << std::scientific;
    if (kind == 'f') one << std::fixed;
    if constexpr (std::is_same_v<T, stopwatch>) one << v.elapsed().count();
    else one << v;
    std::string s = one.str();
    if (width > 0 && (int)s.size() < width) s = std::string(width - s.size(), ' ') + s;
    os << s;
}

inline void format_into(std::ostringstream& os, const char* f) { os << f; }
template <class A, class... Rest>
void format_into(std::ostringstream& os, const char* f, const A& a, const Rest&... rest) {
    while (*f) {
        if (f[0] == '{' && f[1] == '{') { os << '{'; f += 2; continue; }
        if (f[0] == '}' && f[1] == '}') { os << '}'; f += 2; continue; }
        if (f[0] == '{') {
            const char* e = std::strchr(f, '}');
            if (!e) break;
            std::string spec(f + 1, e);
            if (!spec.empty() && spec[0] == ':') spec = spec.substr(1);
            put(os, spec, a);
            format_into(os, e + 1, rest...);
            return;
        }
        os << *f++;
    }
}
template <class... A>
void log(int lv, const char* tag, const std::string& fmt, const A&... a) {
    if (lv < threshold()) return;
    std::ostringstream os;
    format_into(os, fmt.c_str(), a...);
    std::fprintf(stderr, "[ibis-ref %s] %s\n", tag, os.str().c_str());
}
}  // namespace detail

template <class... A>
void trace(const std::string& f, const A&... a) { detail::log(level::trace, "trace", f, a...); }
template <class... A>
void debug(const std::string& f, const A&... a) { detail::log(level::debug, "debug", f, a...); }
template <class... A>
void info(const std::string& f, const A&... a) { detail::log(level::info, "info", f, a...); }
template <class... A>
void warn(const std::string& f, const A&... a) { detail::log(level::warn, "warn", f, a...); }
template <class... A>
void error(const std::string& f, const A&... a) { detail::log(level::err, "error", f, a...); }
template <class... A>
void critical(const std::string& f, const A&... a) { detail::log(level::critical, "critical", f, a...); }
inline void set_level(level::level_enum l) { detail::threshold() = (int)l; }

}  // namespace spdlog

#endif
