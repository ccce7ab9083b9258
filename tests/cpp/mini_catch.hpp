// mini_catch.hpp -- the few Catch2 constructs MAST's own tests use (TEST_CASE
// with tags, REQUIRE, CHECK, Approx, REQUIRE_THROWS), so that tests of the C++
// mirror read like the reference's tests.  Run: ./binary [tag-filter].
#pragma once
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace mini_catch {
struct Case {
    const char *name, *tags;
    std::function<void()> fn;
};
inline std::vector<Case> &registry() {
    static std::vector<Case> r;
    return r;
}
struct Reg {
    Reg(const char *n, const char *t, std::function<void()> f) { registry().push_back({n, t, f}); }
};
struct Failure : std::runtime_error {
    using std::runtime_error::runtime_error;
};
inline int &failures() {
    static int f = 0;
    return f;
}
struct Approx {
    explicit Approx(double v) : v(v) {}
    Approx &epsilon(double e) { eps = e; return *this; }
    Approx &margin(double m) { mar = m; return *this; }
    double v, eps = 1e-12, mar = 0.0;
};
inline bool operator==(double a, const Approx &b) {
    return std::fabs(a - b.v) <= b.mar + b.eps * std::max(std::fabs(a), std::fabs(b.v));
}
inline bool operator==(const Approx &b, double a) { return a == b; }
inline std::string where(const char *f, int l, const char *e) {
    std::ostringstream s;
    s << f << ":" << l << ": " << e;
    return s.str();
}
}  // namespace mini_catch

#define MC_CAT2(a, b) a##b
#define MC_CAT(a, b) MC_CAT2(a, b)
#define TEST_CASE(name, tags)                                                              \
    static void MC_CAT(mc_test_, __LINE__)();                                              \
    static mini_catch::Reg MC_CAT(mc_reg_, __LINE__)(name, tags, &MC_CAT(mc_test_, __LINE__)); \
    static void MC_CAT(mc_test_, __LINE__)()
#define REQUIRE(expr)                                                                     \
    do {                                                                                  \
        if (!(expr)) throw mini_catch::Failure(mini_catch::where(__FILE__, __LINE__, #expr)); \
    } while (0)
#define CHECK(expr)                                                                       \
    do {                                                                                  \
        if (!(expr)) {                                                                    \
            std::fprintf(stderr, "  CHECK failed %s\n", mini_catch::where(__FILE__, __LINE__, #expr).c_str()); \
            mini_catch::failures()++;                                                     \
        }                                                                                 \
    } while (0)
#define REQUIRE_THROWS(expr)                                                              \
    do {                                                                                  \
        bool thrown_ = false;                                                             \
        try { (void)(expr); } catch (...) { thrown_ = true; }                             \
        if (!thrown_) throw mini_catch::Failure(mini_catch::where(__FILE__, __LINE__, "no throw: " #expr)); \
    } while (0)
using mini_catch::Approx;

#define MINI_CATCH_MAIN                                                                   \
    int main(int argc, char **argv) {                                                     \
        const char *filt = argc > 1 ? argv[1] : "";                                        \
        int run = 0, bad = 0;                                                             \
        for (auto &c : mini_catch::registry()) {                                          \
            if (*filt && !std::strstr(c.tags, filt)) continue;                             \
            run++;                                                                        \
            const int f0 = mini_catch::failures();                                        \
            try { c.fn(); } catch (const std::exception &e) {                             \
                std::fprintf(stderr, "FAILED %s: %s\n", c.name, e.what());                  \
                bad++;                                                                    \
                continue;                                                                 \
            }                                                                             \
            if (mini_catch::failures() != f0) { bad++; std::fprintf(stderr, "FAILED %s\n", c.name); } \
            else std::printf("passed %s\n", c.name);                                      \
        }                                                                                 \
        std::printf("%d test cases, %d failed\n", run, bad);                              \
        return bad ? 1 : 0;                                                               \
    }
