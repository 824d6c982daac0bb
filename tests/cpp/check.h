// Minimal assertion helpers for the C++ test programs (they keep going after
// a failure and report the count in the exit status).
#pragma once
#include <cmath>
#include <cstdio>

static int g_failures = 0;
static int g_checks = 0;

#define CHECK(cond)                                                                   \
    do {                                                                              \
        ++g_checks;                                                                   \
        if (!(cond)) {                                                                \
            ++g_failures;                                                             \
            std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);    \
        }                                                                             \
    } while (0)

#define CHECK_THROWS(expr, Exc)                                                       \
    do {                                                                              \
        ++g_checks;                                                                   \
        bool thrown__ = false;                                                        \
        try { expr; } catch (const Exc&) { thrown__ = true; } catch (...) {}          \
        if (!thrown__) {                                                              \
            ++g_failures;                                                             \
            std::fprintf(stderr, "FAILED %s:%d: %s did not throw %s\n", __FILE__,     \
                         __LINE__, #expr, #Exc);                                      \
        }                                                                             \
    } while (0)

// relative comparison of the reference's test/tests.cpp:19-27
inline bool fequal(float a, float b, float diff) {
    return std::fabs(a - b) <= ((std::fabs(a) < std::fabs(b) ? std::fabs(b) : std::fabs(a)) * diff);
}

inline int finish(const char* name) {
    std::printf("%s: %d checks, %d failures\n", name, g_checks, g_failures);
    return g_failures == 0 ? 0 : 1;
}
