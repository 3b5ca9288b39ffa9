// Host check of the integer-pipe binary64 additions and multiply
// (fortran-to-cuda_gb300/csrc/kernels/soft_fp64.cuh) against the host's IEEE
// double arithmetic, which rounds to nearest-even. The header is compiled as
// host C++: the device intrinsics it calls are given their host meaning here,
// and an empty cuda_runtime.h comes first on the include path.
// Usage: soft_fp64_host <pairs per distribution>; prints one JSON line per
// (operation, distribution); exit status 1 on any mismatch.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>

#define __device__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
using std::min;
static inline long long __double_as_longlong(double d) { long long x; std::memcpy(&x, &d, 8); return x; }
static inline double __longlong_as_double(long long x) { double d; std::memcpy(&d, &x, 8); return d; }
static inline double __dadd_rn(double a, double b) { volatile double r = a + b; return r; }
static inline double __dmul_rn(double a, double b) { volatile double r = a * b; return r; }
static inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll((unsigned long long)x); }

#include "soft_fp64.cuh"
#include "cases.h"

int main(int argc, char **argv) {
    const uint64_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1000000;
    int failed = 0;
    for (int op = 0; op < 3; ++op)
        for (int dist = 0; dist < 7; ++dist) {
            uint64_t bad = 0, first_a = 0, first_b = 0;
            const uint64_t seed = 0x5eed0000ull + 131 * (uint64_t)dist + (uint64_t)op;
            for (uint64_t i = 0; i < n; ++i) {
                uint64_t ia, ib;
                soft_cases::pair(dist, seed, i, &ia, &ib);
                const double a = __longlong_as_double((long long)ia), b = __longlong_as_double((long long)ib);
                const double got = op == 0 ? f2c::add_rn_int(a, b) : op == 1 ? f2c::mul_rn_int(a, b) : f2c::add_rn_near(a, b);
                const double want = op == 1 ? __dmul_rn(a, b) : __dadd_rn(a, b);
                const bool both_nan = got != got && want != want;
                if (!both_nan && __double_as_longlong(got) != __double_as_longlong(want)) {
                    if (bad++ == 0) { first_a = ia; first_b = ib; }
                }
            }
            std::printf("{\"op\": \"%s\", \"dist\": %d, \"pairs\": %llu, \"mismatches\": %llu, \"first\": [\"%016llx\", \"%016llx\"]}\n",
                        op == 0 ? "add" : op == 1 ? "mul" : "add_near", dist, (unsigned long long)n, (unsigned long long)bad,
                        (unsigned long long)first_a, (unsigned long long)first_b);
            failed |= bad != 0;
        }
    return failed;
}
