// Host-side check of the multiply-high division used by the cell id decodes
// (FDiv / fdiv in dmtz_common.cuh): exact quotients against the hardware
// division for divisors from 1 to 2^44 and dividends across the 64-bit range.
#include <cstdio>
#include <random>

#include "../../dmtz_gb300/csrc/dmtz_common.cuh"

using namespace dmtz;

int main() {
    std::mt19937_64 rng(12345);
    long long bad = 0, n_tests = 0;
    const unsigned long long ds[] = {1, 2, 3, 5, 7, 255, 256, 1023, 1024, 1025, 16383, 16384,
                                     8191ull * 4095ull, 16383ull * 8192ull, 1ull << 31, (1ull << 32) - 1, 1ull << 40};
    for (unsigned long long d : ds) {
        const FDiv f = make_fdiv(d);
        for (int i = 0; i < 100000; i++) {
            unsigned long long n = rng();
            if (i % 4 == 1) n >>= (rng() % 64);
            if (i % 4 == 2) n = (rng() % 1000) * d + (rng() % d);
            if (i % 4 == 3) n = ~0ull - (rng() % 1000);
            n_tests++;
            if (fdiv(f, n) != n / d) {
                if (bad < 5) printf("d=%llu n=%llu: %llu, want %llu\n", d, n, fdiv(f, n), n / d);
                bad++;
            }
        }
    }
    for (int i = 0; i < 100000; i++) {
        const unsigned long long d = 1 + rng() % (1ull << 44), n = rng() >> (rng() % 20);
        n_tests++;
        if (fdiv(make_fdiv(d), n) != n / d) bad++;
    }
    printf("%lld checks, %lld wrong\n", n_tests, bad);
    return bad != 0;
}
