// scaled_floor (gpvmc_gb300/csrc/device.cuh) against the double product
// floor(double(n) * u) it replaces, for every lattice size on the path and
// many random and edge-case 52-bit mantissas.
#include <cstdio>
#include <random>

#include "device.cuh"

int main()
{
    std::mt19937_64 rng(12345);
    long bad = 0, checked = 0;
    for (int L = 2; L <= 30; L += 2) {
        const uint32_t n = uint32_t(L) * L;
        for (int i = 0; i < 2000000; ++i) {
            uint64_t m = rng() & ((uint64_t(1) << 52) - 1);
            if (i < 64) m = (uint64_t(1) << 52) - 1 - uint64_t(i);   // largest uniforms
            else if (i < 128) m = uint64_t(i - 64);                  // smallest uniforms
            else if (i < 20000) {                                    // near k/n boundaries
                const uint64_t k = rng() % n;
                const long double t = (long double)k / n * 4503599627370496.0L;
                m = uint64_t(t) + (rng() % 5) - 2;
                m &= (uint64_t(1) << 52) - 1;
            }
            const double u = (double(m) + 0.5) * (1.0 / 4503599627370496.0);
            const int want = int(double(n) * u);
            const int got = gv::scaled_floor(n, m);
            ++checked;
            if (got != want) {
                if (bad < 5) std::printf("n=%u m=%llu want %d got %d\n", n, (unsigned long long)m, want, got);
                ++bad;
            }
        }
    }
    std::printf("checked %ld mismatches %ld\n", checked, bad);
    return bad ? 1 : 0;
}
