// CPU check of the product's modular primitives (grns_gb300/csrc/rns_common.cuh
// compiled for the host): Shoup and Barrett multiplication and the branch-free
// add/sub against exact 64-bit arithmetic.  Built and driven by tests/test_host_arith.py.
#include <cstdint>
#include "../../grns_gb300/csrc/rns_common.cuh"

static uint64_t sm(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

extern "C" long check_modular(uint32_t m, long trials, uint64_t seed) {
    uint32_t b = 0;
    for (uint32_t v = m; v; v >>= 1) b++;
    uint32_t mu = (uint32_t)(((unsigned __int128)1 << (2 * b)) / m);
    long bad = 0;
    uint64_t s = seed;
    for (long t = 0; t < trials; t++) {
        uint32_t x, y;
        if (t < 16) { x = (t & 1) ? m - 1 : (uint32_t)t % m; y = (t & 2) ? m - 1 : (uint32_t)(t / 4) % m; }
        else { x = (uint32_t)(sm(s) % m); y = (uint32_t)(sm(s) % m); }
        uint32_t ysh = (uint32_t)(((uint64_t)y << 32) / m);
        uint32_t want = (uint32_t)(((uint64_t)x * y) % m);
        if (grns::mulmod_barrett(x, y, m, mu, b) != want) bad++;
        if (grns::mulmod_shoup(x, y, ysh, m) != want) bad++;
        if (grns::addmod(x, y, m) != (uint32_t)(((uint64_t)x + y) % m)) bad++;
        if (grns::submod(x, y, m) != (uint32_t)(((uint64_t)x + m - y) % m)) bad++;
    }
    return bad;
}

extern "C" int check_er(double x, long expect_exp, double expect_frac) {
    grns::Er e = grns::er_from_double(x);
    return e.exp == expect_exp && e.frac == expect_frac;
}
