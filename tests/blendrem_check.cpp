// Host check of csrc/uds_blendrem.cuh against the double formula it replaces,
// (float)((double)rem * (1.0 - (double)w)), bit for bit.  Prints the number of
// (rem, w) pairs checked, how many took the integer path, and mismatches.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "uds_blendrem.cuh"

static unsigned long long s_state = 0x9e3779b97f4a7c15ull;
static unsigned long long next64() {
    s_state ^= s_state << 13;
    s_state ^= s_state >> 7;
    s_state ^= s_state << 17;
    return s_state;
}
static float from_bits(unsigned u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
static unsigned to_bits(float f) {
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
}
static float uniform01() { return (float)((next64() >> 40) * 0x1p-24); }
// float bits uniform over [lo, hi] bit patterns (log-uniform-ish)
static float bit_uniform(float lo, float hi) {
    unsigned a = to_bits(lo), b = to_bits(hi);
    return from_bits(a + (unsigned)(next64() % (unsigned long long)(b - a + 1u)));
}

static long long cases = 0, fast = 0, bad = 0;
static void check(float r, float w) {
    ++cases;
    float ref = (float)((double)r * (1.0 - (double)w));
    float got;
    if (uds::blend_rem(r, w, &got)) {
        ++fast;
        if (to_bits(got) != to_bits(ref)) {
            if (bad < 10) std::printf("mismatch rem=%a w=%a got=%a ref=%a\n", r, w, got, ref);
            ++bad;
        }
    }
}

int main(int argc, char** argv) {
    long long n = argc > 1 ? std::atoll(argv[1]) : 1000000;
    const float edges_w[] = {0.0f, 1.0f, 0.5f, 0x1p-30f, 0x1.fffffep-31f, 0x1p-24f, 0x1.fffffep-1f, 0x1.fffffcp-1f,
                             0.25f, 0.75f, 0x1.000002p-1f, 0x1p-53f, 1e-38f, 1e-45f, 0x1.000002p+0f};
    const float edges_r[] = {1.0f, 0.0f, 0.5f, 0x1p-100f, 0x1.fffffep-101f, 0x1p-126f, 0x1.fffffep-1f, 0x1p-24f,
                             0.3f, 0x1p+100f, 1e-40f};
    for (float r : edges_r)
        for (float w : edges_w) check(r, w);
    for (long long i = 0; i < n; ++i) {
        check(uniform01(), uniform01());                                  // typical weights
        check(bit_uniform(0x1p-110f, 1.0f), bit_uniform(0x1p-40f, 1.0f));  // wide exponents
        check(uniform01(), from_bits(0x3f800000u - 1u - (unsigned)(next64() % 4096u)));  // w just below 1
        float r = uniform01(), w = uniform01();
        // products near rounding boundaries: w with few significant bits
        w = std::ldexp(std::floor(std::ldexp(w, 12)), -12);
        check(r, w);
    }
    std::printf("%lld %lld %lld\n", cases, fast, bad);
    return bad ? 1 : 0;
}
