// Compares the integer back-projection quotient (uds_backproject.cuh) with
// the double formula it replaces, bit for bit, on random and edge-case
// inputs, and checks the single-operation rule the kernels' *_via_double
// helpers rely on ((float)(a op b in double) == a op b in float for
// + - * /).  Built and run by test_backproject.py (g++ -ffp-contract=off).
// Prints "<quotient cases> <integer-path cases> <single-op cases> <mismatches>".
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "uds_backproject.cuh"

static float reference(float W, float s, float f) {
    // transformation.cuh backproject: (W - 2 s) / (2 f) in double, then float
    volatile double num = (double)W - 2.0 * (double)s;
    volatile double den = 2.0 * (double)f;
    return (float)(num / den);
}

static uint32_t bits(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
}

int main(int argc, char** argv) {
    long n = argc > 1 ? std::atol(argv[1]) : 2000000;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    long cases = 0, fast = 0, ops = 0, bad = 0;
    auto check = [&](float W, float s, float f) {
        ++cases;
        float got;
        if (!uds::bp_quotient(0.5f * W, s, f, &got)) return;
        ++fast;
        float want = reference(W, s, f);
        if (bits(got) != bits(want)) {
            if (bad < 10) std::printf("mismatch W=%a s=%a f=%a got=%a want=%a\n", W, s, f, got, want);
            ++bad;
        }
    };
    for (long i = 0; i < n; ++i) {
        float W = (float)(1 + (rng() % 4096));
        float f = (float)(1.0 + 5000.0 * U(rng));
        if (rng() % 8 == 0) {  // any positive normal focal length
            uint32_t b = (uint32_t)(rng() % 0x7f000000u) + 0x00800000u;
            std::memcpy(&f, &b, 4);
        }
        int kind = (int)(rng() % 10);
        float s;
        double u = U(rng);
        switch (kind) {
            case 0: s = (float)(-W + 3.0 * W * u); break;             // on and around the screen
            case 1: s = (float)(u * W); break;
            case 2: s = (float)(0.5 * W + (u - 0.5) * 1e-3); break;    // near the centre
            case 3: s = (float)((u - 0.5) * 1e-6); break;              // near zero
            case 4: s = (float)(std::floor(u * W) + 0.5); break;       // pixel centres
            case 5: s = (float)std::floor(u * 2 * W); break;           // integers
            case 6: s = (float)((u - 0.5) * 1e8); break;               // far off screen
            case 7: {                                                  // random finite bit patterns
                uint32_t b = (uint32_t)rng();
                std::memcpy(&s, &b, 4);
                if (!std::isfinite(s)) s = 1.0f;
                break;
            }
            case 8: s = std::nextafterf(0.5f * W, (u < 0.5) ? 0.0f : 1e9f); break;
            default: s = (float)(0.5 * W + (u - 0.5) * W * 1e-7); break;
        }
        check(W, s, f);
        check(W, s + 1.0f, f);  // the second back-projected point
    }
    // exhaustive small grid: pixel-ish coordinates and focal lengths
    for (int Wi = 1; Wi <= 64; ++Wi)
        for (int si = -128; si <= 256; ++si)
            for (float f : {1.0f, 3.0f, 7.0f, 100.0f, 525.0f, 1111.1f})
                check((float)Wi, (float)si * 0.25f, f);
    // the single-operation rule behind div_via_double / add_via_double /
    // sub_via_double: (float)(a op b in double) == a op b in float
    auto rnd_float = [&]() {
        uint32_t b = (uint32_t)rng();
        float x;
        std::memcpy(&x, &b, 4);
        return x;
    };
    for (long i = 0; i < n; ++i) {
        float a = rnd_float(), b = (i & 1) ? rnd_float() : (float)(U(rng) * 2.0 - 0.5);
        if (i % 3 == 0) a = 1.0f;  // the reference's 1.0 / x and x + 1.0
        if (!std::isfinite(a) || !std::isfinite(b)) continue;
        volatile double da = a, db = b;
        float pairs[4][2] = {{(float)(da / db), a / b}, {(float)(da + db), a + b},
                             {(float)(da - db), a - b}, {(float)(da * db), a * b}};
        for (auto& p : pairs) {
            ++ops;
            if (!(std::isnan(p[0]) && std::isnan(p[1])) && bits(p[0]) != bits(p[1])) {
                if (bad < 10) std::printf("single-op mismatch a=%a b=%a\n", a, b);
                ++bad;
            }
        }
    }
    std::printf("%ld %ld %ld %ld\n", cases, fast, ops, bad);
    return bad != 0;
}
