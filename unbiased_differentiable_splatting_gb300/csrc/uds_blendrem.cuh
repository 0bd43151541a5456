// The front-to-back blend's remaining transmittance (alphacompositing.cuh:
// 58-68): rem' = (float)((double)rem * (1.0 - (double)w)), without the FP64
// pipe.
//
// With w = mw 2^-k (mw the 24-bit significand, k = 150 - biased exponent) and
// 2^-30 <= w < 1, 1 - w = (2^k - mw) 2^-k has at most k <= 53 significant
// bits, so the double subtraction is exact.  The double product then rounds
// the exact product rem (1 - w) = mr (2^k - mw) 2^(er - k) (mr the 24-bit
// significand of rem) to 53 bits, and the conversion rounds that to 24 bits.
// Both roundings are done here on the exact integer product (at most 77
// bits), each to nearest with ties to even, so the result is the double
// sequence's bit for bit; there is no shortcut through one rounding, because
// 1 - w is not a float.  Inputs outside this path (w < 2^-30, w >= 1 other
// than exactly 1, rem not a normal float in [2^-100, 2^100], non-finite
// values) return false and the caller uses the double arithmetic; w == 0 and
// w == 1 (with rem >= 0) are exact shortcuts.  The header also compiles as
// host C++ so the CPU tests can compare it with the double formula.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define UDS_BR_FN __host__ __device__ __forceinline__
#else
#define UDS_BR_FN static inline
#endif

namespace uds {

UDS_BR_FN uint32_t br_bits(float x) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

UDS_BR_FN float br_float(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

UDS_BR_FN int br_bitlen64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return 64 - __clzll((long long)x);
#else
    return x ? 64 - __builtin_clzll(x) : 0;
#endif
}

// q >> s rounded to nearest, ties to even (1 <= s <= 63)
UDS_BR_FN uint64_t br_round_shift(uint64_t q, int s) {
    uint64_t kept = q >> s, low = q & ((1ull << s) - 1ull), half = 1ull << (s - 1);
    if (low > half || (low == half && (kept & 1ull))) ++kept;
    return kept;
}

// rem' = (float)((double)rem * (1.0 - (double)w)) when the inputs are on the
// exact path (true), else false (out untouched).
UDS_BR_FN bool blend_rem(float rem, float w, float* out) {
    uint32_t uw = br_bits(w), ur = br_bits(rem);
    if (uw == 0u) {  // w == +0: rem * 1
        *out = rem;
        return true;
    }
    if (uw == 0x3f800000u) {  // w == 1: rem * 0
        if (!(ur <= 0x7f800000u)) return false;  // negative rem, or NaN: leave to the double code
        *out = 0.0f;
        return true;
    }
    int ewf = (int)((uw >> 23) & 0xffu), erf = (int)((ur >> 23) & 0xffu);
    // 2^-30 <= w < 1 (sign 0, biased exponent 97 .. 126)
    if ((uw >> 31) || ewf < 97 || ewf > 126) return false;
    if (ur == 0u) {  // rem == +0
        *out = 0.0f;
        return true;
    }
    // rem a positive normal float in [2^-100, 2^100]
    if ((ur >> 31) || erf < 27 || erf > 227) return false;
    int k = 150 - ewf;  // 24 .. 53
    uint64_t mw = (uint64_t)((uw & 0x7fffffu) | 0x800000u);
    uint64_t mr = (uint64_t)((ur & 0x7fffffu) | 0x800000u);
    uint64_t a = (1ull << k) - mw;  // 1 - w = a 2^-k, exactly; a < 2^53
    // exact product P = mr a < 2^77 as hi:lo, with a = ah 2^32 + al
    uint64_t al = a & 0xffffffffull, ah = a >> 32;
    uint64_t lo_part = mr * al;  // < 2^56
    uint64_t mid = mr * ah;      // < 2^45
    uint64_t lo = lo_part + (mid << 32);
    uint64_t hi = (mid >> 32) + (lo < lo_part ? 1ull : 0ull);
    // exponent of the product's unit: 2^(erf - 150 - k)
    int e = erf - 150 - k;
    // round P to 53 significant bits (the double multiplication)
    int nb = hi ? 64 + br_bitlen64(hi) : br_bitlen64(lo);
    uint64_t q;
    if (nb > 53) {
        int s = nb - 53;  // 1 .. 24: the dropped bits straddle lo and hi
        uint64_t kept = (hi << (64 - s)) | (lo >> s);
        uint64_t low = lo & ((1ull << s) - 1ull), half = 1ull << (s - 1);
        if (low > half || (low == half && (kept & 1ull))) ++kept;
        if (kept >> 53) {
            kept >>= 1;
            ++s;
        }
        q = kept;
        e += s;
    } else {
        q = lo;  // at most 53 bits: exact
    }
    // round the double to 24 significant bits (the conversion to float)
    int nb2 = br_bitlen64(q);  // >= 24: mr >= 2^23 and a >= 1
    uint64_t m = q;
    if (nb2 > 24) {
        int s2 = nb2 - 24;
        m = br_round_shift(q, s2);
        e += s2;
        if (m >> 24) {
            m >>= 1;
            ++e;
        }
    }
    int field = e + 23 + 127;  // m in [2^23, 2^24): value m 2^e
    if (field < 1 || field > 254) return false;
    *out = br_float(((uint32_t)field << 23) | ((uint32_t)m & 0x7fffffu));
    return true;
}

}  // namespace uds
