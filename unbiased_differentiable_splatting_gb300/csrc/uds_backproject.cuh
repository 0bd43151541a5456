// backproject's division (transformation.cuh: x = (W - 2 s) / (2 f) in
// double, rounded to float) without the FP64 pipe.
//
// With A = W / 2 the value is RN_f(RN_d(RN_d(A - s) / f)) (halving numerator
// and denominator is exact).  When the exact numerator N = A - s spans at most
// 50 significant bits it is a double, and no float rounding midpoint lies
// within half a double ulp of the quotient N / f unless the quotient is that
// midpoint (|N / f - m| >= 2^(E - 50) for a quotient in [2^E, 2^(E+1))), so
// the double rounding is innocuous and the result is the correctly rounded
// float quotient RN_f(N / f).  That quotient is computed here exactly with
// 64-bit integers: N as an integer times a power of two, a 64-by-24-bit
// division for 24 significant bits, a round bit and a sticky remainder, and
// round-to-nearest-even.  Inputs outside this path (non-finite or subnormal
// operands, f <= 0, both operands zero, a numerator wider than 50 bits, a
// result outside the normal float range) return false and the caller uses
// the double arithmetic.  The header also compiles as host C++ so the CPU
// tests can compare it with the double formula.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define UDS_BP_FN __host__ __device__ __forceinline__
#else
#define UDS_BP_FN static inline
#endif

namespace uds {

UDS_BP_FN int bp_bitlen64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return 64 - __clzll((long long)x);
#else
    return x ? 64 - __builtin_clzll(x) : 0;
#endif
}

UDS_BP_FN int bp_ctz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __ffsll((long long)x) - 1;
#else
    return __builtin_ctzll(x);
#endif
}

UDS_BP_FN uint32_t bp_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

UDS_BP_FN float bp_float(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

// RN_f((a - s) / f) for float a, s and f > 0, exactly; false outside the
// fast path described above.
UDS_BP_FN bool bp_quotient(float a, float s, float f, float* out) {
    uint32_t ua = bp_bits(a), us = bp_bits(s), uf = bp_bits(f);
    int ea = (int)((ua >> 23) & 0xffu), es = (int)((us >> 23) & 0xffu), ef = (int)((uf >> 23) & 0xffu);
    uint32_t fa = ua & 0x7fffffu, fs = us & 0x7fffffu;
    if (ea == 255 || es == 255 || ef == 0 || ef == 255 || (uf >> 31)) return false;
    if ((ea == 0 && fa) || (es == 0 && fs)) return false;  // subnormal operand
    if (ea == 0 && es == 0) return false;                    // both zero: signed-zero rules
    // a = ma 2^(ea - 150), s = ms 2^(es - 150) (a zero takes the other's scale)
    int64_t ma = ea ? (int64_t)(fa | 0x800000u) : 0, ms = es ? (int64_t)(fs | 0x800000u) : 0;
    if (ua >> 31) ma = -ma;
    if (us >> 31) ms = -ms;
    if (!ea) ea = es;
    if (!es) es = ea;
    int e0 = ea < es ? ea : es;
    int da = ea - e0, ds = es - e0;
    if (da > 38 || ds > 38) return false;  // the numerator would not fit 63 bits
    int64_t N = ma * ((int64_t)1 << da) - ms * ((int64_t)1 << ds);
    if (N == 0) {  // a == s: the difference is +0, and so is the quotient
        *out = 0.0f;
        return true;
    }
    bool neg = N < 0;
    uint64_t n = neg ? (uint64_t)(-N) : (uint64_t)N;
    int tz = bp_ctz64(n);
    n >>= tz;
    e0 += tz;  // N = n 2^(e0 - 150)
    int nb = bp_bitlen64(n);
    if (nb > 50) return false;
    // N / f = (n / mf) 2^(e0 - ef); X = n 2^k has its top bit at 2^62
    uint64_t mf = (uint64_t)((uf & 0x7fffffu) | 0x800000u);
    int k = 63 - nb;
    uint64_t X = n << k;
    uint64_t q = X / mf, r = X % mf;  // 39 or 40 bits
    int sh = bp_bitlen64(q) - 25;      // keep 24 bits and the round bit
    bool sticky = r != 0 || (q & (((uint64_t)1 << sh) - 1)) != 0;
    uint64_t q25 = q >> sh;
    uint32_t m = (uint32_t)(q25 >> 1);
    int E = e0 - ef - k + sh + 1;  // N / f ~ m 2^E, m in [2^23, 2^24)
    if ((q25 & 1u) && (sticky || (m & 1u))) {
        ++m;
        if (m == (1u << 24)) {
            m >>= 1;
            ++E;
        }
    }
    int biased = E + 150;
    if (biased <= 0 || biased >= 255) return false;  // subnormal or overflowing result
    *out = bp_float(((uint32_t)neg << 31) | ((uint32_t)biased << 23) | (m & 0x7fffffu));
    return true;
}

}  // namespace uds
