// digit_sum.cuh -- the running sum of gdn_integer_to_float
// (qmctoolscl/c_funcs/gdn_integer_to_float.c:33-39):
//
//     v = 0; for t: v = RN(v + RN(recip_t * digit_t))
//
// where the terms RN(recip_t * digit_t) come from a table, and the adds run in
// integer arithmetic, bit for bit.  The sum is kept unpacked between digits
// -- significand M with its leading one at bit 52 and biased exponent E -- so
// one add is an aligned integer add with its rounding, with no packing and
// unpacking of doubles in between.  Adds that do not fit that fast form (the
// first nonzero term, a carry into the next binade, subnormals) are left to
// the caller's exact fallback.
//
// Host-compilable (g++) so the CPU tests can check it against the host's
// IEEE arithmetic.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define DS_HD __host__ __device__ __forceinline__
#else
#define DS_HD inline
#endif

namespace dsum {

typedef unsigned long long u64;
typedef unsigned int u32;

constexpr u64 FRAC = 0xFFFFFFFFFFFFFull;
constexpr u64 HIDDEN = 1ull << 52;

struct Sum {
    u64 M;  // significand with the leading one at bit 52; 0 for v = 0, the raw fraction for subnormal v
    u32 E;  // biased exponent (0 for zero and subnormal v)
};

DS_HD Sum unpack(u64 bits)
{
    Sum v;
    v.E = (u32)(bits >> 52);
    v.M = v.E ? ((bits & FRAC) | HIDDEN) : bits;
    return v;
}

DS_HD u64 pack(const Sum &v) { return v.E ? ((u64)v.E << 52) | (v.M & FRAC) : v.M; }

// v = RN(v + y) for y the bits of a non-negative double, in the fast form:
// v and y normal, y at least one binade below v, and the rounded sum staying
// in v's binade.  Returns false, with v unchanged, when the form does not
// apply (v or y zero or subnormal, y comparable to v, a carry into the next
// binade); the caller then adds exactly by other means.
DS_HD bool add_fast(Sum &v, u64 y)
{
    const u32 ey = (u32)(y >> 52);
    if (!(v.M >> 52) || !ey) return false;
    // y = my * 2^(ey - 1075), v = M * 2^(E - 1075): k2 bits of my fall below v's last place
    const int k2 = (int)v.E - (int)ey;
    if (k2 >= 55) return true;  // y < 2^53 * ulp(v) / 2^55: RN(v + y) = v
    if (k2 < 1) return false;
    const u64 my = (y & FRAC) | HIDDEN;
    const u64 q = my >> k2;
    const u64 rem2 = my << (64 - k2);  // the dropped bits, left-aligned
    u64 m = v.M + q;
    m += (u64)((rem2 > (1ull << 63)) | ((rem2 == (1ull << 63)) & (m & 1ull)));  // nearest, ties to even
    if (m >> 53) return false;  // reached the next binade, whose grid is twice as coarse
    v.M = m;
    return true;
}

// Bits of RN(r * (double)m) for r the bits of a positive normal double and
// 0 < m < 2^11, in integer arithmetic: the 64-bit product of the significand
// and m, normalised, rounded to 53 bits (nearest, ties to even).  The
// result stays normal and finite for r in [2^-1000, 2^1000).
DS_HD u64 mul_small(u64 r, u32 m)
{
    const u64 P = ((r & FRAC) | HIDDEN) * (u64)m;  // below 2^64, at least 2^52
    u32 lz;
#ifdef __CUDA_ARCH__
    lz = (u32)__clzll((long long)P);
#else
    lz = (u32)__builtin_clzll(P);
#endif
    const u64 Pn = P << lz;                   // leading one at bit 63
    const u64 mant = Pn >> 11, rem = Pn & 0x7FFull;
    const u64 up = (u64)((rem > 0x400ull) | ((rem == 0x400ull) & (mant & 1ull)));
    // value = mant * 2^(E - 1075) with E = Er + 11 - lz; the hidden bit of mant adds one to the
    // exponent field, and a round-up to 2^53 carries into it
    return ((r >> 52) + 10u - lz) * HIDDEN + mant + up;
}

}  // namespace dsum
