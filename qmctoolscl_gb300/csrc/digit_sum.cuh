// digit_sum.cuh -- the running sum of gdn_integer_to_float
// (qmctoolscl/c_funcs/gdn_integer_to_float.c:33-39):
//
//     v = 0; for t: v = RN(v + RN(recip_t * digit_t))
//
// in integer arithmetic, bit for bit.  The sum is kept unpacked between
// digits -- significand M with its leading one at bit 52 and biased exponent
// E -- so one term costs a 53x11-bit product, one rounding of it to 53 bits
// and one aligned add with its rounding, with no packing and unpacking of
// doubles in between.  Terms that do not fit that fast form (the first
// nonzero term, a carry into the next binade, subnormals, digits of 2^11 or
// more) go through the general exact routine.
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

DS_HD u32 clz32(u32 x)
{
#ifdef __CUDA_ARCH__
    return (u32)__clz((int)x);
#else
    return x ? (u32)__builtin_clz(x) : 32u;
#endif
}

DS_HD u32 clz64(u64 x)
{
#ifdef __CUDA_ARCH__
    return (u32)__clzll((long long)x);
#else
    return x ? (u32)__builtin_clzll(x) : 64u;
#endif
}

constexpr u64 FRAC = 0xFFFFFFFFFFFFFull;
constexpr u64 HIDDEN = 1ull << 52;

// RN(a + b) for finite non-negative normal-or-zero doubles given as bits with
// a + b < 2^1023: mantissas at bit 62 with ten guard bits and a sticky bit.
DS_HD u64 add_bits(u64 a, u64 b)
{
    if (a < b) { const u64 t = a; a = b; b = t; }
    if (b == 0) return a;
    const u32 ea = (u32)(a >> 52), eb = (u32)(b >> 52);
    const u64 ma = ((a & FRAC) | HIDDEN) << 10;
    u64 mb = ((b & FRAC) | HIDDEN) << 10;
    const u32 dlt = ea - eb;
    if (dlt) {
        if (dlt >= 64) {
            mb = 1;
        } else {
            const u64 lost = mb & ((1ull << dlt) - 1);
            mb = (mb >> dlt) | (lost != 0);
        }
    }
    u64 s = ma + mb;
    u32 e = ea;
    if (s >> 63) {
        s = (s >> 1) | (s & 1);
        e += 1;
    }
    u64 m = s >> 10;
    const u64 rem = s & 0x3FFull;
    m += (rem > 0x200ull) | ((rem == 0x200ull) & (m & 1ull));
    return ((u64)(e - 1) << 52) + m;
}

// RN(r * s) for a positive normal double r (bits) and 1 <= s < 2^11
DS_HD u64 mul_bits(u64 r, u32 s)
{
    const u64 mr = (r & FRAC) | HIDDEN;
    const u64 p = mr * (u64)s;
    const u32 lz = clz64(p);
    const u64 N = p << lz;
    u64 m = N >> 11;
    const u64 rem = N & 0x7FFull;
    m += (rem > 0x400ull) | ((rem == 0x400ull) & (m & 1ull));
    const u32 er = (u32)(r >> 52);
    return ((u64)(er + 10 - lz) << 52) + m;
}

// true when the general integer routine (add_bits(v, mul_bits(r, s))) is exact
// for these operands; otherwise the caller uses the hardware double operations
DS_HD bool general_ok(u64 vbits, u64 rbits, u32 s)
{
    const u32 er = (u32)(rbits >> 52);
    return s < 2048 && er >= 1 && er < 2036 && (vbits >> 52) < 2000;
}

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

// v = RN(v + RN(r * s)) in the fast form: r = mr * 2^(er - 1075) normal (mr
// with its leading one at bit 52, er its biased exponent), 1 <= s < 2^11, v
// normal, and the rounded sum staying in v's binade.  Returns false, with v
// unchanged, when the fast form does not apply.
DS_HD bool add_term_fast(Sum &v, u64 mr, u32 er, u32 s)
{
    // RN(r * s): the exact product p = mr * s has 64 - clz(p) bits; drop the
    // k1 = 11 - clz(p) below the top 53 to nearest, ties to even
    const u64 p = mr * (u64)s;
    const u32 k1 = 11u - clz32((u32)(p >> 32));  // p >= 2^52, so p_hi >= 2^20 and k1 <= 11
    u64 my = p;
    if (k1) {
        const u32 half = 1u << (k1 - 1);
        const u32 rem = (u32)p & ((half << 1) - 1u);
        my = p >> k1;
        my += (u64)((rem > half) | ((rem == half) & ((u32)my & 1u)));
    }
    // y = my * 2^(er - 1075 + k1), v = M * 2^(E - 1075): k2 bits of my fall
    // below v's last place (my may be 2^53 after rounding: still exact here)
    const int k2 = (int)v.E - (int)er - (int)k1;
    if (k2 <= 0) return false;
    if (k2 >= 64) return true;  // y < ulp(v)/2^10: RN(v + y) = v
    const u64 q = my >> k2;
    const u64 rem2 = my << (64 - k2);
    u64 m = v.M + q;
    m += (u64)((rem2 > (1ull << 63)) | ((rem2 == (1ull << 63)) & (m & 1ull)));
    if (m >> 53) return false;  // reached the next binade, whose grid is twice as coarse
    v.M = m;
    return true;
}

}  // namespace dsum
