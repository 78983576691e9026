// qrng_step.cuh -- one Horner step of halton_qrng
// (qmctoolscl/c_funcs/halton_qrng.c:135-136),
//
//     v = RN(RN(v + c) / b)        (v in [0, 1), integer 0 <= c < b, 2 <= b < 2^12)
//
// in integer arithmetic, bit for bit.  The add is exact in 128-bit fixed point
// (c in the high word, v in units of 2^-64 with a sticky bit for what lies
// below) and rounds once to 53 bits; the quotient by b is taken to 128 bits
// through the precomputed floor(2^64 / b) and 2^64 mod b, with the exact
// remainder as sticky bit, and rounds once.  Cases outside that form (v >= 1,
// results that would come near the subnormal range) report false and the
// caller uses the FP64 operations.
//
// Host-compilable (g++) so the CPU tests can check it against the host's IEEE
// arithmetic.
#pragma once

#ifdef __CUDACC__
#define QS_HD __host__ __device__ __forceinline__
#else
#define QS_HD inline
#endif

namespace qstep {

typedef unsigned long long u64;
typedef unsigned int u32;

struct Div {
    u64 inv;   // floor(2^64 / b)
    u32 rem0;  // 2^64 mod b
    u32 b;
};

QS_HD Div make_div(u32 b)
{
    Div D;
    D.b = b;
    D.inv = ~0ull / b;                    // floor((2^64 - 1) / b): floor(2^64 / b) unless b divides 2^64
    D.rem0 = (u32)((~0ull % b + 1) % b);  // 2^64 mod b
    if (D.rem0 == 0) D.inv += 1;          // b a power of two
    return D;
}

QS_HD int clz64(u64 x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

QS_HD u64 mulhi64(u64 a, u64 b)
{
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (u64)(((unsigned __int128)a * b) >> 64);
#endif
}

// bits of RN(RN(v + c) / b); false (out unchanged) outside the integer form
QS_HD bool step(u64 vbits, u32 c, const Div &D, u64 &out)
{
    const u32 Ev = (u32)(vbits >> 52);
    if (Ev >= 1023) return false;  // v >= 1 (or inf / nan)
    const u64 Mv = Ev ? ((vbits & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : (vbits & 0xFFFFFFFFFFFFFull);
    u64 Mx;      // significand of x = RN(v + c), leading one at bit 52
    int Ex;      // biased exponent of x
    if (c == 0) {
        if (Ev == 0) {
            if (Mv) return false;  // subnormal v
            out = 0;               // 0 / b
            return true;
        }
        Mx = Mv;
        Ex = (int)Ev;
    } else {
        // v in units of 2^-64 (V), with a sticky bit for the bits below
        const int sh = (int)(Ev ? Ev : 1) - 1011;  // v = Mv * 2^(E - 1075) = Mv * 2^(sh - 64)
        u64 V;
        u32 sticky;
        if (sh >= 0) {  // sh <= 11 for v < 1: V < 2^64
            V = Mv << sh;
            sticky = 0;
        } else if (sh > -64) {
            V = Mv >> -sh;
            sticky = (Mv & ((1ull << -sh) - 1)) != 0;
        } else {
            V = 0;
            sticky = Mv != 0;
        }
        const int lc = 63 - clz64((u64)c);            // leading bit of c (c < 2^12)
        const int Dd = 12 + lc;                       // bits of S = c * 2^64 + V below the kept 53
        u64 kept = ((u64)c << (52 - lc)) | (V >> Dd);
        const u64 drop = V & ((1ull << Dd) - 1), half = 1ull << (Dd - 1);
        kept += (u64)((drop > half) | ((drop == half) & ((u64)sticky | (kept & 1ull))));
        // x = kept * 2^(Dd - 64); a round-up to 2^53 moves to the next binade
        Ex = 1011 + Dd;
        if (kept >> 53) {
            kept >>= 1;
            Ex += 1;
        }
        Mx = kept;
    }
    // y = x / b = (Mx * 2^64 / b) * 2^(Ex - 1139): quotient Q = Qh * 2^64 + Ql, remainder R2
    u64 Qh = mulhi64(Mx, D.inv);
    u64 R = Mx - Qh * D.b;
    if (R >= D.b) {
        Qh += 1;
        R -= D.b;
    }
    const u64 t = R * (u64)D.rem0;  // < b^2 < 2^24
    const u64 tq = t / D.b;
    const u64 Ql = R * D.inv + tq;
    const u64 R2 = t - tq * D.b;
    const int p = 63 - clz64(Qh);   // leading bit of Qh: 40 .. 52 (Mx >= 2^52, b < 2^12)
    const int sh = 52 - p;          // 0 .. 12
    u64 mant = sh ? ((Qh << sh) | (Ql >> (64 - sh))) : Qh;
    const u64 rb = Ql << sh;        // the dropped bits of Ql, left-aligned
    const u64 halfq = 1ull << 63;
    mant += (u64)((rb > halfq) | ((rb == halfq) & ((u64)(R2 != 0) | (mant & 1ull))));
    const int Ey = Ex + p - 52;     // biased exponent of y (before a round-up carry)
    if (Ey < 2) return false;       // near the subnormal range
    out = ((u64)(Ey - 1) << 52) + mant;  // the hidden bit adds one; a carry to 2^53 bumps the exponent
    return true;
}

}  // namespace qstep
