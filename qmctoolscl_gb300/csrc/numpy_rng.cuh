// numpy_rng.cuh -- numpy's SFC64 bit generator and the Generator methods the
// randomisation helpers call, on the device, bit for bit:
//
//   * SFC64 (Chris Doty-Humphrey's Small Fast Chaotic generator, 64-bit
//     variant): state a, b, c and a counter w; one step returns a + b + w++
//     and mixes the state with a right shift by 11, a left shift by 3 and a
//     rotation by 24;
//   * numpy's 32-bit outputs are the two halves of one 64-bit output, low half
//     first, the high half buffered in the bit generator (has_uint32,
//     uinteger: the state words 4 and 5);
//   * Generator.random(): the top 53 bits of a 64-bit output times 2^-53;
//   * Generator.integers(low, high): with rng = high - low - 1, no draw when
//     rng = 0, one 32-bit output when rng = 2^32 - 1, Lemire's
//     multiply-and-reject on 32-bit outputs for other rng below 2^32, one
//     64-bit output when rng = 2^64 - 1, Lemire on 64-bit outputs otherwise
//     (D. Lemire, "Fast random integer generation in an interval", ACM TOMS
//     2019: a draw x maps to floor(x * (rng+1) / 2^w), rejected while the low
//     w bits of the product fall below 2^w mod (rng+1));
//   * Generator.permutation(b): Fisher-Yates on arange(b) from the top, each
//     swap index from random_interval(i): outputs masked to the bits of i,
//     drawn again while above i (32-bit outputs for i below 2^32).
//
// State layout shared with the host (six uint64 words): a, b, c, w,
// has_uint32, uinteger -- the fields of numpy's SFC64 state dictionary.
#pragma once
#include "common.cuh"

namespace {

struct Sfc64 {
    u64 a, b, c, w, half;
    u32 has;

    __device__ __forceinline__ u64 next64()
    {
        const u64 out = a + b + w++;
        a = b ^ (b >> 11);
        b = c + (c << 3);
        c = ((c << 24) | (c >> 40)) + out;
        return out;
    }
    __device__ __forceinline__ u64 next32()
    {
        if (has) {
            has = 0;
            return half;
        }
        const u64 x = next64();
        has = 1;
        half = x >> 32;
        return x & 0xFFFFFFFFull;
    }
    // Generator.integers(0, 2**bits) (bits <= 63) and random_tbit_uint64s(rng,
    // bits, 1) (bits <= 64): with a power-of-two range numpy's Lemire rule
    // never rejects, so the value is the top bits of one 32-bit output (range
    // up to 2^32) or one 64-bit output; no draw for bits = 0
    __device__ __forceinline__ u64 bits(u32 nb)
    {
        if (nb == 0) return 0;
        if (nb <= 32) return next32() >> (32 - nb);
        const u64 x = next64();
        return nb == 64 ? x : x >> (64 - nb);
    }
    // Generator.random()
    __device__ __forceinline__ double uniform() { return (double)(next64() >> 11) * (1.0 / 9007199254740992.0); }
    // Generator.integers(off, off + rng + 1) for one value (any integer dtype:
    // numpy fills int64 and uint64 arrays through the same bounded rule).
    // `tries` bounds each rejection loop; a loop that runs out sets *bad.
    __device__ __forceinline__ u64 bounded(u64 off, u64 rng, bool *bad)
    {
        constexpr int TRIES = 64;  // each rejection has probability below 1/2
        if (rng == 0) return off;
        if (rng <= 0xFFFFFFFFull) {
            if (rng == 0xFFFFFFFFull) return off + next32();
            const u32 excl = (u32)rng + 1u;
            u64 m = next32() * (u64)excl;
            u32 left = (u32)m;
            if (left < excl) {
                const u32 thr = (0xFFFFFFFFu - (u32)rng) % excl;
                for (int t = 0; left < thr; t++) {
                    if (t >= TRIES) {
                        *bad = true;
                        break;
                    }
                    m = next32() * (u64)excl;
                    left = (u32)m;
                }
            }
            return off + (m >> 32);
        }
        if (rng == ~0ull) return off + next64();
        const u64 excl = rng + 1;
        u64 x = next64();
        u64 left = x * excl, hi = __umul64hi(x, excl);
        if (left < excl) {
            const u64 thr = (~0ull - rng) % excl;
            for (int t = 0; left < thr; t++) {
                if (t >= TRIES) {
                    *bad = true;
                    break;
                }
                x = next64();
                left = x * excl;
                hi = __umul64hi(x, excl);
            }
        }
        return off + hi;
    }
    // random_interval(max) for 1 <= max < 2^32 (the swap index of one
    // Fisher-Yates step of Generator.permutation)
    __device__ __forceinline__ u32 interval(u32 max, bool *bad)
    {
        constexpr int TRIES = 256;  // each try fails with probability below 1/2
        const u32 mask = 0xFFFFFFFFu >> __clz((int)max);
        for (int t = 0;; t++) {
            const u32 v = (u32)next32() & mask;
            if (v <= max) return v;
            if (t >= TRIES) {
                *bad = true;
                return 0;
            }
        }
    }
    __device__ __forceinline__ void load(const u64 *st)
    {
        a = st[0];
        b = st[1];
        c = st[2];
        w = st[3];
        has = (u32)(st[4] != 0);
        half = st[5];
    }
    __device__ __forceinline__ void store(u64 *st) const
    {
        st[0] = a;
        st[1] = b;
        st[2] = c;
        st[3] = w;
        st[4] = has;
        st[5] = half;
    }
};

}  // namespace
