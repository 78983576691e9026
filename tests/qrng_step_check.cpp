// Checks qstep::step of qrng_step.cuh (one Horner step of halton_qrng:
// RN(RN(v + c) / b)) against the host's IEEE double arithmetic.
// Usage: qrng_step_check <cases> <seed>; prints "ok" or the first mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../qmctoolscl_gb300/csrc/qrng_step.cuh"

using qstep::u32;
using qstep::u64;

static u64 state;
static u64 next()  // splitmix64
{
    u64 z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static u64 bits(double x) { u64 b; std::memcpy(&b, &x, 8); return b; }
static double dbl(u64 b) { double x; std::memcpy(&x, &b, 8); return x; }

int main(int argc, char **argv)
{
    const long cases = argc > 1 ? atol(argv[1]) : 1000000;
    state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    long fast = 0;
    for (long k = 0; k < cases; k++) {
        u32 b = 2 + (u32)(next() % 2422);
        if (k % 7 == 0) b = 1u << (1 + next() % 11);  // powers of two
        const qstep::Div D = qstep::make_div(b);
        u64 vb = ((u64)(1022 - next() % 80) << 52) | (next() & 0xFFFFFFFFFFFFFull);  // v in [2^-80, 1)
        if (k % 11 == 0) vb = 0;
        if (k % 13 == 0) vb = ((u64)(1022 - next() % 1000) << 52) | (next() & 0xFFFFFFFFFFFFFull);  // tiny
        if (k % 17 == 0) vb = bits(1.0) - 1 - (next() % 16);                                       // just below 1
        if (k % 3 == 0) vb &= ~((1ull << (next() % 53)) - 1);  // trailing zeros: exact sums and ties
        u32 c = (u32)(next() % b);
        if (k % 5 == 0) c = 0;
        if (k % 19 == 0) c = b - 1;
        volatile double x = dbl(vb) + (double)c;
        volatile double y = x / (double)b;
        u64 got;
        if (qstep::step(vb, c, D, got)) {
            fast++;
            if (got != bits(y)) {
                printf("mismatch v=%016llx c=%u b=%u got=%016llx want=%016llx\n", vb, c, b, got, bits(y));
                return 1;
            }
        }
    }
    // whole Horner chains as halton_qrng runs them: v = 0; 32 times v = RN(RN(v + c)/b)
    for (long k = 0; k < cases / 32; k++) {
        const u32 b = 2 + (u32)(next() % 2422);
        const qstep::Div D = qstep::make_div(b);
        double hv = 0.0;
        u64 iv = 0;
        for (int t = 0; t < 32; t++) {
            const u32 c = (k % 4 == 0 && t < 20) ? 0u : (u32)(next() % b);
            volatile double x = hv + (double)c;
            hv = x / (double)b;
            u64 o;
            if (qstep::step(iv, c, D, o)) {
                iv = o;
            } else {
                volatile double x2 = dbl(iv) + (double)c;
                volatile double y2 = x2 / (double)b;
                iv = bits(y2);
            }
            if (iv != bits(hv)) {
                printf("chain mismatch b=%u t=%d got=%016llx want=%016llx\n", b, t, iv, bits(hv));
                return 1;
            }
        }
    }
    printf("ok fast=%ld\n", fast);
    return 0;
}
