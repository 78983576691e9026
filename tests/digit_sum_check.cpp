// Checks the integer digit-sum routines of digit_sum.cuh against the host's
// IEEE double arithmetic (built with -ffp-contract=off, so v + r*s is two
// separately rounded operations, as in gdn_integer_to_float.c:37).
// Usage: digit_sum_check <cases> <chains> <seed>; prints "ok" or the first mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../qmctoolscl_gb300/csrc/digit_sum.cuh"

using dsum::u32;
using dsum::u64;

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

static u64 hw_step(u64 v, u64 r, u32 s)
{
    volatile double prod = dbl(r) * (double)s;
    volatile double sum = dbl(v) + prod;
    return bits(sum);
}

// the kernel's step: fast form, else the general routine, else hardware
static dsum::Sum emu_step(dsum::Sum v, u64 r, u32 s)
{
    const u32 er = (u32)(r >> 52);
    const u64 mr = (r & dsum::FRAC) | dsum::HIDDEN;
    if ((v.M >> 52) && s < 2048 && er >= 1 && er < 2036 && dsum::add_term_fast(v, mr, er, s)) return v;
    const u64 vb = dsum::pack(v);
    const u64 nb = dsum::general_ok(vb, r, s) ? dsum::add_bits(vb, dsum::mul_bits(r, s)) : hw_step(vb, r, s);
    return dsum::unpack(nb);
}

int main(int argc, char **argv)
{
    const long cases = argc > 1 ? atol(argv[1]) : 1000000;
    const long chains = argc > 2 ? atol(argv[2]) : 100000;
    state = argc > 3 ? strtoull(argv[3], 0, 10) : 1;
    long fast_hits = 0;
    // single steps: v in [2^-40, 1), r in [2^-120, 1), s in [1, 2^11) plus some wide digits
    for (long c = 0; c < cases; c++) {
        const u64 vb = ((u64)(1023 - 1 - next() % 40) << 52) | (next() & dsum::FRAC);
        const u64 rb = ((u64)(1023 - 1 - next() % 120) << 52) | (next() & dsum::FRAC);
        u32 s = 1 + (u32)(next() % 2047);
        if (c % 64 == 0) s = 1 + (u32)(next() % 100000);
        if (c % 7 == 0) s = 1u << (next() % 11);  // exact products
        dsum::Sum v = dsum::unpack(vb);
        dsum::Sum w = v;
        const u32 er = (u32)(rb >> 52);
        if (s < 2048 && dsum::add_term_fast(w, (rb & dsum::FRAC) | dsum::HIDDEN, er, s)) fast_hits++;
        const u64 got = dsum::pack(emu_step(v, rb, s)), want = hw_step(vb, rb, s);
        if (got != want) {
            printf("step mismatch v=%016llx r=%016llx s=%u got=%016llx want=%016llx\n", vb, rb, s, got, want);
            return 1;
        }
    }
    // whole chains: base b, recip_0 = 1/b, recip_{t+1} = recip_t/b, digits in [0, b)
    for (long c = 0; c < chains; c++) {
        const u32 b = 2 + (u32)(next() % (c % 3 == 0 ? 30 : 2046));
        const u32 tmax = 1 + (u32)(next() % 90);
        volatile double bd = (double)b;
        volatile double rc = 1.0 / bd;
        u64 hv = 0;
        dsum::Sum ev = dsum::unpack(0);
        for (u32 t = 0; t < tmax; t++) {
            u32 s = (u32)(next() % b);
            if (c % 11 == 0 && t < 3) s = 0;        // leading zero digits
            if (c % 13 == 0) s = b - 1;              // all digits maximal: carries into new binades
            if (s) {
                hv = hw_step(hv, bits(rc), s);
                ev = emu_step(ev, bits(rc), s);
            }
            rc = rc / bd;
        }
        if (dsum::pack(ev) != hv) {
            printf("chain mismatch b=%u tmax=%u got=%016llx want=%016llx\n", b, tmax, dsum::pack(ev), hv);
            return 1;
        }
    }
    printf("ok fast=%ld/%ld\n", fast_hits, cases);
    return 0;
}
