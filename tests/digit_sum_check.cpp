// Checks the integer add of digit_sum.cuh against the host's IEEE double
// arithmetic (built with -ffp-contract=off, so v + r*s is two separately
// rounded operations, as in gdn_integer_to_float.c:37).
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

static u64 hw_add(u64 v, u64 y)
{
    volatile double s = dbl(v) + dbl(y);
    return bits(s);
}

static u64 hw_term(u64 r, u64 s)
{
    volatile double p = dbl(r) * (double)s;
    return bits(p);
}

// the kernel's add: the fast form, else the exact fallback (here the host FPU)
static dsum::Sum emu_add(dsum::Sum v, u64 y, long *fast)
{
    if (dsum::add_fast(v, y)) {
        ++*fast;
        return v;
    }
    if (!y) return v;
    return dsum::unpack(v.M ? hw_add(dsum::pack(v), y) : y);
}

int main(int argc, char **argv)
{
    const long cases = argc > 1 ? atol(argv[1]) : 1000000;
    const long chains = argc > 2 ? atol(argv[2]) : 100000;
    state = argc > 3 ? strtoull(argv[3], 0, 10) : 1;
    long fast = 0;
    // single adds: v in [2^-40, 1), y in [2^-130, 1) plus zeros and subnormals
    for (long c = 0; c < cases; c++) {
        u64 vb = ((u64)(1023 - 1 - next() % 40) << 52) | (next() & dsum::FRAC);
        u64 yb = ((u64)(1023 - 1 - next() % 130) << 52) | (next() & dsum::FRAC);
        if (c % 97 == 0) yb = 0;
        if (c % 89 == 0) yb = next() & dsum::FRAC;  // subnormal
        if (c % 83 == 0) vb = next() & dsum::FRAC;
        if (c % 79 == 0) vb = 0;
        if (c % 5 == 0) yb = vb - ((u64)(1 + next() % 60) << 52);  // same significand, lower binade
        if (c % 3 == 0) yb &= ~((1ull << (next() % 53)) - 1);         // trailing zeros: exact halves
        if (c % 7 == 0) yb = ((u64)(1023 - 1 - next() % 60) << 52) | (next() & dsum::FRAC);  // y above v too
        if (c % 11 == 0) yb = ((vb >> 52) << 52) | (next() & dsum::FRAC);                 // same binade
        const u64 got = dsum::pack(emu_add(dsum::unpack(vb), yb, &fast)), want = hw_add(vb, yb);
        if (got != want) {
            printf("add mismatch v=%016llx y=%016llx got=%016llx want=%016llx\n", vb, yb, got, want);
            return 1;
        }
    }
    // products RN(recip * m) for m < 2^11 against the host's multiply
    for (long c = 0; c < cases; c++) {
        u64 rb = ((u64)(1023 - 700 + next() % 1000) << 52) | (next() & dsum::FRAC);
        if (c % 3 == 0) rb &= ~((1ull << (next() % 53)) - 1);  // trailing zeros: exact and tie products
        const u32 m = 1 + (u32)(next() % 2047);
        volatile double p = dbl(rb) * (double)m;
        if (dsum::mul_small(rb, m) != bits(p)) {
            printf("mul mismatch r=%016llx m=%u got=%016llx want=%016llx\n", rb, m, dsum::mul_small(rb, m), bits(p));
            return 1;
        }
    }
    // whole chains: base b, recip_0 = 1/b, recip_{t+1} = recip_t/b, terms RN(recip_t * digit)
    for (long c = 0; c < chains; c++) {
        const u32 b = 2 + (u32)(next() % (c % 3 == 0 ? 30 : 2046));
        const u32 tmax = 1 + (u32)(next() % 90);
        volatile double bd = (double)b;
        volatile double rc = 1.0 / bd;
        u64 hv = 0;
        dsum::Sum ev = dsum::unpack(0);
        for (u32 t = 0; t < tmax; t++) {
            u64 s = next() % b;
            if (c % 11 == 0 && t < 3) s = 0;         // leading zero digits
            if (c % 13 == 0) s = b - 1;               // all digits maximal: carries into new binades
            if (c % 17 == 0) s = next() % 100000;     // digits beyond the base (permutations without a shift)
            const u64 y = s ? hw_term(bits(rc), s) : 0;
            hv = hw_add(hv, y);
            ev = emu_add(ev, y, &fast);
            rc = rc / bd;
        }
        if (dsum::pack(ev) != hv) {
            printf("chain mismatch b=%u tmax=%u got=%016llx want=%016llx\n", b, tmax, dsum::pack(ev), hv);
            return 1;
        }
    }
    printf("ok fast=%ld\n", fast);
    return 0;
}
