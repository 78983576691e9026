// Checks the integer FP64 <-> FP32 conversions of fpconv.cuh against the
// host's conversions (round to nearest even).
// Usage: fpconv_check <cases> <seed>; prints "ok" or the first mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../qmctoolscl_gb300/csrc/fpconv.cuh"

using fpc::u32;
using fpc::u64;

static u64 state;
static u64 next()  // splitmix64
{
    u64 z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main(int argc, char **argv)
{
    const long cases = argc > 1 ? atol(argv[1]) : 1000000;
    state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    long fast64 = 0, fast32 = 0;
    for (long c = 0; c < cases; c++) {
        u64 b = next();
        switch (c % 6) {
        case 0: break;                                                       // any bits
        case 1: b = (b & 0x800FFFFFFFFFFFFFull) | ((u64)(897 + next() % 254) << 52); break;  // FP32 normal range
        case 2: b = (b & 0x800FFFFFE0000000ull) | ((u64)(880 + next() % 290) << 52) | 0x10000000ull; break;  // ties
        case 3: b = (b & 0x8000000000000000ull) | ((u64)(1150) << 52) | 0x000FFFFFF0000000ull; break;  // max: carry to inf
        case 4: b &= 0x8000000000000000ull; break;                           // +-0
        default: b = (b & 0x800FFFFFFFFFFFFFull) | ((u64)(896 - next() % 30) << 52); break;  // FP32 subnormal range
        }
        double x;
        std::memcpy(&x, &b, 8);
        volatile float want = (float)x;
        u32 wb;
        std::memcpy(&wb, (const void *)&want, 4);
        u32 got;
        if (fpc::f64_to_f32_bits(b, got)) {
            fast64++;
            if (got != wb) {
                printf("f64->f32 mismatch %016llx: got %08x want %08x\n", b, got, wb);
                return 1;
            }
        }
        const u32 u = (u32)next();
        float f;
        std::memcpy(&f, &u, 4);
        volatile double wd = (double)f;
        u64 wdb;
        std::memcpy(&wdb, (const void *)&wd, 8);
        u64 gd;
        if (fpc::f32_to_f64_bits(u, gd)) {
            fast32++;
            if (gd != wdb) {
                printf("f32->f64 mismatch %08x: got %016llx want %016llx\n", u, gd, wdb);
                return 1;
            }
        }
    }
    printf("ok fast64=%ld fast32=%ld\n", fast64, fast32);
    return 0;
}
