// common.cuh -- shared device helpers and host plumbing for libqmcgb.
//
// GB300 executes FP64 at about 1.25 TFLOP/s (two DFMA per SM per clock),
// far below its integer issue rate (128 lanes per SM per clock) and below
// what its HBM can feed.  Every kernel whose output must be the bit-exact
// IEEE double the reference C backend produces therefore builds that bit
// pattern with integer operations: the helpers below construct a double
// from a fixed-point integer, round an unsigned integer to nearest-even,
// and add two non-negative doubles with round-to-nearest-even.  Each helper
// states the input domain on which it is exact; kernels test the domain and
// fall back to the FP64 instruction otherwise, so results are identical in
// every case and only the speed differs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qmcgb.h"

typedef unsigned long long u64;
typedef unsigned int u32;
typedef unsigned short u16;

// ---------------------------------------------------------------- bits ----

__device__ __forceinline__ double as_double(u64 b) { return __longlong_as_double((long long)b); }
__device__ __forceinline__ u64 as_bits(double x) { return (u64)__double_as_longlong(x); }

// Shift counts of 64 or more (or "negative" counts that wrapped around as
// unsigned) are undefined in C; gcc on x86-64 and aarch64 emits a hardware
// shift that uses the count mod 64.  The reference's results in those cases
// follow that rule, so the kernels spell it out.
__device__ __forceinline__ u64 shl64(u64 v, u64 s) { return v << (u32)(s & 63); }
__device__ __forceinline__ u64 shr64(u64 v, u64 s) { return v >> (u32)(s & 63); }

// Exact value W * 2^-64 as a double.  Exact when W has at most 53
// significant bits (always true for the callers, which say why).
__device__ __forceinline__ double fix64_to_double(u64 W)
{
    if (W == 0) return 0.0;
    const int lz = __clzll((long long)W);
    const u64 m = (W << lz) >> 11;  // 53 bits, leading one at bit 52
    // biased exponent of W*2^-64 is 1022-lz; adding m (with its leading one)
    // to (1021-lz)<<52 bumps the exponent field by exactly that one
    return as_double(((u64)(1021 - lz) << 52) + m);
}

// RN-even of the unsigned integer x, times 2^e, as a double.  Exact
// emulation of ldexp((double)x, e) whenever the result is a normal number:
// valid for 1 <= 1085 - clz(x) + e (x != 0); x == 0 gives +0.
__device__ __forceinline__ u64 u64_scaled_bits(u64 x, int e)
{
    if (x == 0) return 0;
    const int lz = __clzll((long long)x);
    const u64 N = x << lz;
    u64 m = N >> 11;
    const u64 rem = N & 0x7FFull;
    m += (rem > 0x400ull) | ((rem == 0x400ull) & (m & 1ull));
    return ((u64)(1085 - lz + e) << 52) + m;  // a carry out of m bumps the exponent
}

// fmod(y, 1.0) for any double y, exact (fmod is exact; y - trunc(y) is the
// exact fractional part, and copysign gives fmod's sign of zero).
__device__ __forceinline__ double frac_mod1(double y)
{
    return copysign(__dadd_rn(y, -trunc(y)), y);
}

// If x is in [0, 1) and a multiple of 2^-64, write x*2^64 to *X and return
// true.  Used to move doubles into 0.64 fixed point.
__device__ __forceinline__ bool double_to_fix64(double x, u64 *X)
{
    const u64 b = as_bits(x);
    if (b == 0) { *X = 0; return true; }
    const u32 E = (u32)(b >> 52);  // includes the sign bit: negatives fail below
    if (E == 0 || E >= 1023) return false;  // subnormal, >= 1, negative, inf, nan
    const u64 M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = (int)E - 1023 + 12;  // X = M * 2^(E-1023-52+64)
    if (sh >= 0) { *X = M << sh; return true; }
    if (sh <= -53) return false;
    if (M & ((1ull << (-sh)) - 1)) return false;
    *X = M >> (-sh);
    return true;
}

// fmod(RN(x + s), 1) for x = X*2^-64 and s = S*2^-64, both in [0, 1): the
// double sum rounds to 53 significant bits (ulp 2^-52 once the sum reaches
// 1), then the integer part is dropped.  Returns the 0.64 fixed-point result,
// which has at most 53 significant bits.
__device__ __forceinline__ u64 add_mod1_fix64(u64 X, u64 S)
{
    u64 T = X + S;
    int sh;
    if (T < X) {
        sh = 12;  // sum in [1, 2): spacing 2^-52
    } else {
        const int lz = T ? __clzll((long long)T) : 64;
        sh = 11 - lz;  // sum in [2^-1-lz, 2^-lz): spacing 2^(11-lz) units
    }
    if (sh > 0) {
        const u64 half = 1ull << (sh - 1), mask = (1ull << sh) - 1;
        const u64 rem = T & mask;
        T &= ~mask;
        if (rem > half || (rem == half && ((T >> sh) & 1))) T += 1ull << sh;  // may wrap to 0: sum rounded to 1 or 2
    }
    return T;
}

// ---------------------------------------------------- small integer math --

// Lemire-Kaser-Kurz direct remainder ("Faster remainder by direct
// computation", 2019): with M = floor(2^64 / b) + 1, for every 32-bit x and
// 1 < b < 2^32: x / b = mulhi64(M, x) and x % b = mulhi64(M * x, b).
struct FastDiv32 {
    u64 M;
    u32 b;
};

__host__ __device__ __forceinline__ FastDiv32 fastdiv32_make(u32 b)
{
    FastDiv32 f;
    f.b = b;
    f.M = (b > 1) ? (~0ull / b + 1) : 0;
    return f;
}

__device__ __forceinline__ u32 fd_div(const FastDiv32 &f, u32 x)
{
    return f.b == 1 ? x : (u32)__umul64hi(f.M, (u64)x);
}

__device__ __forceinline__ u32 fd_mod(const FastDiv32 &f, u32 x)
{
    return f.b == 1 ? 0u : (u32)__umul64hi(f.M * (u64)x, (u64)f.b);
}

// ---------------------------------------------------------- host side ----

namespace qmcgb {

void set_error(const char *fmt, ...);
int cuda_status(cudaError_t e, const char *what);
int launch_status(const char *what);

// device-side error word: kernels that meet an index the reference would
// read out of its array record the code here and skip the access
int device_error_reset(cudaStream_t s);
unsigned int *device_error_ptr();

inline unsigned grid_for(u64 work, unsigned per_block, unsigned cap)
{
    u64 g = (work + per_block - 1) / per_block;
    if (g == 0) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

int sm_count();

// Raise the kernel's dynamic shared-memory limit to at least `bytes` (no-op up
// to the default 48 KB).  The limit is one attribute per kernel and device:
// it is only ever raised (a high-water mark kept under a lock), so a launch
// prepared for one size is never broken by a later, smaller setting.
int raise_smem_limit(const void *func, size_t bytes, const char *what);

// base-2 net generation with optional fused digital shift / float output
// (dnb2.cu); stream-ordered, allocates nothing
int dnb2_gen_fused(u64 r, u64 n, u64 d, u64 n_start, u64 mmax, const u64 *C, u64 r_C, int gray,
                   const u64 *lshifts, u64 r_x, const u64 *shifts, const u64 *tmaxes, u64 *xrb, double *x,
                   cudaStream_t s);

}  // namespace qmcgb

#define QMC_REQUIRE(cond, ...)                \
    do {                                      \
        if (!(cond)) {                        \
            qmcgb::set_error(__VA_ARGS__);    \
            return QMC_ERR_ARG;               \
        }                                     \
    } while (0)

#define QMC_REQUIRE_DOMAIN(cond, ...)         \
    do {                                      \
        if (!(cond)) {                        \
            qmcgb::set_error(__VA_ARGS__);    \
            return QMC_ERR_DOMAIN;            \
        }                                     \
    } while (0)

#define QMC_STREAM(s) ((cudaStream_t)(s))
