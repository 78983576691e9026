// lattice_dev.cuh -- per-point device code of the rank-1 lattice kernels,
// shared by the per-call kernels (lattice.cu) and the batched persistent
// kernel (batch.cu).
//
// Reference: qmctoolscl/c_funcs/lat_gen_linear.c:23-33, lat_gen_natural.c:23-58,
// lat_gen_gray.c:23-56, lat_shift_mod_1.c:24-35.
//
// Closed form.  The reference walks a Gray-code recurrence; the value it
// writes is fmod((double)g * V, 1) with V = ldexp(v, -p), where for a row
// whose sequence index is m (m = n_start+k in natural order, the Gray code
// of n_start+i in Gray order), p = bitlen(m) and v = m bit-reversed in p
// bits -- V is the van der Corput radical inverse of m.  With
// B = bitreverse64(m), V = B * 2^-64 exactly, and when bitlen(g) + p <= 53 the
// double product g*V is exact, so fmod(g*V, 1) = (g*B mod 2^64) * 2^-64: one
// integer multiply gives the fraction in 0.64 fixed point.  Columns outside
// that domain take the FP64 instructions the reference's formula names.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace lat {
namespace {  // internal linkage: included by several translation units

enum Order { LINEAR_POW2 = 0, LINEAR_GENERIC = 1, NATURAL = 2, GRAY = 3 };

// Per-column constants, prepared once per thread and column.
struct Col {
    u64 g;
    double gd;       // (double)g, rounded as the reference converts it
    u64 S;           // shift in 0.64 fixed point
    double s;
    bool fast;       // exact integer generation
    u32 shift_kind;  // 0: 0.64 with 11 zero low bits, 1: 0.64, 2: FP64 add
};

// p: bit length of the largest sequence index (log2 n for linear order)
__device__ __forceinline__ Col load_col(u64 g, const double *s_ptr, u32 p, int order)
{
    Col c;
    c.g = g;
    c.gd = __ull2double_rn(g);
    const u32 bits_g = g ? 64 - __clzll((long long)g) : 0;
    c.fast = (order != LINEAR_GENERIC) && (bits_g + p <= 53) && (p <= 53);
    c.S = 0;
    c.s = 0.0;
    c.shift_kind = 2;
    if (s_ptr) {
        c.s = *s_ptr;
        u64 S;
        if (double_to_fix64(c.s, &S)) {
            c.S = S;
            c.shift_kind = (S & 0x7FFull) ? 1u : 0u;
        }
    }
    return c;
}

// fmod(g*V, 1) as the reference computes it, with FP64 instructions.  Kept
// out of line: GB300's FP64 pipe is slow, and if the compiler if-converted
// these fallbacks into the per-element loop their (predicated-off) FP64
// instructions would still be issued for every coordinate and saturate it.
__device__ __noinline__ double value_hw(double gd, int order, u64 m, u64 i, u64 n)
{
    if (order == LINEAR_POW2 || order == LINEAR_GENERIC) {
        const double q = __ddiv_rn(__ull2double_rn(i), __ull2double_rn(n));
        return frac_mod1(__dmul_rn(gd, q));
    }
    const int p = m ? 64 - __clzll((long long)m) : 0;
    const u64 v = m ? (__brevll(m) >> (64 - p)) : 0;
    const double V = scalbn(__ull2double_rn(v), -p);
    return frac_mod1(__dmul_rn(gd, V));
}

// Every case other than the common one: exact integer generation with a
// shift that needs general rounding, or FP64 generation/shift.
__device__ __noinline__ double point_general(const Col &c, int order, u64 B, u64 m, u64 i, u64 n, bool shift)
{
    double x;
    if (c.fast) {
        const u64 W = c.g * B;
        if (!shift) return fix64_to_double(W);
        if (c.shift_kind == 1) return fix64_to_double(add_mod1_fix64(W, c.S));
        x = fix64_to_double(W);
    } else {
        x = value_hw(c.gd, order, m, i, n);
        if (!shift) return x;
    }
    return frac_mod1(__dadd_rn(x, c.s));
}

template <bool SHIFT>
__device__ __forceinline__ double point(const Col &c, int order, u64 B, u64 m, u64 i, u64 n)
{
    if (c.fast && (!SHIFT || c.shift_kind == 0)) {
        const u64 W = c.g * B;  // fraction of g*V in 0.64 fixed point (<= 53 significant bits)
        if (!SHIFT) return fix64_to_double(W);
        // W and S are multiples of 2^-53: the sum needs rounding only when it
        // reaches 1, and then only a tie on bit 11 can occur
        u64 T = W + c.S;
        if (T < W) T = (T + ((T >> 1) & 0x800ull)) & ~0xFFFull;
        return fix64_to_double(T);
    }
    return point_general(c, order, B, m, i, n, SHIFT);
}

// Exact double of (th:tl) * 2^-64 for th != 0 and at most 53 significant
// bits, on 32-bit halves: normalise with one funnel shift, drop 11 bits with
// another, add the exponent into the high word.
__device__ __forceinline__ double fix64_hi_to_double(u32 th, u32 tl)
{
    const u32 lz = __clz(th);
    const u32 hi = __funnelshift_l(tl, th, lz);
    const u32 lo = tl << lz;
    const u32 m_lo = __funnelshift_r(lo, hi, 11);
    const u32 m_hi = (hi >> 11) + ((1021u - lz) << 20);
    return __hiloint2double((int)m_hi, (int)m_lo);
}

// The common case in 32-bit arithmetic: every sequence index below 2^32, so
// B = bitreverse64(m) has a zero low word and the fraction g*B mod 2^64 is
// (g mod 2^32) * bitreverse32(m) in the high word; the shift is on the
// 2^-53 grid, in 0.64 fixed point (sh:sl).
template <bool SHIFT>
__device__ __forceinline__ double point_narrow(u32 g_lo, u32 bh, u32 sh, u32 sl)
{
    const u32 wh = g_lo * bh;
    if (!SHIFT) return wh ? fix64_hi_to_double(wh, 0u) : 0.0;
    u32 th = wh + sh, tl = sl;
    if (th < wh) {  // the sum reached 1: round to the 2^-52 grid (ties to even), drop the 1
        const u64 t = ((((u64)th << 32) | tl) + ((tl >> 1) & 0x800u)) & ~0xFFFull;
        th = (u32)(t >> 32);
        tl = (u32)t;
    }
    if (th) return fix64_hi_to_double(th, tl);
    return fix64_to_double(((u64)th << 32) | tl);  // results below 2^-32
}

// One thread's share of a block of rows for column group jg (VEC consecutive
// columns) of one randomisation: rows i_begin, i_begin+stride, ... < i_end.
//   g_l, s_l: generating vector and shifts of this randomisation (d each; s_l
//             null without SHIFT), out_l: its r-slab of the output (n*d)
//   narrow:   every index n_start + i < 2^32 (and log2 n <= 32 for linear order)
template <int ORDER, bool SHIFT, int VEC>
__device__ __forceinline__ void rows(const u64 *g_l, const double *s_l, double *out_l, u64 d, u64 n, u64 n_start,
                                     u32 p, u64 jg, u64 i_begin, u64 i_end, u64 stride, bool narrow)
{
    const u64 j0 = jg * VEC;
    Col c[VEC];
    bool easy = narrow;
#pragma unroll
    for (int v = 0; v < VEC; v++) {
        c[v] = load_col(g_l[j0 + v], SHIFT ? s_l + j0 + v : nullptr, p, ORDER);
        easy &= c[v].fast && (!SHIFT || c[v].shift_kind == 0);
    }
    double *out = out_l + j0;
    if (easy) {
        u32 g_lo[VEC], sh[VEC], sl[VEC];
#pragma unroll
        for (int v = 0; v < VEC; v++) {
            g_lo[v] = (u32)c[v].g;
            sh[v] = (u32)(c[v].S >> 32);
            sl[v] = (u32)c[v].S;
        }
        const u32 ns = (u32)n_start;
        for (u64 i = i_begin; i < i_end; i += stride) {
            u32 bh;
            if (ORDER == LINEAR_POW2) {
                bh = p ? ((u32)i << (32 - p)) : 0u;
            } else {
                const u32 k = ns + (u32)i;
                bh = __brev(ORDER == GRAY ? (k ^ (k >> 1)) : k);
            }
            double y[VEC];
#pragma unroll
            for (int v = 0; v < VEC; v++) y[v] = point_narrow<SHIFT>(g_lo[v], bh, sh[v], sl[v]);
            if (VEC == 2)
                __stcs((double2 *)(out + i * d), make_double2(y[0], y[VEC - 1]));
            else
                __stcs(out + i * d, y[0]);
        }
        return;
    }
    for (u64 i = i_begin; i < i_end; i += stride) {
        const u64 k = n_start + i;
        const u64 m = (ORDER == GRAY) ? (k ^ (k >> 1)) : k;
        u64 B;
        if (ORDER == LINEAR_POW2 || ORDER == LINEAR_GENERIC)
            B = (ORDER == LINEAR_POW2 && p) ? (i << (64 - p)) : 0;
        else
            B = __brevll(m);
        double y[VEC];
#pragma unroll
        for (int v = 0; v < VEC; v++) y[v] = point<SHIFT>(c[v], ORDER, B, m, i, n);
        if (VEC == 2)
            __stcs((double2 *)(out + i * d), make_double2(y[0], y[VEC - 1]));
        else
            __stcs(out + i * d, y[0]);
    }
}

__host__ __device__ __forceinline__ u32 bitlen(u64 v)
{
#ifdef __CUDA_ARCH__
    return v ? 64u - (u32)__clzll((long long)v) : 0u;
#else
    return v ? 64u - (u32)__builtin_clzll(v) : 0u;
#endif
}

}  // namespace
}  // namespace lat
