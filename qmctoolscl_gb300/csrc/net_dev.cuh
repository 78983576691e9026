// net_dev.cuh -- tile-level device code of the base-2 digital-net
// generator, shared by the per-call kernel (dnb2.cu) and the batched
// persistent kernel (batch.cu).
//
// Reference: qmctoolscl/c_funcs/dnb2_gen_natural.c:23-69,
// dnb2_gen_gray.c:23-68, dnb2_digital_shift.c:25-35,
// dnb2_integer_to_float.c:22-32.
//
// The point with sequence index m (natural order m = n_start+k, Gray order
// m = gray(n_start+i)) is the XOR of the generating-matrix columns picked by
// the set bits of m -- the closed form of the reference's recurrence.  A CTA
// stages, for one randomisation and a tile of up to 64 columns, the table
// T[lo][c] of XORs for the K low index bits (built by doubling) and the
// columns H[b][c] for the high bits.  A coordinate is then T[m mod 2^K] ^
// (XOR of H over the set bits of m >> K), the second term changing only every
// 2^K rows.  The digital shift (x << ls) ^ s distributes over XOR and is
// folded into T and H; the float conversion is done before the store.
#pragma once

#include "common.cuh"

namespace net {
namespace {  // internal linkage: included by several translation units

constexpr int MAX_COLS = 64;  // columns per table
constexpr int MAX_K = 8;      // low index bits resolved by the table

__device__ __forceinline__ u64 seq_index(bool gray, u64 n_start, u64 i)
{
    const u64 k = n_start + i;
    return gray ? (k ^ (k >> 1)) : k;
}

// FP64 fallback kept out of line so its instructions never sit (predicated
// off) in the per-coordinate loop, where they would load GB300's slow FP64 pipe.
__device__ __noinline__ double to_float_hw(u64 v, int e) { return ldexp(__ull2double_rn(v), e); }

// ldexp((double)v, e) (dnb2_integer_to_float.c:29)
__device__ __forceinline__ double to_float_bits(u64 v, int e)
{
    if (v == 0) return 0.0;
    const int lz = __clzll((long long)v);
    const int E = 1085 - lz + e;
    if (E >= 1 && E <= 2045) return as_double(u64_scaled_bits(v, e));
    return to_float_hw(v, e);  // subnormal or overflowing results
}

// Largest K <= min(mmax, MAX_K) whose table of 2^K x ncols words fits 32 KB.
__host__ __device__ __forceinline__ u32 pick_K(u64 mmax, u32 ncols)
{
    u32 K = (u32)(mmax < MAX_K ? mmax : MAX_K);
    while (K > 0 && ((u64)ncols << K) * 8 > 32768) K--;
    return K;
}

__host__ __device__ __forceinline__ size_t table_words(u32 K, u64 mmax, u32 ncols)
{
    return ((size_t(1) << K) + (mmax > K ? mmax - K : 0)) * ncols;
}

// Build T and H for columns [j0, j0+ncols) of one matrix set Cl (d*mmax
// words, column-major per dimension as in the reference), left shift ls and
// digital shifts s_l (d words, or null).  Called by every thread of the CTA;
// ends with a barrier.
__device__ __forceinline__ void build_table(u64 *T, u64 *H, const u64 *Cl, u64 mmax, u64 j0, u32 ncols, u32 K,
                                            u32 ls, const u64 *s_l)
{
    const u32 nhi = mmax > K ? (u32)(mmax - K) : 0u;
    for (u32 e = threadIdx.x; e < nhi * ncols; e += blockDim.x) {
        const u32 b = e / ncols, c = e % ncols;
        H[e] = Cl[(j0 + c) * mmax + K + b] << ls;
    }
    // T[0] holds the digital shift (it reaches every entry through the
    // doubling); T[lo + 2^b] = T[lo] ^ (C[b] << ls)
    for (u32 c = threadIdx.x; c < ncols; c += blockDim.x) T[c] = s_l ? s_l[j0 + c] : 0ull;
    __syncthreads();
    for (u32 b = 0; b < K; b++) {
        const u32 half = 1u << b;
        for (u32 e = threadIdx.x; e < half * ncols; e += blockDim.x) {
            const u32 lo = e / ncols, c = e % ncols;
            T[(half + lo) * ncols + c] = T[lo * ncols + c] ^ (Cl[(j0 + c) * mmax + b] << ls);
        }
        __syncthreads();
    }
}

// Write rows [row_begin, row_end) of the tile.  Each thread owns VEC columns
// (VEC = 2: one adjacent pair, one 16-byte load and store; VEC = 4: two pairs
// half a row apart) and
// walks rows ry, ry + R, ...: R rows per step, so a step of the CTA writes R
// consecutive row segments, and a thread's high-bit term stays cached while
// m >> K holds.  Threads beyond R*groups idle (ncols need not divide the CTA).
// xb_l / x_l point at column j0 of the randomisation's slab (either may be
// null); d is the row pitch.  The per-row index work (sequence index, Gray
// code, high-bit key, store offset) is the kernel's ALU cost, so a thread
// takes four columns where it can and uses 32-bit indices (I = u32) when
// every index stays below 2^32.
template <bool GRAY, int VEC, typename I>
__device__ __forceinline__ void gen_rows_vec(const u64 *T, const u64 *H, u32 K, u32 ncols, u64 n_start, u64 d,
                                             u64 row_begin, u64 row_end, u64 *xb_l, double *x_l, int e_float)
{
    const u32 groups = ncols / VEC;
    const u32 R = blockDim.x / groups;
    if (threadIdx.x >= R * groups) return;
    // VEC = 4: two column pairs half a row apart (2g, 2g+1 and ncols/2 + 2g, +1), so each
    // 16-byte store instruction of a warp covers a contiguous run of the row
    const u32 c0 = (threadIdx.x % groups) * (VEC == 4 ? 2u : (u32)VEC);
    const u32 chalf = VEC == 4 ? ncols / 2 : 2u;  // column offset of the second pair
    const u32 nlo = 1u << K;
    I hi_key = ~(I)0;
    u64 hx[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) hx[v] = 0;
    const I ns = (I)n_start;
    const u64 row0 = row_begin + threadIdx.x / groups;
    u64 o = row0 * d + c0;
    const u64 ostep = (u64)R * d;
    for (I row = (I)row0; row < (I)row_end; row += R, o += ostep) {
        const I k = ns + row;
        const I m = GRAY ? (k ^ (k >> 1)) : k;
        const I hi = m >> K;
        if (hi != hi_key) {  // XOR of the high-bit columns picked by hi: changes every 2^K rows
#pragma unroll
            for (int v = 0; v < VEC; v++) hx[v] = 0;
            for (I hb = hi; hb; hb &= hb - 1) {
                const u32 b = (sizeof(I) == 4 ? __ffs((int)(u32)hb) : __ffsll((long long)hb)) - 1;
#pragma unroll
                for (int v = 0; v < VEC; v++) hx[v] ^= H[b * ncols + c0 + (v >> 1) * chalf + (v & 1)];
            }
            hi_key = hi;
        }
        const u32 ti = (u32)(m & (I)(nlo - 1)) * ncols + c0;
        if (VEC >= 2) {
#pragma unroll
            for (int h = 0; h < VEC / 2; h++) {
                const ulonglong2 t = *(const ulonglong2 *)(T + ti + h * chalf);
                const u64 v0 = t.x ^ hx[2 * h], v1 = t.y ^ hx[2 * h + 1];
                if (xb_l) __stcs((ulonglong2 *)(xb_l + o + h * chalf), make_ulonglong2(v0, v1));
                if (x_l)
                    __stcs((double2 *)(x_l + o + h * chalf),
                           make_double2(to_float_bits(v0, e_float), to_float_bits(v1, e_float)));
            }
        } else {
            const u64 v0 = T[ti] ^ hx[0];
            if (xb_l) __stcs(xb_l + o, v0);
            if (x_l) __stcs(x_l + o, to_float_bits(v0, e_float));
        }
    }
}

template <bool GRAY, typename I>
__device__ __forceinline__ void gen_rows_i(const u64 *T, const u64 *H, u32 K, u32 ncols, u64 n_start, u64 d,
                                           u64 row_begin, u64 row_end, u64 *xb_l, double *x_l, int e_float)
{
    const bool vec2 = (ncols % 2 == 0) && (d % 2 == 0) && !(((uintptr_t)xb_l | (uintptr_t)x_l) & 15);
    if (vec2 && ncols % 4 == 0 && d % 4 == 0)
        gen_rows_vec<GRAY, 4, I>(T, H, K, ncols, n_start, d, row_begin, row_end, xb_l, x_l, e_float);
    else if (vec2)
        gen_rows_vec<GRAY, 2, I>(T, H, K, ncols, n_start, d, row_begin, row_end, xb_l, x_l, e_float);
    else
        gen_rows_vec<GRAY, 1, I>(T, H, K, ncols, n_start, d, row_begin, row_end, xb_l, x_l, e_float);
}

// VEC = 2 and 4 need an even row pitch and 16-byte aligned rows (d even and 16-byte aligned
// bases); 32-bit indices when n_start + row_end stays at or below 2^31, so that neither the
// index nor the row counter (stepped by R <= blockDim.x) can wrap.
template <bool GRAY>
__device__ __forceinline__ void gen_rows(const u64 *T, const u64 *H, u32 K, u32 ncols, u64 n_start, u64 d,
                                         u64 row_begin, u64 row_end, u64 *xb_l, double *x_l, int e_float)
{
    if (n_start + row_end <= (1ull << 31) && n_start + row_end >= n_start)
        gen_rows_i<GRAY, u32>(T, H, K, ncols, n_start, d, row_begin, row_end, xb_l, x_l, e_float);
    else
        gen_rows_i<GRAY, u64>(T, H, K, ncols, n_start, d, row_begin, row_end, xb_l, x_l, e_float);
}

}  // namespace
}  // namespace net
