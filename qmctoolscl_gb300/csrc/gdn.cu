// gdn.cu -- generalized digital nets (a base b per dimension, e.g. Halton):
// point digits in natural order, base-b linear matrix scrambling, digit
// permutation, digital shift, digits-to-float, interlacing and its inverse.
//
// Reference: qmctoolscl/c_funcs/gdn_gen_natural.c:3-53,
// gdn_gen_natural_same_base.c:3-63, gdn_linear_matrix_scramble.c:3-46,
// gdn_digital_permutation.c:3-46, gdn_digital_shift.c:3-45,
// gdn_integer_to_float.c:3-43, gdn_interlace.c:3-39,
// gdn_undo_interlace.c:3-39.
//
// Integer arithmetic.  The reference does everything in 64-bit unsigned
// arithmetic with a `%` after each step.  64-bit division is a long
// software sequence on the GPU, so the common case (base below 2^16, index
// and matrix entries below 2^32) runs in 32 bits with the direct-remainder
// method of Lemire, Kaser and Kurz (FastDiv32 in common.cuh); no
// intermediate value wraps there, so the reductions give the reference's
// numbers exactly.  Anything outside that domain takes a word-for-word
// 64-bit restatement of the reference's step, wrap-around included.
//
// Digits to float.  The reference sums recip_t*digit_t with recip_0 = 1/b
// and recip_{t+1} = recip_t/b, every operation rounded separately.  The
// recip_t depend only on (b, t): each CTA computes them once per dimension.
// The adds run on the FP64 unit (__dadd_rn), one per digit, and bound the
// kernel; the products RN(recip_t * digit) come from a shared-memory table
// of all (t, digit < b) when the CTA's tables fit in 16 KB, else from an
// integer 53x11-bit product with its rounding (dsum::mul_small) for digits
// below 2^11, else from __dmul_rn out of line.  (Emulating the adds in
// integer arithmetic as well measured about a hundred ALU instructions per
// digit with the ALU pipe 91% busy.)
//
// Layout in HBM: xdig is r*n*d*tmax (digit t fastest), C is r*d*mmax*tmax,
// S is r*d*tmax_new*tmax, perms r*d*tmax_new*bmax.  Per-point kernels walk
// (row, dimension, digit) as one flat run so stores are contiguous.
#include "common.cuh"
#include "digit_sum.cuh"

namespace {

constexpr int THREADS = 256;
constexpr u32 DIM_TILE = 256;  // dimensions per CTA (shared per-dimension tables)

struct DimInfo {
    u64 b;
    FastDiv32 fd;
    u32 small;  // b in [2, 2^16): 32-bit fast path
};

__device__ __forceinline__ DimInfo make_dim(u64 b)
{
    DimInfo di;
    di.b = b;
    di.small = (b >= 2 && b < 65536) ? 1u : 0u;
    di.fd = fastdiv32_make(di.small ? (u32)b : 2u);
    return di;
}

// x / d for 32-bit x and a divisor fixed for the launch (d >= 1): the high
// word of the 64x32-bit product M*x with M = floor((2^64-1)/d) + 1
struct Div32 {
    u64 M;
    u32 d;
};

__host__ __device__ inline Div32 div32_make(u32 d) { return Div32{fastdiv32_make(d).M, d}; }
__device__ __forceinline__ Div32 div32_dev(u32 d) { return div32_make(d); }

__device__ __forceinline__ u32 div32(const Div32 &v, u32 x)
{
    if (v.d == 1) return x;
    const u64 lo = (u64)(u32)v.M * x;
    return (u32)(((v.M >> 32) * x + (lo >> 32)) >> 32);
}

// C entry (k, t) of the current (l, j) block, read the way the reference
// reads it (flat index), and recorded as an error when that index falls
// outside the array.
__device__ __forceinline__ u64 read_flat(const u64 *base, u64 flat, u64 total, unsigned *err)
{
    if (flat < total) return base[flat];
    atomicOr(err, 1u);
    return 0;
}

// One digit of a generalized-net point: the reference's loop over the
// base-b digits of itrue (gdn_gen_natural.c:37-50).
__device__ u64 gdn_point_digit(const DimInfo &di, u64 itrue, const u64 *C, u64 c_off, u64 tmax, u64 t,
                               u64 c_total, unsigned *err)
{
    if (di.b < 2) {
        // the reference divides by zero (b = 0) or never leaves its digit
        // loop (b = 1); record the error instead of looping
        atomicOr(err, 2u);
        return 0;
    }
    if (di.small && itrue < (1ull << 32)) {
        // The reference reduces after every digit; with digits below 2^16 and matrix entries
        // below 2^32 each product is below 2^48 and the at most 32 products of a 32-bit index sum
        // to below 2^53 without wrapping, so one reduction at the end gives the same digit.
        u32 x = (u32)itrue;
        const u32 b32 = (u32)di.b;
        u64 acc = 0;
        bool ok = true;
        for (u64 k = 0; x; k++) {
            const u32 q = fd_div(di.fd, x);
            const u32 dig = x - q * b32;
            x = q;
            if (dig) {
                const u64 cv = read_flat(C, c_off + k * tmax + t, c_total, err);
                if (cv >> 32) { ok = false; break; }
                acc += (u64)dig * cv;
            }
        }
        if (ok) return acc < (1ull << 32) ? (u64)fd_mod(di.fd, (u32)acc) : acc % di.b;
    }
    const u64 b = di.b;
    u64 out = 0, icp = itrue;
    for (u64 k = 0; icp > 0; k++) {
        const u64 dig = icp % b;
        icp = (icp - dig) / b;
        if (dig > 0) out = (out + dig * read_flat(C, c_off + k * tmax + t, c_total, err)) % b;
    }
    return out;
}

// Grid: x = row blocks, y = randomisation * dimension tiles.
struct PointGrid {
    u64 rows_per_cta;
    u32 dim_tiles;
    u32 narrow;  // rows_per_cta * (dims per tile * words per point) < 2^32: 32-bit index arithmetic
};

// (row within the CTA's run, dimension within the tile, word within the point) of run offset f
struct RunPos {
    u64 rr, t;
    u32 c;
};

__device__ __forceinline__ RunPos run_pos(u64 f, bool narrow, const Div32 &dv_row, const Div32 &dv_t, u64 per_row,
                                          u64 words)
{
    RunPos p;
    if (narrow) {  // 32-bit index arithmetic by multiply-high (point_grid checked the range)
        const u32 r32 = div32(dv_row, (u32)f), rem = (u32)f - r32 * (u32)per_row;
        p.c = div32(dv_t, rem);
        p.rr = r32;
        p.t = rem - p.c * (u32)words;
    } else {
        p.rr = f / per_row;
        const u64 rem = f - p.rr * per_row;
        p.c = (u32)(rem / words);
        p.t = rem - (u64)p.c * words;
    }
    return p;
}

// streaming kernels handle RUN_UNROLL elements per thread per iteration, all
// loads issued before any is used (bytes in flight to cover HBM latency)
constexpr u32 RUN_UNROLL = 4;
constexpr u32 RUN_UNROLL_1 = 8;  // single-word runs: twice the loads in flight

__device__ __forceinline__ void point_block(const PointGrid &pg, u64 d, u64 &l, u64 &j0, u32 &nd)
{
    l = (u64)blockIdx.y / pg.dim_tiles;
    const u32 tile = (u32)((u64)blockIdx.y % pg.dim_tiles);
    j0 = (u64)tile * DIM_TILE;
    nd = (u32)min((u64)DIM_TILE, d - j0);
}

__global__ void __launch_bounds__(THREADS) gdn_gen_kernel(u64 r, u64 n, u64 d, u64 r_b, u64 mmax, u64 tmax,
                                                          u64 n_start, const u64 *bases, u64 common_b,
                                                          const u64 *C, u64 *xdig, PointGrid pg, u64 l_off,
                                                          unsigned *err)
{
    __shared__ DimInfo dims[DIM_TILE];
    u64 l, j0;
    u32 nd;
    point_block(pg, d, l, j0, nd);
    l += l_off;
    if (l >= r) return;
    for (u32 c = threadIdx.x; c < nd; c += blockDim.x)
        dims[c] = make_dim(bases ? bases[(l % r_b) * d + j0 + c] : common_b);
    __syncthreads();
    const u64 row0 = (u64)blockIdx.x * pg.rows_per_cta;
    if (row0 >= n) return;
    const u64 rows = min(pg.rows_per_cta, n - row0);
    const u64 per_row = (u64)nd * tmax;
    const u64 total = rows * per_row;
    const u64 c_total = r * d * mmax * tmax;
    u64 *out = xdig + l * n * d * tmax + row0 * d * tmax + j0 * tmax;
    if (pg.narrow) {
        // the CTA's run fits 32 bits (point_grid): index arithmetic by multiply-high
        const Div32 dv_row = div32_dev((u32)per_row), dv_t = div32_dev((u32)tmax);  // this CTA's dimension count
        for (u32 f = threadIdx.x; f < (u32)total; f += THREADS) {
            const u32 rr = div32(dv_row, f), rem = f - rr * (u32)per_row;
            const u32 c = div32(dv_t, rem), t = rem - c * (u32)tmax;
            const u64 i = row0 + rr, j = j0 + c;
            out[(u64)rr * d * tmax + rem] =
                gdn_point_digit(dims[c], i + n_start, C, l * d * mmax * tmax + j * mmax * tmax, tmax, t, c_total, err);
        }
        return;
    }
    for (u64 f = threadIdx.x; f < total; f += THREADS) {
        const u64 rr = f / per_row, rem = f - rr * per_row;
        const u32 c = (u32)(rem / tmax);
        const u64 t = rem - (u64)c * tmax;
        const u64 i = row0 + rr, j = j0 + c;
        const u64 c_off = l * d * mmax * tmax + j * mmax * tmax;
        out[rr * d * tmax + rem] = gdn_point_digit(dims[c], i + n_start, C, c_off, tmax, t, c_total, err);
    }
}

// ---------------------------------------------------------------- tiled generation
//
// The common case of gdn_gen_natural (and _same_base): base in [2, 4096),
// indices below 2^32, generating-matrix entries below 2^32, every index with
// at most mmax base-b digits, mmax * tmax <= GT_MAX_CW, tmax <= GT_MAX_TMAX.
// A CTA owns one (randomisation, dimension) and a run of 32-point groups; its
// matrix, reduced mod b, sits in shared memory (with entries below 2^32 a
// digit times an entry cannot wrap, so reducing first gives the reference's
// digits).  Per group, the index splits as hi * b^K + lo with b^K >= 32: the
// 32 points have at most two distinct hi, whose contributions to every
// output digit the warp computes together.  When b^K * tmax words fit, the
// low digits' contributions to every output digit, reduced mod b, are a
// shared-memory table over lo built once per CTA, so an output word is two
// table reads, an add, a conditional subtract of b and a store, the words of
// a group written in order by consecutive lanes (coalesced runs); otherwise
// each lane adds its K low digits and the digits are staged per 32-digit
// chunk in shared memory.  A CTA outside the case runs the per-element code
// above for its block instead.
constexpr u32 GT_MAX_CW = 8192;    // matrix words staged per CTA (32 KB as u32)
constexpr u32 GT_MAX_TMAX = 256;
constexpr u32 GT_WARPS = THREADS / 32;

constexpr u32 GT_LT_WORDS = GT_WARPS * 32 * 33;  // the low-digit table, or the staging of the general loop
constexpr u32 GT_MAX_HD = 64;                      // high digits per index (indices below 2^32)

inline size_t gt_smem(u64 mmax, u64 tmax)
{
    return (((mmax * tmax + 3) & ~3ull) + GT_WARPS * 2 * tmax + GT_LT_WORDS + GT_WARPS * (64 + 2 * GT_MAX_HD)) *
           sizeof(u32);
}

__global__ void __launch_bounds__(THREADS) gdn_gen_tiled_kernel(u64 r, u64 n, u64 d, u64 r_b, u64 mmax, u64 tmax,
                                                                u64 n_start, const u64 *bases, u64 common_b,
                                                                const u64 *C, u64 *xdig, u64 groups_per_cta,
                                                                u64 unit_off, unsigned *err)
{
    extern __shared__ __align__(16) u32 gsm[];
    u32 *Cs = gsm;                                  // [mmax][tmax] entries mod b
    u32 *hi_tab = Cs + ((mmax * tmax + 3) & ~3ull); // [warp][2][tmax] (after the matrix, 16-byte aligned)
    u32 *stage = hi_tab + GT_WARPS * 2 * tmax;      // [warp][32][33], or the low-digit table [b^K][tmax]
    u32 *ptab = stage + GT_LT_WORDS;                // [warp][32][2] per point: high-sum and low-table offsets
    u32 *hdig = ptab + GT_WARPS * 64;               // [warp][2][GT_MAX_HD] high digits of the two high parts
    __shared__ u32 big;
    const u64 unit = unit_off + blockIdx.y;         // = l * d + j
    if (unit >= r * d) return;
    const u64 l = unit / d, j = unit % d;
    const u64 b = bases ? bases[(l % r_b) * d + j] : common_b;
    const u64 g0 = (u64)blockIdx.x * groups_per_cta;
    const u64 ngroups = (n + 31) / 32;
    if (g0 >= ngroups) return;
    const u64 g1 = min(ngroups, g0 + groups_per_cta);
    const u64 c_total = r * d * mmax * tmax, c_off = l * d * mmax * tmax + j * mmax * tmax;
    u64 *out = xdig + l * n * d * tmax + j * tmax;  // point i, digit t at out[i * d * tmax + t]
    const u32 warp = threadIdx.x / 32, lane = threadIdx.x % 32;

    // is this block in the tiled case?
    bool tiled = b >= 2 && b < 4096 && n_start + n <= (1ull << 32);
    if (tiled) {  // the last index has at most mmax base-b digits (else the reference reads past the block)
        u64 x = n_start + n - 1, k = 0;
        while (x) {
            x /= b;
            k++;
        }
        tiled = k <= mmax;
    }
    if (threadIdx.x == 0) big = 0;
    __syncthreads();
    if (tiled)
        for (u32 w = threadIdx.x; w < mmax * tmax; w += THREADS) {
            const u64 cv = C[c_off + w];
            if (cv >> 32) big = 1;
            Cs[w] = (u32)(cv % b);
        }
    __syncthreads();
    if (!tiled || big) {
        // the per-element code (reference order, 64-bit where needed), this CTA's points and dimension
        __shared__ DimInfo di_s;
        if (threadIdx.x == 0) di_s = make_dim(b);
        __syncthreads();
        const u64 i0 = g0 * 32, i1 = min(n, g1 * 32);
        for (u64 f = threadIdx.x; f < (i1 - i0) * tmax; f += THREADS) {
            const u64 i = i0 + f / tmax, t = f % tmax;
            out[i * d * tmax + t] = gdn_point_digit(di_s, i + n_start, C, c_off, tmax, t, c_total, err);
        }
        return;
    }
    const u32 b32 = (u32)b, T = (u32)tmax, M = (u32)mmax;
    const FastDiv32 fb = fastdiv32_make(b32);
    u32 K = 1, bK = b32;
    while (bK < 32) {
        bK *= b32;
        K++;
    }
    const FastDiv32 fK = fastdiv32_make(bK);
    const u32 KL = K < M ? K : M;  // low digits that can be nonzero (indices below b^mmax)
    u32 *ht = hi_tab + warp * 2 * T;
    if ((u64)bK * T <= GT_LT_WORDS && M - KL <= GT_MAX_HD && T >= 2) {
        // LT[lo * T + t]: the low digits' part of output digit t, mod b, for every lo < b^K
        u32 *LT = stage;
        for (u32 w = threadIdx.x; w < bK * T; w += THREADS) {
            const u32 lo = w / T, t = w - lo * T;
            u32 x = lo, acc = 0;
            for (u32 k = 0; k < KL; k++) {
                const u32 q = x / b32;
                acc += (x - q * b32) * Cs[k * T + t];  // < 5 * 4096^2
                x = q;
            }
            LT[w] = acc % b32;
        }
        __syncthreads();
        u32 *pw = ptab + warp * 64, *hd = hdig + warp * 2 * GT_MAX_HD;
        const u32 HD = M - KL;                               // high digits that can be nonzero
        const u32 mT = (u32)((0x100000000ull + T - 1) / T);  // e / T = umulhi(e, mT) for e < 2^13
        const u64 dT = d * tmax;
        for (u64 g = g0 + warp; g < g1; g += GT_WARPS) {
            const u64 i0 = g * 32;
            const u32 base = (u32)(n_start + i0);
            const u32 itrue = i0 + lane < n ? base + lane : base;
            const u32 h0 = fd_div(fK, base), hi = fd_div(fK, itrue);
            __syncwarp();  // the previous group's reads of hd, ht and pw are done
            // the base-b digits of the two high parts h0 and h0 + 1, lane k digit k
            for (u32 k = lane; k < HD; k += 32) {
#pragma unroll
                for (u32 sx = 0; sx < 2; sx++) {
                    u32 h = h0 + sx;
                    for (u32 e = 0; e < k && h; e++) h = fd_div(fb, h);
                    hd[sx * GT_MAX_HD + k] = h - fd_div(fb, h) * b32;
                }
            }
            pw[2 * lane] = (hi - h0) * T;
            pw[2 * lane + 1] = (itrue - hi * bK) * T;
            __syncwarp();
            // high-digit sums of both high parts for every output digit (gdn_gen_natural.c:37-50, k >= K)
            for (u32 t = lane; t < T; t += 32) {
                u32 a0 = 0, a1 = 0;
                for (u32 k = 0; k < HD; k++) {
                    const u32 c = Cs[(KL + k) * T + t];
                    a0 += hd[k] * c;  // < 64 * 4096^2 = 2^30
                    a1 += hd[GT_MAX_HD + k] * c;
                }
                ht[t] = fd_mod(fb, a0);
                ht[T + t] = fd_mod(fb, a1);
            }
            __syncwarp();
            // the group's npts x T words in output order, one per lane
            const u32 words = (u32)min((u64)32, n - i0) * T;
            u64 *ot = out + i0 * dT;
            for (u32 e = lane; e < words; e += 32) {
                const u32 p = __umulhi(e, mT), t = e - p * T;
                const uint2 po = *(const uint2 *)&pw[2 * p];
                u32 acc = ht[po.x + t] + LT[po.y + t];  // both below b
                acc = min(acc, acc - b32);
                if (dT == T)
                    ot[e] = acc;
                else
                    ot[(u64)p * dT + t] = acc;
            }
        }
        return;
    }
    u32 *sg = stage + warp * 32 * 33;
    for (u64 g = g0 + warp; g < g1; g += GT_WARPS) {
        const u64 i0 = g * 32;
        const u32 base = (u32)(n_start + i0);
        const bool active = i0 + lane < n;
        const u32 itrue = active ? base + lane : base;
        const u32 h0 = fd_div(fK, base), hi = fd_div(fK, itrue);
        const u32 sel = hi - h0;  // 0 or 1
        u32 dl[5];
        {
            u32 x = itrue - hi * bK;
#pragma unroll
            for (u32 k = 0; k < 5; k++) {
                const u32 q = fd_div(fb, x);
                dl[k] = x - q * b32;
                x = q;
            }
        }
        // high-digit sums of both hi values for every output digit (gdn_gen_natural.c:37-50 for k >= K)
        __syncwarp();
        for (u32 t = lane; t < T; t += 32) {
#pragma unroll
            for (u32 s = 0; s < 2; s++) {
                u32 h = h0 + s, acc = 0;
                for (u32 k = K; h && k < M; k++) {
                    const u32 q = fd_div(fb, h);
                    acc += (h - q * b32) * Cs[k * T + t];  // < 64 * 4096^2 = 2^30
                    h = q;
                }
                ht[s * T + t] = fd_mod(fb, acc);
            }
        }
        __syncwarp();
        const u32 npts = (u32)min((u64)32, n - i0);
        for (u32 t0 = 0; t0 < T; t0 += 32) {
            const u32 tw = min(32u, T - t0);
            for (u32 tt = 0; tt < tw; tt++) {
                const u32 t = t0 + tt;
                u32 acc = ht[sel * T + t];
#pragma unroll
                for (u32 k = 0; k < 5; k++)
                    if (k < KL) acc += dl[k] * Cs[k * T + t];  // < 4096 + 5 * 4096^2 < 2^27
                sg[lane * 33 + tt] = fd_mod(fb, acc);
            }
            __syncwarp();
            // the npts x tw block: contiguous runs of tw words per point
            if (tw == 32) {
                for (u32 p = 0; p < npts; p++) out[(i0 + p) * d * tmax + t0 + lane] = sg[p * 33 + lane];
            } else if ((tw & (tw - 1)) == 0) {  // a power of two: index by shift and mask
                const u32 sh = 31 - __clz((int)tw);
                for (u32 e = lane; e < npts * tw; e += 32) {
                    const u32 p = e >> sh, tt = e & (tw - 1);
                    out[(i0 + p) * d * tmax + t0 + tt] = sg[p * 33 + tt];
                }
            } else {
                for (u32 e = lane; e < npts * tw; e += 32) {
                    const u32 p = e / tw, tt = e - p * tw;
                    out[(i0 + p) * d * tmax + t0 + tt] = sg[p * 33 + tt];
                }
            }
            __syncwarp();
        }
    }
}

// (digit + shift) mod b as gdn_digital_shift.c:38 computes it (the sum wraps in 64 bits); a base
// of 0 is reported, never divided by
__device__ __forceinline__ u64 shift_mod(const DimInfo &di, u64 sum, unsigned *err)
{
    if (di.b == 0) {
        atomicOr(err, 2u);
        return 0;
    }
    return (di.small && sum < (1ull << 32)) ? (u64)fd_mod(di.fd, (u32)sum) : sum % di.b;
}

// at most 64 registers (4 CTAs per SM): its general path alone would take 72 and leave 3 CTAs, too
// few loads in flight for the streaming paths (0.64-0.82 of the copy peak; 0.74-0.91 capped)
__global__ void __launch_bounds__(THREADS, 4) gdn_shift_kernel(u64 r, u64 n, u64 d, u64 r_x, u64 r_b, u64 tmax,
                                                            u64 tmax_new, const u64 *bases, const u64 *shifts,
                                                            const u64 *xdig, u64 *xdig_new, PointGrid pg,
                                                            u64 l_off, u32 lin, unsigned *err)
{
    __shared__ DimInfo dims[DIM_TILE];
    u64 l, j0;
    u32 nd;
    point_block(pg, d, l, j0, nd);
    l += l_off;
    if (l >= r) return;
    for (u32 c = threadIdx.x; c < nd; c += blockDim.x) dims[c] = make_dim(bases[(l % r_b) * d + j0 + c]);
    __syncthreads();
    const u64 row0 = (u64)blockIdx.x * pg.rows_per_cta;
    if (row0 >= n) return;
    const u64 rows = min(pg.rows_per_cta, n - row0);
    const u64 per_row = (u64)nd * tmax_new;
    const u64 total = rows * per_row;
    const Div32 dv_row = div32_dev(pg.narrow ? (u32)per_row : 1u), dv_t = div32_dev(pg.narrow ? (u32)tmax_new : 1u);
    if (lin == 1) {
        // host-checked: the tile holds every dimension, tmax == tmax_new, per_row even, arrays 16-byte
        // aligned, the run below 2^32 words: input and output are contiguous runs, read and written
        // two words at a time; word f of the run is digit sidx = f mod per_row of its point
        const ulonglong2 *src = (const ulonglong2 *)(xdig + (l % r_x) * n * d * tmax + row0 * per_row);
        ulonglong2 *dst = (ulonglong2 *)(xdig_new + l * n * d * tmax + row0 * per_row);
        const u64 *shl = shifts + l * per_row;
        const u32 npair = (u32)(total / 2);
        for (u32 q0 = threadIdx.x; q0 < npair; q0 += RUN_UNROLL * THREADS) {
            ulonglong2 xv[RUN_UNROLL];
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL; u++) {
                const u32 q = q0 + u * THREADS;
                if (q < npair) xv[u] = src[q];
            }
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL; u++) {
                const u32 q = q0 + u * THREADS;
                if (q >= npair) continue;
                const u32 sidx = 2 * q - div32(dv_row, 2 * q) * (u32)per_row;  // even, sidx + 1 < per_row
                // the sums wrap as in C
                dst[q] = make_ulonglong2(shift_mod(dims[div32(dv_t, sidx)], xv[u].x + shl[sidx], err),
                                         shift_mod(dims[div32(dv_t, sidx + 1)], xv[u].y + shl[sidx + 1], err));
            }
        }
        return;
    }
    if (lin == 2) {
        // contiguous runs read and written one word at a time (odd words per point or unaligned arrays)
        const u64 *src = xdig + (l % r_x) * n * d * tmax + row0 * per_row;
        u64 *dst = xdig_new + l * n * d * tmax + row0 * per_row;
        const u64 *shl = shifts + l * per_row;
        for (u32 f0 = threadIdx.x; f0 < (u32)total; f0 += RUN_UNROLL_1 * THREADS) {
            u64 xv[RUN_UNROLL_1];
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL_1; u++) {
                const u32 f = f0 + u * THREADS;
                if (f < (u32)total) xv[u] = src[f];
            }
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL_1; u++) {
                const u32 f = f0 + u * THREADS;
                if (f >= (u32)total) continue;
                const u32 sidx = f - div32(dv_row, f) * (u32)per_row;
                dst[f] = shift_mod(dims[div32(dv_t, sidx)], xv[u] + shl[sidx], err);  // the sum wraps as in C
            }
        }
        return;
    }
    for (u64 f0 = threadIdx.x; f0 < total; f0 += RUN_UNROLL * THREADS) {
        RunPos ps[RUN_UNROLL];
        u64 sh[RUN_UNROLL], xv[RUN_UNROLL];
#pragma unroll
        for (u32 u = 0; u < RUN_UNROLL; u++) {
            const u64 f = f0 + u * THREADS;
            sh[u] = xv[u] = 0;
            if (f >= total) continue;
            ps[u] = run_pos(f, pg.narrow, dv_row, dv_t, per_row, tmax_new);
            const u64 i = row0 + ps[u].rr, j = j0 + ps[u].c;
            sh[u] = shifts[l * d * tmax_new + j * tmax_new + ps[u].t];
            if (ps[u].t < tmax) xv[u] = xdig[(l % r_x) * n * d * tmax + i * d * tmax + j * tmax + ps[u].t];
        }
#pragma unroll
        for (u32 u = 0; u < RUN_UNROLL; u++) {
            const u64 f = f0 + u * THREADS;
            if (f >= total) continue;
            const u64 i = row0 + ps[u].rr, j = j0 + ps[u].c, t = ps[u].t;
            u64 v;
            if (t < tmax) {
                v = shift_mod(dims[ps[u].c], xv[u] + sh[u], err);  // the sum wraps as in C
            } else {
                v = sh[u];
            }
            xdig_new[l * n * d * tmax_new + i * d * tmax_new + j * tmax_new + t] = v;
        }
    }
}

__global__ void __launch_bounds__(THREADS) gdn_perm_kernel(u64 r, u64 n, u64 d, u64 r_x, u64 tmax, u64 tmax_new,
                                                           u64 bmax, const u64 *perms, const u64 *xdig,
                                                           u64 *xdig_new, PointGrid pg, u64 l_off, u32 lin,
                                                           unsigned *err)
{
    u64 l, j0;
    u32 nd;
    point_block(pg, d, l, j0, nd);
    l += l_off;
    if (l >= r) return;
    const u64 row0 = (u64)blockIdx.x * pg.rows_per_cta;
    if (row0 >= n) return;
    const u64 rows = min(pg.rows_per_cta, n - row0);
    const u64 per_row = (u64)nd * tmax_new;
    const u64 total = rows * per_row, p_total = r * d * tmax_new * bmax;
    const Div32 dv_row = div32_dev(pg.narrow ? (u32)per_row : 1u), dv_t = div32_dev(pg.narrow ? (u32)tmax_new : 1u);
    if (lin == 1) {
        // host-checked as in gdn_shift_kernel: contiguous runs, two words at a time; the table row of
        // digit sidx of the point starts at (l * d * tmax + sidx) * bmax
        const ulonglong2 *src = (const ulonglong2 *)(xdig + (l % r_x) * n * d * tmax + row0 * per_row);
        ulonglong2 *dst = (ulonglong2 *)(xdig_new + l * n * d * tmax + row0 * per_row);
        const u64 prow0 = l * per_row * bmax;
        const u32 npair = (u32)(total / 2);
        for (u32 q0 = threadIdx.x; q0 < npair; q0 += RUN_UNROLL * THREADS) {
            ulonglong2 xv[RUN_UNROLL];
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL; u++) {
                const u32 q = q0 + u * THREADS;
                if (q < npair) xv[u] = src[q];
            }
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL; u++) {
                const u32 q = q0 + u * THREADS;
                if (q >= npair) continue;
                const u32 sidx = 2 * q - div32(dv_row, 2 * q) * (u32)per_row;
                xv[u].x = read_flat(perms, prow0 + (u64)sidx * bmax + xv[u].x, p_total, err);
                xv[u].y = read_flat(perms, prow0 + (u64)(sidx + 1) * bmax + xv[u].y, p_total, err);
            }
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL; u++) {
                const u32 q = q0 + u * THREADS;
                if (q < npair) dst[q] = xv[u];
            }
        }
        return;
    }
    if (lin == 2) {
        // contiguous runs one word at a time (odd words per point or unaligned arrays)
        const u64 *src = xdig + (l % r_x) * n * d * tmax + row0 * per_row;
        u64 *dst = xdig_new + l * n * d * tmax + row0 * per_row;
        const u64 prow0 = l * per_row * bmax;
        for (u32 f0 = threadIdx.x; f0 < (u32)total; f0 += RUN_UNROLL_1 * THREADS) {
            u64 xv[RUN_UNROLL_1];
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL_1; u++) {
                const u32 f = f0 + u * THREADS;
                if (f < (u32)total) xv[u] = src[f];
            }
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL_1; u++) {
                const u32 f = f0 + u * THREADS;
                if (f >= (u32)total) continue;
                const u32 sidx = f - div32(dv_row, f) * (u32)per_row;
                xv[u] = read_flat(perms, prow0 + (u64)sidx * bmax + xv[u], p_total, err);
            }
#pragma unroll
            for (u32 u = 0; u < RUN_UNROLL_1; u++) {
                const u32 f = f0 + u * THREADS;
                if (f < (u32)total) dst[f] = xv[u];
            }
        }
        return;
    }
    for (u64 f0 = threadIdx.x; f0 < total; f0 += RUN_UNROLL * THREADS) {
        RunPos ps[RUN_UNROLL];
        u64 pv[RUN_UNROLL];
#pragma unroll
        for (u32 u = 0; u < RUN_UNROLL; u++) {
            const u64 f = f0 + u * THREADS;
            pv[u] = 0;
            if (f >= total) continue;
            ps[u] = run_pos(f, pg.narrow, dv_row, dv_t, per_row, tmax_new);
            const u64 i = row0 + ps[u].rr, j = j0 + ps[u].c;
            if (ps[u].t < tmax) pv[u] = xdig[(l % r_x) * n * d * tmax + i * d * tmax + j * tmax + ps[u].t];
        }
#pragma unroll
        for (u32 u = 0; u < RUN_UNROLL; u++) {
            const u64 f = f0 + u * THREADS;
            if (f >= total) continue;
            const u64 flat = l * d * tmax_new * bmax + (j0 + ps[u].c) * tmax_new * bmax + ps[u].t * bmax + pv[u];
            pv[u] = read_flat(perms, flat, p_total, err);
        }
#pragma unroll
        for (u32 u = 0; u < RUN_UNROLL; u++) {
            const u64 f = f0 + u * THREADS;
            if (f >= total) continue;
            const u64 i = row0 + ps[u].rr, j = j0 + ps[u].c;
            xdig_new[l * n * d * tmax_new + i * d * tmax_new + j * tmax_new + ps[u].t] = pv[u];
        }
    }
}

// recip_t of gdn_integer_to_float.c:34-38 for t < tmax, per dimension
__device__ __forceinline__ void fill_recips(double *rc, u64 b, u64 tmax)
{
    const double bd = __ull2double_rn(b);
    double rcp = __ddiv_rn(1.0, bd);
    for (u64 t = 0; t < tmax; t++) {
        rc[t] = rcp;
        rcp = __ddiv_rn(rcp, bd);
    }
}

// one step v + recip*digit with FP64 instructions, out of line (see
// to_float_hw in dnb2.cu for why)
__device__ __noinline__ u64 digit_step_hw(u64 v, double rc, u64 dg)
{
    return as_bits(__dadd_rn(as_double(v), __dmul_rn(rc, __ull2double_rn(dg))));
}

// one term of the sum: v = RN(v + RN(recip * digit)), gdn_integer_to_float.c:36-37; the
// product in integer arithmetic for digits below 2^11 (dsum::mul_small, exact RN) and the
// add on the FP64 unit, whose throughput bounds this kernel
__device__ __forceinline__ u64 digit_term(u64 v, double rc, u64 dg)
{
    if (dg == 0) return v;  // adds +0: v unchanged
    const u64 rb = as_bits(rc);
    if (dg < 2048 && rb >= (24ull << 52))  // recip >= 2^-999: the product stays normal
        return as_bits(__dadd_rn(as_double(v), as_double(dsum::mul_small(rb, (u32)dg))));
    return digit_step_hw(v, rc, dg);
}

// v = sum_t recip_t * digit_t with the reference's rounding sequence; the
// digits are read eight at a time (16-byte loads when the run is 16-byte
// aligned and of even length), independent loads in flight
__device__ __forceinline__ double digits_to_double(const double *rc, const u64 *dig, u64 tmax)
{
    u64 v = 0;  // bits of a non-negative double
    if ((tmax & 1) == 0 && ((uintptr_t)dig & 15) == 0) {
        const ulonglong2 *d2 = (const ulonglong2 *)dig;
        for (u64 t0 = 0; t0 < tmax; t0 += 8) {
            ulonglong2 q[4];
#pragma unroll
            for (u32 u = 0; u < 4; u++) q[u] = t0 + 2 * u < tmax ? d2[t0 / 2 + u] : make_ulonglong2(0, 0);
#pragma unroll
            for (u32 u = 0; u < 4; u++) {
                if (t0 + 2 * u >= tmax) break;
                v = digit_term(v, rc[t0 + 2 * u], q[u].x);
                v = digit_term(v, rc[t0 + 2 * u + 1], q[u].y);
            }
        }
        return as_double(v);
    }
    for (u64 t0 = 0; t0 < tmax; t0 += 4) {
        u64 dg4[4];
#pragma unroll
        for (u32 u = 0; u < 4; u++) dg4[u] = t0 + u < tmax ? dig[t0 + u] : 0;
#pragma unroll
        for (u32 u = 0; u < 4; u++)
            if (t0 + u < tmax) v = digit_term(v, rc[t0 + u], dg4[u]);
    }
    return as_double(v);
}

// RN(recip * (double)dg) for the digits beyond the term table, out of line
__device__ __noinline__ double term_hw(double rc, u64 dg) { return __dmul_rn(rc, __ull2double_rn(dg)); }

// term t of a digit: the table entry RN(recip_t * dg) for dg < b (T[t * b + dg]), else the
// product itself (recip_t = T[t * b + 1])
__device__ __forceinline__ double tbl_term(const double *T, u32 b, u64 t, u64 dg)
{
    const u32 row = (u32)t * b;
    return dg < b ? T[row + (u32)dg] : term_hw(T[row + 1], dg);
}

// digits_to_double with the products from the term table: one FP64 operation per digit
__device__ __forceinline__ double digits_to_double_tbl(const double *T, u32 b, const u64 *dig, u64 tmax)
{
    double v = 0.0;
    if ((tmax & 1) == 0 && ((uintptr_t)dig & 15) == 0) {
        const ulonglong2 *d2 = (const ulonglong2 *)dig;
        for (u64 t0 = 0; t0 < tmax; t0 += 8) {
            ulonglong2 q[4];
#pragma unroll
            for (u32 u = 0; u < 4; u++) q[u] = t0 + 2 * u < tmax ? d2[t0 / 2 + u] : make_ulonglong2(0, 0);
#pragma unroll
            for (u32 u = 0; u < 4; u++) {
                if (t0 + 2 * u >= tmax) break;
                v = __dadd_rn(v, tbl_term(T, b, t0 + 2 * u, q[u].x));  // gdn_integer_to_float.c:37
                v = __dadd_rn(v, tbl_term(T, b, t0 + 2 * u + 1, q[u].y));
            }
        }
        return v;
    }
    for (u64 t0 = 0; t0 < tmax; t0 += 8) {
        u64 dg8[8];
#pragma unroll
        for (u32 u = 0; u < 8; u++) dg8[u] = t0 + u < tmax ? dig[t0 + u] : 0;
#pragma unroll
        for (u32 u = 0; u < 8; u++)
            if (t0 + u < tmax) v = __dadd_rn(v, tbl_term(T, b, t0 + u, dg8[u]));
    }
    return v;
}

constexpr u32 I2F_DIMS = 32;            // dimensions per CTA
constexpr u32 I2F_TMAX = 64;            // recip table depth held in shared memory
constexpr u32 I2F_SMEM_WORDS = 2048;    // dynamic shared memory (16 KB, 8 CTAs per SM): term or recip table
enum I2fMode { I2F_LOOP = 0, I2F_RECIP = 1, I2F_TERMS = 2 };

// Each CTA converts a run of points for up to 32 dimensions.  When the CTA's
// term tables -- RN(recip_t * dg) for t < tmax, dg < b, per dimension -- fit
// in 16 KB, the products come from shared memory and only the adds run on the
// FP64 unit; else a table of recip_t (tmax <= 64), else the reference's loop.
__global__ void __launch_bounds__(THREADS) gdn_to_float_kernel(u64 r, u64 n, u64 d, u64 r_b, u64 tmax,
                                                               const u64 *bases, const u64 *xdig, double *x,
                                                               u64 rows_per_cta, u32 dim_tiles, u64 l_off)
{
    extern __shared__ __align__(16) double i2f_sm[];
    __shared__ u32 toff[I2F_DIMS + 1], tb[I2F_DIMS], mode;
    const u64 l = l_off + (u64)blockIdx.y / dim_tiles;
    if (l >= r) return;
    const u64 j0 = (u64)(blockIdx.y % dim_tiles) * I2F_DIMS;
    const u32 nd = (u32)min((u64)I2F_DIMS, d - j0);
    const u64 *bl = bases + (l % r_b) * d + j0;
    if (threadIdx.x == 0) {
        u64 acc = 0;
        bool fits = tmax <= I2F_TMAX;
        for (u32 c = 0; c < nd && fits; c++) {
            const u64 b = bl[c];
            fits = b >= 2 && b <= I2F_SMEM_WORDS;
            toff[c] = (u32)acc;
            tb[c] = (u32)b;
            acc += tmax * b;
            fits = fits && acc <= I2F_SMEM_WORDS;
        }
        toff[nd] = (u32)acc;
        mode = fits ? I2F_TERMS : tmax <= I2F_TMAX ? I2F_RECIP : I2F_LOOP;
    }
    __syncthreads();
    if (mode == I2F_TERMS) {
        // recip_t into column 1 of each row, then every entry from its row's recip
        for (u32 c = threadIdx.x; c < nd; c += blockDim.x) {
            const u32 b = tb[c];
            const double bd = __ull2double_rn(b);
            double rcp = __ddiv_rn(1.0, bd);
            for (u32 t = 0; t < (u32)tmax; t++) {
                i2f_sm[toff[c] + t * b] = 0.0;
                i2f_sm[toff[c] + t * b + 1] = rcp;
                rcp = __ddiv_rn(rcp, bd);
            }
        }
        __syncthreads();
        for (u32 c = 0; c < nd; c++) {
            const u32 b = tb[c], cnt = (u32)tmax * b;
            double *T = i2f_sm + toff[c];
            for (u32 k = threadIdx.x; k < cnt; k += blockDim.x) {
                const u32 t = k / b, dg = k - t * b;
                if (dg >= 2) T[k] = __dmul_rn(T[t * b + 1], (double)dg);
            }
        }
    } else if (mode == I2F_RECIP) {
        for (u32 c = threadIdx.x; c < nd; c += blockDim.x) fill_recips(i2f_sm + c * I2F_TMAX, bl[c], tmax);
    }
    __syncthreads();
    const u64 row0 = (u64)blockIdx.x * rows_per_cta;
    if (row0 >= n) return;
    const u64 rows = min(rows_per_cta, n - row0);
    const u64 total = rows * nd;
    const Div32 dv_nd = div32_dev(nd);
    for (u64 f = threadIdx.x; f < total; f += THREADS) {
        const u64 rr = total < (1ull << 32) ? (u64)div32(dv_nd, (u32)f) : f / nd;
        const u32 c = (u32)(f - rr * nd);
        const u64 i = row0 + rr, j = j0 + c;
        const u64 *dg = xdig + l * n * d * tmax + i * d * tmax + j * tmax;
        double v;
        if (mode == I2F_TERMS) {
            v = digits_to_double_tbl(i2f_sm + toff[c], tb[c], dg, tmax);
        } else if (mode == I2F_RECIP) {
            v = digits_to_double(i2f_sm + c * I2F_TMAX, dg, tmax);
        } else {  // deep digit expansions: the reference's loop as written
            const double bd = __ull2double_rn(bl[c]);
            double rcp = __ddiv_rn(1.0, bd);
            v = 0.0;
            for (u64 t = 0; t < tmax; t++) {
                v = __dadd_rn(v, __dmul_rn(rcp, __ull2double_rn(dg[t])));
                rcp = __ddiv_rn(rcp, bd);
            }
        }
        x[l * n * d + i * d + j] = v;
    }
}

// ---------------------------------------------------------------- matrices

__global__ void gdn_lms_kernel(u64 r, u64 d, u64 mmax, u64 r_C, u64 r_b, u64 tmax, u64 tmax_new, const u64 *bases,
                               const u64 *S, const u64 *C, u64 *C_lms, unsigned *err)
{
    const u64 total = r * d * mmax * tmax_new;
    u64 cached_b = 0;
    DimInfo di = make_dim(2);
    for (u64 f = (u64)blockIdx.x * blockDim.x + threadIdx.x; f < total; f += (u64)gridDim.x * blockDim.x) {
        const u64 t = f % tmax_new, k = (f / tmax_new) % mmax, j = (f / (tmax_new * mmax)) % d;
        const u64 l = f / (tmax_new * mmax * d);
        const u64 b = bases[(l % r_b) * d + j];
        if (b != cached_b) {
            di = make_dim(b);
            cached_b = b;
        }
        if (b == 0) {  // the reference divides by zero
            atomicOr(err, 2u);
            C_lms[f] = 0;
            continue;
        }
        const u64 *col = C + (l % r_C) * d * mmax * tmax + j * mmax * tmax + k * tmax;
        const u64 *srow = S + l * d * tmax_new * tmax + j * tmax_new * tmax + t * tmax;
        u64 acc = 0;
        for (u64 c = 0; c < tmax; c++) {
            const u64 sv = srow[c], cv = col[c];
            if (di.small && !((sv | cv) >> 32)) {
                // both below 2^32: the product does not wrap, reduce the factors first
                acc += fd_mod(di.fd, fd_mod(di.fd, (u32)sv) * fd_mod(di.fd, (u32)cv));
            } else {
                acc += (sv * cv) % b;  // 64-bit product wraps as in C
            }
        }
        C_lms[f] = acc;
    }
}

__global__ void gdn_interlace_kernel(u64 r, u64 d_alpha, u64 mmax, u64 d, u64 tmax, u64 tmax_alpha, u64 alpha,
                                     const u64 *C, u64 *C_alpha, unsigned *err)
{
    const u64 total = r * d_alpha * mmax * tmax_alpha, c_total = r * d * mmax * tmax;
    for (u64 f = (u64)blockIdx.x * blockDim.x + threadIdx.x; f < total; f += (u64)gridDim.x * blockDim.x) {
        const u64 ta = f % tmax_alpha, k = (f / tmax_alpha) % mmax, ja = (f / (tmax_alpha * mmax)) % d_alpha;
        const u64 l = f / (tmax_alpha * mmax * d_alpha);
        const u64 t = ta / alpha, j = ja * alpha + ta % alpha;
        C_alpha[f] = read_flat(C, l * d * mmax * tmax + j * mmax * tmax + k * tmax + t, c_total, err);
    }
}

__global__ void gdn_undo_interlace_kernel(u64 r, u64 d, u64 mmax, u64 d_alpha, u64 tmax, u64 tmax_alpha, u64 alpha,
                                          const u64 *C_alpha, u64 *C, unsigned *err)
{
    const u64 total = r * d * mmax * tmax, a_total = r * d_alpha * mmax * tmax_alpha;
    for (u64 f = (u64)blockIdx.x * blockDim.x + threadIdx.x; f < total; f += (u64)gridDim.x * blockDim.x) {
        const u64 t = f % tmax, k = (f / tmax) % mmax, j = (f / (tmax * mmax)) % d;
        const u64 l = f / (tmax * mmax * d);
        const u64 ja = j / alpha, ta = t * alpha + j % alpha;
        C[f] = read_flat(C_alpha, l * d_alpha * mmax * tmax_alpha + ja * mmax * tmax_alpha + k * tmax_alpha + ta,
                         a_total, err);
    }
}

// ---------------------------------------------------------------- host side

unsigned flat_grid(u64 total) { return qmcgb::grid_for(total, 256, (unsigned)qmcgb::sm_count() * 32); }

// ctas_per_sm: CTAs asked for per SM (several waves of short row runs balance the SMs best for
// the streaming kernels: measured 32 for permutation and shift, 16 for integer-to-float)
PointGrid point_grid(u64 r, u64 n, u64 d, u64 per_point, u32 dim_tile, u64 *splits_out, u32 ctas_per_sm = 8)
{
    PointGrid pg;
    pg.dim_tiles = (u32)((d + dim_tile - 1) / dim_tile);
    const u64 units = r * pg.dim_tiles;
    const u64 want = (u64)qmcgb::sm_count() * ctas_per_sm;
    u64 splits = (want + units - 1) / units;
    // at least ~2 elements per thread in a CTA
    const u64 per_row = (d < dim_tile ? d : dim_tile) * (per_point ? per_point : 1);
    const u64 min_rows = (2 * THREADS + per_row - 1) / per_row;
    const u64 max_splits = (n + min_rows - 1) / min_rows;
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    pg.rows_per_cta = (n + splits - 1) / splits;
    *splits_out = splits;
    pg.narrow = per_row < (1ull << 32) && pg.rows_per_cta * per_row < (1ull << 32) ? 1u : 0u;
    return pg;
}

// launch over blockIdx.y = (randomisation, dimension tile) in chunks of 65535
template <typename F>
int launch_points(u64 r, u32 dim_tiles, F &&launch_chunk, const char *what)
{
    const u64 l_per = 65535 / dim_tiles;
    for (u64 l0 = 0; l0 < r; l0 += l_per) {
        const u64 cnt = (r - l0 < l_per ? r - l0 : l_per) * dim_tiles;
        launch_chunk(l0, (unsigned)cnt);
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    return QMC_OK;
}

// the digit-wise kernels' contiguous-run form: 0 = no (several dimension tiles, digit counts that
// differ, runs of 2^32 words or more), 1 = pairs of words (an even number of words per point,
// 16-byte aligned arrays), 2 = single words
u32 linear_run(const PointGrid &pg, u64 d, u64 tmax, u64 tmax_new, const void *in, const void *out)
{
    if (!(pg.narrow && pg.dim_tiles == 1 && d <= DIM_TILE && tmax == tmax_new)) return 0u;
    return (d * tmax) % 2 == 0 && (((uintptr_t)in | (uintptr_t)out) & 15) == 0 ? 1u : 2u;
}

// grid of the tiled generation: y = (randomisation, dimension) units in chunks of 65535, x = runs of
// 32-point groups sized so the whole launch has about 8 CTAs per SM
int gen_tiled(u64 r, u64 n, u64 d, u64 r_b, u64 mmax, u64 tmax, u64 n_start, const u64 *bases, u64 common_b,
              const u64 *C, u64 *xdig, cudaStream_t st, unsigned *err, const char *what)
{
    const u64 units = r * d, ngroups = (n + 31) / 32;
    const u64 want = (u64)qmcgb::sm_count() * 8;
    u64 splits = (want + units - 1) / units;
    if (splits > ngroups) splits = ngroups;
    if (splits < 1) splits = 1;
    const u64 groups_per_cta = (ngroups + splits - 1) / splits;
    const u64 nx = (ngroups + groups_per_cta - 1) / groups_per_cta;
    const size_t smem = gt_smem(mmax, tmax);
    if (int rc = qmcgb::raise_smem_limit((const void *)gdn_gen_tiled_kernel, smem, what)) return rc;
    for (u64 u0 = 0; u0 < units; u0 += 65535) {
        const unsigned cnt = (unsigned)(units - u0 < 65535 ? units - u0 : 65535);
        gdn_gen_tiled_kernel<<<dim3((unsigned)nx, cnt, 1), THREADS, smem, st>>>(
            r, n, d, r_b, mmax, tmax, n_start, bases, common_b, C, xdig, groups_per_cta, u0, err);
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    return QMC_OK;
}

}  // namespace

extern "C" {

int qmc_gdn_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t r_b, uint64_t mmax, uint64_t tmax,
                        uint64_t n_start, const uint64_t *bases, const uint64_t *C, uint64_t *xdig, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0 || tmax == 0) return QMC_OK;
    QMC_REQUIRE(r_b > 0 && bases && C && xdig, "bad r_b or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    if (mmax * tmax <= GT_MAX_CW && tmax <= GT_MAX_TMAX)
        return gen_tiled(r, n, d, r_b, mmax, tmax, n_start, (const u64 *)bases, 0, (const u64 *)C, (u64 *)xdig,
                         QMC_STREAM(s), err, "gdn_gen_natural");
    u64 splits;
    const PointGrid pg = point_grid(r, n, d, tmax, DIM_TILE, &splits);
    return launch_points(r, pg.dim_tiles, [&](u64 l0, unsigned cnt) {
        gdn_gen_kernel<<<dim3((unsigned)splits, cnt, 1), THREADS, 0, QMC_STREAM(s)>>>(
            r, n, d, r_b, mmax, tmax, n_start, (const u64 *)bases, 0, (const u64 *)C, (u64 *)xdig, pg, l0, err);
    }, "gdn_gen_natural");
}

int qmc_gdn_gen_natural_same_base(uint64_t r, uint64_t n, uint64_t d, uint64_t mmax, uint64_t tmax,
                                  uint64_t n_start, uint64_t b, const uint64_t *C, uint64_t *xdig, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0 || tmax == 0) return QMC_OK;
    QMC_REQUIRE(C && xdig, "null array pointer");
    QMC_REQUIRE_DOMAIN(b >= 2, "base %llu: the reference divides by it (b=0) or never ends (b=1)",
                       (unsigned long long)b);
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    if (mmax * tmax <= GT_MAX_CW && tmax <= GT_MAX_TMAX)
        return gen_tiled(r, n, d, 1, mmax, tmax, n_start, nullptr, b, (const u64 *)C, (u64 *)xdig, QMC_STREAM(s), err,
                         "gdn_gen_natural_same_base");
    u64 splits;
    const PointGrid pg = point_grid(r, n, d, tmax, DIM_TILE, &splits);
    return launch_points(r, pg.dim_tiles, [&](u64 l0, unsigned cnt) {
        gdn_gen_kernel<<<dim3((unsigned)splits, cnt, 1), THREADS, 0, QMC_STREAM(s)>>>(
            r, n, d, 1, mmax, tmax, n_start, nullptr, b, (const u64 *)C, (u64 *)xdig, pg, l0, err);
    }, "gdn_gen_natural_same_base");
}

int qmc_gdn_linear_matrix_scramble(uint64_t r, uint64_t d, uint64_t mmax, uint64_t r_C, uint64_t r_b,
                                   uint64_t tmax, uint64_t tmax_new, const uint64_t *bases, const uint64_t *S,
                                   const uint64_t *C, uint64_t *C_lms, qmc_stream_t s)
{
    const u64 total = r * d * mmax * tmax_new;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(r_C > 0 && r_b > 0 && bases && S && C && C_lms, "bad r_C/r_b or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    gdn_lms_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(r, d, mmax, r_C, r_b, tmax, tmax_new,
                                                                (const u64 *)bases, (const u64 *)S,
                                                                (const u64 *)C, (u64 *)C_lms, err);
    return qmcgb::launch_status("gdn_linear_matrix_scramble");
}

int qmc_gdn_digital_permutation(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t r_b, uint64_t tmax,
                                uint64_t tmax_new, uint64_t bmax, const uint64_t *perms, const uint64_t *xdig,
                                uint64_t *xdig_new, qmc_stream_t s)
{
    (void)r_b;
    const u64 total = r * n * d * tmax_new;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(r_x > 0 && perms && xdig_new && (tmax == 0 || xdig), "bad r_x or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    u64 splits;
    const PointGrid pg = point_grid(r, n, d, tmax_new, DIM_TILE, &splits, 32);
    const u32 lin = linear_run(pg, d, tmax, tmax_new, xdig, xdig_new);
    return launch_points(r, pg.dim_tiles, [&](u64 l0, unsigned cnt) {
        gdn_perm_kernel<<<dim3((unsigned)splits, cnt, 1), THREADS, 0, QMC_STREAM(s)>>>(
            r, n, d, r_x, tmax, tmax_new, bmax, (const u64 *)perms, (const u64 *)xdig, (u64 *)xdig_new, pg, l0, lin,
            err);
    }, "gdn_digital_permutation");
}

int qmc_gdn_digital_shift(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, uint64_t r_b, uint64_t tmax,
                          uint64_t tmax_new, const uint64_t *bases, const uint64_t *shifts, const uint64_t *xdig,
                          uint64_t *xdig_new, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0 || tmax_new == 0) return QMC_OK;
    QMC_REQUIRE(r_x > 0 && r_b > 0 && bases && shifts && xdig_new && (tmax == 0 || xdig),
                "bad r_x/r_b or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    u64 splits;
    const PointGrid pg = point_grid(r, n, d, tmax_new, DIM_TILE, &splits, 32);
    const u32 lin = linear_run(pg, d, tmax, tmax_new, xdig, xdig_new);
    return launch_points(r, pg.dim_tiles, [&](u64 l0, unsigned cnt) {
        gdn_shift_kernel<<<dim3((unsigned)splits, cnt, 1), THREADS, 0, QMC_STREAM(s)>>>(
            r, n, d, r_x, r_b, tmax, tmax_new, (const u64 *)bases, (const u64 *)shifts, (const u64 *)xdig,
            (u64 *)xdig_new, pg, l0, lin, err);
    }, "gdn_digital_shift");
}

int qmc_gdn_integer_to_float(uint64_t r, uint64_t n, uint64_t d, uint64_t r_b, uint64_t tmax, const uint64_t *bases,
                             const uint64_t *xdig, double *x, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(r_b > 0 && bases && x && (tmax == 0 || xdig), "bad r_b or null array pointer");
    u64 splits;
    const PointGrid pg = point_grid(r, n, d, 1, I2F_DIMS, &splits, 16);
    return launch_points(r, pg.dim_tiles, [&](u64 l0, unsigned cnt) {
        gdn_to_float_kernel<<<dim3((unsigned)splits, cnt, 1), THREADS, I2F_SMEM_WORDS * sizeof(double),
                              QMC_STREAM(s)>>>(
            r, n, d, r_b, tmax, (const u64 *)bases, (const u64 *)xdig, x, pg.rows_per_cta, pg.dim_tiles, l0);
    }, "gdn_integer_to_float");
}

int qmc_gdn_interlace(uint64_t r, uint64_t d_alpha, uint64_t mmax, uint64_t d, uint64_t tmax, uint64_t tmax_alpha,
                      uint64_t alpha, const uint64_t *C, uint64_t *C_alpha, qmc_stream_t s)
{
    const u64 total = r * d_alpha * mmax * tmax_alpha;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(alpha > 0 && C && C_alpha, "bad alpha or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    gdn_interlace_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(r, d_alpha, mmax, d, tmax, tmax_alpha, alpha,
                                                                      (const u64 *)C, (u64 *)C_alpha, err);
    return qmcgb::launch_status("gdn_interlace");
}

int qmc_gdn_undo_interlace(uint64_t r, uint64_t d, uint64_t mmax, uint64_t d_alpha, uint64_t tmax,
                           uint64_t tmax_alpha, uint64_t alpha, const uint64_t *C_alpha, uint64_t *C, qmc_stream_t s)
{
    const u64 total = r * d * mmax * tmax;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(alpha > 0 && C_alpha && C, "bad alpha or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    gdn_undo_interlace_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(r, d, mmax, d_alpha, tmax, tmax_alpha,
                                                                           alpha, (const u64 *)C_alpha, (u64 *)C, err);
    return qmcgb::launch_status("gdn_undo_interlace");
}

}  // extern "C"
