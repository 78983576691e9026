// halton.cu -- fused generalized digital net (e.g. randomised Halton): for
// every dimension j with its own base b_j, digit count tmax_j and generating
// matrix (mmax_j columns), the chain
//
//   gdn_linear_matrix_scramble   qmctoolscl/c_funcs/gdn_linear_matrix_scramble.c:3-46
//   gdn_gen_natural              qmctoolscl/c_funcs/gdn_gen_natural.c:3-53
//   gdn_digital_permutation      qmctoolscl/c_funcs/gdn_digital_permutation.c:3-46
//   gdn_digital_shift            qmctoolscl/c_funcs/gdn_digital_shift.c:3-45
//   gdn_integer_to_float         qmctoolscl/c_funcs/gdn_integer_to_float.c:3-43
//
// called once per dimension (d = 1, r_b = 1, tmax_new = tmax_j: the reference
// takes one tmax per call), with the per-dimension results written into
// x[l, i, j] of one r x n x d array -- bit for bit, without ever storing a
// digit in HBM.
//
// Preparation (per plan run, small next to the output):
//  * the scrambled generating matrices reduced mod b, as 32-bit words (the
//    reference's gen step reduces after every column; with entries of at
//    most tmax*(b-1) no 64-bit sum wraps, so one reduction of reduced terms
//    gives the same digits);
//  * recip_t = 1/b^(t+1) as the reference computes it (repeated correctly
//    rounded divisions);
//  * the term table Y[l][j][t][g] = RN(recip_t * digit) for every raw digit
//    g < b, where digit = (perm[l][t][g] + shift[l][t]) mod b (either step
//    left out when its array is absent).  Once the raw digit g of output
//    digit t is known, permutation, shift and the rounded product of
//    gdn_integer_to_float.c:37 are one table read;
//  * the tail table: for each (l, j, t) the largest exponent among the terms
//    of digits t..tmax-1, for an exact early stop.
//
// Generation: a CTA owns a tile of 32 consecutive points of one
// randomisation and all d dimensions.  Each warp takes whole dimensions
// (assigned longest-first to balance the work), one point per lane, so the
// 32 lanes share base, digit count and tables.  The index splits as
// hi * b^K + lo with b^K >= the tile's point count (32 or 64): the tile has at
// most two distinct hi, whose contributions to each output digit the lanes
// compute together, and K <= 6 low digits per point.  With few enough
// dimensions each lane carries two points (two independent chains sharing
// the shuffled per-digit values).  Per output digit t: the raw digit mod b (32-bit
// multiply-high division), the term from the table, and v = RN(v + term) --
// on the FP64 unit or in integer arithmetic on the unpacked sum
// (digit_sum.cuh), chosen per dimension by a share knob.  On GB300 all-FP64
// measures fastest (an integer add is about 30 dependent instructions, and a
// mixed kernel carries both code paths), and an all-FP64 plan launches a
// variant without the integer path.  Once every remaining term of a group of
// four digits is below half an ulp of v the lane stops.  The tile of doubles
// is staged in shared memory and stored as contiguous rows.  The grid holds
// exactly the CTAs resident at once, striding over the equal-cost tiles.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "digit_sum.cuh"

namespace {

constexpr int HT_THREADS = 256;
constexpr int HT_WARPS = HT_THREADS / 32;
constexpr u32 HT_MAX_DIMS = 1024;
constexpr u32 HT_MAX_B = 2048;
constexpr u32 HT_GROUP = 4;  // output digits whose table reads are issued together

enum : u32 { ADD_FP64 = 0, ADD_INT = 1 };

struct HDim {
    u32 b, tmax, mmax;
    u32 K;         // low digits per point: the smallest K with b^K >= points per tile
    u32 Klo;       // min(K, mmax): low digits that can be nonzero (C has mmax rows)
    u32 bK;        // b^K
    u32 m32;       // floor(2^32 / b) + 1: x / b = umulhi(x, m32) for x < 2^32 / b
    u32 wide;      // 1 when digit sums can reach 2^32 / b: 64-bit remainders instead
    u32 add;       // ADD_FP64 or ADD_INT
    u32 tpad;      // tmax rounded up to a multiple of HT_GROUP: term rows past tmax hold +0
    u64 fd_M;      // direct-remainder constant for b (any 32-bit x)
    u64 fdK_M;     // the same for b^K
    u64 c_off;     // offset of this dimension's (mmax x tmax) block inside a randomisation's C block
    u64 y_off;     // offset of its (tpad x b) term rows inside a randomisation's Y block
    u64 s_off;     // offset of its tpad digits inside the request's tail blocks
    u64 r_off;     // offset of its tpad recip_t in the plan's recip array
};

// One request of a batch (device copy): r randomisations of n points from
// index n_start, d dimensions (dims[dim0 ..]), output x (r x n x d).  Its
// tables sit at request-relative bases inside the plan's shared arrays.
struct HReq {
    u64 r, n, n_start, d;
    u64 dim0;              // first HDim / PrepDim of the request
    u64 c_base, c_per_l;   // C words: randomisation l of this request at c_base + l * c_per_l
    u64 y_base, y_per_l;   // term-table words
    u64 t_base, s_per_l;   // tail words (t_base + l * s_per_l + s_off); also the term-row prefix
    u64 tl_base;           // prefix of (l, j) items of the tail kernel
    u64 tile0, tiles_per_l;  // generation tiles
    u32 o_base, pad;       // dimension order of the warps: order[o_base + wstart[q * (HT_WARPS + 1) + w] ...]
    u32 has_lms, has_perm, has_shift, pad2;
    double *x;
};

struct HPlanDev {
    u64 nreq, total_c, rows, titems, ntiles, ndims;
    const HReq *req;
    const HDim *dims;    // all requests' dimensions
    const u32 *C;        // scrambled matrices mod b
    const u64 *Y;        // term bits RN(recip_t * digit)
    const u64 *recip;    // bits of recip_t at HDim::r_off + t
    const u32 *tail;     // largest biased exponent among the terms of digits t.. of (l, j)
    const u16 *order;    // per request, its dimension ids (request-relative) grouped by warp
    const u32 *wstart;   // per request, HT_WARPS + 1 offsets into its order
    unsigned *err;
};

// the request whose prefix field (a non-decreasing u64 member of HReq) holds key
template <typename F>
__device__ __forceinline__ u32 req_of(const HReq *req, u64 nreq, u64 key, F field)
{
    u32 lo = 0, hi = (u32)nreq - 1;
    while (lo < hi) {
        const u32 mid = (lo + hi + 1) >> 1;
        if (field(req[mid]) <= key)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

struct PrepDim {
    u64 b, tmax, mmax;
    const u64 *S, *C, *perms, *shifts;  // caller's per-dimension arrays
};

// floor(x / b) and x mod b for any x < 2^32, b >= 2, from M = floor((2^64-1)/b) + 1;
// hdiv is the high word of the 64x32-bit product M*x / 2^64
__device__ __forceinline__ u32 hdiv(u64 M, u32 x)
{
    const u64 lo = (u64)(u32)M * x;
    return (u32)(((M >> 32) * x + (lo >> 32)) >> 32);
}
__device__ __forceinline__ u32 hmod(u64 M, u32 b, u32 x) { return (u32)__umul64hi(M * (u64)x, (u64)b); }

// the same for x < 2^32 / b, with m32 = floor(2^32/b) + 1: x*m32/2^32 exceeds
// x/b by less than x/2^32 < 1/b, too little to reach the next integer
__device__ __forceinline__ u32 ndiv(u32 m32, u32 x) { return __umulhi(x, m32); }
__device__ __forceinline__ u32 nmod(u32 m32, u32 b, u32 x) { return x - __umulhi(x, m32) * b; }

__device__ __forceinline__ u32 dim_mod(const HDim &D, u32 x)
{
    return D.wide ? hmod(D.fd_M, D.b, x) : nmod(D.m32, D.b, x);
}

// ---------------------------------------------------------------- prep

// the dimension (of dims[0 .. d)) whose block (offset `field` of HDim) holds offset off
template <typename F>
__device__ __forceinline__ u32 dim_of(const HDim *dims, u64 d, u64 off, F field)
{
    u32 lo = 0, hi = (u32)d - 1;
    while (lo < hi) {
        const u32 mid = (lo + hi + 1) >> 1;
        if (field(dims[mid]) <= off)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// one thread per (request, l, j, k, t) word of C
__global__ void halton_lms_kernel(HPlanDev P, const PrepDim *pd, u32 *C)
{
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 w = (u64)blockIdx.x * blockDim.x + threadIdx.x; w < P.total_c; w += stride) {
        const HReq &R = P.req[req_of(P.req, P.nreq, w, [](const HReq &q) { return q.c_base; })];
        const u64 loc0 = w - R.c_base, l = loc0 / R.c_per_l, off = loc0 % R.c_per_l;
        const HDim *dims = P.dims + R.dim0;
        const u32 j = dim_of(dims, R.d, off, [](const HDim &h) { return h.c_off; });
        const HDim &D = dims[j];
        const u64 loc = off - D.c_off, k = loc / D.tmax, t = loc % D.tmax;
        const PrepDim &Q = pd[R.dim0 + j];
        if (R.has_lms) {
            // gdn_linear_matrix_scramble.c:36-42 with d = 1, r_C = 1: sum_c (S[l,t,c]*C[k,c]) % b, no final
            // mod; the sum is at most tmax*(b-1) and the generation step reduces it anyway
            const u64 *srow = Q.S + (l * Q.tmax + t) * Q.tmax;
            const u64 *col = Q.C + k * Q.tmax;
            u64 acc = 0;
            for (u64 c = 0; c < Q.tmax; c++) acc += (srow[c] * col[c]) % Q.b;
            C[w] = (u32)(acc % Q.b);
        } else {
            // the generation step multiplies raw entries by digits below b in 64 bits: entries below
            // 2^32 cannot wrap, so reducing them first gives the same digits
            const u64 c = Q.C[k * Q.tmax + t];
            if (c >> 32) atomicOr(P.err, 8u);
            C[w] = (u32)(c % Q.b);
        }
    }
}

// recip_t of gdn_integer_to_float.c:34-38 for every dimension of every request
__global__ void halton_recip_kernel(HPlanDev P, u64 *recip)
{
    for (u64 g = (u64)blockIdx.x * blockDim.x + threadIdx.x; g < P.ndims; g += (u64)gridDim.x * blockDim.x) {
        const HDim &D = P.dims[g];
        const double bd = (double)D.b;
        double rc = __ddiv_rn(1.0, bd);
        for (u32 t = 0; t < D.tpad; t++) {
            recip[D.r_off + t] = as_bits(rc);
            rc = __ddiv_rn(rc, bd);
        }
    }
}

// One warp per term row (request, l, j, t): Y[g] = RN(recip_t * digit(g)) for
// g < b, digit(g) = (perm[l,t,g] + shift[l,t]) mod b as
// gdn_digital_permutation.c:36-39 and gdn_digital_shift.c:37-39 compute it
// (64-bit wrapping add), then (double)digit * recip_t as
// gdn_integer_to_float.c:36-37.  Lane 0 records the row's largest exponent in
// the tail table (whose words are numbered exactly like the rows).
__global__ void halton_terms_kernel(HPlanDev P, const PrepDim *pd, u64 *Y, u32 *tail)
{
    const u32 lane = threadIdx.x % 32;
    const u64 wstride = (u64)gridDim.x * (blockDim.x / 32);
    for (u64 row = ((u64)blockIdx.x * blockDim.x + threadIdx.x) / 32; row < P.rows; row += wstride) {
        const HReq &R = P.req[req_of(P.req, P.nreq, row, [](const HReq &q) { return q.t_base; })];
        const u64 loc = row - R.t_base, l = loc / R.s_per_l, off = loc % R.s_per_l;
        const HDim *dims = P.dims + R.dim0;
        const u32 j = dim_of(dims, R.d, off, [](const HDim &h) { return h.s_off; });
        const HDim &D = dims[j];
        const PrepDim &Q = pd[R.dim0 + j];
        const u64 t = off - D.s_off;
        u64 *yrow = Y + R.y_base + l * R.y_per_l + D.y_off + t * D.b;
        if (t >= D.tmax) {  // padding row: +0 terms, no tail
            for (u32 g = lane; g < D.b; g += 32) yrow[g] = 0;
            if (lane == 0) tail[row] = 0;
            continue;
        }
        const double rc = as_double(P.recip[D.r_off + t]);
        const u64 sh = R.has_shift ? Q.shifts[l * D.tmax + t] : 0;
        u64 mx = 0;
        for (u32 g = lane; g < D.b; g += 32) {
            const u64 pv = R.has_perm ? Q.perms[(l * D.tmax + t) * D.b + g] : g;
            const u64 dig = R.has_shift ? (pv + sh) % D.b : pv;
            const u64 y = dig ? as_bits(__dmul_rn(rc, __ull2double_rn(dig))) : 0;
            yrow[g] = y;
            mx = max(mx, y);  // non-negative doubles order like their bits
        }
        for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) tail[row] = (u32)(mx >> 52);
    }
}

// suffix maximum over t of the row exponents, per (request, l, j)
__global__ void halton_tail_kernel(HPlanDev P, u32 *tail)
{
    for (u64 w = (u64)blockIdx.x * blockDim.x + threadIdx.x; w < P.titems; w += (u64)gridDim.x * blockDim.x) {
        const HReq &R = P.req[req_of(P.req, P.nreq, w, [](const HReq &q) { return q.tl_base; })];
        const u64 loc = w - R.tl_base, l = loc / R.d, j = loc % R.d;
        const HDim &D = P.dims[R.dim0 + j];
        u32 *tl = tail + R.t_base + l * R.s_per_l + D.s_off;
        u32 m = 0;
        for (u32 t = D.tpad; t-- > 0;) {
            m = max(m, tl[t]);
            tl[t] = m;
        }
    }
}

// ---------------------------------------------------------------- generation

// RN(v + y) for the sums the integer fast form does not take (first term,
// carry into the next binade, subnormal operands): the FP64 unit, out of line
__device__ __noinline__ u64 halton_add_slow(u64 v, u64 y) { return as_bits(__dadd_rn(as_double(v), as_double(y))); }

// v = RN(v + y) on the unpacked sum, y = the bits of a non-negative double
__device__ __forceinline__ void add_term_int(dsum::Sum &v, u64 y)
{
    if (dsum::add_fast(v, y) || !y) return;
    v = dsum::unpack(v.M ? halton_add_slow(dsum::pack(v), y) : y);  // 0 + y = y exactly
}

// sum over the base-b digits k >= K of h (the digits of index / b^K) of
// digit * C[k][t], reduced mod b; h < 2^32 / b^K
__device__ __forceinline__ u32 high_part(const HDim &D, const u32 *Cj, u32 h, u32 t)
{
    u32 acc = 0;
    for (u32 k = D.K; h && k < D.mmax; k++) {
        const u32 q = ndiv(D.m32, h);
        acc += (h - q * D.b) * Cj[k * D.tmax + t];  // < mmax * b^2
        h = q;
    }
    return dim_mod(D, acc);
}

// The values of dimension D for this lane's PPL points (bits of the doubles),
// KL = min(K, mmax) low digits per point.  The CTA's tile holds 32 * PPL
// consecutive points (lane c has points c, c + 32, ...), and b^K >= 32 * PPL,
// so the tile spans at most two values of hi = index / b^K.
//
// Output digits go in chunks of 32: lane c holds, for digit t0 + c, the
// high-digit sums of both hi values (packed), the low-digit matrix entries
// C[k][t0 + c] (k < KL) and the tail exponent, and every lane takes its own
// from lane t - t0 by shuffles, shared by its PPL points.  Within a chunk,
// groups of HT_GROUP digits compute their raw digits and issue their table
// reads (independent of v), then add the terms in order.  The early stop is
// tested once per group: an add after the exact stop point leaves v
// unchanged (the term is below half an ulp), so the group's adds need no
// test; a stopped point adds +0.
template <u32 ADD, u32 KL, u32 PPL>
__device__ __forceinline__ void dim_value(const HDim &D, const u32 *Cj, const u64 *Yj, const u32 *Tj, u32 base,
                                          const u32 (&itrue)[PPL], const bool (&active)[PPL], u32 lane, u64 (&out)[PPL])
{
    const u32 h0 = hdiv(D.fdK_M, base);
    u32 sel[PPL], dl[PPL][KL];
    bool done[PPL];
    dsum::Sum vi[PPL];  // ADD_INT: the running sums, unpacked
    double vd[PPL];     // ADD_FP64: the running sums
#pragma unroll
    for (u32 q = 0; q < PPL; q++) {
        const u32 hi = hdiv(D.fdK_M, itrue[q]);
        sel[q] = (hi - h0) * 16;  // 0 or 16: which half of the packed word
        u32 x = itrue[q] - hi * D.bK;  // < b^K < 64 b
#pragma unroll
        for (u32 k = 0; k < KL; k++) {
            const u32 qq = ndiv(D.m32, x);
            dl[q][k] = x - qq * D.b;
            x = qq;
        }
        done[q] = !active[q];
        vi[q] = dsum::unpack(0);
        vd[q] = 0.0;
    }
    auto all_done = [&]() {
        bool a = true;
#pragma unroll
        for (u32 q = 0; q < PPL; q++) a = a && done[q];
        return a;
    };
    for (u32 t0 = 0; t0 < D.tpad; t0 += 32) {
        if (__all_sync(0xffffffffu, all_done())) break;
        const u32 tc = t0 + lane;
        u32 packed = 0, tailc = 0, cl[KL];
#pragma unroll
        for (u32 k = 0; k < KL; k++) cl[k] = 0;
        if (tc < D.tmax) {
            packed = high_part(D, Cj, h0, tc) | (high_part(D, Cj, h0 + 1, tc) << 16);
            tailc = Tj[tc];
#pragma unroll
            for (u32 k = 0; k < KL; k++) cl[k] = Cj[k * D.tmax + tc];
        }
        const u32 tend = min(D.tpad, t0 + 32);
        for (u32 t = t0; t < tend; t += HT_GROUP) {
            // every remaining term is below 2^(tail - 1022); once that is at most half an ulp of v
            // (2^(E - 1076)), RN(v + term) = v for the rest of the digits
            const u32 tl = __shfl_sync(0xffffffffu, tailc, t - t0);  // every lane takes part in the shuffle
#pragma unroll
            for (u32 q = 0; q < PPL; q++) {
                const u32 E = ADD == ADD_INT ? vi[q].E : (u32)(as_bits(vd[q]) >> 52);
                done[q] = done[q] || tl + 54 <= E;
            }
            if (__all_sync(0xffffffffu, all_done())) break;
            u64 y[PPL][HT_GROUP];
#pragma unroll
            for (u32 u = 0; u < HT_GROUP; u++) {
                const u32 src = t + u - t0;
                // gdn_gen_natural.c:37-50: raw digit t + u of each point, mod b (rows past tmax: +0)
                const u32 pk = __shfl_sync(0xffffffffu, packed, src);
                u32 c[KL];
#pragma unroll
                for (u32 k = 0; k < KL; k++) c[k] = __shfl_sync(0xffffffffu, cl[k], src);
#pragma unroll
                for (u32 q = 0; q < PPL; q++) {
                    u32 acc = (pk >> sel[q]) & 0xFFFFu;
#pragma unroll
                    for (u32 k = 0; k < KL; k++) acc += dl[q][k] * c[k];
                    y[q][u] = done[q] ? 0ull : Yj[(t + u) * D.b + dim_mod(D, acc)];
                }
            }
            // the padded rows past tmax add +0, which leaves v as it is: a group that reaches past
            // tmax (the same for the whole warp: it owns the dimension) skips those adds
            const u32 nu = min(HT_GROUP, D.tmax - t);
            if (ADD == ADD_INT) {
#pragma unroll
                for (u32 u = 0; u < HT_GROUP; u++) {
                    if (u >= nu) break;
#pragma unroll
                    for (u32 q = 0; q < PPL; q++) add_term_int(vi[q], y[q][u]);
                }
            } else {
#pragma unroll
                for (u32 u = 0; u < HT_GROUP; u++) {
                    if (u >= nu) break;
#pragma unroll
                    for (u32 q = 0; q < PPL; q++)
                        vd[q] = __dadd_rn(vd[q], as_double(y[q][u]));  // gdn_integer_to_float.c:37
                }
            }
        }
    }
#pragma unroll
    for (u32 q = 0; q < PPL; q++) out[q] = ADD == ADD_INT ? dsum::pack(vi[q]) : as_bits(vd[q]);
}

template <u32 ADD, u32 PPL>
__device__ __forceinline__ void dim_value_k(const HDim &D, const u32 *Cj, const u64 *Yj, const u32 *Tj, u32 base,
                                            const u32 (&itrue)[PPL], const bool (&active)[PPL], u32 lane,
                                            u64 (&out)[PPL])
{
    switch (D.Klo) {
    case 1: return dim_value<ADD, 1, PPL>(D, Cj, Yj, Tj, base, itrue, active, lane, out);
    case 2: return dim_value<ADD, 2, PPL>(D, Cj, Yj, Tj, base, itrue, active, lane, out);
    case 3: return dim_value<ADD, 3, PPL>(D, Cj, Yj, Tj, base, itrue, active, lane, out);
    case 4: return dim_value<ADD, 4, PPL>(D, Cj, Yj, Tj, base, itrue, active, lane, out);
    case 5: return dim_value<ADD, 5, PPL>(D, Cj, Yj, Tj, base, itrue, active, lane, out);
    default: return dim_value<ADD, 6, PPL>(D, Cj, Yj, Tj, base, itrue, active, lane, out);
    }
}

// A CTA owns tiles of 32 * PPL consecutive points of one randomisation of one
// request and all its d dimensions; tiles of all requests form one list.  The
// tile of doubles is staged in shared memory ([32 * PPL][d]) and stored as
// contiguous rows.  With one request (ONE) its descriptor is a kernel
// parameter (the constant bank, no registers held for it).  Without MIXED
// every dimension adds on the FP64 unit and the integer adds are not compiled
// in (fewer registers and instructions for the common split).
template <u32 PPL, bool ONE, bool MIXED>
__global__ void __launch_bounds__(HT_THREADS, 3) halton_gen_kernel(HPlanDev P, HReq R1)
{
    extern __shared__ __align__(16) unsigned char sm[];
    double *tile = (double *)sm;
    constexpr u32 TP = 32 * PPL;  // points per tile
    const u32 warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (u64 tt = blockIdx.x; tt < P.ntiles; tt += gridDim.x) {
        const u32 q = ONE ? 0u : req_of(P.req, P.nreq, tt, [](const HReq &r_) { return r_.tile0; });
        const HReq R = ONE ? R1 : P.req[q];  // by value: the output stores may not alias it
        const u64 loc = tt - R.tile0, l = loc / R.tiles_per_l, i0 = (loc % R.tiles_per_l) * TP;
        const u32 base = (u32)(R.n_start + i0);
        u32 itrue[PPL];
        bool active[PPL];
#pragma unroll
        for (u32 k = 0; k < PPL; k++) {
            active[k] = i0 + lane + 32 * k < R.n;  // points past the last compute nothing
            itrue[k] = active[k] ? base + lane + 32 * k : base;  // < 2^32 (checked at plan creation)
        }
        const u32 *Cl = P.C + R.c_base + l * R.c_per_l;
        const u64 *Yl = P.Y + R.y_base + l * R.y_per_l;
        const u32 *Tl = P.tail + R.t_base + l * R.s_per_l;
        const HDim *dims = P.dims + R.dim0;
        const u16 *order = P.order + R.o_base;
        const u32 *ws = P.wstart + (u64)q * (HT_WARPS + 1);
        for (u32 oi = ws[warp]; oi < ws[warp + 1]; oi++) {
            const u32 j = order[oi];
            const HDim D = dims[j];
            u64 vb[PPL];
            if (MIXED && D.add == ADD_INT)
                dim_value_k<ADD_INT, PPL>(D, Cl + D.c_off, Yl + D.y_off, Tl + D.s_off, base, itrue, active, lane, vb);
            else
                dim_value_k<ADD_FP64, PPL>(D, Cl + D.c_off, Yl + D.y_off, Tl + D.s_off, base, itrue, active, lane, vb);
#pragma unroll
            for (u32 k = 0; k < PPL; k++) tile[(lane + 32 * k) * R.d + j] = as_double(vb[k]);
        }
        __syncthreads();
        const u64 rows = min((u64)TP, R.n - i0);
        double *out = R.x + (l * R.n + i0) * R.d;
        for (u64 e = threadIdx.x; e < rows * R.d; e += HT_THREADS) __stcs(out + e, tile[e]);
        __syncthreads();
    }
}

u64 ceil_digits(u64 n_last, u64 b)
{
    u64 k = 0;
    for (u64 x = n_last; x; x /= b) k++;
    return k;
}

// The share of the terms (by count) whose adds go to the FP64 unit; the
// other dimensions add in integer arithmetic.  Dimensions are taken in order
// of decreasing tmax for the FP64 side.  Returns whether any dimension adds
// in integer arithmetic.
bool assign_adds(std::vector<HDim> &hd, double share)
{
    bool mixed = false;
    u64 total = 0;
    for (const HDim &h : hd) total += h.tmax;
    std::vector<u32> idx(hd.size());
    for (u32 j = 0; j < hd.size(); j++) idx[j] = j;
    std::stable_sort(idx.begin(), idx.end(), [&](u32 a, u32 b) { return hd[a].tmax > hd[b].tmax; });
    u64 acc = 0;
    for (u32 j : idx) {
        const bool fp = (double)acc + hd[j].tmax / 2.0 < share * (double)total;
        hd[j].add = fp ? ADD_FP64 : ADD_INT;
        if (fp) acc += hd[j].tmax;
        mixed = mixed || !fp;
    }
    return mixed;
}

}  // namespace

struct qmc_halton_plan {
    HPlanDev P{};
    std::vector<HDim> hd;
    std::vector<HReq> hreq;
    std::vector<PrepDim> prep;
    void *d_req = nullptr, *d_dims = nullptr, *d_C = nullptr, *d_Y = nullptr, *d_recip = nullptr, *d_tail = nullptr;
    void *d_order = nullptr, *d_wstart = nullptr, *d_prep = nullptr;
    size_t smem = 0;
    u32 ppl = 1;
    bool mixed = false;  // some dimensions add in integer arithmetic
    bool prepared = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

void drop_graph(qmc_halton_plan *p)
{
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
}

int prepare_launch(qmc_halton_plan *p, cudaStream_t st)
{
    const unsigned cap = (unsigned)qmcgb::sm_count() * 16;
    halton_lms_kernel<<<qmcgb::grid_for(p->P.total_c, 256, cap), 256, 0, st>>>(p->P, (const PrepDim *)p->d_prep,
                                                                              (u32 *)p->d_C);
    if (int rc = qmcgb::launch_status("halton_lms_kernel")) return rc;
    halton_recip_kernel<<<qmcgb::grid_for(p->P.ndims, 128, 1024), 128, 0, st>>>(p->P, (u64 *)p->d_recip);
    if (int rc = qmcgb::launch_status("halton_recip_kernel")) return rc;
    halton_terms_kernel<<<qmcgb::grid_for(p->P.rows * 32, 256, cap), 256, 0, st>>>(p->P, (const PrepDim *)p->d_prep,
                                                                                  (u64 *)p->d_Y, (u32 *)p->d_tail);
    if (int rc = qmcgb::launch_status("halton_terms_kernel")) return rc;
    halton_tail_kernel<<<qmcgb::grid_for(p->P.titems, 128, cap), 128, 0, st>>>(p->P, (u32 *)p->d_tail);
    return qmcgb::launch_status("halton_tail_kernel");
}

// Every tile costs the same, and the CTAs stride over the tiles: a grid of exactly the CTAs
// resident at once keeps every SM busy to the end (a grid of 8 per SM against 3 resident ran
// in 2.67 waves, the last a third idle).
template <u32 PPL, bool ONE, bool MIXED>
unsigned resident_grid(const qmc_halton_plan *p)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, halton_gen_kernel<PPL, ONE, MIXED>, HT_THREADS,
                                                      p->smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    return qmcgb::grid_for(p->P.ntiles, 1, (unsigned)(qmcgb::sm_count() * per_sm));
}

int run_launch(qmc_halton_plan *p, cudaStream_t st)
{
    const HReq &R1 = p->hreq[0];
    const bool one = p->hreq.size() == 1, mixed = p->mixed;
#define HT_LAUNCH(PPL_, ONE_, MIXED_)                                                             \
    halton_gen_kernel<PPL_, ONE_, MIXED_><<<resident_grid<PPL_, ONE_, MIXED_>(p), HT_THREADS, p->smem, st>>>( \
        p->P, R1)
    if (p->ppl == 2) {
        if (one) {
            if (mixed) HT_LAUNCH(2, true, true); else HT_LAUNCH(2, true, false);
        } else {
            if (mixed) HT_LAUNCH(2, false, true); else HT_LAUNCH(2, false, false);
        }
    } else {
        if (one) {
            if (mixed) HT_LAUNCH(1, true, true); else HT_LAUNCH(1, true, false);
        } else {
            if (mixed) HT_LAUNCH(1, false, true); else HT_LAUNCH(1, false, false);
        }
    }
#undef HT_LAUNCH
    return qmcgb::launch_status("halton_gen_kernel");
}

template <u32 PPL>
int gen_smem_attr(size_t smem)
{
    const void *fs[] = {(const void *)halton_gen_kernel<PPL, true, true>, (const void *)halton_gen_kernel<PPL, false, true>,
                        (const void *)halton_gen_kernel<PPL, true, false>, (const void *)halton_gen_kernel<PPL, false, false>};
    for (const void *f : fs)
        if (int rc = qmcgb::raise_smem_limit(f, smem, "halton_gen_kernel smem")) return rc;
    return QMC_OK;
}

}  // namespace

extern "C" {

int qmc_halton_batch_create(const qmc_halton_request *reqs, int nreq, qmc_halton_plan **plan)
{
    QMC_REQUIRE(plan && reqs && nreq >= 1, "null argument or empty batch");
    *plan = nullptr;
    u64 maxd = 0;
    for (int q = 0; q < nreq; q++) {
        const qmc_halton_request &R = reqs[q];
        QMC_REQUIRE(R.dims && R.x, "request %d: null dims or x", q);
        QMC_REQUIRE(R.d >= 1 && R.d <= HT_MAX_DIMS && R.r >= 1 && R.n >= 1,
                    "request %d: need 1 <= d <= %u, r >= 1, n >= 1", q, HT_MAX_DIMS);
        QMC_REQUIRE(R.n_start + R.n <= (1ull << 32) && R.n_start + R.n > R.n_start,
                    "request %d: indices must stay below 2^32", q);
        maxd = std::max<u64>(maxd, R.d);
    }
    QMC_REQUIRE(32 * maxd * sizeof(double) <= 200 * 1024, "d too large for the shared-memory output tile");
    // two points per lane (two independent digit chains, shuffles shared) while the 64-point
    // output tile stays small enough for four CTAs per SM
    const u32 ppl = 64 * maxd * sizeof(double) <= 52 * 1024 ? 2 : 1;
    const u64 tp = 32ull * ppl;
    qmc_halton_plan *p = new qmc_halton_plan();
    p->ppl = ppl;
    p->smem = tp * maxd * sizeof(double);
    std::vector<u16> order;
    std::vector<u32> wstart;
    u64 c_base = 0, y_base = 0, t_base = 0, tl_base = 0, tile0 = 0, r_base = 0;
    for (int q = 0; q < nreq; q++) {
        const qmc_halton_request &Rq = reqs[q];
        const qmc_gdn_dim *dims = Rq.dims;
        const u64 d = Rq.d;
        // a step is applied when its array is given, for every dimension of the request alike
        const bool has_lms = dims[0].S != nullptr, has_perm = dims[0].perms != nullptr,
                   has_shift = dims[0].shifts != nullptr;
        HReq R{};
        R.r = Rq.r;
        R.n = Rq.n;
        R.n_start = Rq.n_start;
        R.d = d;
        R.dim0 = p->hd.size();
        R.has_lms = has_lms;
        R.has_perm = has_perm;
        R.has_shift = has_shift;
        R.x = Rq.x;
        u64 c_off = 0, y_off = 0, s_off = 0;
        for (u64 j = 0; j < d; j++) {
            const qmc_gdn_dim &g = dims[j];
            const char *bad = nullptr;
            if (g.b < 2 || g.b >= HT_MAX_B) bad = "base outside [2, 2048)";
            else if (g.tmax == 0 || g.tmax > 256 || g.mmax == 0 || g.mmax > 64) bad = "tmax in [1,256] and mmax in [1,64]";
            else if (!g.C) bad = "null generating matrix";
            else if ((g.S != nullptr) != has_lms || (g.perms != nullptr) != has_perm ||
                     (g.shifts != nullptr) != has_shift)
                bad = "S, perms and shifts must be given for all dimensions or for none";
            else if (ceil_digits(Rq.n_start + Rq.n - 1, g.b) > g.mmax)
                bad = "mmax smaller than the base-b digits of the last index";
            if (bad) {
                delete p;
                qmcgb::set_error("request %d, dimension %llu: %s", q, (unsigned long long)j, bad);
                return g.b < 2 ? QMC_ERR_DOMAIN : QMC_ERR_ARG;
            }
            HDim h{};
            h.b = (u32)g.b;
            h.tmax = (u32)g.tmax;
            h.mmax = (u32)g.mmax;
            h.K = 1;
            h.bK = h.b;
            while (h.bK < tp) {
                h.bK *= h.b;
                h.K++;
            }
            h.Klo = std::min<u32>(h.K, h.mmax);
            h.m32 = (u32)((1ull << 32) / h.b + 1);
            // digit sums stay below (mmax + 6) * b^2; the 32-bit division needs them below 2^32 / b
            h.wide = (u64)(h.mmax + 6) * h.b * h.b * h.b >= (1ull << 32);
            h.fd_M = fastdiv32_make(h.b).M;
            h.fdK_M = fastdiv32_make(h.bK).M;
            h.tpad = (h.tmax + HT_GROUP - 1) / HT_GROUP * HT_GROUP;
            h.c_off = c_off;
            h.y_off = y_off;
            h.s_off = s_off;
            h.r_off = r_base + s_off;
            c_off += g.mmax * g.tmax;
            y_off += (u64)h.tpad * g.b;
            s_off += h.tpad;
            p->hd.push_back(h);
            p->prep.push_back(PrepDim{g.b, g.tmax, g.mmax, (const u64 *)g.S, (const u64 *)g.C, (const u64 *)g.perms,
                                      (const u64 *)g.shifts});
        }
        R.c_base = c_base;
        R.c_per_l = c_off;
        R.y_base = y_base;
        R.y_per_l = y_off;
        R.t_base = t_base;
        R.s_per_l = s_off;
        R.tl_base = tl_base;
        R.tile0 = tile0;
        R.tiles_per_l = (Rq.n + tp - 1) / tp;
        R.o_base = (u32)order.size();
        c_base += Rq.r * c_off;
        y_base += Rq.r * y_off;
        t_base += Rq.r * s_off;
        tl_base += Rq.r * d;
        tile0 += Rq.r * R.tiles_per_l;
        r_base += s_off;
        // longest-first assignment of the request's dimensions to the warps of a CTA
        std::vector<u32> idx(d);
        for (u32 j = 0; j < d; j++) idx[j] = j;
        const HDim *hj = p->hd.data() + R.dim0;
        auto cost = [&](u32 j) { return (double)hj[j].tmax * 40.0 + (double)hj[j].mmax * 20.0; };
        std::sort(idx.begin(), idx.end(), [&](u32 a, u32 b) { return cost(a) > cost(b); });
        std::vector<std::vector<u32>> per(HT_WARPS);
        std::vector<double> load(HT_WARPS, 0.0);
        for (u32 j : idx) {
            const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            per[w].push_back(j);
            load[w] += cost(j);
        }
        u32 pos = 0;
        for (int w = 0; w < HT_WARPS; w++) {
            wstart.push_back(pos);
            for (u32 j : per[w]) {
                order.push_back((u16)j);
                pos++;
            }
        }
        wstart.push_back(pos);
        p->hreq.push_back(R);
    }
    p->mixed = assign_adds(p->hd, 1.0);
    const u64 ndims = p->hd.size();
    p->P.nreq = (u64)nreq;
    p->P.total_c = c_base;
    p->P.rows = t_base;
    p->P.titems = tl_base;
    p->P.ntiles = tile0;
    p->P.ndims = ndims;
    p->P.err = qmcgb::device_error_ptr();
    int rc = 0;
    auto alloc = [&](void **dst, size_t bytes) {
        if (!rc) rc = qmcgb::cuda_status(cudaMalloc(dst, bytes ? bytes : 16), "cudaMalloc");
    };
    auto put = [&](void *dst, const void *src, size_t bytes) {
        if (!rc && bytes) rc = qmcgb::cuda_status(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "copy");
    };
    alloc(&p->d_req, nreq * sizeof(HReq));
    alloc(&p->d_dims, ndims * sizeof(HDim));
    alloc(&p->d_C, c_base * sizeof(u32));
    alloc(&p->d_Y, y_base * sizeof(u64));
    alloc(&p->d_recip, r_base * sizeof(u64));
    alloc(&p->d_tail, t_base * sizeof(u32));
    alloc(&p->d_order, order.size() * sizeof(u16));
    alloc(&p->d_wstart, wstart.size() * sizeof(u32));
    alloc(&p->d_prep, ndims * sizeof(PrepDim));
    put(p->d_req, p->hreq.data(), nreq * sizeof(HReq));
    put(p->d_dims, p->hd.data(), ndims * sizeof(HDim));
    put(p->d_order, order.data(), order.size() * sizeof(u16));
    put(p->d_wstart, wstart.data(), wstart.size() * sizeof(u32));
    put(p->d_prep, p->prep.data(), ndims * sizeof(PrepDim));
    if (!rc && !p->P.err) rc = QMC_ERR_CUDA;
    if (!rc && p->smem > 48 * 1024) rc = ppl == 2 ? gen_smem_attr<2>(p->smem) : gen_smem_attr<1>(p->smem);
    p->P.req = (const HReq *)p->d_req;
    p->P.dims = (const HDim *)p->d_dims;
    p->P.C = (const u32 *)p->d_C;
    p->P.Y = (const u64 *)p->d_Y;
    p->P.recip = (const u64 *)p->d_recip;
    p->P.tail = (const u32 *)p->d_tail;
    p->P.order = (const u16 *)p->d_order;
    p->P.wstart = (const u32 *)p->d_wstart;
    if (rc) {
        qmc_halton_plan_destroy(p);
        return rc;
    }
    *plan = p;
    return QMC_OK;
}

int qmc_halton_plan_create(uint64_t r, uint64_t n, uint64_t n_start, uint64_t d, const qmc_gdn_dim *dims, double *x,
                           qmc_halton_plan **plan)
{
    const qmc_halton_request one{r, n, n_start, d, dims, x};
    return qmc_halton_batch_create(&one, 1, plan);
}

int qmc_halton_plan_prepare(qmc_halton_plan *p, qmc_stream_t s)
{
    QMC_REQUIRE(p, "null plan");
    if (int rc = prepare_launch(p, QMC_STREAM(s))) return rc;
    p->prepared = true;
    return QMC_OK;
}

int qmc_halton_plan_run(qmc_halton_plan *p, qmc_stream_t s)
{
    QMC_REQUIRE(p && p->prepared, "null or unprepared plan (call qmc_halton_plan_prepare)");
    return run_launch(p, QMC_STREAM(s));
}

int qmc_halton_plan_graph_launch(qmc_halton_plan *p, qmc_stream_t s)
{
    QMC_REQUIRE(p, "null plan");
    QMC_REQUIRE(s != nullptr, "graph capture needs a stream other than the legacy default stream");
    cudaStream_t st = QMC_STREAM(s);
    if (!p->exec) {
        if (int rc = qmcgb::cuda_status(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "capture"))
            return rc;
        int lrc = prepare_launch(p, st);
        if (!lrc) lrc = run_launch(p, st);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        if (lrc) {
            if (g) cudaGraphDestroy(g);
            return lrc;
        }
        if (int rc = qmcgb::cuda_status(e, "end capture")) return rc;
        p->graph = g;
        if (int rc = qmcgb::cuda_status(cudaGraphInstantiate(&p->exec, g, 0), "instantiate")) {
            drop_graph(p);
            return rc;
        }
        p->prepared = true;
    }
    return qmcgb::cuda_status(cudaGraphLaunch(p->exec, st), "cudaGraphLaunch");
}

int qmc_halton_plan_set_fp64_share(qmc_halton_plan *p, double share)
{
    QMC_REQUIRE(p && share >= 0.0 && share <= 1.0, "null plan or share outside [0, 1]");
    p->mixed = assign_adds(p->hd, share);
    // the previous run may still read the descriptors; a captured graph holds the kernel variant
    if (int rc = qmcgb::cuda_status(cudaDeviceSynchronize(), "synchronise before rewriting the descriptors"))
        return rc;
    drop_graph(p);
    return qmcgb::cuda_status(cudaMemcpy(p->d_dims, p->hd.data(), p->hd.size() * sizeof(HDim), cudaMemcpyHostToDevice),
                              "copy");
}

int qmc_halton_plan_destroy(qmc_halton_plan *p)
{
    if (!p) return QMC_OK;
    drop_graph(p);
    for (void *q : {p->d_req, p->d_dims, p->d_C, p->d_Y, p->d_recip, p->d_tail, p->d_order, p->d_wstart, p->d_prep})
        if (q) cudaFree(q);
    delete p;
    return QMC_OK;
}

}  // extern "C"
