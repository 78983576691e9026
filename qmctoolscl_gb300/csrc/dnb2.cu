// dnb2.cu -- digital nets in base 2: point generation in natural and Gray
// order, digital shift, integer-to-float, and the matrix-side operations
// (linear matrix scrambling, interlacing and its inverse, LSB->MSB).
//
// Reference: qmctoolscl/c_funcs/dnb2_gen_natural.c:3-70,
// dnb2_gen_gray.c:3-69, dnb2_digital_shift.c:3-36,
// dnb2_integer_to_float.c:3-32, dnb2_linear_matrix_scramble.c:3-51,
// dnb2_interlace.c:3-45, dnb2_undo_interlace.c:3-45,
// dnb2_gmat_lsb_to_msb.c:3-44.
//
// Generation.  The reference builds point i from point i-1 by XOR-ing the
// generating-matrix column picked by the lowest set bit of the index (a
// serial recurrence).  Its result is linear over GF(2): the point with
// sequence index m is the XOR of the columns C[b] over the set bits b of m
// (natural order: m = n_start+k; Gray order: m = gray(n_start+i)).  Each CTA
// owns one randomisation, a column tile and a run of rows.  It stages in
// shared memory a table T[lo][c] = XOR of the columns picked by the K low
// bits lo, built by doubling from the generating matrix, plus the columns
// for the high bits.  A point is then T[m mod 2^K] XOR H[m >> K], where H
// (the XOR over the high bits) is recomputed only when m >> K changes -- one
// shared-memory load and one XOR per coordinate, independent of the number
// of bits in the index.  A digital shift (x << lshift) ^ s distributes over
// the XOR, so the fused kernel folds it into the table and into H, and the
// integer-to-float conversion is done in registers before the store.
//
// Layout in HBM: xb/xrb/x are r*n*d, d fastest.  Threads walk the CTA's
// tile as one flat run of (row, column) pairs, so each step of the CTA
// writes 256 consecutive words.
#include <type_traits>

#include "net_dev.cuh"

namespace {

using net::MAX_COLS;
using net::to_float_bits;
constexpr int GEN_THREADS = 256;
constexpr int MAX_BITS = 64;  // generating-matrix columns

struct GenArgs {
    u64 r, n, d, n_start, mmax;
    const u64 *C;        // r_C*d*mmax generating matrices
    u64 r_C;             // randomisation l uses matrix set l % r_C
    u64 *xb;             // r*n*d integer output (may be null when only floats are wanted)
    double *x;           // r*n*d float output (may be null)
    const u64 *lshifts;  // r_x-periodic left shifts (with shifts)
    const u64 *shifts;   // r*d digital shifts (may be null)
    u64 r_x;             // period of lshifts
    const u64 *tmaxes;   // r bit counts (with x)
    u32 K;               // low bits resolved by the table
    u32 col_tiles;       // column tiles per randomisation
    u64 rows_per_cta;
    u64 l_off;           // first randomisation of this launch
};

// grid x: row blocks; grid y: (randomisation, column tile)
template <bool GRAY>
__global__ void __launch_bounds__(GEN_THREADS) dnb2_gen_kernel(GenArgs a)
{
    extern __shared__ u64 smem[];
    const u64 l = a.l_off + (u64)blockIdx.y / a.col_tiles;
    if (l >= a.r) return;
    const u32 tile = (u32)((u64)blockIdx.y % a.col_tiles);
    const u64 j0 = (u64)tile * MAX_COLS;
    const u32 ncols = (u32)min((u64)MAX_COLS, a.d - j0);
    u64 *T = smem;
    u64 *H = smem + ((u64)1 << a.K) * ncols;
    const u32 ls = a.shifts ? (u32)(a.lshifts[l % a.r_x] & 63) : 0u;
    net::build_table(T, H, a.C + (l % a.r_C) * a.d * a.mmax, a.mmax, j0, ncols, a.K, ls,
                     a.shifts ? a.shifts + l * a.d : nullptr);
    const int e_float = a.x ? (int)(u32)(0ull - a.tmaxes[l]) : 0;
    const u64 row_begin = (u64)blockIdx.x * a.rows_per_cta;
    if (row_begin >= a.n) return;
    const u64 row_end = min(a.n, row_begin + a.rows_per_cta);
    net::gen_rows<GRAY>(T, H, a.K, ncols, a.n_start, a.d, row_begin, row_end,
                        a.xb ? a.xb + l * a.n * a.d + j0 : nullptr, a.x ? a.x + l * a.n * a.d + j0 : nullptr,
                        e_float);
}

// ---------------------------------------------------------------------------
// elementwise kernels

// Rows per thread per iteration: all loads of a group are issued before any
// arithmetic so each thread keeps several loads outstanding.
constexpr int ROWS_IN_FLIGHT = 4;

template <int VEC>
__global__ void __launch_bounds__(256) dnb2_shift_kernel(u64 r, u64 n, u64 d, u64 r_x, const u64 *lshifts,
                                                         const u64 *xb, const u64 *shiftsb, u64 *xrb)
{
    typedef typename std::conditional<VEC == 2, ulonglong2, u64>::type vec_t;
    const u64 ngroups = (d + VEC - 1) / VEC;
    const u64 row_stride = (u64)gridDim.x * blockDim.y;
    const u64 dv = d / VEC;
    for (u64 l = blockIdx.y; l < r; l += gridDim.y) {
        const u32 ls = (u32)(lshifts[l % r_x] & 63);
        const vec_t *in = (const vec_t *)(xb + (l % r_x) * n * d);
        vec_t *out = (vec_t *)(xrb + l * n * d);
        for (u64 jg = threadIdx.x; jg < ngroups; jg += blockDim.x) {
            u64 s[VEC];
#pragma unroll
            for (int v = 0; v < VEC; v++) s[v] = shiftsb[l * d + jg * VEC + v];
            for (u64 i0 = (u64)blockIdx.x * blockDim.y + threadIdx.y; i0 < n; i0 += ROWS_IN_FLIGHT * row_stride) {
                vec_t w[ROWS_IN_FLIGHT];
#pragma unroll
                for (int u = 0; u < ROWS_IN_FLIGHT; u++) {
                    const u64 i = i0 + u * row_stride;
                    if (i < n) w[u] = __ldcs(in + i * dv + jg);
                }
#pragma unroll
                for (int u = 0; u < ROWS_IN_FLIGHT; u++) {
                    const u64 i = i0 + u * row_stride;
                    if (i >= n) break;
                    if constexpr (VEC == 2)
                        __stcs(out + i * dv + jg, make_ulonglong2((w[u].x << ls) ^ s[0], (w[u].y << ls) ^ s[1]));
                    else
                        __stcs(out + i * dv + jg, (w[u] << ls) ^ s[0]);
                }
            }
        }
    }
}

template <int VEC>
__global__ void __launch_bounds__(256) dnb2_to_float_kernel(u64 r, u64 n, u64 d, const u64 *tmaxes,
                                                            const u64 *xb, double *x)
{
    typedef typename std::conditional<VEC == 2, ulonglong2, u64>::type in_t;
    typedef typename std::conditional<VEC == 2, double2, double>::type out_t;
    const u64 ngroups = (d + VEC - 1) / VEC;
    const u64 row_stride = (u64)gridDim.x * blockDim.y;
    const u64 dv = d / VEC;
    for (u64 l = blockIdx.y; l < r; l += gridDim.y) {
        const int e = (int)(u32)(0ull - tmaxes[l]);
        const in_t *in = (const in_t *)(xb + l * n * d);
        out_t *out = (out_t *)(x + l * n * d);
        for (u64 jg = threadIdx.x; jg < ngroups; jg += blockDim.x) {
            for (u64 i0 = (u64)blockIdx.x * blockDim.y + threadIdx.y; i0 < n; i0 += ROWS_IN_FLIGHT * row_stride) {
                in_t w[ROWS_IN_FLIGHT];
#pragma unroll
                for (int u = 0; u < ROWS_IN_FLIGHT; u++) {
                    const u64 i = i0 + u * row_stride;
                    if (i < n) w[u] = __ldcs(in + i * dv + jg);
                }
#pragma unroll
                for (int u = 0; u < ROWS_IN_FLIGHT; u++) {
                    const u64 i = i0 + u * row_stride;
                    if (i >= n) break;
                    if constexpr (VEC == 2)
                        __stcs(out + i * dv + jg, make_double2(to_float_bits(w[u].x, e), to_float_bits(w[u].y, e)));
                    else
                        __stcs(out + i * dv + jg, to_float_bits(w[u], e));
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// matrix-side kernels: one thread per output column word

__global__ void dnb2_lms_kernel(u64 r, u64 d, u64 mmax, u64 r_C, u64 tmax_new, const u64 *S,
                                const u64 *C, u64 *C_lms)
{
    const u64 total = r * d * mmax, nelem_C = r_C * d * mmax;
    for (u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (u64)gridDim.x * blockDim.x) {
        const u64 lj = idx / mmax;  // l*d + j
        const u64 col = C[idx % nelem_C];
        const u64 *srow = S + lj * tmax_new;
        u64 out = 0;
        for (u64 t = 0; t < tmax_new; t++)
            if (__popcll(srow[t] & col) & 1) out += shl64(1ull, tmax_new - t - 1);
        C_lms[idx] = out;
    }
}

__device__ __forceinline__ u64 read_flat(const u64 *base, u64 flat, u64 total, unsigned *err)
{
    if (flat < total) return base[flat];
    atomicOr(err, 1u);
    return 0;
}

__global__ void dnb2_interlace_kernel(u64 r, u64 d_alpha, u64 mmax, u64 d, u64 tmax, u64 tmax_alpha,
                                      u64 alpha, const u64 *C, u64 *C_alpha, unsigned *err)
{
    const u64 total = r * d_alpha * mmax, c_total = r * d * mmax;
    for (u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (u64)gridDim.x * blockDim.x) {
        const u64 k = idx % mmax, ja = (idx / mmax) % d_alpha, l = idx / (mmax * d_alpha);
        u64 out = 0;
        for (u64 ta = 0; ta < tmax_alpha; ta++) {
            const u64 t = ta / alpha, j = ja * alpha + ta % alpha;
            if (shr64(read_flat(C, l * d * mmax + j * mmax + k, c_total, err), tmax - t - 1) & 1)
                out += shl64(1ull, tmax_alpha - ta - 1);
        }
        C_alpha[idx] = out;
    }
}

__global__ void dnb2_undo_interlace_kernel(u64 r, u64 d, u64 mmax, u64 d_alpha, u64 tmax, u64 tmax_alpha,
                                           u64 alpha, const u64 *C_alpha, u64 *C, unsigned *err)
{
    const u64 total = r * d * mmax, a_total = r * d_alpha * mmax;
    for (u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (u64)gridDim.x * blockDim.x) {
        const u64 k = idx % mmax, j = (idx / mmax) % d, l = idx / (mmax * d);
        const u64 ja = j / alpha, jr = j % alpha;
        const u64 word = read_flat(C_alpha, l * d_alpha * mmax + ja * mmax + k, a_total, err);
        u64 out = 0;
        for (u64 t = 0; t < tmax; t++)
            if (shr64(word, tmax_alpha - (t * alpha + jr) - 1) & 1) out += shl64(1ull, tmax - t - 1);
        C[idx] = out;
    }
}

__global__ void dnb2_lsb_to_msb_kernel(u64 r, u64 d, u64 mmax, const u64 *tmaxes, const u64 *C_lsb, u64 *C_msb)
{
    const u64 total = r * d * mmax;
    for (u64 idx = (u64)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (u64)gridDim.x * blockDim.x) {
        const u64 tmax = tmaxes[idx / (d * mmax)];
        u64 v = C_lsb[idx], out = 0;
        for (u64 t = 0; v; v >>= 1, t++)
            if (v & 1) out += shl64(1ull, tmax - t - 1);
        C_msb[idx] = out;
    }
}

// ---------------------------------------------------------------------------
// host side

struct Shape {
    dim3 grid, block;
};

Shape rows_shape(u64 r, u64 n, u64 ngroups)
{
    u32 bx = 1;
    while (bx < ngroups && bx < 32) bx <<= 1;
    const u32 by = 256 / bx;
    u64 per_l = (u64)qmcgb::sm_count() * 16 / (r ? r : 1);
    if (per_l < 1) per_l = 1;
    u64 gx = (n + by - 1) / by;
    if (gx > per_l) gx = per_l;
    if (gx < 1) gx = 1;
    Shape s;
    s.grid = dim3((unsigned)gx, (unsigned)(r < 65535 ? (r ? r : 1) : 65535), 1);
    s.block = dim3(bx, by, 1);
    return s;
}

unsigned flat_grid(u64 total) { return qmcgb::grid_for(total, 256, (unsigned)qmcgb::sm_count() * 32); }

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

template <bool GRAY>
int launch_gen(GenArgs a, cudaStream_t s, const char *what)
{
    const u32 ncols = (u32)(a.d < MAX_COLS ? a.d : MAX_COLS);
    a.K = net::pick_K(a.mmax, ncols);
    a.col_tiles = (u32)((a.d + MAX_COLS - 1) / MAX_COLS);
    const u64 units = a.r * a.col_tiles;
    // a small problem takes a smaller table, so that row runs of at least four table lengths
    // still give every SM two CTAs (the high bits' XOR is redone once per 2^K rows)
    while (a.K > 4 && units * ((a.n + (4ull << a.K) - 1) / (4ull << a.K)) < (u64)qmcgb::sm_count() * 2) a.K--;
    // enough CTAs to fill the GPU several times; each CTA covers a row run of
    // at least four table lengths so building the table stays a small cost
    const size_t smem = net::table_words(a.K, a.mmax, ncols) * sizeof(u64);
    auto kern = dnb2_gen_kernel<GRAY>;
    if (int rc = qmcgb::raise_smem_limit((const void *)kern, smem, what)) return rc;
    // four waves of resident CTAs (the table's shared memory limits how many fit per SM): short
    // row runs balance the SMs; one wave of long runs, or 8 CTAs per SM against 6 resident (a
    // third of a wave left over), measured slower
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, GEN_THREADS, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const u64 want = (u64)qmcgb::sm_count() * (u64)per_sm * 4;
    u64 splits = want >= units ? want / units : 1;
    const u64 min_rows = 4ull << a.K;
    const u64 max_splits = (a.n + min_rows - 1) / min_rows;
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    a.rows_per_cta = (a.n + splits - 1) / splits;
    // blockIdx.y enumerates (randomisation, column tile), at most 65535 per launch
    const u64 l_per_launch = 65535 / a.col_tiles;
    for (u64 l0 = 0; l0 < a.r; l0 += l_per_launch) {
        const u64 cnt = (a.r - l0 < l_per_launch ? a.r - l0 : l_per_launch) * a.col_tiles;
        a.l_off = l0;
        kern<<<dim3((unsigned)splits, (unsigned)cnt, 1), GEN_THREADS, smem, s>>>(a);
        if (int rc = qmcgb::launch_status(what)) return rc;
    }
    return QMC_OK;
}

// True when the Gray code maps [lo, hi) onto itself, checked on
// the dyadic blocks of the range: the Gray code sends the aligned block
// q*2^k + [0, 2^k) onto gray(q)*2^k + [0, 2^k).
bool gray_closed(u64 lo, u64 hi)
{
    u64 a = lo;
    while (a < hi) {
        u32 k = a ? (u32)__builtin_ctzll(a) : 63;
        while (k > 0 && (k >= 64 || a + (1ull << k) > hi || a + (1ull << k) < a)) k--;
        const u64 q = a >> k;
        const u64 g = q ^ (q >> 1);
        const u64 blo = g << k;
        const u64 bhi = blo + (1ull << k);
        if (blo < lo || bhi > hi) return false;
        a += 1ull << k;
    }
    return true;
}

u32 bitlen(u64 v) { return v ? 64u - (u32)__builtin_clzll(v) : 0u; }

}  // namespace

namespace qmcgb {

// Fused digital-net generation: xrb = (point << lshift) ^ shift and/or
// x = ldexp(xrb, -tmax), with point in natural or Gray order.  Any of the
// shift/float stages can be skipped by passing null pointers.
int dnb2_gen_fused(u64 r, u64 n, u64 d, u64 n_start, u64 mmax, const u64 *C, u64 r_C, int gray,
                   const u64 *lshifts, u64 r_x, const u64 *shifts, const u64 *tmaxes, u64 *xrb, double *x,
                   cudaStream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(mmax <= MAX_BITS, "mmax %llu above 64", (unsigned long long)mmax);
    GenArgs a{};
    a.r = r; a.n = n; a.d = d; a.n_start = n_start; a.mmax = mmax;
    a.C = C; a.r_C = r_C ? r_C : 1;
    a.xb = xrb; a.x = x;
    a.lshifts = lshifts; a.shifts = shifts; a.r_x = r_x ? r_x : 1; a.tmaxes = tmaxes;
    const bool sh = shifts != nullptr, fl = x != nullptr, wi = xrb != nullptr;
    QMC_REQUIRE(!sh || lshifts, "shift stage needs lshifts");
    QMC_REQUIRE(!fl || tmaxes, "float stage needs tmaxes");
    QMC_REQUIRE(fl || wi, "nothing to write");
    (void)sh;
    return gray ? launch_gen<true>(a, s, "dnb2_gen") : launch_gen<false>(a, s, "dnb2_gen");
}

int dnb2_check_gen(u64 n, u64 n_start, u64 mmax, int natural)
{
    if (n == 0) return QMC_OK;
    QMC_REQUIRE_DOMAIN(n_start + n >= n_start, "index range overflows");
    if (natural)
        QMC_REQUIRE_DOMAIN(gray_closed(n_start, n_start + n),
                           "dnb2_gen_natural: the Gray code does not map [n_start, n_start+n) onto itself "
                           "(the reference writes outside xb)");
    QMC_REQUIRE_DOMAIN(bitlen(n_start + n - 1) <= mmax,
                       "sequence index needs %u bits but the generating matrices have mmax=%llu columns",
                       bitlen(n_start + n - 1), (unsigned long long)mmax);
    return QMC_OK;
}

}  // namespace qmcgb

extern "C" {

int qmc_dnb2_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, uint64_t mmax, const uint64_t *C,
                         uint64_t *xb, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(C && xb, "null array pointer");
    if (int rc = qmcgb::dnb2_check_gen(n, n_start, mmax, 1)) return rc;
    return qmcgb::dnb2_gen_fused(r, n, d, n_start, mmax, (const u64 *)C, r, 0, nullptr, 1, nullptr,
                                 nullptr, (u64 *)xb, nullptr, QMC_STREAM(s));
}

int qmc_dnb2_gen_gray(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, uint64_t mmax, const uint64_t *C,
                      uint64_t *xb, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(C && xb, "null array pointer");
    if (int rc = qmcgb::dnb2_check_gen(n, n_start, mmax, 0)) return rc;
    return qmcgb::dnb2_gen_fused(r, n, d, n_start, mmax, (const u64 *)C, r, 1, nullptr, 1, nullptr,
                                 nullptr, (u64 *)xb, nullptr, QMC_STREAM(s));
}

int qmc_dnb2_digital_shift(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, const uint64_t *lshifts,
                           const uint64_t *xb, const uint64_t *shiftsb, uint64_t *xrb, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(r_x > 0 && lshifts && xb && shiftsb && xrb, "bad r_x or null array pointer");
    const bool vec2 = d % 2 == 0 && aligned16(xb) && aligned16(xrb);
    const Shape sh = rows_shape(r, n, vec2 ? d / 2 : d);
    if (vec2)
        dnb2_shift_kernel<2><<<sh.grid, sh.block, 0, QMC_STREAM(s)>>>(r, n, d, r_x, (const u64 *)lshifts,
                                                                      (const u64 *)xb, (const u64 *)shiftsb,
                                                                      (u64 *)xrb);
    else
        dnb2_shift_kernel<1><<<sh.grid, sh.block, 0, QMC_STREAM(s)>>>(r, n, d, r_x, (const u64 *)lshifts,
                                                                      (const u64 *)xb, (const u64 *)shiftsb,
                                                                      (u64 *)xrb);
    return qmcgb::launch_status("dnb2_digital_shift");
}

int qmc_dnb2_integer_to_float(uint64_t r, uint64_t n, uint64_t d, const uint64_t *tmaxes, const uint64_t *xb,
                              double *x, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(tmaxes && xb && x, "null array pointer");
    const bool vec2 = d % 2 == 0 && aligned16(xb) && aligned16(x);
    const Shape sh = rows_shape(r, n, vec2 ? d / 2 : d);
    if (vec2)
        dnb2_to_float_kernel<2><<<sh.grid, sh.block, 0, QMC_STREAM(s)>>>(r, n, d, (const u64 *)tmaxes,
                                                                         (const u64 *)xb, x);
    else
        dnb2_to_float_kernel<1><<<sh.grid, sh.block, 0, QMC_STREAM(s)>>>(r, n, d, (const u64 *)tmaxes,
                                                                         (const u64 *)xb, x);
    return qmcgb::launch_status("dnb2_integer_to_float");
}

int qmc_dnb2_linear_matrix_scramble(uint64_t r, uint64_t d, uint64_t mmax, uint64_t r_C, uint64_t tmax_new,
                                    const uint64_t *S, const uint64_t *C, uint64_t *C_lms, qmc_stream_t s)
{
    const u64 total = r * d * mmax;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(r_C > 0 && S && C && C_lms, "bad r_C or null array pointer");
    dnb2_lms_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(r, d, mmax, r_C, tmax_new, (const u64 *)S,
                                                                 (const u64 *)C, (u64 *)C_lms);
    return qmcgb::launch_status("dnb2_linear_matrix_scramble");
}

int qmc_dnb2_interlace(uint64_t r, uint64_t d_alpha, uint64_t mmax, uint64_t d, uint64_t tmax, uint64_t tmax_alpha,
                       uint64_t alpha, const uint64_t *C, uint64_t *C_alpha, qmc_stream_t s)
{
    const u64 total = r * d_alpha * mmax;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(alpha > 0 && C && C_alpha, "bad alpha or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    dnb2_interlace_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(r, d_alpha, mmax, d, tmax, tmax_alpha,
                                                                       alpha, (const u64 *)C, (u64 *)C_alpha, err);
    return qmcgb::launch_status("dnb2_interlace");
}

int qmc_dnb2_undo_interlace(uint64_t r, uint64_t d, uint64_t mmax, uint64_t d_alpha, uint64_t tmax,
                            uint64_t tmax_alpha, uint64_t alpha, const uint64_t *C_alpha, uint64_t *C,
                            qmc_stream_t s)
{
    const u64 total = r * d * mmax;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(alpha > 0 && C_alpha && C, "bad alpha or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    dnb2_undo_interlace_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(
        r, d, mmax, d_alpha, tmax, tmax_alpha, alpha, (const u64 *)C_alpha, (u64 *)C, err);
    return qmcgb::launch_status("dnb2_undo_interlace");
}

int qmc_dnb2_gmat_lsb_to_msb(uint64_t r, uint64_t d, uint64_t mmax, const uint64_t *tmaxes, const uint64_t *C_lsb,
                             uint64_t *C_msb, qmc_stream_t s)
{
    const u64 total = r * d * mmax;
    if (total == 0) return QMC_OK;
    QMC_REQUIRE(tmaxes && C_lsb && C_msb, "null array pointer");
    dnb2_lsb_to_msb_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(r, d, mmax, (const u64 *)tmaxes,
                                                                        (const u64 *)C_lsb, (u64 *)C_msb);
    return qmcgb::launch_status("dnb2_gmat_lsb_to_msb");
}

// Fused digital-net pipeline: generation in natural (gray=0) or Gray
// (gray=1) order, then (when shiftsb is not null) the digital shift
// (point << lshifts[l % r_x]) ^ shiftsb[l,j], then (when x is not null) the
// conversion ldexp(value, -tmaxes[l]).  xrb may be null when only the
// floats are wanted.  C has r_C*d*mmax words; randomisation l uses matrix
// set l % r_C and left shift lshifts[l % r_x].
int qmc_dnb2_gen_fused(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, uint64_t mmax, const uint64_t *C,
                       uint64_t r_C, int gray, const uint64_t *lshifts, uint64_t r_x, const uint64_t *shiftsb,
                       const uint64_t *tmaxes, uint64_t *xrb, double *x, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(C, "null generating matrices");
    if (int rc = qmcgb::dnb2_check_gen(n, n_start, mmax, !gray)) return rc;
    return qmcgb::dnb2_gen_fused(r, n, d, n_start, mmax, (const u64 *)C, r_C, gray,
                                 (const u64 *)lshifts, r_x, (const u64 *)shiftsb, (const u64 *)tmaxes,
                                 (u64 *)xrb, x, QMC_STREAM(s));
}

}  // extern "C"
