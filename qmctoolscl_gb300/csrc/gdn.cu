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
// recip_t depend only on (b, t): each CTA computes them once per dimension
// into shared memory.  The per-digit multiply and add are emulated with
// integer operations (dmul_small_bits, dadd_pos_bits) so the FP64 unit,
// slow on GB300, is not on the per-digit path.
//
// Layout in HBM: xdig is r*n*d*tmax (digit t fastest), C is r*d*mmax*tmax,
// S is r*d*tmax_new*tmax, perms r*d*tmax_new*bmax.  Per-point kernels walk
// (row, dimension, digit) as one flat run so stores are contiguous.
#include "common.cuh"

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
        u32 x = (u32)itrue, acc = 0;
        bool ok = true;
        for (u64 k = 0; x; k++) {
            const u32 q = fd_div(di.fd, x);
            const u32 dig = x - q * (u32)di.b;
            x = q;
            if (dig) {
                const u64 cv = read_flat(C, c_off + k * tmax + t, c_total, err);
                if (cv >> 32) { ok = false; break; }
                acc = fd_mod(di.fd, acc + dig * fd_mod(di.fd, (u32)cv));  // < b + b^2 < 2^32
            }
        }
        if (ok) return acc;
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
};

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
    for (u64 f = threadIdx.x; f < total; f += THREADS) {
        const u64 rr = f / per_row, rem = f - rr * per_row;
        const u32 c = (u32)(rem / tmax);
        const u64 t = rem - (u64)c * tmax;
        const u64 i = row0 + rr, j = j0 + c;
        const u64 c_off = l * d * mmax * tmax + j * mmax * tmax;
        xdig[l * n * d * tmax + i * d * tmax + j * tmax + t] =
            gdn_point_digit(dims[c], i + n_start, C, c_off, tmax, t, c_total, err);
    }
}

__global__ void __launch_bounds__(THREADS) gdn_shift_kernel(u64 r, u64 n, u64 d, u64 r_x, u64 r_b, u64 tmax,
                                                            u64 tmax_new, const u64 *bases, const u64 *shifts,
                                                            const u64 *xdig, u64 *xdig_new, PointGrid pg,
                                                            u64 l_off, unsigned *err)
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
    for (u64 f = threadIdx.x; f < total; f += THREADS) {
        const u64 rr = f / per_row, rem = f - rr * per_row;
        const u32 c = (u32)(rem / tmax_new);
        const u64 t = rem - (u64)c * tmax_new;
        const u64 i = row0 + rr, j = j0 + c;
        const u64 sh = shifts[l * d * tmax_new + j * tmax_new + t];
        u64 v;
        if (t < tmax) {
            const u64 sum = xdig[(l % r_x) * n * d * tmax + i * d * tmax + j * tmax + t] + sh;  // wraps as in C
            const DimInfo &di = dims[c];
            if (di.b == 0) {
                atomicOr(err, 2u);
                v = 0;
            } else {
                v = (di.small && sum < (1ull << 32)) ? (u64)fd_mod(di.fd, (u32)sum) : sum % di.b;
            }
        } else {
            v = sh;
        }
        xdig_new[l * n * d * tmax_new + i * d * tmax_new + j * tmax_new + t] = v;
    }
}

__global__ void __launch_bounds__(THREADS) gdn_perm_kernel(u64 r, u64 n, u64 d, u64 r_x, u64 tmax, u64 tmax_new,
                                                           u64 bmax, const u64 *perms, const u64 *xdig,
                                                           u64 *xdig_new, unsigned *err)
{
    const u64 total = r * n * d * tmax_new, p_total = r * d * tmax_new * bmax;
    for (u64 f = (u64)blockIdx.x * blockDim.x + threadIdx.x; f < total; f += (u64)gridDim.x * blockDim.x) {
        const u64 t = f % tmax_new, j = (f / tmax_new) % d, i = (f / (tmax_new * d)) % n;
        const u64 l = f / (tmax_new * d * n);
        const u64 p = t < tmax ? xdig[(l % r_x) * n * d * tmax + i * d * tmax + j * tmax + t] : 0;
        const u64 flat = l * d * tmax_new * bmax + j * tmax_new * bmax + t * bmax + p;
        xdig_new[f] = read_flat(perms, flat, p_total, err);
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

// v = sum_t recip_t * digit_t with the reference's rounding sequence
__device__ __forceinline__ double digits_to_double(const double *rc, const u64 *dig, u64 tmax)
{
    u64 v = 0;  // bits of a non-negative double
    for (u64 t = 0; t < tmax; t++) {
        const u64 dg = dig[t];
        if (dg == 0) continue;  // adds +0: v unchanged
        const u64 rb = as_bits(rc[t]);
        const u32 er = (u32)(rb >> 52);
        if (dg < 2048 && er >= 1 && er < 2036 && ((v >> 52) < 2000)) {
            const u64 p = dmul_small_bits(rb, (u32)dg);
            v = dadd_pos_bits(v, p);
        } else {
            v = digit_step_hw(v, rc[t], dg);
        }
    }
    return as_double(v);
}

constexpr u32 I2F_DIMS = 32;   // dimensions per CTA
constexpr u32 I2F_TMAX = 64;   // recip table depth held in shared memory

__global__ void __launch_bounds__(THREADS) gdn_to_float_kernel(u64 r, u64 n, u64 d, u64 r_b, u64 tmax,
                                                               const u64 *bases, const u64 *xdig, double *x,
                                                               u64 rows_per_cta, u32 dim_tiles, u64 l_off)
{
    __shared__ double rc[I2F_DIMS][I2F_TMAX];
    const u64 l = l_off + (u64)blockIdx.y / dim_tiles;
    if (l >= r) return;
    const u64 j0 = (u64)(blockIdx.y % dim_tiles) * I2F_DIMS;
    const u32 nd = (u32)min((u64)I2F_DIMS, d - j0);
    const bool table = tmax <= I2F_TMAX;
    if (table)
        for (u32 c = threadIdx.x; c < nd; c += blockDim.x) fill_recips(rc[c], bases[(l % r_b) * d + j0 + c], tmax);
    __syncthreads();
    const u64 row0 = (u64)blockIdx.x * rows_per_cta;
    if (row0 >= n) return;
    const u64 rows = min(rows_per_cta, n - row0);
    const u64 total = rows * nd;
    for (u64 f = threadIdx.x; f < total; f += THREADS) {
        const u64 rr = f / nd;
        const u32 c = (u32)(f - rr * nd);
        const u64 i = row0 + rr, j = j0 + c;
        const u64 *dg = xdig + l * n * d * tmax + i * d * tmax + j * tmax;
        double v;
        if (table) {
            v = digits_to_double(rc[c], dg, tmax);
        } else {  // deep digit expansions: the reference's loop as written
            const double bd = __ull2double_rn(bases[(l % r_b) * d + j]);
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

PointGrid point_grid(u64 r, u64 n, u64 d, u64 per_point, u32 dim_tile, u64 *splits_out)
{
    PointGrid pg;
    pg.dim_tiles = (u32)((d + dim_tile - 1) / dim_tile);
    const u64 units = r * pg.dim_tiles;
    const u64 want = (u64)qmcgb::sm_count() * 8;
    u64 splits = (want + units - 1) / units;
    // at least ~2 elements per thread in a CTA
    const u64 per_row = (d < dim_tile ? d : dim_tile) * (per_point ? per_point : 1);
    const u64 min_rows = (2 * THREADS + per_row - 1) / per_row;
    const u64 max_splits = (n + min_rows - 1) / min_rows;
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    pg.rows_per_cta = (n + splits - 1) / splits;
    *splits_out = splits;
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

}  // namespace

extern "C" {

int qmc_gdn_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t r_b, uint64_t mmax, uint64_t tmax,
                        uint64_t n_start, const uint64_t *bases, const uint64_t *C, uint64_t *xdig, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0 || tmax == 0) return QMC_OK;
    QMC_REQUIRE(r_b > 0 && bases && C && xdig, "bad r_b or null array pointer");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
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
    gdn_perm_kernel<<<flat_grid(total), 256, 0, QMC_STREAM(s)>>>(r, n, d, r_x, tmax, tmax_new, bmax,
                                                                 (const u64 *)perms, (const u64 *)xdig,
                                                                 (u64 *)xdig_new, err);
    return qmcgb::launch_status("gdn_digital_permutation");
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
    const PointGrid pg = point_grid(r, n, d, tmax_new, DIM_TILE, &splits);
    return launch_points(r, pg.dim_tiles, [&](u64 l0, unsigned cnt) {
        gdn_shift_kernel<<<dim3((unsigned)splits, cnt, 1), THREADS, 0, QMC_STREAM(s)>>>(
            r, n, d, r_x, r_b, tmax, tmax_new, (const u64 *)bases, (const u64 *)shifts, (const u64 *)xdig,
            (u64 *)xdig_new, pg, l0, err);
    }, "gdn_digital_shift");
}

int qmc_gdn_integer_to_float(uint64_t r, uint64_t n, uint64_t d, uint64_t r_b, uint64_t tmax, const uint64_t *bases,
                             const uint64_t *xdig, double *x, qmc_stream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(r_b > 0 && bases && x && (tmax == 0 || xdig), "bad r_b or null array pointer");
    u64 splits;
    const PointGrid pg = point_grid(r, n, d, 1, I2F_DIMS, &splits);
    return launch_points(r, pg.dim_tiles, [&](u64 l0, unsigned cnt) {
        gdn_to_float_kernel<<<dim3((unsigned)splits, cnt, 1), THREADS, 0, QMC_STREAM(s)>>>(
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
