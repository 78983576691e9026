// rand.cu -- the randomisation inputs on the GPU, bit for bit the reference's
// numpy helpers (qmctoolscl/rand_funcs.py:4-153) with numpy's SFC64 streams:
// the same draws in the same order from one Generator, whose six state words
// live in device memory and are advanced in place.
//
// A Generator's stream is serial (SFC64 has no jump-ahead), so one thread runs
// it: it draws exactly what numpy draws, in numpy's order, and stores each
// value where the helper puts it.  The permutation helpers, which draw the
// most, run their stream in one CTA instead: a producer lane steps the
// generator and a warp decides which outputs the masked rejection accepts, 32
// at a time (fy_stream.cuh).  What does not depend on the stream runs wide:
// the zero fill before it, and for the permutation helpers the Fisher-Yates
// swaps themselves -- the stream only writes the swap index j_i into entry i
// of each row, and one thread per row then replays the swaps on arange(b) in
// shared memory and writes the permutation over the indices.
//
// Every rejection loop is bounded; a loop that runs out (an impossible stream)
// sets bit 32 of the device error word.  A base for which numpy would raise
// (below 2 for the scrambling matrices, 0 for the shifts) or one above the
// permutation width sets bit 128 and stops the stream there.
#include "fy_stream.cuh"

namespace {

constexpr unsigned ERR_STREAM = 32u;
constexpr unsigned ERR_BASE = 128u;  // a base the helper cannot draw for (the stream stops there)

// ---- single-thread stream kernels ----------------------------------------------------

// Generator.random(count) (lat_get_shifts: count = r*d)
__global__ void __launch_bounds__(32) rng_uniform_kernel(u64 *state, u64 count, double *out)
{
    if (threadIdx.x != 0) return;
    Sfc64 g;
    g.load(state);
    for (u64 k = 0; k < count; k++) out[k] = g.uniform();
    g.store(state);
}

// random_tbit_uint64s(rng, t, count); with tmax >= 1 the rows of
// dnb2_get_linear_scramble_matrix: value k is row t = k % tmax_new, and rows
// t < tmin keep their bits above position tmin - t and get bit tmax - 1 - t
__global__ void __launch_bounds__(32) rng_tbits_kernel(u64 *state, u32 t, u64 count, u64 *out, u32 lms_tmax,
                                                       u32 lms_tmax_new)
{
    if (threadIdx.x != 0) return;
    Sfc64 g;
    g.load(state);
    if (lms_tmax == 0) {
        for (u64 k = 0; k < count; k++) out[k] = g.bits(t);
    } else {
        u32 row = 0;
        for (u64 k = 0; k < count; k++) {
            u64 x = g.bits(t);
            if (row < t) {
                const u32 drop = t - row;  // numpy's shift by 64 or more gives 0
                x = drop >= 64 ? 0 : (x >> drop) << drop;
                x += 1ull << (lms_tmax - 1 - row);
            }
            out[k] = x;
            if (++row == lms_tmax_new) row = 0;
        }
    }
    g.store(state);
}

__device__ __forceinline__ u64 base_of(const u64 *bases, u64 r_b, u64 d, u64 l, u64 j)
{
    return bases[(l % r_b) * d + j];
}

// gdn_get_linear_scramble_matrix: per (l, j) the strictly lower entries of the
// (tmax_new x tmax) matrix in row-major order from integers(0, b), then the
// tmax diagonal entries from integers(1, b); the rest stays zero (filled
// before)
__global__ void __launch_bounds__(32) gdn_lms_rand_kernel(u64 *state, u64 r, u64 d, u32 tmax, u32 tmax_new, u64 r_b,
                                                          const u64 *bases, u64 *S, unsigned *err)
{
    if (threadIdx.x != 0) return;
    Sfc64 g;
    g.load(state);
    bool bad = false;
    for (u64 l = 0; l < r; l++)
        for (u64 j = 0; j < d; j++) {
            const u64 b = base_of(bases, r_b, d, l, j);
            if (b < 2) {  // numpy refuses integers(1, b) for b < 2
                atomicOr(err, ERR_BASE);
                g.store(state);
                return;
            }
            u64 *M = S + (l * d + j) * tmax_new * tmax;
            for (u32 t = 1; t < tmax_new; t++) {
                const u32 cend = t < tmax ? t : tmax;
                for (u32 c = 0; c < cend; c++) M[(u64)t * tmax + c] = g.bounded(0, b - 1, &bad);
            }
            for (u32 t = 0; t < tmax; t++) M[(u64)t * tmax + t] = g.bounded(1, b - 2, &bad);
        }
    if (bad) atomicOr(err, ERR_STREAM);
    g.store(state);
}

// gdn_get_digital_shifts: per (l, j) tmax_new values from integers(0, b)
__global__ void __launch_bounds__(32) gdn_shift_rand_kernel(u64 *state, u64 r, u64 d, u32 tmax_new, u64 r_b,
                                                            const u64 *bases, u64 *out, unsigned *err)
{
    if (threadIdx.x != 0) return;
    Sfc64 g;
    g.load(state);
    bool bad = false;
    for (u64 l = 0; l < r; l++)
        for (u64 j = 0; j < d; j++) {
            const u64 b = base_of(bases, r_b, d, l, j);
            if (b < 1) {  // numpy refuses integers(0, 0)
                atomicOr(err, ERR_BASE);
                g.store(state);
                return;
            }
            u64 *o = out + (l * d + j) * tmax_new;
            for (u32 t = 0; t < tmax_new; t++) o[t] = g.bounded(0, b - 1, &bad);
        }
    if (bad) atomicOr(err, ERR_STREAM);
    g.store(state);
}

// the swap indices of Generator.permutation(b) for every row: rows of `width`
// entries, row q = (l*d + j)*levels + t with base b(l, j) (bases == nullptr:
// one base b0 for every row); entry i of a row gets j_i, i = b-1 .. 1.  One
// CTA runs the stream (fy_stream.cuh), the (l, j) pairs as runs of rows; a
// base above the row width stops the stream there.  Rows that all share one
// base of at most FY_SMALL_MAX take the small-base decoder as one run.
struct PermRows {
    const u64 *bases;
    u64 r, d, levels, r_b, b0, width;
    u64 *out;
    unsigned *err;
    u64 lj;   // the next (l, j) pair
    u64 *cur;  // rows of the current pair
    __device__ bool next(u32 &b, u64 &rows)
    {
        if (lj >= r * d) return false;
        const u64 bb = bases ? base_of(bases, r_b, d, lj / d, lj % d) : b0;
        if (bb > width) {  // a row holds `width` entries
            atomicOr(err, ERR_BASE);
            lj = r * d;
            return false;
        }
        cur = out + lj * levels * width;
        lj++;
        b = (u32)bb;
        rows = levels;
        return true;
    }
    __device__ void put(u64 q, u32 i, u32 j) { cur[q * width + i] = j; }
};

// all rows of one small base: row q at out + q*width
struct PermRowsFlat {
    u64 *out;
    u64 width;
    __device__ void put(u64 q, u32 i, u32 j) { out[q * width + i] = j; }
};

__global__ void __launch_bounds__(FY_THREADS) perm_stream_kernel(u64 *state, u64 r, u64 d, u64 levels, u64 r_b,
                                                                 const u64 *bases, u64 b0, u64 width, u64 *out,
                                                                 unsigned *err)
{
    __shared__ FyShared sh;
    __shared__ u64 one_base;  // the base of every row, or 0
    if (threadIdx.x == 0) {
        u64 bb = bases ? base_of(bases, r_b, d, 0, 0) : b0;
        if (bases)
            for (u64 lj = 0; lj < (r < r_b ? r : r_b) * d && bb; lj++)
                if (base_of(bases, r_b, d, lj / d, lj % d) != bb) bb = 0;
        one_base = bb;
    }
    __syncthreads();
    const u64 bb = one_base;
    if (bb >= 2 && bb <= FY_SMALL_MAX && bb <= width) {  // one run of a small base
        PermRowsFlat P{out, width};
        fy_stream_small(sh, state, (u32)bb, r * d * levels, P, err, ERR_STREAM);
    } else {
        PermRows R{bases, r, d, levels, r_b, b0, width, out, err, 0, out};
        fy_stream(sh, state, R, err, ERR_STREAM);
    }
}

// ---- wide passes ------------------------------------------------------------------

// one thread per row: arange(b) in column t of a (b x T) shared-memory array
// (lanes never share a bank for T a multiple of 64), the row's swaps replayed
// from the top, the permutation written over the indices
__global__ void perm_shuffle_kernel(u64 rows, u64 d, u64 levels, u64 r_b, const u64 *bases, u64 b0, u64 width,
                                    u64 *out)
{
    extern __shared__ unsigned short col[];
    const u32 T = blockDim.x, t = threadIdx.x;
    const u64 q = (u64)blockIdx.x * T + t;
    if (q >= rows) return;
    const u64 lj = q / levels;
    const u64 bb = bases ? base_of(bases, r_b, d, lj / d, lj % d) : b0;
    if (bb > width) return;  // reported by the stream
    const u32 b = (u32)bb;
    u64 *row = out + q * width;
    unsigned short *A = col + t;
    for (u32 k = 0; k < b; k++) A[(u64)k * T] = (unsigned short)k;
    for (u32 k = b - 1; k >= 1 && b >= 2; k--) {
        const u32 jv = (u32)row[k];
        const unsigned short x = A[(u64)k * T], y = A[(u64)jv * T];
        A[(u64)k * T] = y;
        A[(u64)jv * T] = x;
    }
    for (u32 k = 0; k < b; k++) row[k] = A[(u64)k * T];
}

int one_thread(const char *what) { return qmcgb::launch_status(what); }

// the permutation rows: zero fill (the padding beyond each base), the stream,
// the shuffles
int permutations(u64 *state, u64 r, u64 d, u64 levels, u64 r_b, const u64 *bases, u64 b0, u64 bmax, u64 *out,
                 cudaStream_t st)
{
    const u64 rows = r * d * levels;
    if (rows == 0 || bmax == 0) return QMC_OK;
    QMC_REQUIRE(bmax <= 65536, "permutations on the GPU take bases up to 65536 (bmax = %llu)",
                (unsigned long long)bmax);
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    if (int rc = qmcgb::cuda_status(cudaMemsetAsync(out, 0, rows * bmax * 8, st), "permutation fill")) return rc;
    perm_stream_kernel<<<1, FY_THREADS, 0, st>>>(state, r, d, levels, r_b, bases, b0, bmax, out, err);
    if (int rc = one_thread("perm_stream_kernel")) return rc;
    u32 T = 128;
    while (T > 1 && (u64)T * bmax * 2 > 98304) T >>= 1;
    const size_t smem = (size_t)T * bmax * 2;
    if (int rc = qmcgb::raise_smem_limit((const void *)perm_shuffle_kernel, smem, "permutation smem")) return rc;
    perm_shuffle_kernel<<<(unsigned)((rows + T - 1) / T), T, smem, st>>>(rows, d, levels, r_b, bases, b0, bmax, out);
    return qmcgb::launch_status("perm_shuffle_kernel");
}

}  // namespace

extern "C" {

int qmc_lat_get_shifts(uint64_t *state, uint64_t r, uint64_t d, double *shifts, qmc_stream_t s)
{
    const u64 count = r * d;
    if (count == 0) return QMC_OK;
    QMC_REQUIRE(state && shifts, "lat_get_shifts: null state or output");
    rng_uniform_kernel<<<1, 32, 0, QMC_STREAM(s)>>>((u64 *)state, count, shifts);
    return one_thread("rng_uniform_kernel");
}

int qmc_random_tbit_uint64s(uint64_t *state, uint64_t t, uint64_t count, uint64_t *out, qmc_stream_t s)
{
    QMC_REQUIRE(t <= 64, "t must be between 0 and 64");
    if (count == 0) return QMC_OK;
    QMC_REQUIRE(state && out, "random_tbit_uint64s: null state or output");
    rng_tbits_kernel<<<1, 32, 0, QMC_STREAM(s)>>>((u64 *)state, (u32)t, count, (u64 *)out, 0, 0);
    return one_thread("rng_tbits_kernel");
}

int qmc_dnb2_get_digital_shifts(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax_new, uint64_t *shifts,
                                qmc_stream_t s)
{
    return qmc_random_tbit_uint64s(state, tmax_new, r * d, shifts, s);
}

int qmc_dnb2_get_linear_scramble_matrix(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax, uint64_t tmax_new,
                                        uint64_t *S, qmc_stream_t s)
{
    QMC_REQUIRE(tmax <= tmax_new && tmax >= 1 && tmax <= 64,
                "dnb2_get_linear_scramble_matrix: needs 1 <= tmax <= min(tmax_new, 64) (tmax = %llu, tmax_new = %llu)",
                (unsigned long long)tmax, (unsigned long long)tmax_new);
    const u64 count = r * d * tmax_new;
    if (count == 0) return QMC_OK;
    QMC_REQUIRE(state && S, "dnb2_get_linear_scramble_matrix: null state or output");
    rng_tbits_kernel<<<1, 32, 0, QMC_STREAM(s)>>>((u64 *)state, (u32)tmax, count, (u64 *)S, (u32)tmax, (u32)tmax_new);
    return one_thread("rng_tbits_kernel");
}

int qmc_gdn_get_linear_scramble_matrix(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax, uint64_t tmax_new,
                                       uint64_t r_b, const uint64_t *bases, uint64_t *S, qmc_stream_t s)
{
    QMC_REQUIRE(tmax <= tmax_new && tmax_new < (1ull << 31),
                "gdn_get_linear_scramble_matrix: needs tmax <= tmax_new (tmax = %llu, tmax_new = %llu)",
                (unsigned long long)tmax, (unsigned long long)tmax_new);
    const u64 count = r * d * tmax_new * tmax;
    if (count == 0) return QMC_OK;
    QMC_REQUIRE(state && S && bases && r_b >= 1, "gdn_get_linear_scramble_matrix: null state, bases or output");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    cudaStream_t st = QMC_STREAM(s);
    if (int rc = qmcgb::cuda_status(cudaMemsetAsync(S, 0, count * 8, st), "scramble matrix fill")) return rc;
    gdn_lms_rand_kernel<<<1, 32, 0, st>>>((u64 *)state, r, d, (u32)tmax, (u32)tmax_new, r_b, (const u64 *)bases,
                                          (u64 *)S, err);
    return one_thread("gdn_lms_rand_kernel");
}

int qmc_gdn_get_digital_shifts(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax_new, uint64_t r_b,
                               const uint64_t *bases, uint64_t *shifts, qmc_stream_t s)
{
    QMC_REQUIRE(tmax_new < (1ull << 31), "gdn_get_digital_shifts: tmax_new too large");
    if (r * d * tmax_new == 0) return QMC_OK;
    QMC_REQUIRE(state && shifts && bases && r_b >= 1, "gdn_get_digital_shifts: null state, bases or output");
    unsigned *err = qmcgb::device_error_ptr();
    QMC_REQUIRE(err, "device error word unavailable");
    gdn_shift_rand_kernel<<<1, 32, 0, QMC_STREAM(s)>>>((u64 *)state, r, d, (u32)tmax_new, r_b, (const u64 *)bases,
                                                       (u64 *)shifts, err);
    return one_thread("gdn_shift_rand_kernel");
}

int qmc_gdn_get_digital_permutations(uint64_t *state, uint64_t r, uint64_t d, uint64_t tmax_new, uint64_t r_b,
                                     const uint64_t *bases, uint64_t bmax, uint64_t *perms, qmc_stream_t s)
{
    if (r * d * tmax_new == 0) return QMC_OK;
    QMC_REQUIRE(state && perms && bases && r_b >= 1, "gdn_get_digital_permutations: null state, bases or output");
    return permutations((u64 *)state, r, d, tmax_new, r_b, (const u64 *)bases, 0, bmax, (u64 *)perms,
                        QMC_STREAM(s));
}

int qmc_random_uint64_permutations(uint64_t *state, uint64_t n, uint64_t b, uint64_t *out, qmc_stream_t s)
{
    if (n == 0 || b == 0) return QMC_OK;
    QMC_REQUIRE(state && out, "random_uint64_permutations: null state or output");
    return permutations((u64 *)state, 1, 1, n, 1, nullptr, b, b, (u64 *)out, QMC_STREAM(s));
}

}  // extern "C"
