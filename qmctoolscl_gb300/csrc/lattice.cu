// lattice.cu -- rank-1 lattice generation (linear, natural, Gray order) and
// the mod-1 shift, plus the fused generate+shift kernel used by the batched
// path.
//
// Reference: qmctoolscl/c_funcs/lat_gen_linear.c:3-33,
// lat_gen_natural.c:3-58, lat_gen_gray.c:3-56, lat_shift_mod_1.c:3-35.
//
// Closed form.  The reference walks a Gray-code recurrence; the value it
// writes is fmod((double)g * V, 1) with V = ldexp(v, -p), where for a row
// whose sequence index is m (m = n_start+k in natural order, the Gray code
// of n_start+i in Gray order), p = bitlen(m) and v = m bit-reversed in p
// bits -- i.e. V is the van der Corput radical inverse of m.  With
// B = bitreverse64(m), V = B * 2^-64 exactly.  When bitlen(g) + p <= 53 the
// double product g*V is exact, so fmod(g*V, 1) = (g*B mod 2^64) * 2^-64:
// one 64-bit integer multiply gives the fraction in 0.64 fixed point and
// fix64_to_double turns it into the double bit pattern.  Other columns take
// the FP64 instructions the reference's formula names (same rounding, slower
// on GB300).
//
// The mod-1 shift adds a double shift and drops the integer part.  When
// both operands are multiples of 2^-64 in [0,1) (lattice points are, and
// numpy's random() shifts are multiples of 2^-53) the rounded sum is done in
// 0.64 fixed point by add_mod1_fix64.
//
// Layout in HBM: x and xr are r*n*d doubles, d fastest.  A warp covers one
// row (or several short rows) with 16-byte stores when d is even and the
// output is 16-byte aligned, so each warp store is one contiguous span.
#include "common.cuh"

namespace {

enum LatOrder { ORDER_LINEAR_POW2 = 0, ORDER_LINEAR_GENERIC = 1, ORDER_NATURAL = 2, ORDER_GRAY = 3 };

struct LatArgs {
    u64 r, n, d, n_start;
    const u64 *g;          // r*d
    const double *shifts;  // r*d, only with SHIFT
    double *out;           // r*n*d
    u32 log2n;             // ORDER_LINEAR_POW2
    u32 pmax;              // bit length of the largest sequence index
};

// Per-column constants, prepared once per thread and column.
struct LatCol {
    u64 g;
    double gd;   // (double)g, RN as the reference converts it
    u64 S;       // shift in 0.64 fixed point
    double s;
    bool fast;   // exact integer generation
    u32 shift_kind;  // 0: 0.64 with 11 zero low bits, 1: 0.64, 2: FP64 add
};

__device__ __forceinline__ u64 row_index(int order, u64 n_start, u64 i)
{
    if (order == ORDER_GRAY) {
        const u64 k = n_start + i;
        return k ^ (k >> 1);
    }
    return n_start + i;
}

__device__ __forceinline__ LatCol load_col(const LatArgs &a, u64 l, u64 j, bool with_shift, int order)
{
    LatCol c;
    c.g = a.g[l * a.d + j];
    c.gd = __ull2double_rn(c.g);
    const u32 bits_g = 64 - __clzll((long long)c.g);
    const u32 p = (order == ORDER_LINEAR_POW2) ? a.log2n : a.pmax;
    c.fast = (order != ORDER_LINEAR_GENERIC) && (bits_g + p <= 53) && (p <= 53);
    c.S = 0;
    c.s = 0.0;
    c.shift_kind = 2;
    if (with_shift) {
        c.s = a.shifts[l * a.d + j];
        u64 S;
        if (double_to_fix64(c.s, &S)) {
            c.S = S;
            c.shift_kind = (S & 0x7FFull) ? 1u : 0u;
        }
    }
    return c;
}

// fmod(g*V, 1) as the reference computes it, for sequence index m, with
// FP64 instructions.  Kept out of line: GB300's FP64 pipe is slow, and if
// the compiler if-converted these fallbacks into the per-element loop their
// (predicated-off) FP64 instructions would still be issued for every
// coordinate and saturate that pipe.
__device__ __noinline__ double lat_value_hw(double gd, int order, u64 m, u64 i, u64 n)
{
    if (order == ORDER_LINEAR_POW2 || order == ORDER_LINEAR_GENERIC) {
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
__device__ __noinline__ double lat_point_general(const LatCol &c, int order, u64 B, u64 m, u64 i, u64 n,
                                                 bool shift)
{
    double x;
    if (c.fast) {
        const u64 W = c.g * B;
        if (!shift) return fix64_to_double(W);
        if (c.shift_kind == 1) return fix64_to_double(add_mod1_fix64(W, c.S));
        x = fix64_to_double(W);
    } else {
        x = lat_value_hw(c.gd, order, m, i, n);
        if (!shift) return x;
    }
    return frac_mod1(__dadd_rn(x, c.s));
}

template <bool SHIFT>
__device__ __forceinline__ double lat_point(const LatCol &c, int order, u64 B, u64 m, u64 i, u64 n)
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
    return lat_point_general(c, order, B, m, i, n, SHIFT);
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

// fmod(point + shift, 1) for the narrow case (every sequence index below
// 2^32, so B = bitreverse64(m) has a zero low word and the fraction
// g*B mod 2^64 is (g mod 2^32) * bitreverse32(m) in the high word); the shift
// is a multiple of 2^-53 in 0.64 fixed point (sh:sl).
template <bool SHIFT>
__device__ __forceinline__ double lat_point_narrow(u32 g_lo, u32 bh, u32 sh, u32 sl, const LatCol &c, int order,
                                                   u64 m, u64 i, u64 n)
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

template <int ORDER, bool SHIFT, int VEC>
__global__ void __launch_bounds__(256) lat_gen_narrow_kernel(LatArgs a)
{
    // every index n_start + i < 2^32 and every column on the exact integer
    // path with (for SHIFT) a shift on the 2^-53 grid: checked per column,
    // with the general per-element code for columns that are not
    const u32 ngroups = (u32)((a.d + VEC - 1) / VEC);
    const u32 row_stride = gridDim.x * blockDim.y;
    const u32 n = (u32)a.n, n_start = (u32)a.n_start;
    for (u64 l = blockIdx.y; l < a.r; l += gridDim.y) {
        for (u32 jg = threadIdx.x; jg < ngroups; jg += blockDim.x) {
            const u64 j0 = (u64)jg * VEC;
            LatCol c[VEC];
            bool easy = true;
#pragma unroll
            for (int v = 0; v < VEC; v++) {
                c[v] = load_col(a, l, j0 + v, SHIFT, ORDER);
                easy &= c[v].fast && (!SHIFT || c[v].shift_kind == 0);
            }
            u32 g_lo[VEC], sh[VEC], sl[VEC];
#pragma unroll
            for (int v = 0; v < VEC; v++) {
                g_lo[v] = (u32)c[v].g;
                sh[v] = (u32)(c[v].S >> 32);
                sl[v] = (u32)c[v].S;
            }
            double *out = a.out + l * a.n * a.d + j0;
            for (u32 i = blockIdx.x * blockDim.y + threadIdx.y; i < n; i += row_stride) {
                u32 bh, m32;
                if (ORDER == ORDER_LINEAR_POW2) {
                    m32 = i;
                    bh = a.log2n ? (i << (32 - a.log2n)) : 0u;  // log2n <= 32 here
                } else {
                    const u32 k = n_start + i;
                    m32 = (ORDER == ORDER_GRAY) ? (k ^ (k >> 1)) : k;
                    bh = __brev(m32);
                }
                double y[VEC];
                if (easy) {
#pragma unroll
                    for (int v = 0; v < VEC; v++)
                        y[v] = lat_point_narrow<SHIFT>(g_lo[v], bh, sh[v], sl[v], c[v], ORDER, m32, i, a.n);
                } else {
#pragma unroll
                    for (int v = 0; v < VEC; v++)
                        y[v] = lat_point_general(c[v], ORDER, (u64)bh << 32, m32, i, a.n, SHIFT);
                }
                if (VEC == 2) {
                    __stcs((double2 *)(out + (u64)i * a.d), make_double2(y[0], y[1]));
                } else {
                    __stcs(out + (u64)i * a.d, y[0]);
                }
            }
        }
    }
}

template <int ORDER, bool SHIFT, int VEC>
__global__ void __launch_bounds__(256) lat_gen_kernel(LatArgs a)
{
    const u64 ngroups = (a.d + VEC - 1) / VEC;
    const u64 row_stride = (u64)gridDim.x * blockDim.y;
    for (u64 l = blockIdx.y; l < a.r; l += gridDim.y) {
        for (u64 jg = threadIdx.x; jg < ngroups; jg += blockDim.x) {
            const u64 j0 = jg * VEC;
            LatCol c[VEC];
#pragma unroll
            for (int v = 0; v < VEC; v++) c[v] = load_col(a, l, j0 + v, SHIFT, ORDER);
            double *out = a.out + l * a.n * a.d + j0;
            for (u64 i = (u64)blockIdx.x * blockDim.y + threadIdx.y; i < a.n; i += row_stride) {
                const u64 m = row_index(ORDER, a.n_start, i);
                u64 B;
                if (ORDER == ORDER_LINEAR_POW2)
                    B = a.log2n ? (i << (64 - a.log2n)) : 0;
                else
                    B = __brevll(m);
                double y[VEC];
#pragma unroll
                for (int v = 0; v < VEC; v++) y[v] = lat_point<SHIFT>(c[v], ORDER, B, m, i, a.n);
                if (VEC == 2) {
                    __stcs((double2 *)(out + i * a.d), make_double2(y[0], y[1]));
                } else {
                    __stcs(out + i * a.d, y[0]);
                }
            }
        }
    }
}

struct ShiftArgs {
    u64 r, n, d, r_x;
    const double *x;
    const double *shifts;
    double *xr;
};

__device__ __noinline__ double shift_one_hw(double x, double s) { return frac_mod1(__dadd_rn(x, s)); }

__device__ __forceinline__ double shift_one(double x, u64 S, bool s_ok, double s)
{
    u64 X;
    if (s_ok && double_to_fix64(x, &X)) return fix64_to_double(add_mod1_fix64(X, S));
    return shift_one_hw(x, s);
}

template <int VEC>
__global__ void __launch_bounds__(256) lat_shift_kernel(ShiftArgs a)
{
    const u64 ngroups = (a.d + VEC - 1) / VEC;
    const u64 row_stride = (u64)gridDim.x * blockDim.y;
    for (u64 l = blockIdx.y; l < a.r; l += gridDim.y) {
        for (u64 jg = threadIdx.x; jg < ngroups; jg += blockDim.x) {
            const u64 j0 = jg * VEC;
            double s[VEC];
            u64 S[VEC];
            bool ok[VEC];
#pragma unroll
            for (int v = 0; v < VEC; v++) {
                s[v] = a.shifts[l * a.d + j0 + v];
                ok[v] = double_to_fix64(s[v], &S[v]);
            }
            const double *xin = a.x + (l % a.r_x) * a.n * a.d + j0;
            double *out = a.xr + l * a.n * a.d + j0;
            for (u64 i = (u64)blockIdx.x * blockDim.y + threadIdx.y; i < a.n; i += row_stride) {
                if (VEC == 2) {
                    const double2 xv = __ldcs((const double2 *)(xin + i * a.d));
                    __stcs((double2 *)(out + i * a.d),
                           make_double2(shift_one(xv.x, S[0], ok[0], s[0]), shift_one(xv.y, S[1], ok[1], s[1])));
                } else {
                    __stcs(out + i * a.d, shift_one(__ldcs(xin + i * a.d), S[0], ok[0], s[0]));
                }
            }
        }
    }
}

// Block shape: threadIdx.x over column groups (a warp spans whole rows when
// they are short), threadIdx.y over rows.  Grid: x over row blocks, capped
// so that every thread loops over many rows; y over randomisations.
struct Shape {
    dim3 grid, block;
};

Shape shape_for(u64 r, u64 n, u64 ngroups)
{
    u32 bx = 1;
    while (bx < ngroups && bx < 32) bx <<= 1;
    const u32 by = 256 / bx;
    const u64 want_ctas = (u64)qmcgb::sm_count() * 16;
    u64 per_l = want_ctas / (r ? r : 1);
    if (per_l < 1) per_l = 1;
    u64 gx = (n + by - 1) / by;
    if (gx > per_l) gx = per_l;
    if (gx < 1) gx = 1;
    if (gx > 0x7FFFFFFFull) gx = 0x7FFFFFFFull;
    const u64 gy = r < 65535 ? (r ? r : 1) : 65535;
    Shape s;
    s.grid = dim3((unsigned)gx, (unsigned)gy, 1);
    s.block = dim3(bx, by, 1);
    return s;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

u32 bitlen(u64 v) { return v ? 64u - (u32)__builtin_clzll(v) : 0u; }

template <int ORDER, bool SHIFT>
int launch_gen(const LatArgs &a, cudaStream_t s, const char *what)
{
    const bool vec2 = (a.d % 2 == 0) && aligned16(a.out);
    const u64 ngroups = vec2 ? a.d / 2 : a.d;
    const Shape sh = shape_for(a.r, a.n, ngroups);
    // 32-bit indexing: every sequence index below 2^32
    const bool narrow = ORDER != ORDER_LINEAR_GENERIC && a.n_start + a.n <= (1ull << 32) &&
                        a.n_start + a.n >= a.n_start && (ORDER != ORDER_LINEAR_POW2 || a.log2n <= 32);
    if (narrow) {
        if (vec2)
            lat_gen_narrow_kernel<ORDER, SHIFT, 2><<<sh.grid, sh.block, 0, s>>>(a);
        else
            lat_gen_narrow_kernel<ORDER, SHIFT, 1><<<sh.grid, sh.block, 0, s>>>(a);
    } else if (vec2) {
        lat_gen_kernel<ORDER, SHIFT, 2><<<sh.grid, sh.block, 0, s>>>(a);
    } else {
        lat_gen_kernel<ORDER, SHIFT, 1><<<sh.grid, sh.block, 0, s>>>(a);
    }
    return qmcgb::launch_status(what);
}

int check_common(u64 r, u64 n, u64 d, const void *in, const void *out)
{
    QMC_REQUIRE(r == 0 || n == 0 || d == 0 || (in && out), "null array pointer");
    return QMC_OK;
}

}  // namespace

namespace qmcgb {

// Fused generate+shift over one randomisation batch (used by the batched
// plan and by qmc_lat_gen_shift): xr[l,i,j] = fmod(point(l,i,j) + shifts[l,j], 1)
// with the point in natural or Gray order.
int lat_gen_shift(u64 r, u64 n, u64 d, u64 n_start, int gray, const u64 *g, const double *shifts,
                  double *xr, cudaStream_t s)
{
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    LatArgs a{r, n, d, n_start, g, shifts, xr, 0, bitlen(n_start + n - 1)};
    return gray ? launch_gen<ORDER_GRAY, true>(a, s, "lat_gen_shift")
                : launch_gen<ORDER_NATURAL, true>(a, s, "lat_gen_shift");
}

}  // namespace qmcgb

extern "C" {

int qmc_lat_gen_linear(uint64_t r, uint64_t n, uint64_t d, const uint64_t *g, double *x, qmc_stream_t s)
{
    if (int rc = check_common(r, n, d, g, x)) return rc;
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    const bool pow2 = (n & (n - 1)) == 0;
    LatArgs a{r, n, d, 0, (const u64 *)g, nullptr, x, pow2 ? bitlen(n) - 1 : 0, 0};
    return pow2 ? launch_gen<ORDER_LINEAR_POW2, false>(a, QMC_STREAM(s), "lat_gen_linear")
                : launch_gen<ORDER_LINEAR_GENERIC, false>(a, QMC_STREAM(s), "lat_gen_linear");
}

int qmc_lat_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, const uint64_t *g,
                        double *x, qmc_stream_t s)
{
    QMC_REQUIRE((n_start & (n_start - 1)) == 0 && ((n + n_start) & (n + n_start - 1)) == 0,
                "lat_gen_natural requires n_start and n+n_start are either 0 or powers of 2");
    if (int rc = check_common(r, n, d, g, x)) return rc;
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    LatArgs a{r, n, d, n_start, (const u64 *)g, nullptr, x, 0, bitlen(n_start + n - 1)};
    return launch_gen<ORDER_NATURAL, false>(a, QMC_STREAM(s), "lat_gen_natural");
}

int qmc_lat_gen_gray(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, const uint64_t *g,
                     double *x, qmc_stream_t s)
{
    if (int rc = check_common(r, n, d, g, x)) return rc;
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    LatArgs a{r, n, d, n_start, (const u64 *)g, nullptr, x, 0, bitlen(n_start + n - 1)};
    return launch_gen<ORDER_GRAY, false>(a, QMC_STREAM(s), "lat_gen_gray");
}

int qmc_lat_shift_mod_1(uint64_t r, uint64_t n, uint64_t d, uint64_t r_x, const double *x,
                        const double *shifts, double *xr, qmc_stream_t s)
{
    if (int rc = check_common(r, n, d, x, xr)) return rc;
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    QMC_REQUIRE(r_x > 0 && shifts, "lat_shift_mod_1 needs r_x > 0 and a shifts array");
    ShiftArgs a{r, n, d, r_x, x, shifts, xr};
    const bool vec2 = (d % 2 == 0) && aligned16(x) && aligned16(xr);
    const u64 ngroups = vec2 ? d / 2 : d;
    const Shape sh = shape_for(r, n, ngroups);
    if (vec2)
        lat_shift_kernel<2><<<sh.grid, sh.block, 0, QMC_STREAM(s)>>>(a);
    else
        lat_shift_kernel<1><<<sh.grid, sh.block, 0, QMC_STREAM(s)>>>(a);
    return qmcgb::launch_status("lat_shift_mod_1");
}

// Fused lattice generation (natural: gray=0, Gray: gray=1) and mod-1 shift:
// the output of lat_gen_{natural,gray} followed by lat_shift_mod_1 with
// r_x = r, in one pass that writes only xr.
int qmc_lat_gen_shift(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, int gray,
                      const uint64_t *g, const double *shifts, double *xr, qmc_stream_t s)
{
    if (int rc = check_common(r, n, d, g, xr)) return rc;
    QMC_REQUIRE(r == 0 || n == 0 || d == 0 || shifts, "null shifts pointer");
    if (!gray)
        QMC_REQUIRE((n_start & (n_start - 1)) == 0 && ((n + n_start) & (n + n_start - 1)) == 0,
                    "lat_gen_natural requires n_start and n+n_start are either 0 or powers of 2");
    return qmcgb::lat_gen_shift(r, n, d, n_start, gray, (const u64 *)g, shifts, xr, QMC_STREAM(s));
}

}  // extern "C"
