// lattice.cu -- rank-1 lattice generation (linear, natural, Gray order) and
// the mod-1 shift, plus the fused generate+shift kernel used by the batched
// path.
//
// Reference: qmctoolscl/c_funcs/lat_gen_linear.c:3-33,
// lat_gen_natural.c:3-58, lat_gen_gray.c:3-56, lat_shift_mod_1.c:3-35.
//
// The per-point arithmetic (closed form of the reference's recurrence,
// exact integer emulation of its FP64 roundings) is in lattice_dev.cuh.
//
// The mod-1 shift adds a double shift and drops the integer part.  When
// both operands are multiples of 2^-64 in [0,1) (lattice points are, and
// numpy's random() shifts are multiples of 2^-53) the rounded sum is done in
// 0.64 fixed point by add_mod1_fix64.
//
// Layout in HBM: x and xr are r*n*d doubles, d fastest.  A warp covers one
// row (or several short rows) with 16-byte stores when d is even and the
// output is 16-byte aligned, so each warp store is one contiguous span.
#include "lattice_dev.cuh"

namespace {

using lat::bitlen;

struct LatArgs {
    u64 r, n, d, n_start;
    const u64 *g;          // r*d
    const double *shifts;  // r*d, only with SHIFT
    double *out;           // r*n*d
    u32 p;                 // bit length of the largest sequence index (log2 n for linear order)
    bool narrow;           // every sequence index below 2^32
};

// threadIdx.x over column groups, threadIdx.y over rows; grid x over row
// blocks, y over randomisations
template <int ORDER, bool SHIFT, int VEC>
__global__ void __launch_bounds__(256) lat_gen_kernel(LatArgs a)
{
    const u64 ngroups = (a.d + VEC - 1) / VEC;
    const u64 row_stride = (u64)gridDim.x * blockDim.y;
    for (u64 l = blockIdx.y; l < a.r; l += gridDim.y)
        for (u64 jg = threadIdx.x; jg < ngroups; jg += blockDim.x)
            lat::rows<ORDER, SHIFT, VEC>(a.g + l * a.d, SHIFT ? a.shifts + l * a.d : nullptr, a.out + l * a.n * a.d,
                                         a.d, a.n, a.n_start, a.p, jg, (u64)blockIdx.x * blockDim.y + threadIdx.y,
                                         a.n, row_stride, a.narrow);
}

struct ShiftArgs {
    u64 r, n, d, r_x;
    const double *x;
    const double *shifts;
    double *xr;
};

__device__ __noinline__ double shift_one_hw(double x, double s) { return frac_mod1(__dadd_rn(x, s)); }

__device__ __noinline__ double shift_one_fix64(double x, u64 S, bool s_ok, double s)
{
    u64 X;
    if (s_ok && double_to_fix64(x, &X)) return fix64_to_double(add_mod1_fix64(X, S));
    return shift_one_hw(x, s);
}

// fmod(RN(x + s), 1) when s is on the 2^-53 grid in [0,1) (K = s*2^53, as
// numpy's random() draws) and x is too (lattice points with up to 2^53
// points are): F = x*2^53 is then an integer, the sum F+K needs rounding only
// when it reaches 2^53 (spacing 2 there, ties to even), and the result is
// exact.  Other inputs take the general 0.64 fixed-point or FP64 path.
__device__ __forceinline__ double shift_one(double x, u64 K, bool k_ok, u64 S, bool s_ok, double s)
{
    const u64 b = as_bits(x);
    const u32 E = (u32)(b >> 52);  // sign bit included: negatives fail
    const u32 sh = 1022u - E;      // x = M * 2^(E-1075) = (M >> sh) * 2^-53
    const u64 M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    if (k_ok && E <= 1022u && sh <= 52u && (M & ((1ull << sh) - 1)) == 0) {
        u64 T = (M >> sh) + K;
        if (T >> 53) {  // sum in [1, 2): round to even on bit 0, drop the 1
            T += (T & 1) & (T >> 1);
            T = (T & ~1ull) - (1ull << 53);
            T &= (1ull << 53) - 1;  // a sum that rounded up to 2 leaves 0
        }
        return T ? fix64_to_double(T << 11) : 0.0;
    }
    if (b == 0 && k_ok) return s;  // x = +0: the sum is s itself
    return shift_one_fix64(x, S, s_ok, s);
}

// Rows per thread per iteration: all loads of a group are issued before
// any arithmetic, so each thread keeps ROWS_IN_FLIGHT loads outstanding (the
// bytes in flight per SM that a streaming kernel needs to reach HBM speed).
constexpr int ROWS_IN_FLIGHT = 4;

template <int VEC>
__global__ void __launch_bounds__(256) lat_shift_kernel(ShiftArgs a)
{
    typedef typename std::conditional<VEC == 2, double2, double>::type vec_t;
    const u64 ngroups = (a.d + VEC - 1) / VEC;
    const u64 row_stride = (u64)gridDim.x * blockDim.y;
    for (u64 l = blockIdx.y; l < a.r; l += gridDim.y) {
        for (u64 jg = threadIdx.x; jg < ngroups; jg += blockDim.x) {
            const u64 j0 = jg * VEC;
            double s[VEC];
            u64 S[VEC], K[VEC];
            bool ok[VEC], kok[VEC];
#pragma unroll
            for (int v = 0; v < VEC; v++) {
                s[v] = a.shifts[l * a.d + j0 + v];
                ok[v] = double_to_fix64(s[v], &S[v]);
                kok[v] = ok[v] && (S[v] & 0x7FFull) == 0;
                K[v] = S[v] >> 11;
            }
            const vec_t *xin = (const vec_t *)(a.x + (l % a.r_x) * a.n * a.d + j0);
            vec_t *out = (vec_t *)(a.xr + l * a.n * a.d + j0);
            const u64 dv = a.d / VEC;  // row pitch in vec_t units (d % VEC == 0 when VEC == 2)
            for (u64 i0 = (u64)blockIdx.x * blockDim.y + threadIdx.y; i0 < a.n; i0 += ROWS_IN_FLIGHT * row_stride) {
                vec_t xv[ROWS_IN_FLIGHT];
#pragma unroll
                for (int u = 0; u < ROWS_IN_FLIGHT; u++) {
                    const u64 i = i0 + u * row_stride;
                    if (i < a.n) xv[u] = __ldcs(xin + i * dv);
                }
#pragma unroll
                for (int u = 0; u < ROWS_IN_FLIGHT; u++) {
                    const u64 i = i0 + u * row_stride;
                    if (i >= a.n) break;
                    vec_t y;
                    if constexpr (VEC == 2) {
                        y = make_double2(shift_one(xv[u].x, K[0], kok[0], S[0], ok[0], s[0]),
                                         shift_one(xv[u].y, K[1], kok[1], S[1], ok[1], s[1]));
                    } else {
                        y = shift_one(xv[u], K[0], kok[0], S[0], ok[0], s[0]);
                    }
                    __stcs(out + i * dv, y);
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

template <int ORDER, bool SHIFT>
int launch_gen(LatArgs a, cudaStream_t s, const char *what)
{
    const bool vec2 = (a.d % 2 == 0) && aligned16(a.out);
    const u64 ngroups = vec2 ? a.d / 2 : a.d;
    const Shape sh = shape_for(a.r, a.n, ngroups);
    a.narrow = ORDER != lat::LINEAR_GENERIC && a.n_start + a.n <= (1ull << 32) && a.n_start + a.n >= a.n_start &&
               a.p <= 32;
    if (vec2)
        lat_gen_kernel<ORDER, SHIFT, 2><<<sh.grid, sh.block, 0, s>>>(a);
    else
        lat_gen_kernel<ORDER, SHIFT, 1><<<sh.grid, sh.block, 0, s>>>(a);
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
    LatArgs a{r, n, d, n_start, g, shifts, xr, bitlen(n_start + n - 1), false};
    return gray ? launch_gen<lat::GRAY, true>(a, s, "lat_gen_shift")
                : launch_gen<lat::NATURAL, true>(a, s, "lat_gen_shift");
}

}  // namespace qmcgb

extern "C" {

int qmc_lat_gen_linear(uint64_t r, uint64_t n, uint64_t d, const uint64_t *g, double *x, qmc_stream_t s)
{
    if (int rc = check_common(r, n, d, g, x)) return rc;
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    const bool pow2 = (n & (n - 1)) == 0;
    LatArgs a{r, n, d, 0, (const u64 *)g, nullptr, x, pow2 ? bitlen(n) - 1 : 64, false};
    return pow2 ? launch_gen<lat::LINEAR_POW2, false>(a, QMC_STREAM(s), "lat_gen_linear")
                : launch_gen<lat::LINEAR_GENERIC, false>(a, QMC_STREAM(s), "lat_gen_linear");
}

int qmc_lat_gen_natural(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, const uint64_t *g,
                        double *x, qmc_stream_t s)
{
    QMC_REQUIRE((n_start & (n_start - 1)) == 0 && ((n + n_start) & (n + n_start - 1)) == 0,
                "lat_gen_natural requires n_start and n+n_start are either 0 or powers of 2");
    if (int rc = check_common(r, n, d, g, x)) return rc;
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    LatArgs a{r, n, d, n_start, (const u64 *)g, nullptr, x, bitlen(n_start + n - 1), false};
    return launch_gen<lat::NATURAL, false>(a, QMC_STREAM(s), "lat_gen_natural");
}

int qmc_lat_gen_gray(uint64_t r, uint64_t n, uint64_t d, uint64_t n_start, const uint64_t *g,
                     double *x, qmc_stream_t s)
{
    if (int rc = check_common(r, n, d, g, x)) return rc;
    if (r == 0 || n == 0 || d == 0) return QMC_OK;
    LatArgs a{r, n, d, n_start, (const u64 *)g, nullptr, x, bitlen(n_start + n - 1), false};
    return launch_gen<lat::GRAY, false>(a, QMC_STREAM(s), "lat_gen_gray");
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
